"""Device-generated initial conditions against the oracle's, and the
mixed-precision form (FP32 fields and FFTs, FP64 positions, int64 fixed-point
deposits) against the FP64 form."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


# The modes take the reference's float logarithm of the uniform draw r1 (log of a
# float is <cmath>'s float overload).  The device rounds the FP64 log to float, the
# C library computes logf: on rare draws the two differ by one unit in the last
# place, 3e-8 of that mode's amplitude, and the kernel spectrum comes from two
# different FFTs (1e-16).  Positions then agree to ~1e-11 cell, fields to ~1e-10;
# B, the transverse remainder of the momentum deposit, cancels most of it and
# magnifies the difference a hundredfold.
TOL_IC_POS, TOL_IC_REL, TOL_IC_B = 1e-10, 1e-9, 1e-8


@pytest.mark.parametrize("N", [16, 32])
def test_device_ic_matches_oracle(gpu, oracle, N):
    """The device IC against the oracle's (whose displacement field, CIC kernel and
    random stream are bit-identical to the reference's own, tests/test_oracle_golden.py)."""
    L = 5.0 * N
    o = oracle.Sim(N).ic(**oracle.default_icparams(N, L, seed=21))
    ctx = gpu.Context(N)
    s = gpu.Sim(ctx, N ** 3)
    s.ic_generate(**gpu.ic_params(L, seed=21))
    st = s.state()
    for k in ("a", "dtau", "fourpiG", "mass"):
        assert abs(st[k] - o.scalars()[k]) <= 1e-14 * abs(o.scalars()[k]), k
    assert abs(st["tau"] - o.s.tau) <= 1e-12 * o.s.tau
    got = s.particles().download()
    ref = o.particles
    assert (got["ID"] == ref["ID"]).all()
    assert np.abs(got["pos"] - ref["pos"]).max() * N < TOL_IC_POS
    assert rel(got["vel"], ref["vel"]) < TOL_IC_REL
    for name in ("phi", "chi"):
        assert rel(s.field(name).download(), o.field(name)) < TOL_IC_REL, name
    assert rel(s.field("Bi").download(), o.field("Bi")) < TOL_IC_B
    assert rel(s.field("BiFT").download(), o.spectrum("BiFT")) < TOL_IC_B


@pytest.mark.parametrize("N", [16, 32, 48])
def test_mixed_operators_against_fp64(gpu, oracle, N):
    rng = np.random.default_rng(7 + N)
    c64, c32 = gpu.Context(N, gpu.PREC_FP64), gpu.Context(N, gpu.PREC_MIXED)
    x = rng.standard_normal((6, N, N, N))
    out = {}
    for c in (c64, c32):
        r = c.real(6).upload(x)
        sp = c.spectrum(6)
        gpu.fft_r2c(r, sp)
        one = c.spectrum(1)
        gpu.project_scalar(sp, one, 0)
        back = c.real(1)
        gpu.fft_c2r(one, back)
        out[c.precision] = (sp.download(), back.download())
    assert rel(out[1][0], out[0][0]) < 1e-5
    assert rel(out[1][1], out[0][1]) < 1e-4


@pytest.mark.parametrize("N", [16, 32])
def test_mixed_deposits_reproducible_and_close(gpu, oracle, N):
    rng = np.random.default_rng(3 * N)
    n = N ** 3
    p = np.zeros(n, oracle.PART)
    p["pos"] = rng.random((n, 3))
    p["pos"][:300] = 0.25 + rng.random((300, 3)) * (0.4 / N)  # a dense clump
    p["vel"] = rng.standard_normal((n, 3)) * 1e-3
    p["ID"] = np.arange(n)
    phi_h = rng.standard_normal((1, N, N, N)) * 1e-5
    res = {}
    for prec in (gpu.PREC_FP64, gpu.PREC_MIXED):
        c = gpu.Context(N, prec)
        pc = c.particles(n, 1.0 / n).upload(p)
        phi = c.real(1).upload(phi_h)
        fs = []
        for _ in range(2):
            T = c.real(6)
            gpu.projection_Tij(pc, T, 0.05, phi)
            f0 = c.real(1)
            gpu.projection_T00(pc, f0, 0.05, phi)
            fs.append((f0.download(), T.download()))
        assert np.array_equal(fs[0][0], fs[1][0]) and np.array_equal(fs[0][1], fs[1][1])
        res[prec] = fs[0]
    assert rel(res[1][0], res[0][0]) < 1e-6
    assert rel(res[1][1], res[0][1]) < 1e-5


@pytest.mark.parametrize("qscale", [1e-8, 1e-6, 1e-2])
def test_mixed_deposit_scale_follows_momenta(gpu, oracle, qscale):
    """The fixed-point scale comes from the particles' largest |q| and the fullest
    cell: with the momenta of a high-redshift start (|q| ~ 1e-6) and with large
    ones, every component of T0i and Tij (which carry q and q^2) stays at FP32
    accuracy against the FP64 form, in rms and per cell."""
    N = 32
    rng = np.random.default_rng(17)
    n = N ** 3
    p = np.zeros(n, oracle.PART)
    p["pos"] = rng.random((n, 3))
    p["pos"][:500] = 0.5 + rng.random((500, 3)) * (0.5 / N)  # one crowded cell region
    p["vel"] = rng.standard_normal((n, 3)) * qscale
    p["ID"] = np.arange(n)
    phi_h = rng.standard_normal((1, N, N, N)) * 1e-5
    res = {}
    for prec in (gpu.PREC_FP64, gpu.PREC_MIXED):
        c = gpu.Context(N, prec)
        pc = c.particles(n, 1.0 / n).upload(p)
        phi = c.real(1).upload(phi_h)
        T = c.real(6)
        gpu.projection_Tij(pc, T, 0.02, phi)
        B = c.real(3)
        gpu.projection_T0i(pc, B, phi)
        res[prec] = (T.download(), B.download())
    for k in range(2):
        got, ref = res[gpu.PREC_MIXED][k], res[gpu.PREC_FP64][k]
        for comp in range(ref.shape[0]):
            d, r = got[comp] - ref[comp], ref[comp]
            assert np.sqrt((d ** 2).mean() / (r ** 2).mean()) < 1e-6, (k, comp)
            assert np.abs(d).max() <= 1e-5 * np.abs(r).max(), (k, comp)


def test_mixed_cycles_track_fp64(gpu, oracle):
    """A few cycles from the same device IC: mixed positions stay within 1e-4 of a cell."""
    N = 32
    sims = {}
    for prec in (gpu.PREC_FP64, gpu.PREC_MIXED):
        c = gpu.Context(N, prec)
        s = gpu.Sim(c, N ** 3)
        s.ic_generate(**gpu.ic_params(160.0, seed=4))
        for _ in range(8):
            s.step()
        sims[prec] = (c, s, s.particles().download())
    a, b = sims[0][2], sims[1][2]
    order_a, order_b = np.argsort(a["ID"]), np.argsort(b["ID"])
    d = (a["pos"][order_a] - b["pos"][order_b] + 0.5) % 1.0 - 0.5
    assert np.abs(d).max() * N < 1e-4


@pytest.mark.parametrize("prec", [0, 1])
def test_fused_entry_points_match_separate_calls(gpu, oracle, prec):
    """gev_projection_T00_Tij equals projection_init + T00 and projection_init + Tij, and
    gev_update_q_pos equals update_q followed by update_pos (downloaded in (cell, ID)
    order), bit for bit in both forms."""
    N = 16
    rng = np.random.default_rng(23)
    n = N ** 3
    p = np.zeros(n, oracle.PART)
    p["pos"] = rng.random((n, 3))
    p["vel"] = rng.standard_normal((n, 3)) * 1e-4
    p["ID"] = rng.permutation(n)
    fields = [rng.standard_normal((c, N, N, N)) * 1e-5 for c in (1, 1, 3)]
    out = []
    for fused in (True, False):
        c = gpu.Context(N, prec)
        pc = c.particles(n, 1.0 / n).upload(p)
        phi, chi, Bi = (c.real(f.shape[0]).upload(f) for f in fields)
        T00, Tij = c.real(1), c.real(6)
        T00.upload(np.full((1, N, N, N), 7.0))  # replaced, not accumulated into
        Tij.upload(np.full((6, N, N, N), 7.0))
        if fused:
            gpu.projection_T00_Tij(pc, T00, Tij, 0.03, phi)
            mv = gpu.update_q_pos(pc, 2e-3, 0.03, 3, 2e-3, 0.031, 3, phi, chi, Bi)
        else:
            T00.zero()
            Tij.zero()
            gpu.projection_T00(pc, T00, 0.03, phi)
            gpu.projection_Tij(pc, Tij, 0.03, phi)
            mv = gpu.update_q(pc, 0, 2e-3, phi, chi, Bi, 3, 0.03, 0.03 * 0.03 * N)
            gpu.update_pos(pc, 0, 2e-3, phi, chi, Bi, 3, 0.031, 0.031 * 0.031 * N)
        first = (T00.download(), Tij.download())
        # a deposit from the moved store: its cell keys and in-cell offsets (the fused
        # path splits the offsets from the positions again as it moves them)
        gpu.projection_T00_Tij(pc, T00, Tij, 0.031, phi)
        out.append(first + (mv, pc.download(), T00.download(), Tij.download()))
    a, b = out
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert a[2] == b[2]
    assert np.array_equal(a[3]["ID"], b[3]["ID"])
    assert np.array_equal(a[3]["pos"], b[3]["pos"]) and np.array_equal(a[3]["vel"], b[3]["vel"])
    assert np.array_equal(a[4], b[4]) and np.array_equal(a[5], b[5])


@pytest.mark.parametrize("prec", [0, 1])
def test_particle_store_returns_its_bytes(gpu, oracle, prec):
    """A particle store gives back every device byte it counted, including the
    deposit's prefactor scratch that it allocates on first use.  The context's own
    deposit scratch stays (it is sized by the grid), so the count is compared after
    a first store has come and gone."""
    import gc
    N = 16
    c = gpu.Context(N, prec)
    phi = c.real(1).zero()
    T00, Tij = c.real(1), c.real(6)
    rng = np.random.default_rng(3)
    p = np.zeros(N ** 3, oracle.PART)
    p["pos"] = rng.random((N ** 3, 3))
    p["vel"] = rng.standard_normal((N ** 3, 3)) * 1e-3
    p["ID"] = np.arange(N ** 3)

    def one_store():
        pc = c.particles(N ** 3, 1.0 / N ** 3).upload(p)
        gpu.projection_T00_Tij(pc, T00, Tij, 0.02, phi)
        c.sync()
        held = c.bytes_in_use()
        del pc
        gc.collect()
        return held

    one_store()
    base = c.bytes_in_use()
    held = one_store()
    assert held >= base + N ** 3 * 56
    assert c.bytes_in_use() == base


@pytest.mark.parametrize("N", [12, 16, 32])
def test_clustered_deposits(gpu, oracle, N):
    """Mixed-form T00, Tij and T00+Tij gathers on clustered particles (clumps from a few
    hundred particles in one cell down to a few, at the periodic edges too, beside empty
    cells): the fused deposit gives the same bits as the two separate ones, and both
    follow the FP64 restatement within the form's rounding (the fixed-point scale is
    set by the fullest cell)."""
    rng = np.random.default_rng(N)
    n = 4 * N ** 3
    p = np.zeros(n, gpu.PART)
    p["pos"] = rng.random((n, 3))
    k = 0
    for centre, count, spread in (((0.5, 0.5, 0.5), 600, 0.4), ((0.0, 0.0, 0.0), 300, 0.9), ((0.99, 0.2, 0.7), 40, 2.0),
                                  ((0.3, 0.999, 0.001), 12, 1.0), ((0.7, 0.6, 0.1), 9, 0.5)):
        pts = (np.array(centre) + (rng.random((count, 3)) - 0.5) * spread / N) % 1.0
        p["pos"][k:k + count] = pts
        k += count
    p["vel"] = rng.standard_normal((n, 3)) * 1e-3
    p["ID"] = rng.permutation(n)
    phi_h = rng.standard_normal((1, N, N, N)) * 1e-5
    ctx = gpu.Context(N, gpu.PREC_MIXED)
    pc = ctx.particles(n, 2e-4).upload(p)
    phi = ctx.real(1).upload(phi_h)
    f1, f6, g1, g6 = ctx.real(1), ctx.real(6), ctx.real(1), ctx.real(6)
    gpu.projection_T00(pc, f1, 0.03, phi)
    gpu.projection_Tij(pc, f6, 0.03, phi)
    gpu.projection_T00_Tij(pc, g1, g6, 0.03, phi)
    assert f1.download().tobytes() == g1.download().tobytes()
    assert f6.download().tobytes() == g6.download().tobytes()
    for which, got in (("T00", f1.download()), ("Tij", f6.download())):
        ref = oracle.deposit(which, N, p, 2e-4, 0.03, phi_h, 1.0)
        assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max(), which


def test_dense_cells_beyond_the_slots_are_walked(gpu, oracle):
    """A store holds one dense-cell slot for 64 particles (at least 1024): with many
    cells above the dense threshold most of them get no slot and are walked.  The same
    particles in a store with room for every dense cell give the same bits (integer
    sums do not depend on which cells are summed apart), and both follow the FP64
    restatement within the form's rounding."""
    N = 64
    rng = np.random.default_rng(7)
    # 16,000 cells of 12 particles (small dense cells) and 2,000 of 70 (big ones, a warp
    # each) beside sparse particles: 192,000 + 140,000 + 60,000 particles
    cells = rng.choice(N ** 3, 18000, replace=False)
    corner = np.stack([cells % N, (cells // N) % N, cells // (N * N)], 1).astype(float)
    small = (corner[:16000, None, :] + rng.random((16000, 12, 3))) / N
    big = (corner[16000:, None, :] + rng.random((2000, 70, 3))) / N
    sparse = rng.random((60000, 3))
    pos = np.concatenate([small.reshape(-1, 3), big.reshape(-1, 3), sparse]) % 1.0
    n = len(pos)
    p = np.zeros(n, gpu.PART)
    p["pos"] = pos
    p["vel"] = rng.standard_normal((n, 3)) * 1e-3
    p["ID"] = rng.permutation(n)
    phi_h = rng.standard_normal((1, N, N, N)) * 1e-5
    ctx = gpu.Context(N, gpu.PREC_MIXED)
    phi = ctx.real(1).upload(phi_h)
    out = []
    # capacity n: 6,125 small and 1,531 big slots for 16,000 and 2,000 dense cells;
    # capacity 64 n: room for all of them
    for cap in (n, 64 * n):
        pc = ctx.particles(cap, 2e-4).upload(p)
        t00, tij = ctx.real(1), ctx.real(6)
        gpu.projection_T00_Tij(pc, t00, tij, 0.03, phi)
        out.append((t00.download(), tij.download()))
        del pc
    assert out[0][0].tobytes() == out[1][0].tobytes() and out[0][1].tobytes() == out[1][1].tobytes()
    for which, got in (("T00", out[0][0]), ("Tij", out[0][1])):
        ref = oracle.deposit(which, N, p, 2e-4, 0.03, phi_h, 1.0)
        assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max(), which


def test_dense_tables_of_a_sparse_store(gpu, oracle):
    """Fewer particles than cells: the dense-cell tables (4 B a cell) do not fit behind
    the prefactor records in the store's second array set and get an allocation of
    their own; the clustered deposit still follows the FP64 restatement and the fused
    deposit gives the separate ones' bits."""
    N = 64
    rng = np.random.default_rng(11)
    cells = rng.choice(N ** 3, 4000, replace=False)
    corner = np.stack([cells % N, (cells // N) % N, cells // (N * N)], 1).astype(float)
    pos = ((corner[:, None, :] + rng.random((4000, 12, 3))) / N).reshape(-1, 3) % 1.0
    n = len(pos)
    p = np.zeros(n, gpu.PART)
    p["pos"] = pos
    p["vel"] = rng.standard_normal((n, 3)) * 1e-3
    p["ID"] = rng.permutation(n)
    phi_h = rng.standard_normal((1, N, N, N)) * 1e-5
    ctx = gpu.Context(N, gpu.PREC_MIXED)
    phi = ctx.real(1).upload(phi_h)
    pc = ctx.particles(n, 2e-4).upload(p)
    f1, f6, g1, g6 = ctx.real(1), ctx.real(6), ctx.real(1), ctx.real(6)
    before = ctx.bytes_in_use()
    gpu.projection_T00_Tij(pc, g1, g6, 0.03, phi)
    assert ctx.bytes_in_use() - before >= 4 * N ** 3  # the tables' own allocation
    gpu.projection_T00(pc, f1, 0.03, phi)
    gpu.projection_Tij(pc, f6, 0.03, phi)
    assert f1.download().tobytes() == g1.download().tobytes()
    assert f6.download().tobytes() == g6.download().tobytes()
    for which, got in (("T00", g1.download()), ("Tij", g6.download())):
        ref = oracle.deposit(which, N, p, 2e-4, 0.03, phi_h, 1.0)
        assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max(), which
