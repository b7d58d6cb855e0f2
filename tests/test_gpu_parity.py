"""CUDA path (libgev_gb300.so through its C-ABI) against the CPU oracle and the
reference's golden vectors.  FP64 form: every operator within TOL_* of the
oracle (relative to the field's maximum); particle order identical; deposits
bit-reproducible run to run, and bit-identical to the oracle away from the periodic
fold."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

TOL_OP = 1e-13    # per-operator FP64 agreement, relative to max |reference|
TOL_FFT = 2e-14   # FFT, relative to max |reference| (different butterfly order)


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


def rand_parts(rng, G, N, n, vscale=2e-3):
    p = np.zeros(n, G.PART)
    p["pos"] = rng.random((n, 3))
    k = min(n, 6)
    p["pos"][:k] = np.array([[0.0, 0.0, 0.0], [1.0 / N, 2.0 / N, 0.5], [np.nextafter(1.0, 0.0)] * 3,
                             [0.5, np.nextafter(1.0, 0.0), 0.0], [3.0 / N, 3.0 / N, 3.0 / N],
                             [0.25, 0.75, 1.0 / N]])[:k]
    p["vel"] = rng.standard_normal((n, 3)) * vscale
    p["ID"] = rng.permutation(3 * n)[:n]
    return p


@pytest.mark.parametrize("N", [8, 12, 16, 24, 32, 48, 64, 96])
def test_fft(gpu, oracle, N):
    rng = np.random.default_rng(N)
    ctx = gpu.Context(N)
    x = rng.standard_normal((3, N, N, N))
    r = ctx.real(3).upload(x)
    s = ctx.spectrum(3)
    gpu.fft_r2c(r, s)
    F = s.download()
    assert rel(F, oracle.fft_r2c(x)) < TOL_FFT
    # c2r of an arbitrary spectrum (not Hermitian in the kx = 0 / N/2 planes)
    Fr = rng.standard_normal(F.shape) + 1j * rng.standard_normal(F.shape)
    s.upload(Fr)
    out = ctx.real(3)
    gpu.fft_c2r(s, out)
    assert rel(out.download(), oracle.fft_c2r(Fr)) < TOL_FFT
    assert np.array_equal(s.download(), Fr), "c2r modified its input spectrum"
    # round trip
    gpu.fft_r2c(out, s)
    back = ctx.real(3)
    gpu.fft_c2r(s, back)
    assert rel(back.download() / N ** 3, out.download()) < TOL_FFT


@pytest.mark.parametrize("N", [8, 12])
def test_operators_against_reference_golden(gpu, N):
    """Every operator on the golden inputs against the outputs of the reference's
    own gevolution.hpp."""
    g = golden("golden_N%d.npz" % N)
    ctx = gpu.Context(N)
    phi = ctx.real(1).upload(g["phi"])
    chi = ctx.real(1).upload(g["chi"])
    src = ctx.real(1).upload(g["src"])
    T = ctx.real(6).upload(g["T"])
    S = ctx.real(6)
    gpu.prepare_source_tensor(phi, T, S, 0.37)
    assert rel(S.download(), g["out_pst"]) < TOL_OP
    res = ctx.real(1)
    gpu.prepare_source_scalar(phi, chi, src, 0.32, res, 1.3e-3, 2.1e-4, 3.7e-5)
    assert rel(res.download(), g["out_pss"]) < TOL_OP
    s1 = ctx.spectrum(1).upload(g["s1"])
    SF = ctx.spectrum(6).upload(g["S"])
    BF = ctx.spectrum(3).upload(g["B"])
    out1 = ctx.spectrum(1)
    gpu.solve_poisson(s1, out1, 3.0, 0.0)
    assert rel(out1.download(), g["out_poisson"]) < TOL_OP
    gpu.solve_poisson(s1, out1, 3.0, 0.7)
    assert rel(out1.download(), g["out_poisson_modif"]) < TOL_OP
    gpu.project_scalar(SF, out1, 0)
    assert rel(out1.download(), g["out_pscalar"]) < TOL_OP
    out1.upload(g["s1"])
    gpu.project_scalar(SF, out1, 1)
    assert rel(out1.download(), g["out_pscalar_add"]) < TOL_OP
    out3 = ctx.spectrum(3).upload(g["B"])
    gpu.evolve_vector(SF, out3, 0.013)
    assert rel(out3.download(), g["out_evolve"]) < TOL_OP
    gpu.project_vector(BF, out3, 0.3, 0.1)
    assert rel(out3.download(), g["out_pvector"]) < TOL_OP
    gpu.project_vector(BF, BF, 0.3, 0.1)  # in place, as main.cpp:580 calls it
    assert rel(BF.download(), g["out_pvector"]) < TOL_OP
    out6 = ctx.spectrum(6)
    gpu.project_tensor(SF, out6)
    assert rel(out6.download(), g["out_ptensor"]) < TOL_OP
    # deposits
    p = g["parts"]
    pc = ctx.particles(len(p), 1e-3).upload(p)
    for w, nc, fn in (("T00", 1, lambda f: gpu.projection_T00(pc, f, 0.02, phi)),
                      ("T0i", 3, lambda f: gpu.projection_T0i(pc, f, phi)),
                      ("Tij", 6, lambda f: gpu.projection_Tij(pc, f, 0.02, phi))):
        f = ctx.real(nc)
        fn(f)
        assert rel(f.download(), g["out_dep_" + w]) < TOL_OP, w
    f = ctx.real(1)
    gpu.projection_T00(pc, f, 0.02, None)
    assert rel(f.download(), g["out_dep_T00_nophi"]) < TOL_OP
    # particle updates
    Bi = ctx.real(3).upload(g["Bi"])
    a, a2N = 0.02, 0.02 ** 2 * N
    for kind in (0, 1):
        for nf in (1, 2, 3):
            pc.upload(p)
            v = gpu.update_q(pc, kind, 0.011, phi, chi, Bi, nf, a, a2N)
            got = pc.download()
            ref = g["out_kick_%d_%d" % (kind, nf)]
            assert (got["ID"] == ref["ID"]).all()
            assert rel(got["vel"], ref["vel"]) < TOL_OP, (kind, nf)
            assert abs(v - float(g["out_kick_max_%d_%d" % (kind, nf)])) <= 1e-12 * v
        for nf in (0, 1, 2, 3):
            pc.upload(p)
            gpu.update_pos(pc, kind, 0.37, phi, chi, Bi, nf, a, a2N)
            got = pc.download()
            ref = g["out_drift_%d_%d" % (kind, nf)]
            assert (got["ID"] == ref["ID"]).all(), (kind, nf)
            assert np.abs(got["pos"] - ref["pos"]).max() < 1e-14, (kind, nf)


@pytest.mark.parametrize("N", [16, 24, 32])
def test_deposits_and_sort(gpu, oracle, N):
    rng = np.random.default_rng(100 + N)
    n = 2 * N ** 3
    p = rand_parts(rng, oracle, N, n)
    # a dense clump so that some cells hold more than 32 particles
    p["pos"][:200] = 0.5 + rng.random((200, 3)) * (0.5 / N)
    ctx = gpu.Context(N)
    pc = ctx.particles(n, 2e-4).upload(p)
    ps, _ = oracle.sort(N, p)
    got = pc.download()
    assert (got["ID"] == ps["ID"]).all(), "store order differs from (cell, ID)"
    assert np.array_equal(got["pos"], ps["pos"])
    phi_h = rng.standard_normal((1, N, N, N)) * 1e-5
    phi = ctx.real(1).upload(phi_h)
    for which, nc in (("T00", 1), ("T0i", 3), ("Tij", 6), ("mass", 1)):
        f1, f2 = ctx.real(nc), ctx.real(nc)
        for f in (f1, f2):
            if which == "T00":
                gpu.projection_T00(pc, f, 0.03, phi)
            elif which == "T0i":
                gpu.projection_T0i(pc, f, phi)
            elif which == "Tij":
                gpu.projection_Tij(pc, f, 0.03, phi)
            else:
                gpu.projection_mass(pc, f)
        a1, a2 = f1.download(), f2.download()
        assert np.array_equal(a1, a2), "deposit is not bit-reproducible"
        ref = oracle.deposit(which, N, p, 2e-4, 0.03, None if which == "mass" else phi_h, 1.0)
        assert rel(a1, ref) < TOL_OP, which
        # Each cell's sums follow the reference's order of operations (cells above a
        # few particles summed by a warp, the rest by a thread), and each node adds its
        # cells' terms in the reference's order: bit-identical to the oracle at every
        # node that the periodic fold does not reach (all three indices >= 1)
        inner = (slice(None), slice(1, None), slice(1, None), slice(1, None))
        assert np.array_equal(a1.reshape(nc, N, N, N)[inner], np.asarray(ref).reshape(nc, N, N, N)[inner]), which


@pytest.mark.parametrize("N", [16, 24])
def test_sim_cycles(gpu, oracle, N):
    """IC from the oracle, then 6 cycles of the main loop on both."""
    o = oracle.Sim(N).ic(**oracle.default_icparams(N, 5.0 * N, seed=3))
    ctx = gpu.Context(N)
    s = gpu.Sim(ctx, N ** 3)
    load_sim(gpu, s, o)
    for k in range(6):
        o.step()
        s.step()
    st = s.state()
    assert abs(st["a"] - o.s.a) <= 1e-15 * o.s.a
    got = s.particles().download()
    ref = o.particles
    assert (got["ID"] == ref["ID"]).all()
    assert np.abs(got["pos"] - ref["pos"]).max() * N < 1e-9
    assert rel(got["vel"], ref["vel"]) < 1e-10
    for name in ("phi", "chi", "Bi"):
        assert rel(s.field(name).download(), o.field(name)) < 1e-10, name
    assert rel(s.field("BiFT").download(), o.spectrum("BiFT")) < 1e-10
    assert abs(st["T00hom"] - o.s.T00hom) <= 1e-12 * abs(o.s.T00hom)


def load_sim(gpu, s, o):
    """Copies an oracle simulation state into a device simulation."""
    s.particles().upload(o.particles)
    for name in ("phi", "chi", "Bi", "source", "Sij"):
        s.field(name).upload(o.field(name))
    for name in ("scalarFT", "SijFT", "BiFT"):
        s.field(name).upload(o.spectrum(name))
    sc = o.scalars()
    s.set_state(a=sc["a"], tau=sc["tau"], dtau=sc["dtau"], dtau_old=sc["dtau_old"], fourpiG=sc["fourpiG"],
                Cf=sc["Cf"], steplimit=sc["steplimit"], z_relax=sc["z_relax"], mass=sc["mass"], cycle=sc["cycle"],
                vector_elliptic=sc["vector_elliptic"], cosmo=o.cosmo)


@pytest.mark.parametrize("prec", [0, 1])
def test_project_scalar_evolve_vector_fused_equals_separate(gpu, prec):
    """gev_project_scalar_evolve_vector (the cycle's one pass over SijFT) equals
    projectFTscalar followed by evolveFTvector, bit for bit in both forms, k = 0 included."""
    N = 16
    rng = np.random.default_rng(40 + prec)
    ctx = gpu.Context(N, prec)
    S = ctx.spectrum(6)
    shp = S.shape
    S.upload(rng.standard_normal(shp) + 1j * rng.standard_normal(shp))
    B0 = rng.standard_normal((3,) + shp[1:]) + 1j * rng.standard_normal((3,) + shp[1:])
    chi1, B1 = ctx.spectrum(1), ctx.spectrum(3).upload(B0)
    gpu.project_scalar(S, chi1, 0)
    gpu.evolve_vector(S, B1, 3.7e-3)
    chi2, B2 = ctx.spectrum(1), ctx.spectrum(3).upload(B0)
    gpu.project_scalar_evolve_vector(S, chi2, B2, 3.7e-3)
    assert np.array_equal(chi1.download(), chi2.download())
    assert np.array_equal(B1.download(), B2.download())


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("N", [16, 24])
@pytest.mark.parametrize("modif", [0.0, 0.37])
def test_c2r_poisson_equals_solve_then_c2r(gpu, prec, N, modif):
    """gev_fft_c2r_poisson equals solveModifiedPoissonFT in place followed by the c2r, bit
    for bit, and keeps its input spectrum: the mixed form on power-of-two grids applies the
    factor inside the first pass, the other cases solve into the context's scratch."""
    rng = np.random.default_rng(N + 3 * prec)
    ctx = gpu.Context(N, prec)
    S = ctx.spectrum(1)
    shp = S.shape
    X = rng.standard_normal(shp) + 1j * rng.standard_normal(shp)
    S.upload(X)
    P = ctx.spectrum(1).upload(X)
    r1, r2 = ctx.real(1), ctx.real(1)
    gpu.solve_poisson(P, P, 2.3e3, modif)
    gpu.fft_c2r(P, r1)
    gpu.fft_c2r_poisson(S, r2, 2.3e3, modif)
    assert np.array_equal(r1.download(), r2.download())
    assert np.array_equal(S.download(), X.astype(np.complex64) if prec == 1 else X)
