"""On-device power and cross spectra (gev_cross_spectrum) against the oracle's
restatement of extractCrossSpectrum (tools.hpp:53-212), and the precision-form
criterion: mixed-form power spectra of phi, chi, B and the source within 1e-3 of
the FP64 form up to k_Nyquist / 2 after several cycles from the same initial
conditions."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_K = 1e-13  # mean k per bin: the same terms summed in another order
TOL_P = 1e-12  # mean power per bin, relative (FMA contraction on the device, order)
TOL_SCATTER = 1e-7  # scatters are square roots of differences of sums: absolute, relative to the mean
TOL_MIXED_PK = 1e-3  # mixed vs FP64 power per bin up to k_Nyquist / 2


def relmax(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


@pytest.mark.parametrize("N,sym,deconv", [(16, False, True), (24, True, True), (32, False, False), (32, True, True)])
def test_spectrum_matches_oracle(gpu, oracle, N, sym, deconv):
    rng = np.random.default_rng(N + 7 * sym)
    ncomp = 6 if sym else 3
    NH = N // 2 + 1
    F = rng.standard_normal((ncomp, N, N, NH)) + 1j * rng.standard_normal((ncomp, N, N, NH))
    ctx = gpu.Context(N)
    s = ctx.spectrum(ncomp).upload(F)
    nb = 20
    kb, pw, ks, ps, occ = gpu.cross_spectrum(s, numbins=nb, deconvolve=deconv, symmetric=sym)
    okb, opw, oks, ops, oocc = oracle.power_spectrum(F, nb, symmetric=sym, deconvolve=deconv)
    assert (occ == oocc).all()
    m = occ > 0
    assert relmax(kb[m], okb[m]) < TOL_K
    assert relmax(pw[m], opw[m]) < TOL_P
    assert np.all(np.abs(ks[m] - oks[m]) <= TOL_SCATTER * kb[m])
    assert np.all(np.abs(ps[m] - ops[m]) <= TOL_SCATTER * np.abs(pw[m]))
    # integer sums: a second call gives the same bits
    again = gpu.cross_spectrum(s, numbins=nb, deconvolve=deconv, symmetric=sym)
    for x, y in zip((kb, pw, ks, ps, occ), again):
        assert np.array_equal(x, y)


def test_spectrum_of_fp32_spectrum(gpu, oracle):
    """Mixed form: the FP32 spectrum is read and the per-mode arithmetic stays FP64."""
    N, rng = 32, np.random.default_rng(5)
    NH = N // 2 + 1
    F = (rng.standard_normal((1, N, N, NH)) + 1j * rng.standard_normal((1, N, N, NH))).astype(np.complex64)
    ctx = gpu.Context(N, gpu.PREC_MIXED)
    s = ctx.spectrum(1).upload(F.astype(np.complex128))
    kb, pw, ks, ps, occ = gpu.cross_spectrum(s, numbins=16)
    okb, opw, oks, ops, oocc = oracle.power_spectrum(F.astype(np.complex128), 16)
    assert (occ == oocc).all()
    m = occ > 0
    assert relmax(pw[m], opw[m]) < TOL_P


def test_cross_spectrum_components_and_grid_k(gpu):
    """comp1/comp2 select single components; a component against itself equals the
    power spectrum of that component alone.  The grid-k binning (KTYPE_GRID) is
    checked against a direct numpy count of the same bins."""
    N, rng = 16, np.random.default_rng(9)
    NH = N // 2 + 1
    F = rng.standard_normal((3, N, N, NH)) + 1j * rng.standard_normal((3, N, N, NH))
    ctx = gpu.Context(N)
    s = ctx.spectrum(3).upload(F)
    one = ctx.spectrum(1).upload(F[1:2])
    a = gpu.cross_spectrum(s, s, numbins=12, comp1=1, comp2=1)
    b = gpu.cross_spectrum(one, numbins=12)
    assert (a[4] == b[4]).all()
    assert relmax(a[1][a[4] > 0], b[1][b[4] > 0]) < TOL_P
    # cross of components 0 and 2: mean of Re(f0 conj f2) k^3 / s with the reference's weights
    kb, pw, _, _, occ = gpu.cross_spectrum(s, s, numbins=12, comp1=0, comp2=2, deconvolve=False, ktype=0)
    i = np.arange(N)
    tk2 = (2.0 * N * np.sin(np.pi * i / N)) ** 2
    k2 = tk2[None, None, :NH] + tk2[None, :, None] + tk2[:, None, None]
    w = np.full((N, N, NH), 2.0)
    w[:, :, 0] = 1.0
    w[:, :, N // 2] = 1.0
    w[0, 0, 0] = 0.0
    k2max = 3.0 * tk2[N // 2]
    b = np.floor(12 * np.sqrt(k2 / k2max)).astype(int)
    p = (F[0] * np.conj(F[2])).real
    keep = (w > 0) & (b < 12)
    occ_np = np.bincount(b[keep], weights=w[keep], minlength=12)
    pw_np = np.bincount(b[keep], weights=(w * p * k2 * np.sqrt(k2))[keep], minlength=12)
    assert np.array_equal(occ, occ_np.astype(int))
    m = occ > 0
    assert np.allclose(pw[m], pw_np[m] / occ_np[m], rtol=1e-11, atol=1e-12 * np.abs(pw_np[m] / occ_np[m]).max())


def test_mixed_power_spectra_track_fp64(gpu):
    """The precision form's spectra stay within 1e-3 of the FP64 form's up to
    k_Nyquist / 2 (linear k: k_Nyquist = pi N in the units of typek2)."""
    N, cycles, nb = 64, 10, 32
    spectra = {}
    for prec in (gpu.PREC_FP64, gpu.PREC_MIXED):
        ctx = gpu.Context(N, prec)
        s = gpu.Sim(ctx, N ** 3)
        s.ic_generate(**gpu.ic_params(320.0, seed=6))
        for _ in range(cycles):
            s.step()
        out = {}
        for name, nc in (("phi", 1), ("chi", 1), ("Bi", 3), ("source", 1)):
            sp = ctx.spectrum(nc)
            gpu.fft_r2c(s.field(name), sp)
            out[name] = gpu.cross_spectrum(sp, numbins=nb)
        spectra[prec] = out
    for name in ("phi", "chi", "Bi", "source"):
        kb, p64, _, _, occ = spectra[gpu.PREC_FP64][name]
        p32 = spectra[gpu.PREC_MIXED][name][1]
        m = (occ > 0) & (kb <= 0.5 * np.pi * N)
        assert m.sum() > 5
        assert relmax(p32[m], p64[m]) < TOL_MIXED_PK, name


GOLDEN_CASES = (("auto1_dec", "F1", None, True, -1, -1), ("auto1", "F1", None, False, -1, -1),
                ("auto3", "F3", None, False, -1, -1), ("auto6", "F6", None, False, -1, -1),
                ("auto6_dec", "F6", None, True, -1, -1), ("cross1", "F1", "G1", True, -1, -1),
                ("comps6", "F6", None, True, 0, 3))


@pytest.mark.parametrize("name,f1,f2,dec,c1,c2", GOLDEN_CASES)
def test_spectrum_matches_reference_golden(gpu, name, f1, f2, dec, c1, c2):
    """gev_cross_spectrum against the reference's own extractCrossSpectrum
    (golden vectors from tools.hpp), including a cross spectrum and the
    component pair of the ncdm cross spectra."""
    from conftest import golden
    g = golden("golden_spectra_N12.npz")
    ctx = gpu.Context(12)
    a = ctx.spectrum(g[f1].shape[0]).upload(g[f1])
    b = a if f2 is None else ctx.spectrum(g[f2].shape[0]).upload(g[f2])
    kb, pw, ks, ps, occ = gpu.cross_spectrum(a, b, 10, dec, 1, g[f1].shape[0] == 6, c1, c2)
    assert (occ == g[name + "_occupation"]).all()
    m = occ > 0
    assert relmax(kb[m], g[name + "_kbin"][m]) <= TOL_K
    scale = np.abs(g[name + "_power"][m]).max()
    assert np.abs(pw[m] - g[name + "_power"][m]).max() <= TOL_P * scale
    assert np.abs(ks[m] - g[name + "_kscatter"][m]).max() <= TOL_SCATTER * np.abs(g[name + "_kbin"][m]).max()
    assert np.abs(ps[m] - g[name + "_pscatter"][m]).max() <= TOL_SCATTER * scale


def read_table(path):
    lines = open(path).read().splitlines()
    z = float(lines[1].split("=")[1])
    rows = np.array([[float(x) for x in ln.split()] for ln in lines[3:]])
    return lines[0][2:], z, rows


def expected_tables(oracle, s, nb, boxsize):
    """writeSpectra's sequence (output.hpp:1785-2152) redone with the oracle on the
    simulation's downloaded state: name -> (description, k, P, count)."""
    N = s.ctx.N
    st = s.state()
    a, fourpiG, cm = st["a"], st["fourpiG"], st["cosmo"]
    parts, mass = s.particles().download(), st["mass"]
    phi, chi, BiFT = s.field("phi").download(), s.field("chi").download(), s.field("BiFT").download()
    base = float(N ** 3) * float(N ** 3) * 2. * np.pi * np.pi
    out = {}

    def table(name, desc, F, dec, rescalep, sym=False):
        kb, pw, ks, ps, occ = oracle.power_spectrum(F, nb, symmetric=sym, deconvolve=dec)
        m = occ > 0
        out[name] = (desc, kb[m] / boxsize, pw[m] / rescalep, occ[m])

    rho = oracle.fft_r2c(oracle.deposit("mass", N, parts, mass))
    table("rhoN", "power spectrum of rho_N", rho, True, base * a ** 6.0)
    table("deltaN", "power spectrum of delta_N", rho, True, base * cm["Omega_m"] * cm["Omega_m"])
    table("psiN", "power spectrum of psi_N", oracle.poisson(rho, fourpiG / a), False, base)
    table("phi", "power spectrum of phi", oracle.fft_r2c(phi), False, base)
    table("chi", "power spectrum of chi", oracle.fft_r2c(chi), False, base)
    T = oracle.deposit("Tij", N, parts, mass, a, phi)
    S = oracle.prepare_source_tensor(phi, T, 2. * fourpiG / N / N / a)
    table("hij", "power spectrum of hij", oracle.project_tensor(oracle.fft_r2c(S)), False, 2. * np.pi * np.pi, True)
    T00 = oracle.fft_r2c(oracle.deposit("T00", N, parts, mass, a, phi))
    table("T00", "power spectrum of T00", T00, True, base * a ** 6.0)
    om = cm["Omega_cdm"] + cm["Omega_b"]
    table("delta", "power spectrum of delta", T00, True, base * om * om)
    table("B", "power spectrum of B", BiFT, False, a * a * a * a * N * N * 2. * np.pi * np.pi)
    return out


ALL_PK = 1 | 2 | 4 | 8 | 16 | 64 | 128 | 4096 | 8192


def test_write_spectra_against_oracle(gpu, oracle, tmp_path):
    """writeSpectra between the field solves and the particle update, as main.cpp
    calls it: every table (phi, chi, psi_N, rho_N, delta_N, hij, T00, delta, B)
    against the oracle's deposits, FFTs and spectra of the same state."""
    N, nb, L = 16, 12, 80.0
    c = gpu.Context(N, gpu.PREC_FP64)
    s = gpu.Sim(c, N ** 3)
    s.ic_generate(**gpu.ic_params(L, seed=8))
    s.step()
    s.step_fields()
    s.write_spectra(ALL_PK, nb, L, 7, str(tmp_path) + "/", "pk_")
    want = expected_tables(oracle, s, nb, L)
    z = 1.0 / s.state()["a"] - 1.0
    for name, (desc, k, P, occ) in want.items():
        d, zf, rows = read_table(tmp_path / ("pk_007_%s.dat" % name))
        assert d == desc, name
        assert abs(zf - z) <= 1e-6, name
        assert rows.shape[0] == len(k), name
        assert (rows[:, 4] == occ).all(), name
        assert np.allclose(rows[:, 0], k, rtol=2e-6, atol=0), name
        assert np.allclose(rows[:, 1], P, rtol=2e-6, atol=1e-7 * np.abs(P).max()), name
    s.step_particles()


@pytest.mark.parametrize("prec", [0, 1])
def test_step_halves_equal_the_step(gpu, prec):
    N = 16
    runs = []
    for split in (False, True):
        c = gpu.Context(N, prec)
        s = gpu.Sim(c, N ** 3)
        s.ic_generate(**gpu.ic_params(5.0 * N, seed=3))
        for _ in range(3):
            if split:
                s.step_fields()
                s.step_particles()
            else:
                s.step()
        runs.append((s.particles().download(), s.field("phi").download(), s.field("BiFT").download(),
                     s.state()["a"]))
    for x, y in zip(*runs):
        assert np.asarray(x).tobytes() == np.asarray(y).tobytes()


def test_exact_output_redshift_interpolation(gpu, tmp_path):
    """EXACT_OUTPUT_REDSHIFTS: written one cycle before z_target and again one
    cycle after it, a table ends at z_target, interpolated linearly in redshift
    between the two cycles' spectra (tools.hpp:279-316)."""
    N, nb, L = 16, 10, 80.0
    c = gpu.Context(N, gpu.PREC_FP64)
    s = gpu.Sim(c, N ** 3)
    s.ic_generate(**gpu.ic_params(L, seed=6))
    s.step()
    s.step_fields()
    z1 = 1.0 / s.state()["a"] - 1.0
    phi1 = gpu.cross_spectrum(_fft(gpu, c, s.field("phi")), None, nb, False)
    out, plain = str(tmp_path) + "/", str(tmp_path / "plain") + "/"
    os.makedirs(plain)
    s.step_particles()
    z2 = 1.0 / s.state()["a"] - 1.0
    zt = 0.5 * (z1 + z2)
    # cycle 1 (before z_target): the table as it is
    c1 = gpu.Context(N, gpu.PREC_FP64)
    s1 = gpu.Sim(c1, N ** 3)
    s1.ic_generate(**gpu.ic_params(L, seed=6))
    s1.step()
    s1.step_fields()
    s1.write_spectra(1, nb, L, 0, out, "pk_", zt, True)
    s1.step_particles()
    # cycle 2 (after it): interpolated
    s1.step_fields()
    phi2 = gpu.cross_spectrum(_fft(gpu, c1, s1.field("phi")), None, nb, False)
    s1.write_spectra(1, nb, L, 0, out, "pk_", zt, True)
    s1.write_spectra(1, nb, L, 0, plain, "pk_", zt, False)
    _, zf, rows = read_table(tmp_path / "pk_000_phi.dat")
    _, zp, rows_plain = read_table(tmp_path / "plain" / "pk_000_phi.dat")
    assert zf == float("%f" % zt) and abs(zp - z2) <= 1e-6
    base = float(N ** 3) ** 2 * 2. * np.pi * np.pi
    m = phi1[4] > 0
    p1, p2 = phi1[1][m] / base, phi2[1][m] / base
    # the first table is re-read with its printed digits, its redshift too
    z1p = float("%f" % z1)
    w = (z1p - zt) / (1. + z1p - 1. / s1.state()["a"])
    p1 = np.array([float("%e" % v) for v in p1])
    assert np.allclose(rows[:, 1], (1. - w) * p1 + w * p2, rtol=2e-6, atol=0)
    assert np.allclose(rows_plain[:, 1], p2, rtol=2e-6, atol=0)


def _fft(gpu, c, real):
    F = c.spectrum(1)
    gpu.fft_r2c(real, F)
    return F
