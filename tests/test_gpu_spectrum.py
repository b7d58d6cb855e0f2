"""On-device power and cross spectra (gev_cross_spectrum) against the oracle's
restatement of extractCrossSpectrum (tools.hpp:53-212), and the precision-form
criterion: mixed-form power spectra of phi, chi, B and the source within 1e-3 of
the FP64 form up to k_Nyquist / 2 after several cycles from the same initial
conditions."""
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
