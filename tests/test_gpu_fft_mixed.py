"""Mixed form (FP32) 3-D transforms at the grids the bench and the serving runs
use (256 and 512), against numpy's FFT of the same FP32 input.

The forward transform is checked against numpy directly, including the kx = 0
and Nyquist kx = N/2 columns, whose rows the real-to-complex split treats apart.
The backward one is checked on the Hermitian spectrum of a real field (where
c2r is unambiguous), through the round trip, and on the Hermitian part of a
random spectrum against numpy's inverse.  Tolerance: FP32 butterflies over
log2(N^3) = 24 or 27 stages, relative to the largest magnitude of the reference."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_F32 = 2e-5
AXES = (0, 1, 2)


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


@pytest.mark.parametrize("N", [256, 512])
def test_mixed_fft_against_numpy(gpu, N):
    rng = np.random.default_rng(7 + N)
    ctx = gpu.Context(N, gpu.PREC_MIXED)
    x = rng.standard_normal((N, N, N)).astype(np.float32)
    r = ctx.real(1).upload(x)
    s = ctx.spectrum(1)
    gpu.fft_r2c(r, s)
    F = s.download().reshape(N, N, N // 2 + 1)
    ref = np.fft.rfftn(x, axes=AXES)  # axes (z, y, x), x fastest: the same layout
    assert rel(F, ref) < TOL_F32
    assert rel(F[:, :, N // 2], ref[:, :, N // 2]) < TOL_F32
    assert rel(F[:, :, 0], ref[:, :, 0]) < TOL_F32
    del ref
    # backward of the Hermitian spectrum: N^3 x, and the input spectrum kept
    out = ctx.real(1)
    gpu.fft_c2r(s, out)
    back = out.download().reshape(N, N, N)
    assert rel(back / float(N) ** 3, x) < TOL_F32
    assert np.array_equal(s.download().reshape(N, N, N // 2 + 1), F), "c2r modified its input spectrum"
    # backward of the Hermitian part of a random spectrum against numpy's inverse
    G = (rng.standard_normal((N, N, N // 2 + 1)) + 1j * rng.standard_normal((N, N, N // 2 + 1))).astype(np.complex64)
    herm = np.fft.rfftn(np.fft.irfftn(G, s=(N, N, N), axes=AXES), axes=AXES)
    s.upload(herm)
    gpu.fft_c2r(s, out)
    want = np.fft.irfftn(herm, s=(N, N, N), axes=AXES) * float(N) ** 3
    assert rel(out.download().reshape(N, N, N), want) < TOL_F32


@pytest.mark.parametrize("N", [32, 256])
def test_tile_widths_give_the_same_bits(gpu, N):
    """The mixed form's FFT tile widths are chosen by timing (once per context); every
    width computes the same butterflies on the same values, so each combination gives
    the same bits, and the timed choice is one of them."""
    rng = np.random.default_rng(N)
    x = rng.standard_normal((N, N, N)).astype(np.float32)
    ref = None
    # one pass's width varied at a time around (rows 2, y 3, z 4)
    combos = sorted({(r, 3, 4) for r in (1, 2, 3)} | {(2, y, 4) for y in (2, 3, 4)} | {(2, 3, z) for z in (2, 3, 4)})
    for r, y, z in combos:
        ctx = gpu.Context(N, gpu.PREC_MIXED)
        ctx.set_fft_tiles(r, y, z, r)
        real, spec, back = ctx.real(1).upload(x), ctx.spectrum(1), ctx.real(1)
        gpu.fft_r2c(real, spec)
        gpu.fft_c2r(spec, back)
        got = (spec.download(), back.download())
        if ref is None:
            ref = got
        assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1]), (r, y, z)
    ctx = gpu.Context(N, gpu.PREC_MIXED)
    real, spec = ctx.real(1).upload(x), ctx.spectrum(1)
    gpu.fft_r2c(real, spec)
    tiles = ctx.fft_tiles()
    assert 1 <= tiles["r2c_rows"] <= 3 and 2 <= tiles["y"] <= 4 and 2 <= tiles["z"] <= 4, tiles
    assert np.array_equal(spec.download(), ref[0])
    with pytest.raises(RuntimeError):
        gpu.Context(N, gpu.PREC_FP64).set_fft_tiles(2, 2, 2, 2)
