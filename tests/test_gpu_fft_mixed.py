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
