"""The mixed form's source stencils (prepareFTsource scalar and tensor,
gevolution.hpp:56-192) give the same bits whatever launch shape the context's
tuner picks or the caller pins (include/gev_gb300.h, gev_ctx_set_stencil_shapes)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(256, 16), (64, 1), (128, 4), (512, 32), (128, 64)]


def run_stencils(gpu, N, shape, inputs):
    ctx = gpu.Context(N, gpu.PREC_MIXED)
    if shape is not None:
        ctx.set_stencil_shapes(shape, shape)
    phi, chi, src, Tij = ctx.real(1), ctx.real(1), ctx.real(1), ctx.real(6)
    phi.upload(inputs["phi"])
    chi.upload(inputs["chi"])
    src.upload(inputs["src"])
    Tij.upload(inputs["Tij"])
    gpu.prepare_source_scalar(phi, chi, src, 0.32, src, 2e-3, 3e-2, 5e-4)  # in place, as the cycle calls it
    gpu.prepare_source_tensor(phi, Tij, Tij, 7e-3)
    return src.download(), Tij.download(), ctx.stencil_shapes()


@pytest.mark.parametrize("N", [32, 64, 96])
def test_every_launch_shape_gives_the_same_bits(gpu, N):
    rng = np.random.default_rng(N)
    inputs = {"phi": 1e-5 * rng.standard_normal((N, N, N)), "chi": 1e-6 * rng.standard_normal((N, N, N)),
              "src": rng.random((N, N, N)), "Tij": rng.standard_normal((6, N, N, N))}
    ref_s, ref_t, sh = run_stencils(gpu, N, SHAPES[0], inputs)
    assert sh == {"scalar": SHAPES[0], "tensor": SHAPES[0]}
    for shape in SHAPES[1:] + [None]:  # None: the context's tuner picks
        s, t, sh = run_stencils(gpu, N, shape, inputs)
        assert np.array_equal(s, ref_s) and np.array_equal(t, ref_t), shape
        if shape is None:
            for th, ps in sh.values():
                assert th in (128, 256, 512) and ps in (4, 8, 16, 32)


def test_pinning_rejects_bad_shapes(gpu):
    ctx = gpu.Context(32, gpu.PREC_MIXED)
    for bad in [((96, 8), (256, 16)), ((256, 0), (256, 16)), ((256, 16), (1024, 16)), ((256, 16), (256, 65))]:
        with pytest.raises(gpu.GevError):
            ctx.set_stencil_shapes(*bad)
