"""Device timing of the library's kernels and cycle phases (gev_ctx_set_timing /
gev_ctx_timing_report): every kernel of the cycle and the phases of main.cpp's
BENCHMARK breakdown (main.cpp:907-922) are reported, the counts follow the
launches, and timing changes no result."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [0, 1])
def test_cycle_timing_report(gpu, prec):
    N, cycles = 32, 3
    runs = []
    for timing in (False, True):
        ctx = gpu.Context(N, prec)
        s = gpu.Sim(ctx, N ** 3)
        s.ic_generate(**gpu.ic_params(5.0 * N, seed=4))
        s.step()
        ctx.set_timing(timing)
        for _ in range(cycles):
            s.step()
        ctx.set_timing(False)
        rep = ctx.timing()
        runs.append((s.particles().download(), s.field("phi").download(), rep))
    (p0, f0, r0), (p1, f1, r1) = runs
    assert r0 == {}
    assert p0.tobytes() == p1.tobytes() and f0.tobytes() == f1.tobytes()
    for name in ("phase:projections", "phase:gravity solver", "phase:fft", "phase:update particles", "k_kick_drift",
                 "k_source_scalar", "k_source_tensor"):
        assert name in r1, name
        cnt, ms = r1[name]
        assert ms > 0.0
    assert r1["phase:projections"][0] == cycles and r1["phase:update particles"][0] == cycles
    assert r1["k_kick_drift"][0] == cycles
    # one region per transform call (all components of a field in one call): phi's r2c and
    # c2r, Sij's r2c (6 components), chi's c2r, B's c2r (3 components)
    assert r1["phase:fft"][0] == 5 * cycles
    if prec == 1:
        assert r1["k_dep_gather"][0] == cycles and r1["k_move"][0] == cycles
    # the FFT phase lies inside the gravity solver phase
    assert r1["phase:fft"][1] <= r1["phase:gravity solver"][1]
    # a second report without reset adds nothing new
    assert ctx_report_empty_after_reset(gpu)


def ctx_report_empty_after_reset(gpu):
    ctx = gpu.Context(16, 1)
    ctx.set_timing(True)
    s = gpu.Sim(ctx, 16 ** 3)
    s.ic_generate(**gpu.ic_params(80.0, seed=1))
    s.step()
    first = ctx.timing(reset=True)
    ctx.set_timing(False)
    s.step()
    return len(first) > 0 and ctx.timing() == {}
