"""gev_batch_step / gev_batch_run (include/gev_sim.h): one cycle of many simulations
with one launch per kernel for each cohort of one grid size.

- Batched cycles are deterministic: the same simulations batched twice, or one
  simulation batched alone and inside a cohort of others, give the same bits.
- Against gev_sim_step they agree to FP32 rounding.  The batched forms are compiled
  apart from the kernels, so the FP32 bodies that leave multiply-add fusion to the
  compiler may round differently in the last bit; the tolerances below (fields 1e-5
  of their largest value, positions 1e-5 of a cell, T00hom 1e-8 relative after ten
  cycles from z = 100) are far above that and far below the mixed form's own error
  against FP64 (1e-3 in P(k)).
- Cohorts of power-of-two and radix-3 grids, several cosmologies in one cohort, and
  simulations that take direct cycles (FP64 form, timers on) in the same call."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STATE_KEYS = ("a", "tau", "dtau", "dtau_old", "T00hom", "maxvel", "phik0", "cycle")
FIELD_TOL = 1e-5   # of the field's largest |value|
POS_TOL = 1e-5     # cells
T00_TOL = 1e-8     # relative


def make(gpu, N, prec, seed, **cosmo):
    c = gpu.Context(N, prec)
    s = gpu.Sim(c, N ** 3)
    s.ic_generate(**gpu.ic_params(2.5 * N, seed=seed, **cosmo))
    return c, s


def by_id(s):
    p = s.particles().download()
    return p[np.argsort(p["ID"], kind="stable")]


def assert_same_bits(s1, s2):
    st1, st2 = s1.state(), s2.state()
    for k in STATE_KEYS:
        assert st1[k] == st2[k], k
    assert by_id(s1).tobytes() == by_id(s2).tobytes()
    for name in ("phi", "chi", "Bi"):
        assert np.array_equal(s1.field(name).download(), s2.field(name).download()), name


def assert_close(sb, sd, N):
    """batched sb against direct sd, within the FP32-rounding tolerances; returns the
    largest deviations seen"""
    stb, std = sb.state(), sd.state()
    for k in ("a", "tau", "dtau", "dtau_old", "cycle", "phik0"):
        assert stb[k] == std[k], k
    assert abs(stb["T00hom"] - std["T00hom"]) <= T00_TOL * abs(std["T00hom"])
    assert abs(stb["maxvel"] - std["maxvel"]) <= 1e-5 * std["maxvel"]
    pb, pd = by_id(sb), by_id(sd)
    assert np.array_equal(pb["ID"], pd["ID"])
    d = np.abs(pb["pos"] - pd["pos"])
    dpos = float(np.minimum(d, 1.0 - d).max()) * N
    assert dpos <= POS_TOL, dpos
    dev = {"pos_cells": dpos}
    for name in ("phi", "chi", "Bi"):
        fb, fd = sb.field(name).download(), sd.field(name).download()
        rel = float(np.abs(fb - fd).max() / np.abs(fd).max())
        assert rel <= FIELD_TOL, (name, rel)
        dev[name] = rel
    return dev


SPECS = [(32, "PREC_MIXED", 1, {}), (32, "PREC_MIXED", 2, {"Omega_cdm": 0.3}),
         (32, "PREC_MIXED", 3, {"sigma8": 0.85}), (48, "PREC_MIXED", 4, {}),
         (48, "PREC_MIXED", 5, {"n_s": 0.95}), (64, "PREC_MIXED", 6, {}), (32, "PREC_FP64", 7, {})]


def test_batched_cycles_match_direct_cycles(gpu):
    batched = [make(gpu, N, getattr(gpu, f), seed, **c) for N, f, seed, c in SPECS]
    direct = [make(gpu, N, getattr(gpu, f), seed, **c) for N, f, seed, c in SPECS]
    b = gpu.Batch()
    cycles = 10
    for _ in range(cycles):
        b.step([s for _, s in batched])
        for _, s in direct:
            s.step()
    for (N, f, _, _), (_, sb), (_, sd) in zip(SPECS, batched, direct):
        if f == "PREC_FP64":
            assert_same_bits(sb, sd)  # its cycles were direct
        else:
            assert_close(sb, sd, N)
    nb, nd, nl = b.info()
    mixed = sum(1 for spec in SPECS if spec[1] == "PREC_MIXED")
    # the first two cycles and the FP64 simulation's cycles run directly
    assert nb == mixed * (cycles - 2) and nd == 2 * mixed + cycles
    # three cohorts (32^3, 48^3, 64^3): one launch per kernel of a cycle for each
    cohort_cycles = 3 * (cycles - 2)
    assert 30 * cohort_cycles <= nl <= 90 * cohort_cycles


def test_batched_cycles_are_deterministic(gpu):
    """The same four simulations batched twice give the same bits, and a simulation
    batched alone gives the same bits as inside the cohort."""
    specs = [(32, 51, {}), (32, 52, {"Omega_cdm": 0.3}), (32, 53, {"sigma8": 0.75}), (32, 54, {})]
    runs = []
    for _ in range(2):
        sims = [make(gpu, N, gpu.PREC_MIXED, seed, **c) for N, seed, c in specs]
        b = gpu.Batch()
        for _ in range(8):
            b.step([s for _, s in sims])
        runs.append(sims)
    alone = make(gpu, 32, gpu.PREC_MIXED, 51)
    b = gpu.Batch()
    for _ in range(8):
        b.step([alone[1]])
    for (_, s1), (_, s2) in zip(runs[0], runs[1]):
        assert_same_bits(s1, s2)
    assert_same_bits(runs[0][0][1], alone[1])


def test_batched_and_direct_cycles_interleave(gpu):
    """A one-simulation cohort, batched and direct cycles in turn on one simulation."""
    _, s = make(gpu, 32, gpu.PREC_MIXED, 11)
    _, ref = make(gpu, 32, gpu.PREC_MIXED, 11)
    b = gpu.Batch()
    for k in range(9):
        if k % 3 == 1:
            s.step()
        else:
            b.step([s])
        ref.step()
    assert_close(s, ref, 32)
    assert b.info()[0] == 5  # k = 2, 3, 5, 6, 8 (k = 0 and 1 are the first two cycles)


def test_timed_simulations_take_direct_cycles(gpu):
    c, s = make(gpu, 32, gpu.PREC_MIXED, 21)
    _, ref = make(gpu, 32, gpu.PREC_MIXED, 21)
    c.set_timing(True)
    b = gpu.Batch()
    for _ in range(4):
        b.step([s])
        ref.step()
    assert b.info()[:2] == (0, 4)
    assert_same_bits(s, ref)
    c.set_timing(False)
    b.step([s])
    ref.step()
    assert b.info()[0] == 1
    assert_close(s, ref, 32)


def test_batch_rejects_bad_calls(gpu):
    _, s = make(gpu, 32, gpu.PREC_MIXED, 31)
    b = gpu.Batch()
    with pytest.raises(gpu.GevError):
        b.step([s, s])  # the same simulation twice


def test_batch_run_to_targets_matches_direct_loops(gpu):
    """gev_batch_run: each simulation stops at the first cycle past its own target, as
    main.cpp's loop does (a is computed on the host, so the cycle counts are exact)."""
    specs = [(32, 41, 60.0), (32, 42, 40.0), (48, 43, 50.0), (64, 44, 70.0)]
    runs = [make(gpu, N, gpu.PREC_MIXED, seed) for N, seed, _ in specs]
    targets = [1.0 / (1.0 + z) for _, _, z in specs]
    b = gpu.Batch()
    cycles = b.run([s for _, s in runs], targets)
    for (N, seed, z), (_, s), ncyc in zip(specs, runs, cycles):
        _, ref = make(gpu, N, gpu.PREC_MIXED, seed)
        k = 0
        while ref.state()["a"] < 1.0 / (1.0 + z):
            ref.step()
            k += 1
        assert ncyc == k
        assert_close(s, ref, N)


def test_small_and_radix3_grids_and_an_empty_call(gpu):
    """12^3 (the deposit walks nodes in lines: 12 is no multiple of its 8 x 2 x 2 patch;
    radix-3 transforms) and 24^3 (patch walk, radix-3 transforms) in one call; an empty
    call does nothing."""
    specs = [(12, 61), (12, 62), (24, 63), (24, 64)]
    batched = [make(gpu, N, gpu.PREC_MIXED, seed) for N, seed in specs]
    direct = [make(gpu, N, gpu.PREC_MIXED, seed) for N, seed in specs]
    b = gpu.Batch()
    b.step([])
    for _ in range(8):
        b.step([s for _, s in batched])
        for _, s in direct:
            s.step()
    for (N, _), (_, sb), (_, sd) in zip(specs, batched, direct):
        assert_close(sb, sd, N)
    assert b.info()[0] == len(specs) * 6
