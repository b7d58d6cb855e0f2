"""Continuous batching (include/gev_serve.h): each request's result is the same
bits alone and among others; admission follows the device-byte budget; the
result is the run main.cpp would make, cycle for cycle."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def run_alone(gpu, req):
    """The same request driven directly through gev_sim.h, cycle by cycle."""
    c = gpu.Context(req.N, req.prec)
    s = gpu.Sim(c, req.N ** 3)
    s.ic_generate(**gpu.ic_params(req.boxsize, seed=req.seed, z_in=req.z_in, Omega_cdm=req.Omega_cdm,
                                  Omega_b=req.Omega_b, sigma8=req.sigma8, n_s=req.n_s, h=req.h))
    a_target = 1.0 / (1.0 + req.z_target)
    cycles = 0
    while s.state()["a"] < a_target:
        s.step()
        cycles += 1
    F = c.spectrum(1)
    gpu.fft_r2c(s.field("phi"), F)
    kb, pw, _, _, occ = gpu.cross_spectrum(F, None, req.numbins, False)
    n3 = float(req.N) ** 3
    # the table's normalisation, (N^3)^2 2 pi^2, in the order writeSpectra writes it
    return {"a": s.state()["a"], "cycles": cycles, "kbin": kb / req.boxsize, "power": pw / (n3 * n3 * 2. * np.pi * np.pi),
            "occupation": occ}


@pytest.mark.parametrize("workers", [1, 4])
def test_results_same_alone_and_in_the_mix(gpu, workers):
    """With one scheduler thread and with four (each simulation's cycles enqueued by
    one of them), every result is the same bits as the request run alone."""
    reqs = [gpu.request(32, seed=11, z_target=60.0), gpu.request(48, seed=12, z_target=80.0, Omega_cdm=0.3),
            gpu.request(32, seed=13, z_target=70.0, sigma8=0.85, prec=gpu.PREC_FP64),
            gpu.request(64, seed=14, z_target=75.0, n_s=0.95), gpu.request(32, seed=15, z_target=60.0)]
    srv = gpu.Server(workers=workers)
    ids = [srv.submit(r) for r in reqs]
    srv.drain(120.0)
    got = {r["id"]: r for r in srv.poll()}
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["max_active_seen"] >= 2  # their work overlapped
    for i, req in zip(ids, reqs):
        mix, alone = got[i], run_alone(gpu, req)
        assert mix["status"] == 0
        assert mix["cycles"] == alone["cycles"] and mix["a"] == alone["a"]
        for k in ("kbin", "power", "occupation"):
            assert np.array_equal(mix[k], alone[k]), (i, k)
        assert mix["t_done"] >= mix["t_admit"] >= mix["t_submit"]


def test_admission_follows_the_byte_budget(gpu):
    """A budget with room for one 64^3 simulation: requests wait their turn, never
    more than one is on the device, all complete; a request larger than the whole
    budget fails without blocking the rest."""
    fp = gpu.footprint(64)
    srv = gpu.Server(bytes_budget=int(fp * 1.6))
    for k in range(3):
        srv.submit(gpu.request(64, seed=20 + k, z_target=90.0))
    big = srv.submit(gpu.request(128, seed=30, z_target=90.0))
    srv.submit(gpu.request(64, seed=31, z_target=90.0))
    srv.drain(120.0)
    res = {r["id"]: r for r in srv.poll()}
    st = srv.stats()
    srv.close()
    assert st["max_active_seen"] == 1
    assert st["completed"] == 4 and st["failed"] == 1
    assert res[big]["status"] != 0
    assert st["bytes_peak"] <= fp * 1.6


def test_requests_arriving_while_others_run(gpu):
    """Submissions during a run are admitted as they come; the first request's
    time to result is not held up by later ones."""
    srv = gpu.Server()
    first = srv.submit(gpu.request(64, seed=40, z_target=70.0))
    time.sleep(0.05)
    later = [srv.submit(gpu.request(32, seed=41 + k, z_target=80.0)) for k in range(4)]
    srv.drain(120.0)
    res = {r["id"]: r for r in srv.poll()}
    srv.close()
    assert all(res[i]["status"] == 0 for i in [first] + later)
    assert all(res[i]["t_submit"] > res[first]["t_submit"] for i in later)


def test_drain_returns_every_result_one_slot_at_a_time(gpu):
    """With one simulation on the device at a time each request is admitted as the
    previous one finishes; drain must not return while the last one is between the
    queue and the device."""
    srv = gpu.Server(max_active=1)
    ids = [srv.submit(gpu.request(32, seed=60 + k, z_target=90.0)) for k in range(6)]
    srv.drain(120.0)
    res = {r["id"]: r for r in srv.poll()}
    st = srv.stats()
    srv.close()
    assert sorted(res) == sorted(ids)
    assert all(r["status"] == 0 for r in res.values())
    assert st["completed"] == 6 and st["active"] == 0 and st["pending"] == 0
