"""gev_sim_step_graph (include/gev_sim.h): the main-loop cycle enqueued as one
CUDA graph, updated in place from cycle to cycle, gives the same bits as
gev_sim_step in both precision forms -- alone, mixed with direct cycles on the
same simulation, and through the server (include/gev_serve.h)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STATE_KEYS = ("a", "tau", "dtau", "dtau_old", "T00hom", "maxvel", "phik0", "cycle")


def new_sim(gpu, N, prec, seed):
    c = gpu.Context(N, prec)
    s = gpu.Sim(c, N ** 3)
    s.ic_generate(**gpu.ic_params(2.5 * N, seed=seed))
    return c, s


def assert_same_bits(s1, s2):
    st1, st2 = s1.state(), s2.state()
    for k in STATE_KEYS:
        assert st1[k] == st2[k], k
    p1, p2 = s1.particles().download(), s2.particles().download()
    assert p1.tobytes() == p2.tobytes()
    for name in ("phi", "chi", "Bi"):
        assert np.array_equal(s1.field(name).download(), s2.field(name).download()), name


@pytest.mark.parametrize("form", ["PREC_MIXED", "PREC_FP64"])
def test_graph_cycles_same_bits_as_direct(gpu, form):
    prec = getattr(gpu, form)
    N, cycles = 32, 12
    _, direct = new_sim(gpu, N, prec, seed=5)
    _, graph = new_sim(gpu, N, prec, seed=5)
    for _ in range(cycles):
        direct.step()
        graph.step_graph()
    assert_same_bits(direct, graph)
    launches, builds, ndirect = graph.graph_info()
    # the first two cycles run directly (first-use set-up), the rest as graphs
    assert ndirect == 2 and launches == cycles - 2
    assert 1 <= builds <= 3  # updated in place, not rebuilt every cycle


def test_graph_and_direct_cycles_interleave(gpu):
    """Switching between the two entry points on one simulation keeps the host's
    side of the cycle (background state, the particle arrays' halves) in step."""
    N = 32
    _, ref = new_sim(gpu, N, gpu.PREC_MIXED, seed=9)
    _, mix = new_sim(gpu, N, gpu.PREC_MIXED, seed=9)
    for k, use_graph in enumerate([0, 0, 1, 1, 0, 1, 0, 0, 1, 1, 1]):
        ref.step()
        (mix.step_graph if use_graph else mix.step)()
        if k == 5:
            assert_same_bits(ref, mix)
    assert_same_bits(ref, mix)
    assert mix.graph_info()[0] == 6 and mix.graph_info()[2] == 0


def run_alone(gpu, req):
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
    return {"a": s.state()["a"], "cycles": cycles, "kbin": kb / req.boxsize,
            "power": pw / (n3 * n3 * 2. * np.pi * np.pi), "occupation": occ}


def test_server_with_graph_cycles_same_bits(gpu):
    """A server that enqueues every simulation's cycles as graphs (four scheduler
    threads capturing at once) returns the same bits as each request run alone
    with direct cycles, and its pooled simulations reuse their graphs."""
    reqs = [gpu.request(32, seed=71, z_target=60.0), gpu.request(48, seed=72, z_target=75.0, Omega_cdm=0.3),
            gpu.request(32, seed=73, z_target=70.0, prec=gpu.PREC_FP64), gpu.request(64, seed=74, z_target=80.0),
            gpu.request(32, seed=75, z_target=65.0), gpu.request(48, seed=76, z_target=70.0, sigma8=0.85)]
    srv = gpu.Server(workers=4, graphs=True)
    ids = [srv.submit(r) for r in reqs]
    srv.drain(180.0)
    got = {r["id"]: r for r in srv.poll()}
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["graph_cycles"] > 0
    for i, req in zip(ids, reqs):
        mix, alone = got[i], run_alone(gpu, req)
        assert mix["status"] == 0
        assert mix["cycles"] == alone["cycles"] and mix["a"] == alone["a"]
        for k in ("kbin", "power", "occupation"):
            assert np.array_equal(mix[k], alone[k]), (i, k)


def test_graph_cycles_radix3_and_line_walk_grids(gpu):
    """24^3 (radix-3 transforms) and 12^3 (the deposit's line walk): graph cycles give the
    same bits as direct ones."""
    for N in (24, 12):
        _, direct = new_sim(gpu, N, gpu.PREC_MIXED, seed=N)
        _, graph = new_sim(gpu, N, gpu.PREC_MIXED, seed=N)
        for _ in range(8):
            direct.step()
            graph.step_graph()
        assert_same_bits(direct, graph)
        assert graph.graph_info()[0] == 6
