"""bench.py's ensemble orchestration (run_ensemble) on the host, no GPU: the same 48
requests through the server three ways and through batched steps in one batch, one
batch per grid size and round-robin lanes, with a stand-in for the library's Python
binding whose simulations end after a number of cycles and with a power spectrum
that depend only on the request.  It checks the request mix the ensemble
configuration names, that every variant sees every request, and the comparisons the
bench line reports (cycles and P(k) against the server's, lanes against one batch)."""
import os
import sys
import threading
from types import SimpleNamespace

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _cycles(seed):
    return 110 + seed % 13


def _pw(seed, nb):
    return np.arange(1.0, nb + 1.0) * (1.0 + (seed % 5))


class FakeGpu:
    PREC_MIXED, PREC_FP64 = 1, 0

    def __init__(self):
        self.requests_seen = []
        self.batches = []
        self.lock = threading.Lock()

    def request(self, N, seed, z_target=0.0, prec=1, Omega_cdm=0.27, sigma8=0.81, n_s=0.96, numbins=32):
        return SimpleNamespace(N=N, seed=seed, z_target=z_target, prec=prec, Omega_cdm=Omega_cdm, Omega_b=0.05,
                               sigma8=sigma8, n_s=n_s, h=0.67, z_in=100.0, boxsize=2.5 * N, numbins=numbins)

    def Request(self, N, prec, boxsize, Omega_cdm, Omega_b, sigma8, n_s, h, z_in, z_target, seed, numbins):
        return SimpleNamespace(N=N, seed=seed, z_target=z_target, prec=prec, Omega_cdm=Omega_cdm, Omega_b=Omega_b,
                               sigma8=sigma8, n_s=n_s, h=h, z_in=z_in, boxsize=boxsize, numbins=numbins)

    def ic_params(self, boxsize, **kw):
        return dict(boxsize=boxsize, **kw)

    class Field:
        def zero(self):
            return self

    def prepare_source_tensor(self, phi, Tij, Sij, coeff):
        pass

    def fft_r2c(self, real, spec):
        spec.seed = real.seed

    def cross_spectrum(self, F, G, nb, deconvolve):
        return None, _pw(F.seed, nb), None, None, None

    def Context(self, N, prec):
        gpu = self

        class Ctx:
            def real(self, n):
                return FakeGpu.Field()

            def spectrum(self, n):
                return SimpleNamespace(seed=None)

            def stencil_shapes(self):
                return {"scalar": (256, 16), "tensor": (256, 16)}

        return Ctx()

    def Sim(self, ctx, n):
        class S:
            seed = None

            def ic_generate(self, **p):
                self.seed = p["seed"]

            def field(self, name):
                return SimpleNamespace(seed=self.seed)

        return S()

    def Server(self, workers=0, graphs=False, max_active=0):
        gpu = self

        class Srv:
            def __init__(self):
                self.reqs = []

            def submit(self, r):
                self.reqs.append(r)
                gpu.requests_seen.append(r.seed)
                gpu.last_requests = self.reqs
                return len(self.reqs)

            def drain(self, t):
                pass

            def poll(self, n):
                n3 = lambda r: float(r.N) ** 3  # noqa: E731
                return [{"id": i + 1, "status": 0, "N": r.N, "cycles": _cycles(r.seed), "a": 1.0 + 1e-3 * r.seed % 7,
                         "t_submit": 0.0,
                         "t_done": 1.0 + 0.01 * i,
                         "power": _pw(r.seed, r.numbins) / (n3(r) * n3(r) * 2. * np.pi * np.pi)}
                        for i, r in enumerate(self.reqs)]

            def stats(self):
                return {"max_active_seen": max_active or len(self.reqs), "workers": workers or 4,
                        "graph_cycles": 5000 if graphs else 0, "failed": 0}

            def close(self):
                pass

        return Srv()

    def Batch(self):
        gpu = self

        class B:
            def __init__(self):
                self.n = 0
                with gpu.lock:
                    gpu.batches.append(self)

            def run(self, sims, targets):
                assert len(sims) == len(targets) and all(t == 1.0 for t in targets)
                self.n += len(sims)
                return [_cycles(s.seed) for s in sims]

            def info(self):
                return (self.n * 100, self.n * 2, 55)

            def close(self):
                pass

        return B()


def test_run_ensemble_orchestration():
    gpu = FakeGpu()
    out = bench.run_ensemble(gpu, 1, lanes=(1, "size", 2))
    # the ensemble configuration: 16 simulations each at 64^3, 96^3, 128^3, distinct seeds
    assert out["simulations"] == 48
    assert len(gpu.requests_seen) == 3 * 48 and len(set(gpu.requests_seen)) == 48
    reqs = gpu.last_requests
    assert sorted(r.N for r in reqs) == [64] * 16 + [96] * 16 + [128] * 16
    assert all(r.boxsize == 2.5 * r.N and r.z_in == 100.0 and r.z_target == 0.0 for r in reqs)
    assert all(0.25 <= r.Omega_cdm <= 0.35 and 0.75 <= r.sigma8 <= 0.87 and 0.94 <= r.n_s <= 0.98 for r in reqs)
    b1 = out["batched_per_phase"]
    assert b1["simulations"] == 48 and b1["lanes"] == 1
    assert b1["same_cycles_as_server"] and b1["max_rel_pk_dev_vs_server"] == 0.0
    lanes = out["batched_per_phase_lanes"]
    assert [x["lanes"] for x in lanes] == [3, 2]
    assert lanes[0]["cohorts"] == "one lane per grid size"
    assert all(x["same_bits_as_one_lane"] for x in lanes)
    # every batch of a variant together ran every simulation once
    assert sum(b.n for b in gpu.batches) == 48 * 3
    assert out["graph_cycles"]["graph_cycles"] == 5000 and out["graph_cycles"]["same_bits_as_direct"]
    assert set(out["stencil_shapes"]) == {"64", "96", "128"}


def test_run_serve_assembles_the_serving_object():
    """run_serve with a short window of Poisson arrivals, a burst of four and the same
    burst in the plain FP64 form one at a time; the serving object carries the
    percentiles, the capacity ratio and the ensemble."""
    gpu = FakeGpu()
    args = SimpleNamespace(seed=1, serve_rate=40.0, serve_seconds=0.25, serve_burst=4)
    out = bench.run_serve(args, gpu)
    assert out["completed"] >= 1 and out["failed"] == 0
    assert 0.0 < out["p50_s"] <= out["p99_s"] <= out["max_s"]
    assert out["burst"]["requests"] == 4 and out["sequential_fp64"]["requests"] == 4
    assert out["capacity_vs_sequential_fp64"] > 0.0
    assert out["ensemble"]["simulations"] == 48 and out["ensemble"]["batched_per_phase"]["same_cycles_as_server"]
