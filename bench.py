"""Benchmark of the per-step particle-mesh hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--grid 512] [--prec mixed|fp64]
    python bench.py --op NAME [--grid N] ...      one operation, for profiler captures

Workload (default): the precision form at 512^3 grid and 512^3 particles in a
1 Gpc/h box (FP32 fields and FFTs, FP64 positions, int64 fixed-point
deposits), seeded BBKS Zel'dovich initial conditions at z = 100 generated on
the device, GR mode with phi, chi, B_i and T_ij active (parabolic vector
method), run to z = 0 as gevolution's main loop runs it (main.cpp:372-879; the
loop ends at the first cycle whose a has passed 1, main.cpp:639-692).  A step
is one cycle: the T00 and Tij deposits, the phi / chi / B solves with 12 FFTs,
the kick, the drift with the relink and the background update.  Metric:
particle-steps/s.

value        device-timed throughput with the state resident in HBM: the LAST K
             cycles before z = 0 (clustered particles), after untimed evolution
             from z = 100; CUDA events on the library's stream between two
             synchronised barriers.  full_run gives the mean over every cycle of
             the run, early_cycles the first K.
e2e          the same K cycles through the C-ABI with the particle state copied
             in from pinned host memory and back out every cycle.
kernels      each kernel's device time in the timed cycles (CUDA events the
             library records around its launches, gev_ctx_set_timing), its
             algorithmic bytes and fraction of the measured HBM bandwidth;
             roofline is the largest of them.
phases_gpu / cpu_baseline.phases   time per cycle in the layout of main.cpp's
             BENCHMARK breakdown (main.cpp:907-922).
pk_check     the precision form against the plain FP64 form from the same seeded
             IC, z = 100 -> 0: per-bin power deviation of phi, chi, B and delta at
             every Pk redshift up to k_Nyquist / 2 (criterion 1e-3), the rms
             difference of the final positions (particles matched by ID), and the
             FP64 form's throughput over the same cycles.
cpu_baseline the CPU restatement of the path (oracle/, FP64, OpenMP on all host
             threads) on a bounded sample of the workload: a 256^3 simulation in
             a 500 Mpc/h box (the 512^3 run's cell size and particle density).

--impl reference runs that CPU implementation of the path alone (the oracle's
port of the reference; the reference itself needs LATfield2, FFTW, MPI and
HDF5, which the GPU hosts do not have), one cycle of the 256^3 sample per step,
and prints the same metric.  With --gpus N > 1 each rank runs its own
simulation (replicas, no data exchange); the value is the sum over ranks of
particles x steps divided by the slowest rank's time.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "gevolution-1.2_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0
PK_REDSHIFTS = (10.0, 3.0, 1.0, 0.5, 0.0)
PK_BINS = 64
CPU_SAMPLE_GRID, CPU_SAMPLE_BOX = 256, 500.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--grid", type=int, default=512)
    ap.add_argument("--prec", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-hbm-fit", action="store_true", help="skip the 1024^3 HBM-fit demonstration")
    ap.add_argument("--no-pk-check", action="store_true", help="skip the FP64-form run and spectrum comparison")
    ap.add_argument("--serve-seconds", type=float, default=120.0,
                    help="length of the serving run's Poisson arrivals (0: no serving measurement)")
    ap.add_argument("--serve-rate", type=float, default=2.0, help="serving requests per second")
    ap.add_argument("--serve-burst", type=int, default=24, help="requests submitted at once for the capacity run")
    ap.add_argument("--op", default=None,
                    help="one operation instead of the benchmark: prepare, cycle, table, r2c_alone, c2r_alone, "
                         "fft_axis_y, fft_axis_z, ensemble, batch_cycle")
    ap.add_argument("--reps", type=int, default=3, help="--op: timed calls")
    ap.add_argument("--z-op", type=float, default=0.0,
                    help="--op prepare / table: evolve from z = 100 until this redshift first")
    ap.add_argument("--state", default=None,
                    help="--op prepare: hibernation file to write; cycle / table: to restart from")
    return ap.parse_args()


def reduce_max_ms(ms, world, device):
    """The slowest rank's time: every rank's timed region ends at a barrier and the
    maximum over ranks is what the aggregate is measured against."""
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def aggregate_value(N, steps, world, ms_max):
    """Whole-job particle-steps/s: every rank advances its own N^3 replica (replicas
    only, weak scaling) for `steps` cycles within the slowest rank's time."""
    return float(N) ** 3 * steps * world / (ms_max / 1e3)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def replica_seed(base, rank):
    """The seed of rank `rank`'s replica: every rank runs an independent simulation."""
    return base + 1000 * rank


# ------------------------------------------------------------ clocks --------
class ClockSampler:
    """nvidia-smi sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def hbm_peak():
    try:
        with open(PEAKS) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


# ------------------------------------------------- the cycle schedule --------
def _hconf(a, fourpiG, c):
    # background.hpp:137-140 without ncdm and fluid terms, as the library's host code
    return math.sqrt((2. * fourpiG / 3.) * (((c["Omega_cdm"] + c["Omega_b"]) / a) + (c["Omega_Lambda"] * a * a) +
                                            (c["Omega_rad"] / a / a)))


def _rk4bg(a, fourpiG, c, dtau):
    # background.hpp:167-177
    k1 = a * _hconf(a, fourpiG, c)
    k2 = (a + k1 * dtau / 2.) * _hconf(a + k1 * dtau / 2., fourpiG, c)
    k3 = (a + k2 * dtau / 2.) * _hconf(a + k2 * dtau / 2., fourpiG, c)
    k4 = (a + k3 * dtau) * _hconf(a + k3 * dtau, fourpiG, c)
    return a + dtau * (k1 + 2. * k2 + 2. * k3 + k4) / 6.


def full_cycles_to(st, N, z_end=0.0):
    """Cycles the main loop completes before it ends at z_end: a(tau) and dtau follow
    from the background alone (main.cpp:792-872), so the count is known up front.
    The loop ends in the fields part of the first cycle whose a has passed 1/(1+z_end)."""
    a, dtau = st["a"], st["dtau"]
    dx = 1.0 / N
    n = 0
    while not (1.0 / a < z_end + 1.0):
        a = _rk4bg(_rk4bg(a, st["fourpiG"], st["cosmo"], 0.5 * dtau), st["fourpiG"], st["cosmo"], 0.5 * dtau)
        H = _hconf(a, st["fourpiG"], st["cosmo"])
        dtau = st["Cf"] * dx if st["Cf"] * dx < st["steplimit"] / H else st["steplimit"] / H
        n += 1
    return n


# ------------------------------------------------- algorithmic bytes --------
def cycle_bytes(N, prec):
    """Compulsory HBM bytes of one cycle (every persistent or intermediate array read
    or written once per use, each 3-D FFT at its three-pass minimum), with r the real
    size of the form and a half-spectrum component of about r bytes a cell:
      particles: the deposit reads pos + q, the kick+drift reads and writes them
                 (ID, cell keys and the relink excluded): 3 (3*8 + 3*r) a particle;
      fields a cell: T00 + 6 Tij written 7r; phi read by the deposit r; scalar solve
                 3r read, half spectrum r, z pass with the Poisson factor 2r, c2r 2r;
                 tensor: phi + Sij read 7r, SijFT 6r, the k-space pass reads 6r + 3r
                 and writes r + 3r, the c2r reads 4r and writes 4r; the kick+drift
                 reads phi, chi and B 5r.
    Mixed form (r = 4): 108 B a particle + 220 B a cell = 328 B a particle-step.
    FP64 form (r = 8): 144 + 440 = 584 (the same terms; the 544 often quoted for it
    leaves out the kick's field reads)."""
    r = 8 if prec == "fp64" else 4
    per_particle = 3 * (3 * 8 + 3 * r)
    per_cell = r * (7 + 1 + (3 + 1 + 2 + 2) + (7 + 6 + 9 + 4 + 8) + 5)
    return (per_particle + per_cell) * N ** 3, per_particle, per_cell


def kernel_alg_bytes(name, N, prec, n=None):
    """Algorithmic bytes of one launch of a kernel of the cycle (the terms of
    cycle_bytes that the kernel covers); None for bookkeeping kernels (the relink,
    scales, sums), which move no bytes the path itself requires."""
    r = 8 if prec == "fp64" else 4
    C = N ** 3
    n = C if n is None else n
    K = N * N * (N // 2 + 1) * 2 * r  # one half-spectrum component
    table = {
        "k_kick_drift": n * 2 * (3 * 8 + 3 * r) + C * 5 * r,
        "k_dep_gather": n * (3 * 8 + 3 * r) + C * 8 * r,
        "k_cube_fp64+k_gather": n * (3 * 8 + 3 * r) + C * 8 * r,
        "k_fft_cols_reg": 2 * K,
        "k_fft_cols": 2 * K,
        "k_fft_r2c_rows_reg": C * r + K,
        "k_fft_r2c_rows": C * r + K,
        "k_fft_c2r_rows_reg": C * r + K,
        "k_fft_c2r_rows": C * r + K,
        "k_source_tensor": C * 13 * r,
        "k_source_scalar": C * 4 * r,
        "k_project_evolve": 13 * K,
        "k_poisson": 2 * K,
    }
    return table.get(name)


# DRAM traffic per launch (dram__bytes_read.sum + dram__bytes_write.sum) from ncu
# --set full captures at late time, keyed by (kernel, grid, precision): the 256^3
# mixed simulation (500 Mpc/h, the 512^3 workload's cell size) evolved to z = 0.28
# and restarted from its hibernation file (bench.py --op prepare / --op cycle), the
# second cycle's launch.  Particles and cells both grow as N^3, so the 512^3 entry is
# the 256^3 capture times 8.
_LATE_256 = {
    "k_dep_gather": 0.884165e9 + 0.526542e9,
    "k_fx_prep": 0.404148e9 + 0.747557e9,
    "k_dense_sums": 0.281905e9 + 0.050591e9,
}
KERNEL_TRAFFIC = {}
for _k, _v in _LATE_256.items():
    KERNEL_TRAFFIC[(_k, 256, "mixed")] = _v
    KERNEL_TRAFFIC[(_k, 512, "mixed")] = 8 * _v


# ------------------------------------------------------------ our arm --------
def _events(torch, n):
    return [torch.cuda.Event(enable_timing=True) for _ in range(n)]


def run_ours(args, rank, world, local):
    import torch
    import gev_gb300 as gpu

    torch.cuda.set_device(local)
    N = args.grid
    prec = gpu.PREC_FP64 if args.prec == "fp64" else gpu.PREC_MIXED
    box = 1000.0 * N / 512
    seed = replica_seed(args.seed, rank)
    ctx = gpu.Context(N, prec, device=local)
    sim = gpu.Sim(ctx, N ** 3)
    sim.ic_generate(**gpu.ic_params(box, seed=seed))
    st0 = sim.state()
    n_full = full_cycles_to(st0, N)
    K = args.steps
    n_pre = max(n_full - K, args.warmup)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device("cuda", local))
    # untimed evolution from z = 100, one event after every cycle for the full-run mean
    ev = _events(torch, n_pre + 1)
    ev[0].record(stream)
    for c in range(n_pre):
        sim.step()
        ev[c + 1].record(stream)
    ctx.sync()
    a_start = sim.state()["a"]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    ctx.timing(reset=True)
    ctx.set_timing(True)
    e0, e1 = _events(torch, 2)
    l0 = ctx.launches()
    e0.record(stream)
    for _ in range(K):
        sim.step()
    e1.record(stream)
    e1.synchronize()
    launches = ctx.launches() - l0
    ms = e0.elapsed_time(e1)
    clk = clocks.stop()
    ctx.set_timing(False)
    kt = ctx.timing(reset=True)
    torch.cuda.synchronize()
    ms_max = reduce_max_ms(ms, world, "cuda")
    value = aggregate_value(N, K, world, ms_max)
    st = sim.state()
    pre_ms = ev[0].elapsed_time(ev[-1])
    k_early = min(K, n_pre)
    full = {"cycles": n_pre + K, "ms_per_step": (pre_ms + ms) / (n_pre + K),
            "value": N ** 3 * (n_pre + K) / ((pre_ms + ms) / 1e3), "z_end": 1.0 / st["a"] - 1.0}
    early = {"cycles": "0..%d" % (k_early - 1), "ms_per_step": ev[0].elapsed_time(ev[k_early]) / k_early}
    early["value"] = N ** 3 / (early["ms_per_step"] / 1e3)
    kernels, phases, roof = kernel_table(kt, K, ms / K, N, args.prec)
    tiles = ctx.fft_tiles()
    tiles["stencils"] = ctx.stencil_shapes()
    timed = {"first": n_pre, "last": n_pre + K - 1, "of": n_full, "z_from": 1.0 / a_start - 1.0,
             "z_to": 1.0 / st["a"] - 1.0}
    cufft = fft_vs_cufft(gpu, ctx, stream, N, args.prec, torch) if world == 1 else None
    del sim, ctx, stream
    torch.cuda.synchronize()
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(gpu, N, prec, box, seed, n_pre, K, local, torch)
    pk = None
    if not args.no_pk_check and prec == gpu.PREC_MIXED and world == 1:
        pk = pk_check_z0(gpu, N, box, args.seed, K, local, torch)
    e2e2 = None
    if not args.no_e2e and world == 1:
        e2e2 = run_e2e_two_sims(gpu, N, args.steps, box, local, torch)
    serve = None
    if args.serve_seconds > 0 and world == 1:
        serve = run_serve(args, gpu)
    hbm = None
    if not args.no_hbm_fit and world == 1 and prec == gpu.PREC_MIXED and N == 512:
        hbm = run_hbm_fit(gpu, local, torch)
    return dict(value=value, ms=ms_max / K, launches=launches, tiles=tiles, clocks=clk, state=st, roofline=roof,
                kernels=kernels, phases=phases, full=full, early=early, timed=timed, cufft=cufft, e2e=e2e, e2e2=e2e2,
                box=box, pk=pk, serve=serve, hbm=hbm)


PHASE_KEYS = (("projections", "phase:projections"), ("gravity solver", "phase:gravity solver"),
              ("thereof FFTs", "phase:fft"), ("update momenta + move particles (one fused pass with the relink)",
                                               "phase:update particles"))


def kernel_table(kt, cycles, ms_cycle, N, prec):
    """Per-kernel device time of the timed cycles with its algorithmic bytes and HBM
    fraction; the per-phase breakdown; the roofline object of the largest kernel."""
    peak, kind = hbm_peak()
    rows = {}
    for name, (cnt, tot) in kt.items():
        if name.startswith("phase:"):
            continue
        alg = kernel_alg_bytes(name, N, prec)
        per = tot / cnt
        row = {"launches_per_step": cnt / cycles, "ms_per_step": tot / cycles, "share": tot / cycles / ms_cycle,
               "ms_per_launch": per}
        if alg:
            row["alg_bytes_per_launch"] = alg
            row["achieved_gbs"] = alg / (per / 1e3) / 1e9
            row["frac"] = row["achieved_gbs"] / peak
        rows[name] = row
    phases = {label: kt[key][1] / cycles for label, key in PHASE_KEYS if key in kt}
    top = max(rows, key=lambda k: rows[k]["ms_per_step"]) if rows else None
    roof = None
    if top:
        r = rows[top]
        alg = kernel_alg_bytes(top, N, prec)
        achieved = alg / (r["ms_per_launch"] / 1e3) / 1e9 if alg else None
        traffic = KERNEL_TRAFFIC.get((top, N, prec))
        roof = {"kernel": top, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak if achieved else None, "traffic": traffic, "peak_kind": kind,
                "ms_per_launch": r["ms_per_launch"], "alg_bytes": alg,
                "share_of_cycle": r["share"],
                "timing": "CUDA events around each launch on the library's stream, over the timed cycles"}
    return rows, phases, roof


def fft_vs_cufft(gpu, ctx, stream, N, prec, torch, reps=5):
    """One component's 3-D r2c and c2r, the library's own FFT against NVIDIA's cuFFT
    (through torch.fft) on the same grid and precision.  CUDA events on each one's
    stream, after a warm-up call (plan creation), mean of reps.  cuFFT's inverse runs
    unnormalised (norm="forward"), as the library's c2r does; its c2r may overwrite
    its input, so torch works on a copy, where the library's keeps its input."""
    import numpy as np
    rng = np.random.default_rng(3)
    real, spec = ctx.real(1), ctx.spectrum(1)
    real.upload(rng.standard_normal(real.shape))

    def timed(fn, st):
        fn()
        torch.cuda.synchronize()
        e0, e1 = _events(torch, 2)
        e0.record(st)
        for _ in range(reps):
            fn()
        e1.record(st)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    ours_r2c = timed(lambda: gpu.fft_r2c(real, spec), stream)
    ours_c2r = timed(lambda: gpu.fft_c2r(spec, real), stream)
    del real, spec
    dt = torch.float64 if prec == "fp64" else torch.float32
    x = torch.randn((N, N, N), dtype=dt, device="cuda")
    cur = torch.cuda.current_stream()
    cu_r2c = timed(lambda: torch.fft.rfftn(x), cur)
    y = torch.fft.rfftn(x)
    cu_c2r = timed(lambda: torch.fft.irfftn(y, s=(N, N, N), norm="forward"), cur)
    del x, y
    torch.cuda.empty_cache()
    return {"grid": N, "precision": prec, "ours_r2c_ms": ours_r2c, "cufft_r2c_ms": cu_r2c, "ours_c2r_ms": ours_c2r,
            "cufft_c2r_ms": cu_c2r, "library": "cuFFT via torch.fft (torch %s)" % torch.__version__}


def run_e2e(gpu, N, prec, box, seed, n_pre, K, device, torch):
    """The timed cycles again through the public C-ABI with host buffers: a fresh
    simulation from the same IC evolves untimed to the same cycle, then each of the
    K cycles uploads the particle records from pinned host memory, runs the cycle
    and downloads the records into pinned host memory (waiting for them)."""
    ctx = gpu.Context(N, prec, device=device)
    sim = gpu.Sim(ctx, N ** 3)
    sim.ic_generate(**gpu.ic_params(box, seed=seed))
    for _ in range(n_pre):
        sim.step()
    pcls = sim.particles()
    n = N ** 3
    host = torch.empty(n * 56, dtype=torch.uint8, pin_memory=True)
    arr = host.numpy().view(gpu.PART)
    back = torch.empty(n * 56, dtype=torch.uint8, pin_memory=True)
    barr = back.numpy().view(gpu.PART)
    pcls.download(out=arr)
    ctx.sync()
    t0 = time.perf_counter()
    for _ in range(K):
        pcls.upload(arr)
        sim.step()
        pcls.download(out=barr)  # into pinned memory; synchronises the stream
        arr, barr = barr, arr
    dt = time.perf_counter() - t0
    del sim, ctx, host, back
    torch.cuda.synchronize()
    return {"value": n * K / dt, "unit": "particle-steps/s", "h2d_bytes_per_step": n * 56,
            "d2h_bytes_per_step": n * 56, "cycles": "the same late cycles as value, host wall clock"}


def _spectra(gpu, ctx, sim, nb):
    """The parity tables of writeSpectra (output.hpp:1762-2204, CDM in GR): phi and chi
    (r2c, no deconvolution), B (BiFT), delta (projection_T00_project with phi, r2c,
    CIC deconvolution)."""
    st = sim.state()
    out = {}
    for name in ("phi", "chi"):
        sp = ctx.spectrum(1)
        gpu.fft_r2c(sim.field(name), sp)
        out[name] = gpu.cross_spectrum(sp, numbins=nb, deconvolve=False)
    out["B"] = gpu.cross_spectrum(sim.field("BiFT"), numbins=nb, deconvolve=False)
    T = ctx.real(1)
    gpu.projection_T00(sim.particles(), T, st["a"], sim.field("phi"))
    sp = ctx.spectrum(1)
    gpu.fft_r2c(T, sp)
    out["delta"] = gpu.cross_spectrum(sp, numbins=nb, deconvolve=True)
    return out


def run_to_z0_with_spectra(gpu, ctx, sim, stream, torch, nb=PK_BINS):
    """gevolution's loop to z = 0 with the spectra where main.cpp takes them
    (main.cpp:639-692): after the field solves of the first cycle past each Pk
    redshift; ends after the last.  Returns (records, device ms of each full cycle,
    spectra excluded)."""
    out, cyc_ms = [], []
    k = 0
    while True:
        e = _events(torch, 4)
        e[0].record(stream)
        sim.step_fields()
        e[1].record(stream)
        a = sim.state()["a"]
        if 1.0 / a < PK_REDSHIFTS[k] + 1.0:
            rec = {"z": PK_REDSHIFTS[k], "a": a}
            rec.update(_spectra(gpu, ctx, sim, nb))
            out.append(rec)
            k += 1
            if k == len(PK_REDSHIFTS):
                return out, cyc_ms
        e[2].record(stream)
        sim.step_particles()
        e[3].record(stream)
        e[3].synchronize()
        cyc_ms.append(e[0].elapsed_time(e[1]) + e[2].elapsed_time(e[3]))


def _by_id(gpu, sim, n):
    import numpy as np
    p = sim.particles().download()
    pos = np.empty((n, 3))
    pos[p["ID"]] = p["pos"]
    return pos


def pk_check_z0(gpu, N, box, seed, K, device, torch):
    """The precision form against the plain FP64 form, both from device IC of the same
    seed at z = 100, run to z = 0: per-bin power deviations up to k_Nyquist / 2 at every
    Pk redshift, the rms difference of the final positions (particles matched by ID),
    and both forms' device-timed throughput over the last K cycles and the whole run."""
    import numpy as np
    runs = {}
    for name, prec in (("mixed", gpu.PREC_MIXED), ("fp64", gpu.PREC_FP64)):
        ctx = gpu.Context(N, prec, device=device)
        sim = gpu.Sim(ctx, N ** 3)
        sim.ic_generate(**gpu.ic_params(box, seed=seed))
        pos0 = _by_id(gpu, sim, N ** 3) if name == "fp64" else None
        stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device("cuda", device))
        recs, cyc = run_to_z0_with_spectra(gpu, ctx, sim, stream, torch)
        pos = _by_id(gpu, sim, N ** 3)
        runs[name] = (recs, cyc, pos, pos0)
        del sim, ctx, stream
        torch.cuda.synchronize()
    (r32, c32, p32, _), (r64, c64, p64, p0) = runs["mixed"], runs["fp64"]
    kmax = 0.5 * np.pi * N
    dev, ok = {}, True
    for a, b in zip(r32, r64):
        row = {}
        for name in ("phi", "chi", "B", "delta"):
            kb, p, occ = b[name][0], b[name][1], b[name][4]
            m = (occ > 0) & (kb <= kmax)
            row[name] = float(np.max(np.abs(a[name][1][m] - p[m]) / np.abs(p[m])))
            ok = ok and row[name] <= 1e-3
        dev["z=%g" % b["z"]] = row
    d = p32 - p64
    d -= np.round(d)
    d *= N
    disp = p64 - p0
    disp -= np.round(disp)
    disp *= N
    rms = float(np.sqrt((d ** 2).sum(axis=1).mean()))
    rms_disp = float(np.sqrt((disp ** 2).sum(axis=1).mean()))

    def form(cyc):
        last = cyc[-K:]
        return {"value": N ** 3 * len(last) / (sum(last) / 1e3), "ms_per_step": sum(last) / len(last),
                "full_run_ms_per_step": sum(cyc) / len(cyc), "cycles": len(cyc)}

    f64, f32 = form(c64), form(c32)
    return {"fp64_form": dict(f64, unit="particle-steps/s",
                              note="the same last %d cycles before z = 0, CUDA events around each cycle" % K),
            "pk_check": {"against": "the FP64 form on the GPU, device IC of the same seed at z = 100, run to z = 0",
                         "numbins": PK_BINS, "k_max": "k_Nyquist/2", "pk_redshifts": list(PK_REDSHIFTS),
                         "max_rel_dev": dev, "tolerance": 1e-3, "pass": ok,
                         "rms_position_difference_cells": rms, "max_position_difference_cells": float(np.abs(d).max()),
                         "rms_displacement_since_ic_cells": rms_disp,
                         "mixed_over_fp64_speed": f32["value"] / f64["value"],
                         "mixed_form_same_loop": f32}}


# ------------------------------------------------------------ serving --------
SERVE_SIZES = (64, 96, 128, 192, 256)
SERVE_Z = (1.0, 0.5, 0.0)


def serve_requests(gpu, rng, n, first_seed, prec=None):
    """Requests of the serving workload: grid drawn from SERVE_SIZES, box 2.5 N Mpc/h,
    Omega_cdm U[0.25, 0.35], sigma8 U[0.75, 0.87], n_s U[0.94, 0.98], target
    redshift from SERVE_Z, BBKS Zel'dovich IC at z = 100, distinct seeds."""
    out = []
    for k in range(n):
        N = int(rng.choice(SERVE_SIZES))
        out.append(gpu.request(N, seed=first_seed + k, z_target=float(rng.choice(SERVE_Z)),
                               Omega_cdm=float(rng.uniform(0.25, 0.35)), sigma8=float(rng.uniform(0.75, 0.87)),
                               n_s=float(rng.uniform(0.94, 0.98)), prec=gpu.PREC_MIXED if prec is None else prec))
    return out


def as_fp64(gpu, req):
    """The same simulation request in the plain FP64 form."""
    return gpu.Request(req.N, gpu.PREC_FP64, req.boxsize, req.Omega_cdm, req.Omega_b, req.sigma8, req.n_s, req.h,
                       req.z_in, req.z_target, req.seed, req.numbins)


def run_serve(args, gpu):
    """The serving loop under load: Poisson arrivals at --serve-rate for
    --serve-seconds (time to result p50 / p99, sustained sims/hour), then a burst of
    --serve-burst requests at once (capacity), against the same burst run one request
    at a time in the plain FP64 form on the same GPU (a server with one slot)."""
    import numpy as np
    rng = np.random.default_rng(args.seed + 77)
    n_poisson = max(1, int(args.serve_seconds * args.serve_rate * 1.5) + 8)
    reqs = serve_requests(gpu, rng, n_poisson, 100000)
    srv = gpu.Server()
    t_start = time.perf_counter()
    t_next, sent = 0.0, 0
    while True:
        t_next += float(rng.exponential(1.0 / args.serve_rate))
        if t_next > args.serve_seconds or sent == len(reqs):
            break
        dt = t_start + t_next - time.perf_counter()
        if dt > 0:
            time.sleep(dt)
        srv.submit(reqs[sent])
        sent += 1
    srv.drain(900.0)
    res = [r for r in srv.poll(100000) if r["status"] == 0]
    st = srv.stats()
    srv.close()
    lat = sorted(r["t_done"] - r["t_submit"] for r in res)
    span = max(r["t_done"] for r in res) - min(r["t_submit"] for r in res)
    # capacity: a burst of requests at once
    burst = serve_requests(gpu, rng, args.serve_burst, 200000)
    srv = gpu.Server()
    for r in burst:
        srv.submit(r)
    srv.drain(900.0)
    bres = [r for r in srv.poll(100000) if r["status"] == 0]
    bst = srv.stats()
    srv.close()
    b_span = max(r["t_done"] for r in bres) - min(r["t_submit"] for r in bres)
    # the same burst in the plain FP64 form, one request at a time
    srv = gpu.Server(max_active=1)
    t0 = time.perf_counter()
    for r in burst:
        srv.submit(as_fp64(gpu, r))
    srv.drain(1800.0)
    sall = srv.poll(100000)
    sres = [r for r in sall if r["status"] == 0]
    sfail = [{"N": r["N"], "status": r["status"]} for r in sall if r["status"] != 0]
    s_span = time.perf_counter() - t0
    srv.close()
    cap = len(bres) / b_span * 3600.0
    seq_rate = len(sres) / s_span * 3600.0
    pct = lambda q: lat[min(len(lat) - 1, int(round(q * (len(lat) - 1))))]  # noqa: E731
    return {
        "precision": "mixed", "arrivals": "Poisson %.3g/s for %.3g s" % (args.serve_rate, args.serve_seconds),
        "sizes": list(SERVE_SIZES), "z_target": list(SERVE_Z), "completed": len(res), "failed": st["failed"],
        "p50_s": pct(0.50), "p99_s": pct(0.99), "max_s": lat[-1],
        "sims_per_hour_offered_load": len(res) / span * 3600.0,
        "max_active_seen": st["max_active_seen"],
        "burst": {"requests": len(bres), "makespan_s": b_span, "sims_per_hour": cap,
                  "max_active_seen": bst["max_active_seen"]},
        "sequential_fp64": {"requests": len(sres), "failed": sfail, "makespan_s": s_span, "sims_per_hour": seq_rate,
                            "note": "the burst's own requests in the plain FP64 form, run one at a time (a server "
                                    "with one slot) on the same GPU"},
        "capacity_vs_sequential_fp64": cap / seq_rate,
        "ensemble": run_ensemble(gpu, args.seed),
    }


def run_ensemble(gpu, seed, lanes=(1, "size")):
    """The batched ensemble: 16 simulations each at 64^3, 96^3 and 128^3, box 2.5 N,
    Omega_cdm U[0.25, 0.35], sigma8 U[0.75, 0.87], n_s U[0.94, 0.98], distinct seeds,
    all to z = 0, admitted at once.  Run four ways on the same requests: through the
    server with cycles enqueued directly by the default scheduler threads, the same
    with each cycle enqueued as one CUDA graph, and with one scheduler thread; and in
    batched steps (gev_batch_run: one launch per kernel of a cycle for each grid
    size's cohort of 16)."""
    import numpy as np
    rng = np.random.default_rng(seed + 301)
    ens = []
    for k, N in enumerate([64] * 16 + [96] * 16 + [128] * 16):
        ens.append(gpu.request(N, seed=300000 + k, z_target=0.0, Omega_cdm=float(rng.uniform(0.25, 0.35)),
                               sigma8=float(rng.uniform(0.75, 0.87)), n_s=float(rng.uniform(0.94, 0.98)),
                               prec=gpu.PREC_MIXED))

    def ensemble(workers, graphs):
        srv = gpu.Server(workers=workers, graphs=graphs)
        ids = [srv.submit(r) for r in ens]
        srv.drain(900.0)
        got = {r["id"]: r for r in srv.poll(100000)}
        stats = srv.stats()
        srv.close()
        res = [got[i] for i in ids if i in got and got[i]["status"] == 0]
        span = max(r["t_done"] for r in res) - min(r["t_submit"] for r in res)
        steps = sum(float(r["N"]) ** 3 * r["cycles"] for r in res)
        return res, stats, {"simulations": len(res), "makespan_s": span, "particle_steps_per_s": steps / span,
                            "max_active_seen": stats["max_active_seen"], "scheduler_threads": stats["workers"]}

    shapes = {}
    for N in (64, 96, 128):  # the launch shapes the stencil tuner picks for each size
        ctx = gpu.Context(N, gpu.PREC_MIXED)
        phi, Tij = ctx.real(1), ctx.real(6)
        gpu.prepare_source_tensor(phi.zero(), Tij.zero(), Tij, 1e-3)
        shapes[str(N)] = ctx.stencil_shapes()
        del phi, Tij, ctx
    def ensemble_batched(lanes=1):
        # the same requests advanced by gev_batch_run: one launch per kernel of a cycle for
        # each grid size's cohort; contexts and initial conditions made by four host
        # threads; timed from the first context to the last result's spectrum, as the
        # server runs are.  lanes > 1: the requests dealt round-robin to that many batches,
        # each run by its own host thread, so that the lanes' cohorts drift out of step and
        # different phases of the cycle share the GPU
        from concurrent.futures import ThreadPoolExecutor

        def make(r):
            c = gpu.Context(r.N, gpu.PREC_MIXED)
            sim = gpu.Sim(c, r.N ** 3)
            sim.ic_generate(**gpu.ic_params(r.boxsize, seed=r.seed, z_in=r.z_in, Omega_cdm=r.Omega_cdm,
                                            Omega_b=r.Omega_b, sigma8=r.sigma8, n_s=r.n_s, h=r.h))
            return c, sim

        t0 = time.perf_counter()
        with ThreadPoolExecutor(4) as ex:
            runs = list(ex.map(make, ens))
        # lanes == "size": one batch per grid size, so that no cohort waits for another's steps
        sizes = sorted({r.N for r in ens})
        if lanes == "size":
            lane_of = [sizes.index(r.N) for r in ens]
            lanes = len(sizes)
        else:
            lane_of = [k % lanes for k in range(len(ens))]
        batches = [gpu.Batch() for _ in range(lanes)]

        def run_lane(li):
            ks = [k for k in range(len(ens)) if lane_of[k] == li]
            cyc = batches[li].run([runs[k][1] for k in ks], [1.0 / (1.0 + ens[k].z_target) for k in ks])
            return dict(zip(ks, cyc))

        cycles = [0] * len(ens)
        with ThreadPoolExecutor(lanes) as ex:
            for part in ex.map(run_lane, range(lanes)):
                for k, c in part.items():
                    cycles[k] = c
        powers = []
        for (c, sim), r in zip(runs, ens):
            F = c.spectrum(1)
            gpu.fft_r2c(sim.field("phi"), F)
            _, pw, _, _, _ = gpu.cross_spectrum(F, None, r.numbins, False)
            n3 = float(r.N) ** 3
            powers.append(pw / (n3 * n3 * 2. * np.pi * np.pi))
        span = time.perf_counter() - t0
        info = [b.info() for b in batches]
        steps = sum(float(r.N) ** 3 * k for r, k in zip(ens, cycles))
        for b in batches:
            b.close()
        del runs
        return cycles, powers, {"simulations": len(ens), "lanes": lanes, "makespan_s": span,
                                "particle_steps_per_s": steps / span, "cycles_batched": sum(i[0] for i in info),
                                "cycles_direct": sum(i[1] for i in info), "batched_launches": sum(i[2] for i in info),
                                "cohorts": ("one lane per grid size" if len(set(lane_of)) == len(sizes) and all(
                                    lane_of[k] == sizes.index(ens[k].N) for k in range(len(ens)))
                                            else "per lane: 64^3, 96^3 and 128^3, %d simulations each" % (16 // lanes))}

    res_d, _, direct = ensemble(0, False)
    res_g, st_g, graph = ensemble(0, True)
    _, _, one = ensemble(1, False)
    cyc_b, pow_b, batched = ensemble_batched()
    more_lanes = []
    for nl_ in lanes[1:]:
        cyc_l, pow_l, bl = ensemble_batched(nl_)
        bl["same_bits_as_one_lane"] = cyc_l == cyc_b and all(np.array_equal(a, b) for a, b in zip(pow_l, pow_b))
        more_lanes.append(bl)
    # against the server's (direct) cycles: the same cycle counts, P(k) of phi to FP32
    # rounding (the batched kernels are compiled apart and may fuse multiply-adds
    # differently)
    batched["same_cycles_as_server"] = len(res_d) == len(ens) and all(
        a["cycles"] == k for a, k in zip(res_d, cyc_b))
    batched["max_rel_pk_dev_vs_server"] = max(
        float(np.max(np.abs(pw - a["power"]) / np.abs(a["power"]))) for a, pw in zip(res_d, pow_b))
    graph["graph_cycles"] = st_g["graph_cycles"]
    graph["same_bits_as_direct"] = len(res_g) == len(res_d) and all(
        a["cycles"] == b["cycles"] and a["a"] == b["a"] and np.array_equal(a["power"], b["power"])
        for a, b in zip(res_d, res_g))
    out = {"sizes": "16 x 64^3, 16 x 96^3, 16 x 128^3, z = 100 -> 0",
           "cuda_device_max_connections": os.environ.get("CUDA_DEVICE_MAX_CONNECTIONS"),
           "stencil_shapes": shapes}
    out.update(direct)
    out["graph_cycles"] = graph
    out["batched_per_phase"] = batched
    out["batched_per_phase_lanes"] = more_lanes
    out["one_scheduler_thread"] = one
    return out


def run_hbm_fit(gpu, device, torch, N=1024, steps=2):
    """The 1024^3 HBM-fit demonstration of the precision form: 1024^3 particles on a
    1024^3 grid in a 2 Gpc/h box, device initial conditions at z = 100, one warm-up
    cycle and `steps` timed cycles.  Reports the device bytes the simulation holds
    against the GPU's memory; a simulation that does not fit is reported, not raised."""
    free0, total = torch.cuda.mem_get_info(device)
    out = {"grid": N, "particles": N ** 3, "box_mpc_h": 2000.0, "gpu_bytes": total, "free_bytes_before": free0}
    try:
        ctx = gpu.Context(N, gpu.PREC_MIXED, device=device)
        sim = gpu.Sim(ctx, N ** 3)
        t0 = time.perf_counter()
        sim.ic_generate(**gpu.ic_params(2000.0, seed=11))
        ctx.sync()
        out["ic_s"] = time.perf_counter() - t0
        sim.step()
        ctx.sync()
        stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device("cuda", device))
        e0, e1 = _events(torch, 2)
        e0.record(stream)
        for _ in range(steps):
            sim.step()
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / steps
        out.update({"fits": True, "device_bytes": ctx.bytes_in_use(), "ms_per_step": ms, "steps": steps,
                    "particle_steps_per_s": N ** 3 / (ms / 1e3), "a": sim.state()["a"]})
        del sim, ctx
    except gpu.GevError as e:
        out.update({"fits": False, "error": str(e)[:200]})
    torch.cuda.synchronize()
    return out


def run_e2e_two_sims(gpu, N, steps, box, device, torch):
    """The e2e loop of two independent simulations at once, each driven by its own host
    thread through the same calls (upload from pinned memory, cycle, download into pinned
    memory): one simulation's transfers over the host link overlap the other's cycle, and
    its uploads the other's downloads.  Value: both simulations' particle-steps over the
    wall time.  Early cycles (z near 100)."""
    n = N ** 3
    sims = []
    for k in range(2):
        ctx = gpu.Context(N, gpu.PREC_MIXED, device=device)
        sim = gpu.Sim(ctx, n)
        sim.ic_generate(**gpu.ic_params(box, seed=7 + k))
        sim.step()
        host = torch.empty(n * 56, dtype=torch.uint8, pin_memory=True)
        back = torch.empty(n * 56, dtype=torch.uint8, pin_memory=True)
        arr, barr = host.numpy().view(gpu.PART), back.numpy().view(gpu.PART)
        sim.particles().download(out=arr)
        ctx.sync()
        sims.append((ctx, sim, host, back, arr, barr))
    start = threading.Barrier(3)
    errors = []

    def loop(ctx, sim, host, back, arr, barr):
        try:
            pcls = sim.particles()
            start.wait()
            for _ in range(steps):
                pcls.upload(arr)
                sim.step()
                pcls.download(out=barr)
        except Exception as e:  # reported after the join
            errors.append(e)

    threads = [threading.Thread(target=loop, args=s) for s in sims]
    for t in threads:
        t.start()
    start.wait()
    t0 = time.perf_counter()
    for t in threads:
        t.join()
    dt = time.perf_counter() - t0
    if errors:
        raise errors[0]
    del sims
    torch.cuda.empty_cache()
    return {"value": 2 * n * steps / dt, "unit": "particle-steps/s", "simulations": 2,
            "h2d_bytes_per_step": n * 56, "d2h_bytes_per_step": n * 56}


# ---------------------------------------------------------- CPU side --------
def _cpu_worker(args):
    """The oracle (FP64 CPU restatement, OpenMP over the host's threads) on the CPU
    sample: IC at z = 100, `warm` untimed cycles, then `steps` timed cycles."""
    N, box, warm, steps, seed = args
    import gevoracle as G
    s = G.Sim(N).ic(**G.default_icparams(N, box, seed=seed))
    for _ in range(warm):
        s.step()
    t0s = s.phase_seconds()
    per = []
    for _ in range(steps):
        t0 = time.perf_counter()
        s.step()
        per.append(time.perf_counter() - t0)
    t1s = s.phase_seconds()
    phases = {k: (t1s[k] - t0s[k]) / max(steps, 1) for k in G.PHASES}
    phases["fft_count_per_cycle"] = (t1s["fft_count"] - t0s["fft_count"]) / max(steps, 1)
    return per, phases, os.cpu_count()


def cpu_sample(N, box, warm, steps):
    """Runs the CPU sample in a spawned process (its own OpenMP runtime, no CUDA)."""
    import multiprocessing as mp
    import gevoracle
    gevoracle.build()
    ctx = mp.get_context("spawn")
    with ctx.Pool(1) as pool:
        return pool.apply(_cpu_worker, ((N, box, warm, steps, 1),))


def cpu_line(per, phases, threads, what):
    n = CPU_SAMPLE_GRID ** 3
    v = n * len(per) / sum(per)
    return {"value": v, "unit": "particle-steps/s", "cores": threads, "kind": "port",
            "sample": "%s of a %d^3 simulation in a %g Mpc/h box (the 512^3 workload's cell size and particle "
                      "density), BBKS Zel'dovich IC at z = 100; FP64 CPU restatement of the path on %d OpenMP threads; "
                      "its FFT is the oracle's, not FFTW" % (what, CPU_SAMPLE_GRID, CPU_SAMPLE_BOX, threads),
            "phases_s_per_cycle": phases}


def config_of(args):
    N = args.grid
    return {"workload": "gevolution GR PM cycle, %d^3 grid, %d^3 CDM particles, box %g Mpc/h, %s form, "
                        "BBKS Zel'dovich IC at z=100 (sigma8 0.81, h 0.67, Omega_cdm 0.27 + Omega_b 0.05), "
                        "parabolic B, 12 FFTs per cycle, run to z=0" % (N, N, 1000.0 * N / 512, args.prec),
            "grid": N, "particles": N ** 3, "precision": args.prec,
            "l2": "inputs larger than L2 (fields >= %d MB each)" % (N ** 3 * (8 if args.prec == "fp64" else 4) // 2 ** 20)}


def main_reference(args, rank):
    if rank != 0:
        return
    t0 = time.perf_counter()
    per, phases, threads = cpu_sample(CPU_SAMPLE_GRID, CPU_SAMPLE_BOX, args.warmup, args.steps)
    cb = cpu_line(per, phases, threads, "%d cycles after %d warm-up cycles" % (args.steps, args.warmup))
    N = args.grid
    line = {"impl": "reference", "metric": "particle-steps/s %d^3 %s" % (N, args.prec), "value": cb["value"],
            "unit": "particle-steps/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": sum(per) / len(per) * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config_of(args),
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": time.perf_counter() - t0}
    print(json.dumps(line))


# ------------------------------------------------------ single operations --
def run_op(args):
    """One operation for profiler captures and per-operation timing (CUDA events on
    the context's stream, --reps calls after one untimed call):
      prepare    IC at z = 100, evolve to --z-op, write the hibernation file --state
      cycle      restart from --state, --reps cycles (the late-time cycle for ncu)
      table      restart from --state (or a fresh IC), time each operation of a cycle
      ensemble   the 48-simulation ensemble alone (server direct, graph and one-thread runs;
                 batched in 1, 2, 4 and 8 lanes)
      batch_cycle  16 simulations of --grid^3: --reps batched steps, then --reps direct
                 cycles of each (one cohort, for launch lists)
      r2c_alone, c2r_alone, fft_axis_y, fft_axis_z   one component of random values"""
    import numpy as np
    import gev_gb300 as gpu
    if args.op == "ensemble":
        print(json.dumps(run_ensemble(gpu, args.seed, lanes=(1, "size", 2, 4, 8))))
        return
    if args.op == "batch_cycle":
        # 16 simulations of --grid^3 (mixed form): two direct cycles each, then --reps
        # batched steps (one launch per kernel for the cohort), then --reps direct cycles of
        # each simulation; host wall time of each phase with the device synchronised
        N = args.grid
        sims = []
        for k in range(16):
            c = gpu.Context(N, gpu.PREC_MIXED)
            sim = gpu.Sim(c, N ** 3)
            sim.ic_generate(**gpu.ic_params(2.5 * N, seed=args.seed + k))
            sims.append((c, sim))
        b = gpu.Batch()
        for _ in range(2):
            b.step([sim for _, sim in sims])
        for c, _ in sims:
            c.sync()
        t0 = time.perf_counter()
        for _ in range(args.reps):
            b.step([sim for _, sim in sims])
        for c, _ in sims:
            c.sync()
        t1 = time.perf_counter()
        for _ in range(args.reps):
            for _, sim in sims:
                sim.step()
        for c, _ in sims:
            c.sync()
        t2 = time.perf_counter()
        print(json.dumps({"grid": N, "simulations": 16, "steps": args.reps, "batch_info": b.info(),
                          "batched_ms_per_step": (t1 - t0) / args.reps * 1e3,
                          "direct_ms_per_step": (t2 - t1) / args.reps * 1e3}))
        return
    import torch
    N = args.grid
    prec = gpu.PREC_MIXED if args.prec == "mixed" else gpu.PREC_FP64
    ctx = gpu.Context(N, prec)
    st = torch.cuda.ExternalStream(ctx.stream())

    def timed(fn):
        fn()
        ctx.sync()
        e0, e1 = _events(torch, 2)
        e0.record(st)
        for _ in range(args.reps):
            fn()
        e1.record(st)
        e1.synchronize()
        return e0.elapsed_time(e1) / args.reps

    rng = np.random.default_rng(1)
    if args.op in ("r2c_alone", "c2r_alone"):
        real, spec = ctx.real(1), ctx.spectrum(1)
        real.upload(rng.standard_normal(real.shape))
        gpu.fft_r2c(real, spec)
        fn = (lambda: gpu.fft_r2c(real, spec)) if args.op == "r2c_alone" else (lambda: gpu.fft_c2r(spec, real))
        print("grid %d^3, %s form, one component; %s %.3f ms per call" % (N, args.prec, args.op, timed(fn)))
        return
    if args.op in ("fft_axis_y", "fft_axis_z"):
        spec = ctx.spectrum(1)
        spec.upload(rng.standard_normal(spec.shape) + 1j * rng.standard_normal(spec.shape))
        axis = 1 if args.op == "fft_axis_y" else 2
        print("grid %d^3, %s form, one spectrum component; %s %.3f ms per call"
              % (N, args.prec, args.op, timed(lambda: gpu.fft_axis(spec, axis, -1))))
        return
    sim = gpu.Sim(ctx, N ** 3)
    box = 1000.0 * N / 512
    if args.op == "prepare":
        sim.ic_generate(**gpu.ic_params(box, seed=args.seed))
        n = full_cycles_to(sim.state(), N, args.z_op)
        for _ in range(n):
            sim.step()
        sim.hibernate(args.state)
        s = sim.state()
        print("grid %d^3, %s form: %d cycles to z = %.4f, hibernation file %s"
              % (N, args.prec, n, 1.0 / s["a"] - 1.0, args.state))
        return
    if args.state:
        sim.restart(args.state)
    else:
        sim.ic_generate(**gpu.ic_params(box, seed=args.seed))
        sim.step()
    z = 1.0 / sim.state()["a"] - 1.0
    if args.op == "cycle":
        print("grid %d^3, %s form, z = %.4f: cycle %.3f ms" % (N, args.prec, z, timed(sim.step)))
        return
    if args.op != "table":
        raise SystemExit("unknown --op %r" % args.op)
    p = sim.particles()
    phi, chi, Bi, src, Sij = (sim.field(k) for k in ("phi", "chi", "Bi", "source", "Sij"))
    sFT, SFT, BFT = (sim.field(k) for k in ("scalarFT", "SijFT", "BiFT"))
    a = sim.state()["a"]
    ops = [
        ("cycle", sim.step),
        ("T00+Tij", lambda: gpu.projection_T00_Tij(p, src, Sij, a, phi)),
        ("source_scalar", lambda: gpu.prepare_source_scalar(phi, chi, src, 0.32, src, 1e-3, 1e-3, 1e-3)),
        ("r2c_x1", lambda: gpu.fft_r2c(src, sFT)),
        ("c2r_x1", lambda: gpu.fft_c2r(sFT, phi)),
        ("source_tensor", lambda: gpu.prepare_source_tensor(phi, Sij, Sij, 1e-3)),
        ("r2c_x6", lambda: gpu.fft_r2c(Sij, SFT)),
        ("project_evolve", lambda: gpu.project_scalar_evolve_vector(SFT, sFT, BFT, 1e-9)),
        ("c2r_x3", lambda: gpu.fft_c2r(BFT, Bi)),
        ("kick_drift_move", lambda: gpu.update_q_pos(p, 1e-9, a, 3, 1e-9, a, 3, phi, chi, Bi, wait=False)),
    ]
    print("grid %d^3, %s form, z = %.4f; ms per call (CUDA events), %d calls" % (N, args.prec, z, args.reps))
    for name, fn in ops:
        print("%-16s %9.3f ms" % (name, timed(fn)), flush=True)


def main():
    args = parse()
    if args.op:
        run_op(args)
        return
    rank, world, local = dist_env()
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl" if args.impl == "ours" else "gloo")
    if args.impl == "reference":
        main_reference(args, rank)
        return
    res = run_ours(args, rank, world, local)
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline:
        per, phases, threads = cpu_sample(CPU_SAMPLE_GRID, CPU_SAMPLE_BOX, 1, 2)
        cpu = cpu_line(per, phases, threads, "2 cycles after 1 warm-up cycle")
    N = args.grid
    alg, per_particle, per_cell = cycle_bytes(N, args.prec)
    config = config_of(args)
    config["timed_cycles"] = res["timed"]
    line = {"metric": "particle-steps/s %d^3 %s" % (N, args.prec), "value": res["value"], "unit": "particle-steps/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": res["ms"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.prec == "fp64" else "f32+f64pos+i64dep",
            "data": "synthetic (device-generated BBKS Zel'dovich IC)", "config": config,
            "roofline": res["roofline"], "kernels": res["kernels"], "phases_gpu_ms_per_cycle": res["phases"],
            "full_run": res["full"], "early_cycles": res["early"],
            "fft_vs_cufft": res["cufft"], "fft_tiles": res["tiles"], "cpu_baseline": cpu, "e2e": res["e2e"],
            "e2e_two_sims": res["e2e2"], "hbm_fit_1024": res["hbm"], "gpu_launches": res["launches"],
            "clocks": res["clocks"],
            "bytes_per_cycle_alg": {"bytes": alg, "per_particle": per_particle, "per_cell": per_cell,
                                    "achieved_gbs": alg / (res["ms"] / 1e3) / 1e9,
                                    "frac": alg / (res["ms"] / 1e3) / 1e9 / hbm_peak()[0]},
            "final_a": res["state"]["a"]}
    if res.get("pk"):
        line.update(res["pk"])
    if res.get("serve"):
        line["serve"] = res["serve"]
    print(json.dumps(line))


if __name__ == "__main__":
    main()
