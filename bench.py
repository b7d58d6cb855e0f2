"""Benchmark of the per-step particle-mesh hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--grid 512] [--prec mixed|fp64]

Workload (default): the precision form at 512^3 grid and 512^3 particles in a
1 Gpc/h box (FP32 fields and FFTs, FP64 positions, int64 fixed-point
deposits), seeded BBKS Zel'dovich initial conditions at z = 100 generated on
the device, GR mode with phi, chi, B_i and T_ij active (parabolic vector
method).  A step is one cycle of gevolution's main loop (main.cpp:372-879):
the three deposits, the phi / chi / B solves with 12 FFTs, the kick, the drift
with the relink, and the background update.  Metric: particle-steps/s.

value    device-timed throughput with the state resident in HBM (CUDA events on
         the library's stream, K cycles between two synchronised barriers);
e2e      the same cycles through the C-ABI with the particle state copied in
         from pinned host memory and back out every step;
roofline the dominant kernel's algorithmic bytes per launch over its event-
         timed duration, against the measured HBM copy bandwidth;
cpu_baseline  the CPU restatement of the same path (oracle/) timed on this
         host on a bounded sample (rank 0, N = 1 only).

--impl reference runs the CPU implementation of the path (the oracle's port of
the reference; the reference itself needs LATfield2, FFTW, MPI and HDF5, which
the GPU hosts do not have) on all host cores, one independent simulation per
core, and prints the same metric.  With --gpus N > 1 each rank runs its own
simulation (replicas, no data exchange); the value is the sum over ranks of
particles x steps divided by the slowest rank's time.
"""
import argparse
import json
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
    ap.add_argument("--serve-seconds", type=float, default=20.0,
                    help="length of the serving run's Poisson arrivals (0: no serving measurement)")
    ap.add_argument("--serve-rate", type=float, default=2.0, help="serving requests per second")
    ap.add_argument("--serve-burst", type=int, default=24, help="requests submitted at once for the capacity run")
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


# ------------------------------------------------- algorithmic bytes --------
def cycle_bytes(N, prec):
    """Compulsory HBM bytes of one cycle: every persistent or intermediate array
    read or written once per use, FFTs at three passes (one read and one write of
    the array per pass).  Particles: deposit reads pos+vel, kick/drift read pos+vel
    and write them back."""
    r = 8 if prec == "fp64" else 4
    V = N ** 3
    K = N * N * (N // 2 + 1) * 2 * r  # bytes of one half spectrum component
    pcl_state = 3 * 8 + 3 * r
    particles = V * (pcl_state + 2 * pcl_state)
    fields = 0
    fields += V * r * (1 + 6)          # T00 and Tij written by the deposits
    fields += V * r * 1                # phi read by the deposits
    fields += V * r * 3 + V * r        # prepareFTsource (scalar): phi, chi, source in, source out
    fields += 12 * 3 * 2 * K           # 12 FFTs x 3 passes x (read + write) of one component
    fields += K * 2                    # Poisson in place
    fields += V * r * 7 + V * r * 6    # prepareFTsource (tensor): phi + Sij in, Sij out
    fields += 6 * K + K                # projectFTscalar
    fields += 6 * K + 2 * 3 * K        # evolveFTvector (Sij in, B in/out)
    fields += V * r * (1 + 1 + 3)      # kick/drift gather phi, chi, Bi
    return particles + fields


def run_ours(args, rank, world, local):
    import torch
    import gev_gb300 as gpu

    torch.cuda.set_device(local)
    N = args.grid
    prec = gpu.PREC_FP64 if args.prec == "fp64" else gpu.PREC_MIXED
    box = 1000.0 * N / 512
    ctx = gpu.Context(N, prec, device=local)
    sim = gpu.Sim(ctx, N ** 3)
    sim.ic_generate(**gpu.ic_params(box, seed=args.seed + 1000 * rank))
    stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device("cuda", local))
    for _ in range(args.warmup):
        sim.step()
    ctx.sync()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = ctx.launches()
    e0.record(stream)
    for _ in range(args.steps):
        sim.step()
    e1.record(stream)
    e1.synchronize()
    launches = ctx.launches() - l0
    tiles = ctx.fft_tiles()
    ms = e0.elapsed_time(e1)
    clk = clocks.stop()
    torch.cuda.synchronize()
    ms_max = reduce_max_ms(ms, world, "cuda")
    value = aggregate_value(N, args.steps, world, ms_max)
    st = sim.state()
    pk = None
    if not args.no_pk_check and prec == gpu.PREC_MIXED and world == 1:
        pk = spectra_of(gpu, ctx, sim)

    # roofline of the dominant kernel (the T00 + Tij deposit) and of the FFT column pass
    roof = deposit_roofline(gpu, ctx, sim, stream, N, args.prec)
    roof_fft = dominant_kernel_roofline(gpu, ctx, sim, stream, N, args.prec)
    roof_pcl = particle_update_roofline(gpu, ctx, sim, stream, N, args.prec)
    cufft = fft_vs_cufft(gpu, ctx, stream, N, args.prec, torch) if world == 1 else None

    # e2e: particle state from pinned host memory in, cycle, particle state out
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(gpu, ctx, sim, stream, N, args.steps, torch)
    del sim, ctx, stream  # the measurements below make their own simulations
    torch.cuda.synchronize()
    fp64 = None
    if pk is not None:
        fp64 = fp64_form_check(args, gpu, N, box, local, pk, torch)
    e2e2 = None
    if not args.no_e2e and world == 1:
        e2e2 = run_e2e_two_sims(gpu, N, args.steps, box, local, torch)
    serve = None
    if args.serve_seconds > 0 and world == 1:
        serve = run_serve(args, gpu)
    hbm = None
    if not args.no_hbm_fit and world == 1 and prec == gpu.PREC_MIXED and N == 512:
        hbm = run_hbm_fit(gpu, local, torch)
    return dict(value=value, ms=ms_max / args.steps, launches=launches, tiles=tiles, clocks=clk, state=st, roofline=roof,
                roofline_fft=roof_fft, roofline_pcl=roof_pcl, cufft=cufft, e2e=e2e, e2e2=e2e2, box=box, fp64=fp64,
                serve=serve, hbm=hbm)


PK_FIELDS = (("phi", 1), ("chi", 1), ("Bi", 3), ("source", 1))
PK_BINS = 64


def spectra_of(gpu, ctx, sim):
    """Power spectra (device FFT + gev_cross_spectrum) of phi, chi, B_i and the
    source field of a simulation."""
    out = {}
    for name, nc in PK_FIELDS:
        sp = ctx.spectrum(nc)
        gpu.fft_r2c(sim.field(name), sp)
        out[name] = gpu.cross_spectrum(sp, numbins=PK_BINS)
        del sp
    return out


def fp64_form_check(args, gpu, N, box, local, pk_mixed, torch):
    """The plain FP64 form from the same initial conditions for the same cycles:
    its device-timed throughput, and the largest per-bin relative deviation of the
    mixed form's power spectra from it up to k_Nyquist / 2 (criterion 1e-3)."""
    import numpy as np
    ctx = gpu.Context(N, gpu.PREC_FP64, device=local)
    sim = gpu.Sim(ctx, N ** 3)
    sim.ic_generate(**gpu.ic_params(box, seed=args.seed))
    stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device("cuda", local))
    for _ in range(args.warmup):
        sim.step()
    ctx.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        sim.step()
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    pk64 = spectra_of(gpu, ctx, sim)
    dev = {}
    for name, _ in PK_FIELDS:
        kb, p64, _, _, occ = pk64[name]
        p32 = pk_mixed[name][1]
        m = (occ > 0) & (kb <= 0.5 * np.pi * N)
        dev[name] = float(np.max(np.abs(p32[m] - p64[m]) / np.maximum(np.abs(p64[m]), 1e-300)))
    return {"fp64_form": {"value": N ** 3 * args.steps / (ms / 1e3), "unit": "particle-steps/s",
                          "ms_per_step": ms / args.steps},
            "pk_check": {"against": "the FP64 form on the GPU, same initial conditions, %d cycles"
                         % (args.warmup + args.steps), "numbins": PK_BINS, "k_max": "k_Nyquist/2",
                         "max_rel_dev": dev, "tolerance": 1e-3, "pass": all(v <= 1e-3 for v in dev.values())}}


# DRAM traffic per launch of the column pass (dram__bytes_read.sum +
# dram__bytes_write.sum) from an ncu capture of the same kernel on one 512^3
# spectrum component (gevolution-1.2_gb300/opbench.py --only fft_axis_z), keyed by
# (grid, precision): 556.2 MB read + 511.3 MB written
COLS_TRAFFIC = {(512, "mixed"): 1.0675e9}


# DRAM traffic per call of the T00 + Tij deposit: its prefactor pass (k_fx_prep) and
# its gather (k_dep_gather), from an ncu capture of the same kernels on the 256^3
# cycle (opbench --grid 256 --only step), scaled by 8 to 512^3: particles and fields
# both grow as N^3.  k_fx_prep 403.9 MB read + 746.9 MB written, k_dep_gather
# 1410.0 MB read + 502.4 MB written; (3063.2 MB) x 8
DEPOSIT_TRAFFIC = {(512, "mixed"): 24.506e9}


def deposit_roofline(gpu, ctx, sim, stream, N, prec):
    """The largest kernel of the cycle in the ncu launch list: the deposit of T00 and
    Tij in one call (projection_init + projection_T00 + projection_Tij), timed with
    its scale pass and its prefactor pass.  Its algorithmic bytes per call: each
    particle's cell, in-cell offset and momentum read once (4 + 3r + 3r bytes), phi
    read once and the 7 target components written once per cell (8 r bytes), r the
    real size of the form.  The prefactor records the gather writes and reads back
    (48 B a particle) are not algorithmic and show in the traffic."""
    import torch
    r = 8 if prec == "fp64" else 4
    p, src, Sij, phi = sim.particles(), sim.field("source"), sim.field("Sij"), sim.field("phi")
    a = sim.state()["a"]
    reps = 4
    gpu.projection_T00_Tij(p, src, Sij, a, phi)
    ctx.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        gpu.projection_T00_Tij(p, src, Sij, a, phi)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    n = C = N ** 3
    alg = n * (4 + 6 * r) + C * 8 * r
    peak, kind = hbm_peak()
    achieved = alg / (ms / 1e3) / 1e9
    return {"kernel": "k_fx_prep + k_dep_gather<T00+Tij> (the T00 and Tij deposits in one gather; timed with the "
                      "scale pass)",
            "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": DEPOSIT_TRAFFIC.get((N, prec)), "peak_kind": kind, "ms_per_launch": ms, "alg_bytes": alg}


def dominant_kernel_roofline(gpu, ctx, sim, stream, N, prec):
    """The FFT column pass (k_fft_cols_reg, the y / z passes of every transform; 24
    launches a cycle, the largest kernel family by count).  One launch transforms one
    spectrum component along y or z in place: its algorithmic bytes are one read
    and one write of the component, 2 * N^2 (N/2+1) * sizeof(complex)."""
    import torch
    csz = 16 if prec == "fp64" else 8
    spec = sim.field("scalarFT")
    reps = 6
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    gpu.fft_axis(spec, 1, -1)
    ctx.sync()
    e0.record(stream)
    for i in range(reps):
        gpu.fft_axis(spec, 1 + (i & 1), -1)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    alg = 2 * N * N * (N // 2 + 1) * csz
    peak, kind = hbm_peak()
    achieved = alg / (ms / 1e3) / 1e9
    return {"kernel": "k_fft_cols_reg (one y or z pass of the 3-D FFT over one spectrum component)", "bound": "hbm",
            "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": COLS_TRAFFIC.get((N, prec)), "peak_kind": kind, "ms_per_launch": ms, "alg_bytes": alg}


# DRAM traffic per call of the particle update: k_kick_drift and k_move from an ncu
# capture of the 256^3 cycle (opbench --grid 256 --only step), scaled by 8 to 512^3.
# k_kick_drift 1624.8 MB read + 973.8 MB written, k_move 1140.9 MB read + 958.6 MB
# written; (4698.1 MB) x 8.  The scan's three kernels (about 1 GB at 512^3) are not in it.
PARTICLE_TRAFFIC = {(512, "mixed"): 37.585e9}


def particle_update_roofline(gpu, ctx, sim, stream, N, prec):
    """The cycle's particle update, whose kick+drift kernel is the largest single kernel
    of the launch list: gev_update_q_pos (updateVel + moveParticles with the relink),
    kick+drift+histogram, scan and move in one call, timed with CUDA events.  Its
    algorithmic bytes per call: kick+drift reads each particle's cell, offset, momentum
    and position and writes them back with its rank (52 + 56 B in the mixed form), and
    reads phi, chi and B once per cell (20 B); the scan reads the counts and writes the
    starts (8 B a cell); the move reads and writes the payload with its rank and start
    (128 B a particle).  The particles move by about 1e-9 of a cell per call here."""
    import torch
    r = 8 if prec == "fp64" else 4
    p, phi, chi, Bi = sim.particles(), sim.field("phi"), sim.field("chi"), sim.field("Bi")
    a = sim.state()["a"]
    reps = 4
    gpu.update_q_pos(p, 1e-9, a, 3, 1e-9, a, 3, phi, chi, Bi, wait=False)
    ctx.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        gpu.update_q_pos(p, 1e-9, a, 3, 1e-9, a, 3, phi, chi, Bi, wait=False)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    n = C = N ** 3
    payload = 3 * 8 + 3 * r + 4 + (3 * 4 if r == 4 else 0)  # pos, q, cell, FP32 offset
    alg = n * (2 * payload + 4) + C * 5 * r + C * 8 + n * (2 * (payload + 8) + 4)
    peak, kind = hbm_peak()
    achieved = alg / (ms / 1e3) / 1e9
    return {"kernel": "k_kick_drift + k_scan_* + k_move (gev_update_q_pos: kick, drift, relink)", "bound": "hbm",
            "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": PARTICLE_TRAFFIC.get((N, prec)), "peak_kind": kind, "ms_per_launch": ms, "alg_bytes": alg}


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
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
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


# ------------------------------------------------------------ serving --------
SERVE_SIZES = (64, 96, 128, 192, 256)
SERVE_Z = (1.0, 0.5, 0.0)


def serve_requests(gpu, rng, n, first_seed):
    """Requests of the serving workload: grid drawn from SERVE_SIZES, box 2.5 N Mpc/h,
    Omega_cdm U[0.25, 0.35], sigma8 U[0.75, 0.87], n_s U[0.94, 0.98], target
    redshift from SERVE_Z, BBKS Zel'dovich IC at z = 100, distinct seeds."""
    out = []
    for k in range(n):
        N = int(rng.choice(SERVE_SIZES))
        out.append(gpu.request(N, seed=first_seed + k, z_target=float(rng.choice(SERVE_Z)),
                               Omega_cdm=float(rng.uniform(0.25, 0.35)), sigma8=float(rng.uniform(0.75, 0.87)),
                               n_s=float(rng.uniform(0.94, 0.98)), prec=gpu.PREC_MIXED))
    return out


def fp64_sequential_seconds(gpu, sizes):
    """Per grid size, the wall time of a plain FP64 run on this GPU: the initial
    conditions, and one cycle (the median of 3 after one warm-up)."""
    out = {}
    for N in sizes:
        c = gpu.Context(N, gpu.PREC_FP64)
        s = gpu.Sim(c, N ** 3)
        t0 = time.perf_counter()
        s.ic_generate(**gpu.ic_params(2.5 * N, seed=7))
        c.sync()
        t_ic = time.perf_counter() - t0
        s.step()
        c.sync()
        ts = []
        for _ in range(3):
            t0 = time.perf_counter()
            s.step()
            c.sync()
            ts.append(time.perf_counter() - t0)
        out[N] = (t_ic, sorted(ts)[1])
        del s, c
    return out


def run_serve(args, gpu):
    """The serving loop under load: Poisson arrivals at --serve-rate for
    --serve-seconds (time to result p50 / p99, sustained sims/hour), then a burst of
    --serve-burst requests at once (capacity), against sequential plain FP64 runs of
    the same requests on the same GPU (their IC and cycle times measured per size)."""
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
    seq = fp64_sequential_seconds(gpu, sorted({r["N"] for r in res} | {r["N"] for r in bres} | {64, 96, 128}))

    def seq_seconds(rs):
        return sum(seq[r["N"]][0] + r["cycles"] * seq[r["N"]][1] for r in rs)

    cap = len(bres) / b_span * 3600.0
    seq_rate = len(bres) / seq_seconds(bres) * 3600.0
    # the batched ensemble: 16 simulations each at 64^3, 96^3 and 128^3, box 2.5 N,
    # cosmologies and seeds as above, all to z = 0, admitted at once
    ens = []
    for k, N in enumerate([64] * 16 + [96] * 16 + [128] * 16):
        ens.append(gpu.request(N, seed=300000 + k, z_target=0.0, Omega_cdm=float(rng.uniform(0.25, 0.35)),
                               sigma8=float(rng.uniform(0.75, 0.87)), n_s=float(rng.uniform(0.94, 0.98)),
                               prec=gpu.PREC_MIXED))
    srv = gpu.Server()
    for r in ens:
        srv.submit(r)
    srv.drain(900.0)
    eres = [r for r in srv.poll(100000) if r["status"] == 0]
    est = srv.stats()
    srv.close()
    e_span = max(r["t_done"] for r in eres) - min(r["t_submit"] for r in eres)
    e_steps = sum(float(r["N"]) ** 3 * r["cycles"] for r in eres)
    pct = lambda q: lat[min(len(lat) - 1, int(round(q * (len(lat) - 1))))]  # noqa: E731
    return {
        "precision": "mixed", "arrivals": "Poisson %.3g/s for %.3g s" % (args.serve_rate, args.serve_seconds),
        "sizes": list(SERVE_SIZES), "z_target": list(SERVE_Z), "completed": len(res), "failed": st["failed"],
        "p50_s": pct(0.50), "p99_s": pct(0.99), "max_s": lat[-1],
        "sims_per_hour_offered_load": len(res) / span * 3600.0,
        "max_active_seen": st["max_active_seen"],
        "burst": {"requests": len(bres), "makespan_s": b_span, "sims_per_hour": cap,
                  "max_active_seen": bst["max_active_seen"]},
        "sequential_fp64": {"sims_per_hour": seq_rate,
                            "per_size_s": {str(N): {"ic": v[0], "cycle": v[1]} for N, v in seq.items()},
                            "note": "the burst's requests run one after another in the plain FP64 form: IC time plus "
                                    "their cycles times the measured FP64 cycle time of their size"},
        "capacity_vs_sequential_fp64": cap / seq_rate,
        "ensemble": {"simulations": len(eres), "sizes": "16 x 64^3, 16 x 96^3, 16 x 128^3, z = 100 -> 0",
                     "makespan_s": e_span, "particle_steps_per_s": e_steps / e_span,
                     "max_active_seen": est["max_active_seen"],
                     "sequential_fp64_s": seq_seconds(eres) if all(r["N"] in seq for r in eres) else None},
    }


def run_e2e(gpu, ctx, sim, stream, N, steps, torch):
    import numpy as np
    pcls = sim.particles()
    n = N ** 3
    host = torch.empty(n * 56, dtype=torch.uint8, pin_memory=True)
    arr = host.numpy().view(gpu.PART)
    back = torch.empty(n * 56, dtype=torch.uint8, pin_memory=True)
    barr = back.numpy().view(gpu.PART)
    pcls.download(out=arr)
    ctx.sync()
    t0 = time.perf_counter()
    for _ in range(steps):
        pcls.upload(arr)
        sim.step()
        pcls.download(out=barr)  # into pinned memory; synchronises the stream
    dt = time.perf_counter() - t0
    return {"value": n * steps / dt, "unit": "particle-steps/s", "h2d_bytes_per_step": n * 56,
            "d2h_bytes_per_step": n * 56}


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
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
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
    wall time."""
    import threading
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
    N, steps, seed = args
    import gevoracle as G
    s = G.Sim(N).ic(**G.default_icparams(N, 1000.0 * N / 512, seed=seed))
    s.step()  # the first cycle skips the phi solve (dtau_old = 0)
    t0 = time.perf_counter()
    for _ in range(steps):
        s.step()
    return N ** 3 * steps, time.perf_counter() - t0


def cpu_sample(N, steps, workers):
    """particle-steps/s of the oracle on `workers` independent simulations."""
    import multiprocessing as mp
    import gevoracle
    gevoracle.build()
    if workers == 1:
        n, t = _cpu_worker((N, steps, 1))
        return n / t
    ctx = mp.get_context("spawn")
    with ctx.Pool(workers) as pool:
        res = pool.map(_cpu_worker, [(N, steps, 1 + i) for i in range(workers)])
    return sum(r[0] for r in res) / max(r[1] for r in res)


def main():
    args = parse()
    rank, world, local = dist_env()
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl" if args.impl == "ours" else "gloo")
    N = args.grid
    metric = "particle-steps/s %d^3 %s" % (N, args.prec)
    config = {"workload": "gevolution GR PM cycle, %d^3 grid, %d^3 CDM particles, box %g Mpc/h, %s form, "
                          "BBKS Zel'dovich IC at z=100 (sigma8 0.81, h 0.67, Omega_cdm 0.27 + Omega_b 0.05), "
                          "parabolic B, 12 FFTs per cycle" % (N, N, 1000.0 * N / 512, args.prec),
              "grid": N, "particles": N ** 3, "precision": args.prec,
              "l2": "inputs larger than L2 (fields >= %d MB each)" % (N ** 3 * (8 if args.prec == "fp64" else 4) // 2 ** 20)}
    if args.impl == "reference":
        if rank != 0:
            return
        workers = os.cpu_count() or 1
        sampleN = 64
        t0 = time.perf_counter()
        cpu_sample(sampleN, 1, workers)  # warm-up (builds, spawns)
        vals = []
        for _ in range(args.steps):
            vals.append(cpu_sample(sampleN, 1, workers))
        v = sorted(vals)[len(vals) // 2]
        line = {"impl": "reference", "metric": metric, "value": v, "unit": "particle-steps/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": config,
                "cpu_baseline": {"value": v, "unit": "particle-steps/s", "cores": workers, "kind": "port",
                                 "sample": "one cycle per worker of an independent %d^3 simulation (same IC recipe "
                                           "and box per particle), %d workers; the FFT is the oracle's, not FFTW"
                                           % (sampleN, workers)},
                "e2e": {"value": v, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "wall_s": time.perf_counter() - t0}
        print(json.dumps(line))
        return
    res = run_ours(args, rank, world, local)
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline:
        sampleN = 64
        v = cpu_sample(sampleN, 3, 1)
        cpu = {"value": v, "unit": "particle-steps/s", "cores": 1, "kind": "port",
               "sample": "3 cycles of one %d^3 simulation with the same IC recipe (CPU restatement, FP64, single "
                         "thread); the FFT is the oracle's, not FFTW" % sampleN}
    line = {"metric": metric, "value": res["value"], "unit": "particle-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": res["ms"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.prec == "fp64" else "f32+f64pos+i64dep",
            "data": "synthetic (device-generated BBKS Zel'dovich IC)", "config": config,
            "roofline": res["roofline"], "roofline_fft_cols": res["roofline_fft"], "roofline_particle_update": res["roofline_pcl"], "fft_vs_cufft": res["cufft"], "fft_tiles": res["tiles"], "cpu_baseline": cpu, "e2e": res["e2e"], "e2e_two_sims": res["e2e2"], "hbm_fit_1024": res["hbm"], "gpu_launches": res["launches"],
            "clocks": res["clocks"], "bytes_per_cycle_alg": cycle_bytes(N, args.prec),
            "final_a": res["state"]["a"]}
    if res.get("fp64"):
        line.update(res["fp64"])
    if res.get("serve"):
        line["serve"] = res["serve"]
    print(json.dumps(line))


if __name__ == "__main__":
    main()
