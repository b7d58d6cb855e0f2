"""Per-operation timings of the pieces of one simulation cycle, and a
single-operation mode for profiler captures.

    python gevolution-1.2_gb300/opbench.py --grid 512                 # table, mixed form
    python gevolution-1.2_gb300/opbench.py --grid 512 --prec fp64
    python gevolution-1.2_gb300/opbench.py --grid 256 --only fft_axis_z --reps 3

The simulation is the bench workload scaled to the grid: N^3 particles from the
device-generated Zel'dovich initial conditions in a box of 1000 Mpc/h * N / 512,
after two cycles.  Each operation is timed with CUDA events on the context's
stream over --reps back-to-back calls, after one untimed call.  Times are per
call.  Operations on the particles change the state (every call kicks or moves
them); the table is for timing, not for physics.
"""
import argparse
import os
import sys
import time

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

import gev_gb300 as gpu  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--grid", type=int, default=512)
    ap.add_argument("--prec", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--only", default=None, help="time one operation (names as in the table)")
    args = ap.parse_args()
    import torch

    N = args.grid
    ctx = gpu.Context(N, gpu.PREC_MIXED if args.prec == "mixed" else gpu.PREC_FP64)
    if args.only in ("r2c_alone", "c2r_alone"):
        # one real component and its spectrum and nothing else: the row and column kernels
        # of one 3-D transform, small enough for a full profiler capture at 512^3
        import numpy as np
        rng = np.random.default_rng(1)
        real, spec = ctx.real(1), ctx.spectrum(1)
        real.upload(rng.standard_normal(real.shape))
        gpu.fft_r2c(real, spec)
        fn = (lambda: gpu.fft_r2c(real, spec)) if args.only == "r2c_alone" else (lambda: gpu.fft_c2r(spec, real))
        st = torch.cuda.ExternalStream(ctx.stream())
        fn()
        ctx.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(args.reps):
            fn()
        e1.record(st)
        e1.synchronize()
        print("grid %d^3, %s form, one component; %s %.3f ms per call (CUDA events), %d calls"
              % (N, args.prec, args.only, e0.elapsed_time(e1) / args.reps, args.reps))
        return
    if args.only in ("fft_axis_y", "fft_axis_z"):
        # one spectrum component of random values and nothing else (small enough for a
        # full profiler capture at 512^3): the same kernel as inside the cycle
        import numpy as np
        rng = np.random.default_rng(1)
        spec = ctx.spectrum(1)
        spec.upload(rng.standard_normal(spec.shape) + 1j * rng.standard_normal(spec.shape))
        axis = 1 if args.only == "fft_axis_y" else 2
        st = torch.cuda.ExternalStream(ctx.stream())
        gpu.fft_axis(spec, axis, -1)
        ctx.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(args.reps):
            gpu.fft_axis(spec, axis, -1)
        e1.record(st)
        e1.synchronize()
        print("grid %d^3, %s form, one spectrum component; %s %.3f ms per call (CUDA events), %d calls"
              % (N, args.prec, args.only, e0.elapsed_time(e1) / args.reps, args.reps))
        return
    s = gpu.Sim(ctx, N ** 3)
    s.ic_generate(**gpu.ic_params(1000.0 * N / 512, seed=1))
    for _ in range(2):
        s.step()
    ctx.sync()
    st = torch.cuda.ExternalStream(ctx.stream())
    p = s.particles()
    phi, chi, Bi, src, Sij = (s.field(k) for k in ("phi", "chi", "Bi", "source", "Sij"))
    sFT, SFT, BFT = (s.field(k) for k in ("scalarFT", "SijFT", "BiFT"))
    a = s.state()["a"]
    ops = [
        ("step", s.step),
        ("zero_Sij", lambda: Sij.zero()),
        ("T00", lambda: gpu.projection_T00(p, src, a, phi)),
        ("Tij", lambda: gpu.projection_Tij(p, Sij, a, phi)),
        ("source_scalar", lambda: gpu.prepare_source_scalar(phi, chi, src, 0.32, src, 1e-3, 1e-3, 1e-3)),
        ("r2c_x1", lambda: gpu.fft_r2c(src, sFT)),
        ("poisson", lambda: gpu.solve_poisson(sFT, sFT, 1.0, 0.1)),
        ("c2r_x1", lambda: gpu.fft_c2r(sFT, phi)),
        ("source_tensor", lambda: gpu.prepare_source_tensor(phi, Sij, Sij, 1e-3)),
        ("r2c_x6", lambda: gpu.fft_r2c(Sij, SFT)),
        ("project_scalar", lambda: gpu.project_scalar(SFT, sFT, 0)),
        ("evolve_vector", lambda: gpu.evolve_vector(SFT, BFT, 1e-9)),
        ("project_evolve", lambda: gpu.project_scalar_evolve_vector(SFT, sFT, BFT, 1e-9)),
        ("c2r_x3", lambda: gpu.fft_c2r(BFT, Bi)),
        ("fft_axis_y", lambda: gpu.fft_axis(sFT, 1, -1)),
        ("fft_axis_z", lambda: gpu.fft_axis(sFT, 2, -1)),
        ("kick", lambda: gpu.update_q(p, 0, 1e-9, phi, chi, Bi, 3, a, a * a * N)),
        ("drift_relink", lambda: gpu.update_pos(p, 0, 1e-9, phi, chi, Bi, 3, a, a * a * N)),
        # the cycle's own particle path: kick, drift and histogram in one pass, scan, move
        ("kick_drift_move", lambda: gpu.update_q_pos(p, 1e-9, a, 3, 1e-9, a, 3, phi, chi, Bi, wait=False)),
    ]
    names = [n for n, _ in ops]
    if args.only and args.only not in names:
        raise SystemExit("unknown operation %r; one of %s" % (args.only, ", ".join(names)))
    print("grid %d^3, %s form, %d particles; ms per call (CUDA events), %d calls" % (N, args.prec, N ** 3, args.reps))
    for name, fn in ops:
        if args.only and name != args.only:
            continue
        fn()
        ctx.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        e0.record(st)
        for _ in range(args.reps):
            fn()
        e1.record(st)
        e1.synchronize()
        wall = (time.perf_counter() - t0) / args.reps * 1e3
        print("%-16s %9.3f ms  (host wall %9.3f ms)" % (name, e0.elapsed_time(e1) / args.reps, wall), flush=True)


if __name__ == "__main__":
    main()
