"""Writes tests/golden/z0_N<N>.npz: the oracle's FP64 run of gevolution's main
loop from z = 100 to z = 0 on the 256^3 configuration (256^3 grid, 256^3 CDM
particles, box 1280 Mpc/h, seeded BBKS Zel'dovich IC: sigma8 0.81, h 0.67,
Omega_cdm 0.27 + Omega_b 0.05, n_s 0.96, Courant factor 48, time-step limit 0.04).

    OMP_NUM_THREADS=8 python tests/golden/make_z0_fixture.py [--grid 256] [--box 1280]

The oracle is the CPU restatement in oracle/ (bit-identical to the reference's
own gevolution.hpp compiled against the LATfield2 shim; see
tests/test_oracle_golden.py).  Stored per Pk redshift (tests/z0_common.py):
the binned power of phi, chi, B and delta with their occupations, a and the
cycle; at the end: the positions of every 1024th particle ID, the SHA-256 of
the initial and the final particle arrays (positions ordered by ID), and the
oracle's per-phase wall time.  tests/test_gpu_parity_z0.py runs the GPU's FP64
form from the oracle's initial conditions and compares against it.  It takes
about 15 minutes on 8 threads.
"""
import argparse
import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.dirname(HERE))

import gevoracle as O  # noqa: E402
import z0_common as Z  # noqa: E402

ID_STRIDE = 1024


def pos_hash(parts):
    return hashlib.sha256(np.ascontiguousarray(Z.by_id(parts)).tobytes()).hexdigest()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--grid", type=int, default=256)
    ap.add_argument("--box", type=float, default=1280.0)
    ap.add_argument("--seed", type=int, default=1)
    a = ap.parse_args()
    N = a.grid
    t0 = time.time()
    o = O.Sim(N).ic(**O.default_icparams(N, a.box, seed=a.seed))
    ic_hash = pos_hash(o.particles)
    print("IC %.1f s, sha256 %s" % (time.time() - t0, ic_hash), flush=True)
    t0 = time.time()
    recs = Z.oracle_run(O, o, on_output=lambda r: print("z %g cycle %d a %.6f %.0f s" % (
        r["z"], r["cycle"], r["a"], time.time() - t0), flush=True))
    out = {"grid": N, "box": a.box, "seed": a.seed, "numbins": Z.NUMBINS, "id_stride": ID_STRIDE,
           "z_pk": np.array([r["z"] for r in recs]), "a_pk": np.array([r["a"] for r in recs]),
           "cycle_pk": np.array([r["cycle"] for r in recs]), "ic_sha256": ic_hash,
           "final_sha256": pos_hash(o.particles)}
    for i, r in enumerate(recs):
        for name in Z.SPECTRA:
            kb, pw, ks, ps, occ = r[name]
            out["%d_%s_k" % (i, name)] = kb
            out["%d_%s_p" % (i, name)] = pw
            out["%d_%s_occ" % (i, name)] = occ
    pos = Z.by_id(o.particles)
    out["pos_subset"] = pos[::ID_STRIDE].copy()
    ph = o.phase_seconds()
    out["phase_names"] = np.array(list(O.PHASES))
    out["phase_seconds"] = np.array([ph[k] for k in O.PHASES])
    out["fft_count"] = ph["fft_count"]
    out["threads"] = int(os.environ.get("OMP_NUM_THREADS", "0") or 0)
    path = os.path.join(HERE, "z0_N%d.npz" % N)
    np.savez_compressed(path, **out)
    print("wrote", path, "%.0f s" % (time.time() - t0))


if __name__ == "__main__":
    main()
