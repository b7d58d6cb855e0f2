"""The oracle's OpenMP loops keep the bits of its serial code: the same simulation
run on one thread and on four gives identical particles, fields and spectra."""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

SCRIPT = r"""
import sys
sys.path.insert(0, %r)
import numpy as np
import gevoracle as go
go.build()
N = 24
s = go.Sim(N)
s.ic(**go.default_icparams(N, 60.0, seed=5))
for _ in range(4):
    s.step()
p = s.particles
o = np.argsort(p["ID"])
np.savez(sys.argv[1], pos=p["pos"][o], vel=p["vel"][o], phi=s.field("phi"), Bi=s.field("Bi"),
         a=s.s.a, T00hom=s.s.T00hom)
"""


def run(threads, out):
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    subprocess.run([sys.executable, "-c", SCRIPT % os.path.join(ROOT, "oracle"), out], env=env, check=True,
                   timeout=600)
    return np.load(out)


def test_oracle_bits_do_not_depend_on_threads(tmp_path):
    a = run(1, str(tmp_path / "t1.npz"))
    b = run(4, str(tmp_path / "t4.npz"))
    for k in ("pos", "vel", "phi", "Bi", "a", "T00hom"):
        assert np.array_equal(a[k], b[k]), k
