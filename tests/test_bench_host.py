"""bench.py's host-side logic, no GPU: the cycle schedule to z = 0 that the timed
window is placed by, and the algorithmic byte accounting of the roofline."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_cycle_count_to_z0_matches_the_oracle_loop(oracle):
    """full_cycles_to replays the background (rk4bg and the dtau rule) and must give
    the number of cycles the main loop completes before its z = 0 output."""
    N = 16
    o = oracle.Sim(N).ic(**oracle.default_icparams(N, 5.0 * N, seed=1))
    sc = o.scalars()
    st = {k: sc[k] for k in ("a", "dtau", "fourpiG", "Cf", "steplimit")}
    st["cosmo"] = o.cosmo
    n = bench.full_cycles_to(st, N, 0.0)
    for _ in range(n):
        assert not (1.0 / o.s.a < 1.0)
        o.step()
    assert 1.0 / o.s.a < 1.0
    assert n == 117  # 5 Mpc/h cells from z = 100 (Courant 48, limit 0.04)


def test_cycle_bytes_restate_the_per_particle_step_sums():
    alg, pp, pc = bench.cycle_bytes(512, "mixed")
    assert (pp, pc) == (108, 220) and alg == 328 * 512 ** 3
    alg, pp, pc = bench.cycle_bytes(64, "fp64")
    assert (pp, pc) == (144, 440)
    # the kick+drift kernel: positions (FP64) and momenta (FP32) read and written, phi chi B read
    assert bench.kernel_alg_bytes("k_kick_drift", 512, "mixed") == 512 ** 3 * (72 + 20)
    assert bench.kernel_alg_bytes("k_move", 512, "mixed") is None


def test_kernel_table_picks_the_largest_kernel():
    kt = {"k_kick_drift": (20, 120.0), "k_fft_cols_reg": (480, 100.0), "phase:fft": (240, 200.0),
          "k_move": (20, 50.0)}
    rows, phases, roof = bench.kernel_table(kt, 20, 30.0, 512, "mixed")
    assert roof["kernel"] == "k_kick_drift"
    assert abs(roof["ms_per_launch"] - 6.0) < 1e-12
    assert abs(roof["achieved"] - 512 ** 3 * 92 / 6e-3 / 1e9) < 1e-6
    assert phases == {"thereof FFTs": 10.0}
    assert "frac" not in rows["k_move"]
