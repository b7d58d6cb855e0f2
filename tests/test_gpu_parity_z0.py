"""The FP64 form against the oracle over whole runs, z = 100 -> 0, on the two FP64
configurations, and the precision form against the FP64 form over the same run.

Tolerances of the FP64 parity criterion: the power spectra of phi, chi, B and
delta within TOL_PK relative in every occupied bin at every Pk redshift, and
every compared particle position within TOL_POS of a cell at the end (z = 0).
How far the oracle moves under round-off alone: with every initial position
moved by one ulp, the 64^3 run ends 5.5e-13 of a cell away and its spectra
within 7e-12 (the margin below these tolerances).

Configurations (BBKS Zel'dovich IC at z = 100, sigma8 0.81, h 0.67, Omega_cdm
0.27 + Omega_b 0.05 folded into CDM, Courant factor 48, time-step limit 0.04,
phi, chi, B and T_ij active):
  64^3 grid and particles, box 320 Mpc/h: the oracle runs here, beside the GPU;
  256^3 grid and particles, box 1280 Mpc/h: the oracle's run is the committed
  fixture tests/golden/z0_N256.npz (written by tests/golden/make_z0_fixture.py);
  the oracle's initial conditions are regenerated here and checked against the
  fixture's hash.
"""
import hashlib
import os

import numpy as np
import pytest

import z0_common as Z

pytestmark = pytest.mark.gpu

TOL_PK = 1e-10   # FP64 form vs oracle, per bin, relative
TOL_POS = 1e-9   # FP64 form vs oracle, final positions, in cells
TOL_MIXED_PK = 1e-3  # precision form vs FP64 form, per bin up to k_Nyquist / 2
TOL_MIXED_RMS = 2e-2  # precision form vs FP64 form, rms displacement difference at z = 0, in cells

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "z0_N256.npz")


def _report(tag, recs_gpu, recs_ref):
    worst = {}
    for rg, ro in zip(recs_gpu, recs_ref):
        for name in Z.SPECTRA:
            d = Z.pk_max_rel(rg[name], ro[name])
            worst[name] = max(worst.get(name, 0.0), d)
    print("%s: max per-bin relative P(k) deviation over all Pk redshifts: %s" % (
        tag, ", ".join("%s %.2e" % kv for kv in worst.items())))
    return worst


def test_fp64_64_to_z0_matches_oracle(gpu, oracle):
    """Configuration 1 (64^3, 320 Mpc/h) run to z = 0 on both, from the oracle's IC."""
    N, L = 64, 320.0
    o = oracle.Sim(N).ic(**oracle.default_icparams(N, L, seed=1))
    ctx = gpu.Context(N, gpu.PREC_FP64)
    s = gpu.Sim(ctx, N ** 3)
    Z.load_sim(s, o)
    rg = Z.gpu_run(gpu, ctx, s)
    ro = Z.oracle_run(oracle, o)
    assert [r["cycle"] for r in rg] == [r["cycle"] for r in ro]
    for a, b in zip(rg, ro):
        assert abs(a["a"] - b["a"]) <= 1e-15 * b["a"]
    worst = _report("64^3 FP64 vs oracle", rg, ro)
    for name, d in worst.items():
        assert d <= TOL_PK, name
    got = s.particles().download()
    dpos = np.abs(Z.periodic_delta(Z.by_id(got), Z.by_id(o.particles))).max() * N
    print("64^3 FP64 vs oracle: max |dpos| at z = 0: %.2e cells (%d cycles)" % (dpos, ro[-1]["cycle"]))
    assert dpos <= TOL_POS
    assert rg[-1]["z"] == 0.0 and 1.0 / rg[-1]["a"] - 1.0 < 0.0


@pytest.mark.skipif(not os.path.exists(FIXTURE), reason="fixture tests/golden/z0_N256.npz not written")
def test_fp64_256_to_z0_matches_oracle_fixture(gpu, oracle):
    """Configuration 2 (256^3, 1280 Mpc/h) run to z = 0 on the GPU from the oracle's
    IC, against the oracle's committed run."""
    f = np.load(FIXTURE)
    N, L = int(f["grid"]), float(f["box"])
    o = oracle.Sim(N).ic(**oracle.default_icparams(N, L, seed=int(f["seed"])))
    ic_hash = hashlib.sha256(np.ascontiguousarray(Z.by_id(o.particles)).tobytes()).hexdigest()
    print("256^3 oracle IC here %s the fixture's (sha256)" % ("matches" if ic_hash == str(f["ic_sha256"]) else
                                                             "differs from"))
    ctx = gpu.Context(N, gpu.PREC_FP64)
    s = gpu.Sim(ctx, N ** 3)
    Z.load_sim(s, o)
    del o
    rg = Z.gpu_run(gpu, ctx, s, nb=int(f["numbins"]))
    assert [r["cycle"] for r in rg] == list(f["cycle_pk"])
    worst = {}
    for i, r in enumerate(rg):
        assert abs(r["a"] - f["a_pk"][i]) <= 1e-15 * f["a_pk"][i]
        for name in Z.SPECTRA:
            ref = (f["%d_%s_k" % (i, name)], f["%d_%s_p" % (i, name)], None, None, f["%d_%s_occ" % (i, name)])
            worst[name] = max(worst.get(name, 0.0), Z.pk_max_rel(r[name], ref))
    print("256^3 FP64 vs oracle fixture: max per-bin relative P(k) deviation: %s" % (
        ", ".join("%s %.2e" % kv for kv in worst.items())))
    for name, d in worst.items():
        assert d <= TOL_PK, name
    pos = Z.by_id(s.particles().download())[::int(f["id_stride"])]
    dpos = np.abs(Z.periodic_delta(pos, f["pos_subset"])).max() * N
    print("256^3 FP64 vs oracle fixture: max |dpos| at z = 0 over %d IDs: %.2e cells" % (len(pos), dpos))
    assert dpos <= TOL_POS


def test_mixed_64_to_z0_tracks_fp64(gpu, oracle):
    """The precision form against the FP64 form, both from the oracle's 64^3 IC, run
    to z = 0: power spectra of phi, chi, B and delta within 1e-3 per bin up to
    k_Nyquist / 2 at every Pk redshift, and the rms difference of the particles'
    final positions (matched by ID).  Late times are where the deposit's fixed-point
    scale, set by the fullest cell, is smallest."""
    N, L = 64, 320.0
    o = oracle.Sim(N).ic(**oracle.default_icparams(N, L, seed=2))
    runs = {}
    for prec in (gpu.PREC_FP64, gpu.PREC_MIXED):
        ctx = gpu.Context(N, prec)
        s = gpu.Sim(ctx, N ** 3)
        Z.load_sim(s, o)
        recs = Z.gpu_run(gpu, ctx, s)
        runs[prec] = (recs, Z.by_id(s.particles().download()))
    r64, p64 = runs[gpu.PREC_FP64]
    r32, p32 = runs[gpu.PREC_MIXED]
    assert [r["cycle"] for r in r64] == [r["cycle"] for r in r32]
    kmax = 0.5 * np.pi * N
    worst = {}
    for a, b in zip(r32, r64):
        for name in Z.SPECTRA:
            worst["%s z=%g" % (name, b["z"])] = Z.pk_max_rel(a[name], b[name], kmax)
    print("64^3 mixed vs FP64, k <= k_Ny/2: " + ", ".join("%s %.2e" % kv for kv in worst.items()))
    d = Z.periodic_delta(p32, p64) * N
    rms = float(np.sqrt((d ** 2).sum(axis=1).mean()))
    disp = Z.periodic_delta(p64, Z.by_id(o.particles)) * N
    rms_disp = float(np.sqrt((disp ** 2).sum(axis=1).mean()))
    print("64^3 mixed vs FP64 at z = 0: rms position difference %.3e cells (max %.3e) against an rms "
          "displacement since z = 100 of %.3f cells" % (rms, np.abs(d).max(), rms_disp))
    for k, v in worst.items():
        assert v <= TOL_MIXED_PK, k
    assert rms <= TOL_MIXED_RMS
