"""The C++ drop-in surface (gevolution-1.2_gb300/host/gevolution_gpu.hpp) driven
by a main loop written with the reference's own call sequence
(tests/cpp/main_loop_gpu.cpp), compiled with g++ against libgev_gb300.so, and
compared with the oracle after several cycles."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_binary(tmp_path):
    exe = str(tmp_path / "main_loop_gpu")
    libdir = os.path.join(ROOT, "gevolution-1.2_gb300")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "main_loop_gpu.cpp"), "-o", exe, "-L" + libdir, "-lgev_gb300",
                    "-Wl,-rpath," + libdir], check=True)
    return exe


def test_cpp_main_loop_matches_oracle(gpu, oracle, tmp_path):
    N, steps = 16, 4
    o = oracle.Sim(N).ic(**oracle.default_icparams(N, 5.0 * N, seed=13))
    sc = o.scalars()
    cm = o.cosmo
    state = tmp_path / "state.bin"
    with open(state, "wb") as f:
        f.write(np.array([N, 0], np.int32).tobytes())
        f.write(np.array([sc["a"], sc["tau"], sc["dtau"], sc["dtau_old"], sc["fourpiG"], sc["Cf"], sc["steplimit"],
                          sc["z_relax"], sc["mass"], cm["Omega_cdm"], cm["Omega_b"], cm["Omega_Lambda"],
                          cm["Omega_rad"]], np.float64).tobytes())
        f.write(np.ascontiguousarray(o.particles).tobytes())
        for name in ("phi", "chi", "Bi"):
            f.write(np.ascontiguousarray(o.field(name)).tobytes())
        f.write(np.ascontiguousarray(o.spectrum("BiFT")).tobytes())
    exe = build_binary(tmp_path)
    out = tmp_path / "out.bin"
    subprocess.run([exe, str(state), str(steps), str(out)], check=True)
    raw = open(out, "rb").read()
    a = np.frombuffer(raw[:8], np.float64)[0]
    npart = N ** 3
    got = np.frombuffer(raw[8:8 + 56 * npart], oracle.PART)
    pk = np.frombuffer(raw[8 + 56 * npart:8 + 56 * npart + 8 * 8], np.float64)
    occ = np.frombuffer(raw[8 + 56 * npart + 8 * 8:], np.int32)
    for _ in range(steps):
        o.step()
    assert abs(a - o.s.a) <= 1e-15 * a
    ref = o.particles
    assert (got["ID"] == ref["ID"]).all()
    assert np.abs(got["pos"] - ref["pos"]).max() * N < 1e-9
    assert np.abs(got["vel"] - ref["vel"]).max() <= 1e-10 * np.abs(ref["vel"]).max()
    # extractPowerSpectrum of BiFT through the drop-in layer vs the oracle's restatement
    _, opw, _, _, oocc = oracle.power_spectrum(o.spectrum("BiFT"), 8)
    assert (occ == oocc).all()
    m = occ > 0
    # the fields agree to 1e-10 of their maximum, so the power per bin to ~1e-9 of the largest bin
    assert np.max(np.abs(pk[m] - opw[m])) <= 1e-8 * np.abs(opw[m]).max()


def test_cpp_snapshot_and_hibernation(gpu, oracle, tmp_path):
    """The drop-in's saveGadget2 and hibernate, called from the C++ loop at its
    end: the snapshot is the restatement's file for the run's final particles,
    and the hibernation point loads back into those particles and scalars."""
    N, steps, L = 16, 3, 80.0
    o = oracle.Sim(N).ic(**oracle.default_icparams(N, L, seed=13))
    sc, cm = o.scalars(), o.cosmo
    state = tmp_path / "state.bin"
    with open(state, "wb") as f:
        f.write(np.array([N, 0], np.int32).tobytes())
        f.write(np.array([sc["a"], sc["tau"], sc["dtau"], sc["dtau_old"], sc["fourpiG"], sc["Cf"], sc["steplimit"],
                          sc["z_relax"], sc["mass"], cm["Omega_cdm"], cm["Omega_b"], cm["Omega_Lambda"],
                          cm["Omega_rad"]], np.float64).tobytes())
        f.write(np.ascontiguousarray(o.particles).tobytes())
        for name in ("phi", "chi", "Bi"):
            f.write(np.ascontiguousarray(o.field(name)).tobytes())
        f.write(np.ascontiguousarray(o.spectrum("BiFT")).tobytes())
    exe = build_binary(tmp_path)
    out, snap, hib = tmp_path / "out.bin", tmp_path / "snap", tmp_path / "hib"
    subprocess.run([exe, str(state), str(steps), str(out), str(snap), str(hib), repr(L)], check=True)
    raw = open(out, "rb").read()
    a = np.frombuffer(raw[:8], np.float64)[0]
    got = np.frombuffer(raw[8:8 + 56 * N ** 3], oracle.PART)
    # the snapshot: the restatement's writer on the same particles and header
    snap_bytes = open(snap, "rb").read()
    hdr = snap_bytes[4:260]
    ref = tmp_path / "ref_snap"
    oracle.gadget2_save(str(ref), N, got, hdr, 1)
    assert snap_bytes == open(ref, "rb").read()
    assert np.frombuffer(hdr[72:80], np.float64)[0] == a  # hdr.time
    # the hibernation point
    info = gpu.checkpoint_info(str(hib))
    assert info.a == a and info.cycle == steps and info.numpcl == N ** 3 and info.has_state == 0
    c = gpu.Context(N, gpu.PREC_FP64)
    pc = c.particles(N ** 3, 1.0)
    phi, chi, Bi, BiFT = c.real(1), c.real(1), c.real(3), c.spectrum(3)
    gpu.checkpoint_load(c, str(hib), pc, phi, chi, Bi, BiFT)
    assert pc.download().tobytes() == got.tobytes()
