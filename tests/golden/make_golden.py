"""Generates the golden vectors in tests/golden/ from gevolution 1.2's own
gevolution.hpp / background.hpp compiled against the single-rank LATfield2 shim
(oracle/_ref/libgevref.so, built by `make -C oracle ref REF_SRC=<tree>`, or here
from the tree that GEV_REFERENCE_SRC names).

    GEV_REFERENCE_SRC=<gevolution-1.2 source tree> python tests/golden/make_golden.py

    python tests/golden/make_golden.py gadget     # only the Gadget-2 files
    python tests/golden/make_golden.py spectra    # only the power spectra
    python tests/golden/make_golden.py run        # only the initial conditions and cycles
    python tests/golden/make_golden.py ic         # only the random stream, kernel, displacement field

Every hot-path function is run on seeded random inputs at N = 8 and N = 12
(a radix-3 size), and a full initial condition plus three cycles of the main
loop are run at N = 8.  Gadget-2 snapshots are written and read back by the
reference's own Particles_gevolution.hpp (oracle/_ref/libgevref_gadget.so) in
three of its build variants, and tools.hpp's spectra and table writer are run
on random spectra.  Inputs and the reference's outputs are stored in
golden_N{8,12}.npz, golden_run_N8.npz, golden_gadget2_N8.npz,
golden_spectra_N12.npz and golden_ic.npz (the sitmo stream, generateCICKernel and
generateDisplacementField of ic_basic.hpp, oracle/_ref/libgevref_ic.so);
tests/test_oracle_golden.py checks the CPU restatement against them and the GPU
tests check the CUDA path.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import gevoracle as G  # noqa: E402


def particles(rng, N, n):
    p = np.zeros(n, G.PART)
    p["pos"] = rng.random((n, 3))
    # edge cases: on a vertex, on cell faces, just below 1, exactly 0
    k = min(n, 6)
    p["pos"][:k] = np.array([[0.0, 0.0, 0.0], [1.0 / N, 2.0 / N, 0.5], [np.nextafter(1.0, 0.0)] * 3,
                             [0.5, np.nextafter(1.0, 0.0), 0.0], [3.0 / N, 3.0 / N, 3.0 / N], [0.25, 0.75, 1.0 / N]])[:k]
    p["vel"] = rng.standard_normal((n, 3)) * 2e-3
    p["ID"] = rng.permutation(n * 3)[:n]
    return p


def one(N, seed):
    R = G.ref()
    rng = np.random.default_rng(seed)
    d = {}
    phi = rng.standard_normal((1, N, N, N)) * 1e-5
    chi = rng.standard_normal((1, N, N, N)) * 1e-5
    src = 0.3 + rng.standard_normal((1, N, N, N)) * 0.1
    T = rng.standard_normal((6, N, N, N)) * 1e-3
    Bi = rng.standard_normal((3, N, N, N)) * 1e-8
    d.update(phi=phi, chi=chi, src=src, T=T, Bi=Bi)
    d["out_pst"] = G.prepare_source_tensor(phi, T, 0.37, impl=R)
    d["out_pss"] = G.prepare_source_scalar(phi, chi, src, 0.32, 1.3e-3, 2.1e-4, 3.7e-5, impl=R)
    S = G.fft_r2c(T)
    B = G.fft_r2c(rng.standard_normal((3, N, N, N)))
    s1 = G.fft_r2c(src)
    d.update(S=S, B=B, s1=s1)
    d["out_poisson"] = G.poisson(s1, 3.0, 0.0, impl=R)
    d["out_poisson_modif"] = G.poisson(s1, 3.0, 0.7, impl=R)
    d["out_pscalar"] = G.project_scalar(S, None, 0, impl=R)
    d["out_pscalar_add"] = G.project_scalar(S, s1, 1, impl=R)
    d["out_evolve"] = G.evolve_vector(S, B, 0.013, impl=R)
    d["out_pvector"] = G.project_vector(B, 0.3, 0.1, impl=R)
    d["out_ptensor"] = G.project_tensor(S, impl=R)
    n = N ** 3
    p = particles(rng, N, n)
    d["parts"] = p
    for w, a in (("T00", 0.02), ("T0i", 0.02), ("Tij", 0.02)):
        d["out_dep_" + w] = G.deposit(w, N, p, 1e-3, a, phi, 1.0, impl=R)
    d["out_dep_T00_nophi"] = G.deposit("T00", N, p, 1e-3, 0.02, None, 1.0, impl=R)
    a, a2N = 0.02, 0.02 ** 2 * N
    for kind in (0, 1):
        for nf in (1, 2, 3):
            pk, vk = G.kick(N, p, kind, 0.011, phi, chi, Bi, nf, a, a2N, impl=R)
            d["out_kick_%d_%d" % (kind, nf)] = pk
            d["out_kick_max_%d_%d" % (kind, nf)] = np.array(vk)
        for nf in (0, 1, 2, 3):
            d["out_drift_%d_%d" % (kind, nf)] = G.drift(N, p, kind, 0.37, phi, chi, Bi, nf, a, a2N, impl=R)
    cm = dict(Omega_cdm=0.27, Omega_b=0.05, Omega_m=0.32, Omega_Lambda=0.68, Omega_rad=0.0)
    av = np.geomspace(0.005, 1.0, 9)
    d["bg_a"] = av
    d["out_hconf"] = np.array([G.hconf(x, 0.0123, cm, impl=R) for x in av])
    d["out_rk4"] = np.array([G.rk4bg(x, 0.0123, cm, 0.5, impl=R) for x in av])
    np.savez_compressed(os.path.join(HERE, "golden_N%d.npz" % N), **d)


def run(N=8, steps=3):
    R = G.ref()
    s = G.Sim(N).ic(**G.default_icparams(N, 40.0, seed=11))
    d = {"ic_parts": s.particles.copy(), "ic_phi": s.field("phi").copy(), "ic_chi": s.field("chi").copy(),
         "ic_Bi": s.field("Bi").copy(), "ic_BiFT": s.spectrum("BiFT").copy(),
         "ic_scalars": np.array([s.s.a, s.s.tau, s.s.dtau, s.s.dtau_old, s.s.fourpiG, s.s.mass, s.s.maxvel])}
    for k in range(steps):
        s.step(impl=R)
        d["step%d_parts" % k] = s.particles.copy()
        d["step%d_phi" % k] = s.field("phi").copy()
        d["step%d_chi" % k] = s.field("chi").copy()
        d["step%d_Bi" % k] = s.field("Bi").copy()
        d["step%d_scalars" % k] = np.array([s.s.a, s.s.tau, s.s.dtau, s.s.dtau_old, s.s.maxvel, s.s.T00hom])
    np.savez_compressed(os.path.join(HERE, "golden_run_N%d.npz" % N), **d)


GADGET_VARIANTS = (("plain", False, 8), ("exact", True, 8), ("id4", False, 4))


def gadget_header(npart, time, boxsize):
    """The 256 header bytes of one CDM snapshot, filled as output.hpp:362-403 does."""
    import struct
    u6 = [0, npart, 0, 0, 0, 0]
    mass = [0.0, 1.5e-3, 0.0, 0.0, 0.0, 0.0]
    b = struct.pack("<6I6d2d2i6I2i4d2i6I", *u6, *mass, time, 1.0 / time - 1.0, 0, 0, *u6, 0, 1,
                    boxsize / 0.001, 0.32, 0.68, 0.67, 0, 0, 0, 0, 0, 0, 0, 0)
    return b + bytes(256 - len(b))


def gadget(N=8, seed=103):
    """Gadget-2 files written and read back by the reference's own
    Particles_gevolution.hpp (three build variants, tracer factors 1 and 3)."""
    import tempfile
    rng = np.random.default_rng(seed)
    n = 700
    p = particles(rng, N, n)
    p["ID"] = rng.permutation(n) + 5
    phi = rng.standard_normal(N ** 3) * 1e-5
    time, box, dtau_pos, dtau_vel = 0.02, 320.0, 0.01, 0.015
    d = {"parts": p, "phi": phi, "params": np.array([time, box, dtau_pos, dtau_vel])}
    with tempfile.TemporaryDirectory() as tmp:
        for tf in (1, 3):
            S = int((p["ID"] % tf == 0).sum())
            hdr = gadget_header(S, time, box)
            d["hdr_tf%d" % tf] = np.frombuffer(hdr, np.uint8).copy()
            for tag, exact, idb in GADGET_VARIANTS:
                f = os.path.join(tmp, "snap")
                G.gadget2_save(f, N, p, hdr, tf, dtau_pos, dtau_vel, phi if exact else None, exact, idb, impl="ref")
                d["file_%s_tf%d" % (tag, tf)] = np.frombuffer(open(f, "rb").read(), np.uint8).copy()
                parts, _ = G.gadget2_load(f, N, n, idb, impl="ref")
                d["load_%s_tf%d" % (tag, tf)] = parts
    np.savez_compressed(os.path.join(HERE, "golden_gadget2_N%d.npz" % N), **d)


SPECTRA_CASES = (  # (name, field, field2 or None, deconvolve, comp1, comp2)
    ("auto1_dec", "F1", None, 1, -1, -1), ("auto1", "F1", None, 0, -1, -1), ("auto3", "F3", None, 0, -1, -1),
    ("auto6", "F6", None, 0, -1, -1), ("auto6_dec", "F6", None, 1, -1, -1), ("cross1", "F1", "G1", 1, -1, -1),
    ("comps6", "F6", None, 1, 0, 3))


def spectra(N=12, seed=104, numbins=10):
    """extractCrossSpectrum and writePowerSpectrum of the reference's own tools.hpp."""
    import tempfile
    rng = np.random.default_rng(seed)
    NH = N // 2 + 1
    d = {}
    for name, nc in (("F1", 1), ("G1", 1), ("F3", 3), ("F6", 6)):
        d[name] = rng.standard_normal((nc, N, N, NH)) + 1j * rng.standard_normal((nc, N, N, NH))
    for name, f1, f2, dec, c1, c2 in SPECTRA_CASES:
        out = G.cross_spectrum_ref(d[f1], d[f2 or f1], numbins, bool(dec), 1, c1, c2)
        for k, v in zip(("kbin", "power", "kscatter", "pscatter", "occupation"), out):
            d["%s_%s" % (name, k)] = v
    # the table writer: default build; EXACT_OUTPUT_REDSHIFTS before and after z_target = 2
    kb, pw, ks, ps, occ = (d["auto1_dec_" + k] for k in ("kbin", "power", "kscatter", "pscatter", "occupation"))
    occ = occ.copy()
    occ[3] = 0  # an empty bin: no row, skipped by the interpolation's reader
    d["table_occupation"] = occ
    pw2 = pw * 1.37
    d["table_power2"] = pw2
    with tempfile.TemporaryDirectory() as tmp:
        f = os.path.join(tmp, "pk.dat")
        G.write_power_spectrum(kb, pw, ks, ps, occ, 320.0, 7.5e5, f, "power spectrum of phi", 0.3, 2.0, impl="ref")
        d["table_plain"] = np.frombuffer(open(f, "rb").read(), np.uint8).copy()
        os.remove(f)
        # one cycle before z = 2 (1/a - 1 = 2.1 > 2), then one after (1.9 < 2)
        G.write_power_spectrum(kb, pw, ks, ps, occ, 320.0, 7.5e5, f, "power spectrum of phi", 1 / 3.1, 2.0, True,
                               impl="ref")
        d["table_exact_before"] = np.frombuffer(open(f, "rb").read(), np.uint8).copy()
        G.write_power_spectrum(kb, pw2, ks, ps, occ, 320.0, 7.5e5, f, "power spectrum of phi", 1 / 2.9, 2.0, True,
                               impl="ref")
        d["table_exact_after"] = np.frombuffer(open(f, "rb").read(), np.uint8).copy()
    np.savez_compressed(os.path.join(HERE, "golden_spectra_N%d.npz" % N), **d)


def ic(seed=105):
    """The reference's sitmo stream, CIC kernel and displacement field."""
    d = {}
    for s, d0 in ((7, 0), (7, 1000003), (4294967295, 3 * 65536 ** 3 + 65536 * 17 + 5)):
        d["draws_%d_%d" % (s, d0)] = G.sitmo_draws(s, d0, 40, impl="ref")
    for N, nt in ((8, 2), (12, 3), (16, 4)):
        d["kernel_sc1_N%d" % N] = G.cic_kernel(N, G.sc1_pcldata(), nt, impl="ref")
    d["kernel_std_N16"] = G.cic_kernel(16, None, 1, impl="ref")
    rng = np.random.default_rng(seed)
    for N in (8, 12, 16):
        K = np.fft.rfftn(d["kernel_sc1_N%d" % N] if N != 16 else d["kernel_sc1_N16"])
        x, y = G.ic_spline_knots(N, **G.default_icparams(N, 5.0 * N))
        d["dfield_in_N%d" % N] = K
        d["dfield_x_N%d" % N], d["dfield_y_N%d" % N] = x, y
        for ks in (0, 1):
            d["dfield_out_N%d_ks%d" % (N, ks)] = G.displacement_field(K, 0.37, x, y, 777 + N, ks, impl="ref")
    np.savez_compressed(os.path.join(HERE, "golden_ic.npz"), **d)


if __name__ == "__main__":
    if G.ref() is None:
        sys.exit("the reference sources are not available here; golden vectors cannot be regenerated")
    which = sys.argv[1:] or ["hotpath", "gadget", "spectra", "ic"]
    if "hotpath" in which:
        one(8, 101)
        one(12, 102)
    if "hotpath" in which or "run" in which:
        run(8, 3)
    if "gadget" in which:
        gadget(8, 103)
    if "spectra" in which:
        spectra(12, 104)
    if "ic" in which:
        ic(105)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))
