"""The CPU restatement (oracle/) against the golden vectors produced by the
reference's own gevolution.hpp (tests/golden/make_golden.py).  With the same
compile flags the two agree bit for bit; the assertions allow one rounding of
slack so that a different compiler or CPU (the Arm GPU hosts) still passes."""
import os

import numpy as np
import pytest

from conftest import golden

TOL = 1e-14


def close(a, b, tol=TOL):
    a = np.asarray(a)
    b = np.asarray(b)
    scale = max(np.abs(b).max(), 1e-300)
    assert np.abs(a - b).max() <= tol * scale, np.abs(a - b).max() / scale


@pytest.mark.parametrize("N", [8, 12])
def test_sources_and_kspace(oracle, N):
    g = golden("golden_N%d.npz" % N)
    G = oracle
    close(G.prepare_source_tensor(g["phi"], g["T"], 0.37), g["out_pst"])
    close(G.prepare_source_scalar(g["phi"], g["chi"], g["src"], 0.32, 1.3e-3, 2.1e-4, 3.7e-5), g["out_pss"])
    close(G.poisson(g["s1"], 3.0, 0.0), g["out_poisson"])
    close(G.poisson(g["s1"], 3.0, 0.7), g["out_poisson_modif"])
    close(G.project_scalar(g["S"], None, 0), g["out_pscalar"])
    close(G.project_scalar(g["S"], g["s1"], 1), g["out_pscalar_add"])
    close(G.evolve_vector(g["S"], g["B"], 0.013), g["out_evolve"])
    close(G.project_vector(g["B"], 0.3, 0.1), g["out_pvector"])
    close(G.project_tensor(g["S"]), g["out_ptensor"])


@pytest.mark.parametrize("N", [8, 12])
def test_deposits(oracle, N):
    g = golden("golden_N%d.npz" % N)
    p = g["parts"]
    for w in ("T00", "T0i", "Tij"):
        close(oracle.deposit(w, N, p, 1e-3, 0.02, g["phi"], 1.0), g["out_dep_" + w])
    close(oracle.deposit("T00", N, p, 1e-3, 0.02, None, 1.0), g["out_dep_T00_nophi"])


@pytest.mark.parametrize("N", [8, 12])
def test_particle_updates(oracle, N):
    g = golden("golden_N%d.npz" % N)
    p = g["parts"]
    a, a2N = 0.02, 0.02 ** 2 * N
    for kind in (0, 1):
        for nf in (1, 2, 3):
            pk, vk = oracle.kick(N, p, kind, 0.011, g["phi"], g["chi"], g["Bi"], nf, a, a2N)
            ref = g["out_kick_%d_%d" % (kind, nf)]
            assert (pk["ID"] == ref["ID"]).all()
            close(pk["vel"], ref["vel"])
            assert abs(vk - float(g["out_kick_max_%d_%d" % (kind, nf)])) <= TOL * vk
        for nf in (0, 1, 2, 3):
            pd = oracle.drift(N, p, kind, 0.37, g["phi"], g["chi"], g["Bi"], nf, a, a2N)
            ref = g["out_drift_%d_%d" % (kind, nf)]
            assert (pd["ID"] == ref["ID"]).all()
            close(pd["pos"], ref["pos"])


def test_background(oracle):
    g = golden("golden_N8.npz")
    cm = dict(Omega_cdm=0.27, Omega_b=0.05, Omega_m=0.32, Omega_Lambda=0.68, Omega_rad=0.0)
    close([oracle.hconf(x, 0.0123, cm) for x in g["bg_a"]], g["out_hconf"])
    close([oracle.rk4bg(x, 0.0123, cm, 0.5) for x in g["bg_a"]], g["out_rk4"])


def test_full_cycles(oracle):
    """Initial conditions plus three cycles of the main loop (main.cpp:372-879)."""
    g = golden("golden_run_N8.npz")
    N = 8
    s = oracle.Sim(N).ic(**oracle.default_icparams(N, 40.0, seed=11))
    close(s.particles["pos"], g["ic_parts"]["pos"])
    close(s.particles["vel"], g["ic_parts"]["vel"])
    close(s.field("phi"), g["ic_phi"])
    close(s.field("chi"), g["ic_chi"])
    close(s.spectrum("BiFT"), g["ic_BiFT"])
    for k in range(3):
        s.step()
        ref = g["step%d_parts" % k]
        assert (s.particles["ID"] == ref["ID"]).all()
        close(s.particles["pos"], ref["pos"])
        close(s.particles["vel"], ref["vel"])
        close(s.field("phi"), g["step%d_phi" % k])
        close(s.field("chi"), g["step%d_chi" % k])
        close(s.field("Bi"), g["step%d_Bi" % k])
        sc = g["step%d_scalars" % k]
        close([s.s.a, s.s.tau, s.s.dtau, s.s.dtau_old], sc[:4])


def test_fft_against_numpy(oracle):
    """The oracle's project-written FFT (not FFTW) against numpy's pocketfft."""
    rng = np.random.default_rng(5)
    for N in (8, 12, 16, 24, 32, 48):
        x = rng.standard_normal((N, N, N))
        F = oracle.fft_r2c(x)
        close(F, np.fft.rfftn(x), 1e-14)
        close(oracle.fft_c2r(F) / N ** 3, x, 1e-14)


def test_known_answers(oracle):
    """Known answers of the reference's maths (single modes, projections)."""
    N = 16
    rng = np.random.default_rng(9)
    g2, ks = oracle.kspace_tables(N)
    # Poisson of a single mode: -coeff / N^3 / (gridk2 sum + modif)  (gevolution.hpp:511-531)
    src = np.zeros((1, N, N, N // 2 + 1), complex)
    src[0, 3, 2, 1] = 1.0
    pot = oracle.poisson(src, 2.0, 0.5)
    assert np.isclose(pot[0, 3, 2, 1].real, -2.0 / N ** 3 / (g2[1] + g2[2] + g2[3] + 0.5), rtol=1e-14)
    # projectFTvector output is transverse: sum_i kshift_i B_i = 0
    B = oracle.project_vector(oracle.fft_r2c(rng.standard_normal((3, N, N, N))), 1.0, 0.0)
    kx, ky, kz = np.arange(N // 2 + 1), np.arange(N), np.arange(N)
    div = ks[kx][None, None, :] * B[0] + ks[ky][None, :, None] * B[1] + ks[kz][:, None, None] * B[2]
    assert np.abs(div).max() <= 1e-12 * np.abs(B).max() * np.abs(ks).max()
    # projectFTscalar of an isotropic tensor s * delta_ij is zero
    Sx = oracle.fft_r2c(rng.standard_normal((1, N, N, N)))[0]
    S = np.zeros((6, N, N, N // 2 + 1), complex)
    S[0] = S[3] = S[5] = Sx
    assert np.abs(oracle.project_scalar(S)).max() <= 1e-14 * np.abs(Sx).max()
    # projectFTtensor output is traceless
    h = oracle.project_tensor(oracle.fft_r2c(rng.standard_normal((6, N, N, N))))
    assert np.abs(h[0] + h[3] + h[5]).max() <= 1e-12 * np.abs(h).max()


def test_single_particle_conserves_T00(oracle):
    """A particle on a vertex deposits all of its energy into one cell
    (gevolution.hpp:995-1018): sum T00 = m e / (dx^3 a) with e = sqrt(q^2 + a^2)."""
    N = 8
    p = np.zeros(1, oracle.PART)
    p["pos"] = [[2.0 / N, 3.0 / N, 5.0 / N]]
    p["vel"] = [[1e-3, -2e-3, 5e-4]]
    a = 0.05
    T = oracle.deposit("T00", N, p, 1e-3, a, None, 1.0)
    assert np.count_nonzero(T) == 1
    assert np.isclose(T[0, 5, 3, 2], 1e-3 * N ** 3 / a * a, rtol=1e-15)
    Tphi = oracle.deposit("T00", N, p, 1e-3, a, np.zeros((1, N, N, N)), 1.0)
    q2 = (p["vel"] ** 2).sum()
    assert np.isclose(Tphi.sum(), 1e-3 * N ** 3 / a * np.sqrt(q2 + a * a), rtol=1e-14)


def test_free_streaming_drift(oracle):
    """update_pos with zero fields moves by dtau q / sqrt(q^2 + a^2) (gevolution.hpp:842-869)."""
    N = 8
    p = np.zeros(1, oracle.PART)
    p["pos"] = [[0.3, 0.4, 0.5]]
    p["vel"] = [[1e-2, 0.0, -3e-2]]
    z = np.zeros((1, N, N, N))
    out = oracle.drift(N, p, 0, 0.1, z, z, np.zeros((3, N, N, N)), 3, 0.5, 0.25 * N)
    e = np.sqrt((p["vel"] ** 2).sum() + 0.25)
    assert np.allclose(out["pos"][0], p["pos"][0] + 0.1 * p["vel"][0] / e, rtol=1e-15, atol=1e-16)


GADGET_VARIANTS = (("plain", False, 8), ("exact", True, 8), ("id4", False, 4))


@pytest.mark.parametrize("tf", [1, 3])
@pytest.mark.parametrize("tag,exact,idb", GADGET_VARIANTS)
def test_gadget2_files_match_reference(oracle, tmp_path, tag, exact, idb, tf):
    """saveGadget2 / loadGadget2 (Particles_gevolution.hpp) restated: the files
    are byte-identical to the reference's own, and reading them back gives the
    reference's particles."""
    g = golden("golden_gadget2_N8.npz")
    time, box, dtau_pos, dtau_vel = g["params"]
    f = str(tmp_path / "snap")
    oracle.gadget2_save(f, 8, g["parts"], g["hdr_tf%d" % tf].tobytes(), tf, dtau_pos, dtau_vel,
                        g["phi"] if exact else None, exact, idb)
    assert open(f, "rb").read() == g["file_%s_tf%d" % (tag, tf)].tobytes()
    parts, hdr = oracle.gadget2_load(f, 8, len(g["parts"]), idb)
    assert hdr == g["hdr_tf%d" % tf].tobytes()
    assert parts.tobytes() == g["load_%s_tf%d" % (tag, tf)].tobytes()


def test_gadget2_against_live_reference(oracle, tmp_path):
    """Where the reference sources are present, its own Gadget-2 code on fresh
    random particles (a 12^3 grid) against the restatement."""
    if oracle._gadget_ref() is None:
        pytest.skip("reference sources not present")
    N, n = 12, 2000
    rng = np.random.default_rng(77)
    p = np.zeros(n, oracle.PART)
    p["pos"] = rng.random((n, 3))
    p["vel"] = rng.standard_normal((n, 3)) * 1e-2
    p["ID"] = rng.permutation(n)
    phi = rng.standard_normal(N ** 3) * 1e-4
    import struct
    for tag, exact, idb in GADGET_VARIANTS:
        hdr = struct.pack("<6I6d2d", 0, n, 0, 0, 0, 0, *([0.0] * 6), 0.5, 1.0) + bytes(8) + bytes(24) + \
            struct.pack("<2i4d", 0, 1, 2.5e5, 0.3, 0.7, 0.7)
        hdr = hdr + bytes(256 - len(hdr))
        a, b = str(tmp_path / "a"), str(tmp_path / "b")
        oracle.gadget2_save(a, N, p, hdr, 1, 0.03, 0.02, phi if exact else None, exact, idb)
        oracle.gadget2_save(b, N, p, hdr, 1, 0.03, 0.02, phi if exact else None, exact, idb, impl="ref")
        assert open(a, "rb").read() == open(b, "rb").read(), tag
        pa, _ = oracle.gadget2_load(a, N, n, idb)
        pb, _ = oracle.gadget2_load(b, N, n, idb, impl="ref")
        assert pa.tobytes() == pb.tobytes(), tag


SPECTRA_AUTO = (("auto1_dec", "F1", True), ("auto1", "F1", False), ("auto3", "F3", False), ("auto6", "F6", False),
                ("auto6_dec", "F6", True))


@pytest.mark.parametrize("name,field,dec", SPECTRA_AUTO)
def test_power_spectrum_matches_reference(oracle, name, field, dec):
    """extractPowerSpectrum (tools.hpp:53-240) restated: bit-identical to the
    reference's own on scalar, vector and symmetric-tensor spectra."""
    g = golden("golden_spectra_N12.npz")
    F = g[field]
    got = oracle.power_spectrum(F, 10, symmetric=F.shape[0] == 6, deconvolve=dec)
    for k, v in zip(("kbin", "power", "kscatter", "pscatter", "occupation"), got):
        assert v.tobytes() == g["%s_%s" % (name, k)].tobytes(), k


def _table_inputs(g):
    return (g["auto1_dec_kbin"], g["auto1_dec_power"], g["auto1_dec_kscatter"], g["auto1_dec_pscatter"],
            g["table_occupation"])


def _write_tables(write, tmp_path):
    """The golden sequence: a default-build table, then an EXACT_OUTPUT_REDSHIFTS
    table one cycle before z = 2 and its interpolated successor one cycle after."""
    g = golden("golden_spectra_N12.npz")
    kb, pw, ks, ps, occ = _table_inputs(g)
    f = str(tmp_path / "pk.dat")
    write(kb, pw, ks, ps, occ, 320.0, 7.5e5, f, "power spectrum of phi", 0.3, 2.0, False)
    plain = open(f, "rb").read()
    os.remove(f)
    write(kb, pw, ks, ps, occ, 320.0, 7.5e5, f, "power spectrum of phi", 1 / 3.1, 2.0, True)
    before = open(f, "rb").read()
    write(kb, g["table_power2"], ks, ps, occ, 320.0, 7.5e5, f, "power spectrum of phi", 1 / 2.9, 2.0, True)
    after = open(f, "rb").read()
    assert plain == g["table_plain"].tobytes()
    assert before == g["table_exact_before"].tobytes()
    assert after == g["table_exact_after"].tobytes()


def test_power_spectrum_table_matches_reference(oracle, tmp_path):
    """writePowerSpectrum (tools.hpp:268-345) restated, with its
    EXACT_OUTPUT_REDSHIFTS interpolation: byte-identical tables."""
    _write_tables(lambda *a: oracle.write_power_spectrum(*a[:11], exact=a[11]), tmp_path)


def test_library_table_writer_matches_reference(tmp_path):
    """The library's own table writer (host code of the C-ABI, no GPU involved)."""
    import build
    build.build()
    import gev_gb300
    _write_tables(lambda *a: gev_gb300.write_power_spectrum(*a[:11], exact_output=a[11]), tmp_path)


def test_sitmo_stream_matches_reference(oracle):
    """sitmo::prng_engine (prng_engine.hpp) restated: the reference's own draws,
    at the start of a stream, past a block boundary and deep in the fourth
    quadrant's lines of generateDisplacementField."""
    g = golden("golden_ic.npz")
    for key in g.files:
        if key.startswith("draws_"):
            _, seed, d0 = key.split("_")
            assert (oracle.sitmo_draws(int(seed), int(d0), 40) == g[key]).all(), key


@pytest.mark.parametrize("N,nt", [(8, 2), (12, 3), (16, 4)])
def test_cic_kernel_matches_reference(oracle, N, nt):
    """generateCICKernel (ic_basic.hpp:737-1052) of the sc1 template tiled nt
    times, and the standard kernel: bit-identical."""
    g = golden("golden_ic.npz")
    assert oracle.cic_kernel(N, oracle.sc1_pcldata(), nt).tobytes() == g["kernel_sc1_N%d" % N].tobytes()
    if N == 16:
        assert oracle.cic_kernel(16).tobytes() == g["kernel_std_N16"].tobytes()


@pytest.mark.parametrize("N", [8, 12, 16])
@pytest.mark.parametrize("ks", [0, 1])
def test_displacement_field_matches_reference(oracle, N, ks):
    """generateDisplacementField (ic_basic.hpp:1089-1379): the sitmo stream laid
    over the four k-space quadrants, the reused and conjugated kx = 0 lines, the
    zeroed modes, the spline of the spectrum -- bit-identical."""
    g = golden("golden_ic.npz")
    F = oracle.displacement_field(g["dfield_in_N%d" % N], 0.37, g["dfield_x_N%d" % N], g["dfield_y_N%d" % N],
                                  777 + N, ks)
    assert F.tobytes() == g["dfield_out_N%d_ks%d" % (N, ks)].tobytes()
