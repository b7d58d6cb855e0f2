"""Particle snapshots and hibernation points through the C-ABI (include/gev_io.h).

Gadget-2: the GPU writer's files are byte-identical to the reference's own
saveGadget2 (golden files from Particles_gevolution.hpp, tests/golden/), and
the GPU reader gives the reference's loadGadget2 particles.  Hibernation: a
run restarted from a hibernation point continues bit for bit; the B section
follows hibernate / readIC's a^2 N convention; damaged files are refused."""
import os

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

VARIANTS = (("plain", False, 8), ("exact", True, 8), ("id4", False, 4))


def header_from(gpu, raw):
    h = gpu.Gadget2Header()
    import ctypes
    ctypes.memmove(ctypes.addressof(h), bytes(raw), 256)
    return h


@pytest.mark.parametrize("tf", [1, 3])
@pytest.mark.parametrize("tag,exact,idb", VARIANTS)
def test_gadget2_save_matches_reference_file(gpu, tmp_path, tag, exact, idb, tf):
    g = golden("golden_gadget2_N8.npz")
    time, box, dtau_pos, dtau_vel = g["params"]
    c = gpu.Context(8, gpu.PREC_FP64)
    pc = c.particles(len(g["parts"]), 1.0).upload(g["parts"])
    phi = c.real(1).upload(g["phi"].reshape(1, 8, 8, 8))
    f = str(tmp_path / "snap")
    gpu.gadget2_save(pc, f, header_from(gpu, g["hdr_tf%d" % tf]), tf, dtau_pos, dtau_vel, phi if exact else None,
                     exact, idb)
    got = open(f, "rb").read()
    want = g["file_%s_tf%d" % (tag, tf)].tobytes()
    assert len(got) == len(want)
    assert got == want


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("tag,exact,idb", VARIANTS)
def test_gadget2_load_matches_reference(gpu, tmp_path, prec, tag, exact, idb):
    g = golden("golden_gadget2_N8.npz")
    f = str(tmp_path / "snap")
    open(f, "wb").write(g["file_%s_tf1" % tag].tobytes())
    c = gpu.Context(8, prec)
    pc = c.particles(len(g["parts"]), 1.0)
    hdr = gpu.gadget2_load(pc, f, idb)
    assert bytes(hdr) == g["hdr_tf1"].tobytes()
    got = pc.download()
    # the file holds FP32 values, which both forms store exactly
    assert got.tobytes() == g["load_%s_tf1" % tag].tobytes()


def test_gadget2_load_appends(gpu, tmp_path):
    """loadGadget2 adds to the store (addParticle_global): two files, one store."""
    g = golden("golden_gadget2_N8.npz")
    a, b = str(tmp_path / "a"), str(tmp_path / "b")
    open(a, "wb").write(g["file_plain_tf3"].tobytes())
    open(b, "wb").write(g["file_plain_tf1"].tobytes())
    c = gpu.Context(8, gpu.PREC_FP64)
    n3, n1 = len(g["load_plain_tf3"]), len(g["load_plain_tf1"])
    pc = c.particles(n1 + n3, 1.0)
    gpu.gadget2_load(pc, a)
    gpu.gadget2_load(pc, b)
    got = pc.download()
    want = np.concatenate([g["load_plain_tf3"], g["load_plain_tf1"]])
    key = lambda p: np.lexsort((p["ID"], p["pos"][:, 0]))  # noqa: E731
    assert len(got) == n1 + n3
    assert np.sort(got["ID"]).tolist() == np.sort(want["ID"]).tolist()
    assert got[key(got)].tobytes() == want[key(want)].tobytes()


def test_gadget2_mixed_form_matches_oracle(gpu, oracle, tmp_path):
    """The mixed form (FP32 momenta and phi on the device) against the restatement
    run on the same, downloaded, values."""
    N, n = 16, 5000
    rng = np.random.default_rng(31)
    p = np.zeros(n, oracle.PART)
    p["pos"] = rng.random((n, 3))
    p["vel"] = rng.standard_normal((n, 3)) * 1e-2
    p["ID"] = rng.permutation(n)
    c = gpu.Context(N, gpu.PREC_MIXED)
    pc = c.particles(n, 1.0).upload(p)
    phi = c.real(1).upload(rng.standard_normal((1, N, N, N)) * 1e-4)
    dev_p, dev_phi = pc.download(), phi.download().reshape(-1)
    for exact in (False, True):
        for tf in (1, 7):
            S = int((p["ID"] % tf == 0).sum())
            hdr = gpu.gadget2_header(S, 0.25, 400.0)
            a, b = str(tmp_path / "gpu"), str(tmp_path / "cpu")
            gpu.gadget2_save(pc, a, hdr, tf, 0.02, 0.03, phi if exact else None, exact)
            oracle.gadget2_save(b, N, dev_p, bytes(hdr), tf, 0.02, 0.03, dev_phi if exact else None, exact)
            assert open(a, "rb").read() == open(b, "rb").read(), (exact, tf)


def test_gadget2_large_store_in_batches(gpu, tmp_path):
    """7.1 M particles (192^3): more than one file batch and thousands of
    selection chunks; the file against a vectorised restatement of the default
    build's conversion (positions * BoxSize, velocities * rescale / time)."""
    N = 192
    n = N ** 3
    rng = np.random.default_rng(5)
    p = np.zeros(n, gpu.PART)
    p["pos"] = rng.random((n, 3))
    p["vel"] = rng.standard_normal((n, 3)) * 1e-3
    p["ID"] = rng.permutation(n)
    c = gpu.Context(N, gpu.PREC_FP64)
    pc = c.particles(n, 1.0).upload(p)
    ordered = pc.download()  # (cell, ID) order, the file's order
    time, box = 0.1, 1000.0
    rescale = 1.0 / np.sqrt(time) / gpu.GADGET_VELOCITY_CONVERSION
    for tf in (1, 3):
        sel = ordered[ordered["ID"] % tf == 0]
        S = len(sel)
        hdr = gpu.gadget2_header(S, time, box / 1000.0 * 1000.0)
        f = str(tmp_path / ("big%d" % tf))
        gpu.gadget2_save(pc, f, hdr, tf)
        raw = np.fromfile(f, np.uint8)
        assert raw.size == 288 + 32 * S
        marks = lambda off: int(raw[off:off + 4].view(np.uint32)[0])  # noqa: E731
        o_pos, o_vel = 268, 276 + 12 * S
        o_id = o_vel + 8 + 12 * S
        assert marks(0) == 256 and marks(260) == 256
        assert marks(264) == (12 * S) % 2 ** 32 and marks(o_vel - 4) == (12 * S) % 2 ** 32
        assert marks(o_id - 4) == 8 * S and marks(o_id + 8 * S) == 8 * S
        pos = raw[o_pos:o_pos + 12 * S].view(np.float32).reshape(S, 3)
        vel = raw[o_vel:o_vel + 12 * S].view(np.float32).reshape(S, 3)
        ids = raw[o_id:o_id + 8 * S].view(np.int64)
        assert np.array_equal(ids, sel["ID"])
        assert np.array_equal(pos, (sel["pos"] * hdr.BoxSize).astype(np.float32))
        assert np.array_equal(vel, (sel["vel"] * rescale / time).astype(np.float32))


def test_gadget2_refuses_bad_requests(gpu, tmp_path):
    g = golden("golden_gadget2_N8.npz")
    c = gpu.Context(8, gpu.PREC_FP64)
    pc = c.particles(len(g["parts"]), 1.0).upload(g["parts"])
    f = str(tmp_path / "snap")
    hdr = header_from(gpu, g["hdr_tf1"])
    hdr.npart[1] = hdr.npart[1] - 1  # the count does not match the tracers
    with pytest.raises(gpu.GevError):
        gpu.gadget2_save(pc, f, hdr, 1)
    hdr = header_from(gpu, g["hdr_tf1"])
    hdr.num_files = 2
    with pytest.raises(gpu.GevError):
        gpu.gadget2_save(pc, f, hdr, 1)
    hdr.num_files = 1
    with pytest.raises(gpu.GevError):  # the exact-output correction needs phi
        gpu.gadget2_save(pc, f, hdr, 1, 0.01, 0.01, None, True)
    small = c.particles(10, 1.0)
    gpu.gadget2_save(pc, f, hdr, 1)
    with pytest.raises(gpu.GevError):  # no room in the store
        gpu.gadget2_load(small, f)
    open(f, "wb").write(b"\x00" * 64)
    with pytest.raises(gpu.GevError):  # not a Gadget-2 file
        gpu.gadget2_load(pc, f)


def sim_snapshot(s):
    st = s.state()
    return {"parts": s.particles().download(), "phi": s.field("phi").download(), "chi": s.field("chi").download(),
            "BiFT": s.field("BiFT").download(),
            "scalars": np.array([st["a"], st["tau"], st["dtau"], st["dtau_old"], st["cycle"]], np.float64)}


@pytest.mark.parametrize("prec", [0, 1])
def test_restart_continues_bit_for_bit(gpu, tmp_path, prec):
    N = 16
    path = str(tmp_path / "hib")
    c = gpu.Context(N, prec)
    s = gpu.Sim(c, N ** 3)
    s.ic_generate(**gpu.ic_params(5.0 * N, seed=9))
    for _ in range(2):
        s.step()
    s.hibernate(path)
    info = gpu.checkpoint_info(path)
    assert info.N == N and info.prec == prec and info.numpcl == N ** 3 and info.has_state == 1
    assert info.cycle == s.state()["cycle"] and info.a == s.state()["a"]
    for _ in range(3):
        s.step()
    want = sim_snapshot(s)
    c2 = gpu.Context(N, prec)
    s2 = gpu.Sim(c2, N ** 3).restart(path)
    for _ in range(3):
        s2.step()
    got = sim_snapshot(s2)
    for k in want:
        assert got[k].tobytes() == want[k].tobytes(), k


def test_restart_from_B_follows_readIC(gpu, tmp_path):
    """hibernate stores B / (a^2 N); readIC multiplies by a^2 / N^2 and transforms
    forward (ic_read.hpp:307-318), which gives back BiFT."""
    N = 16
    path = str(tmp_path / "hib")
    c = gpu.Context(N, gpu.PREC_FP64)
    s = gpu.Sim(c, N ** 3)
    s.ic_generate(**gpu.ic_params(5.0 * N, seed=4))
    for _ in range(2):
        s.step()
    s.hibernate(path)
    Bi0, BiFT0, a = s.field("Bi").download(), s.field("BiFT").download(), s.state()["a"]
    Bi, BiFT = c.real(3), c.spectrum(3)
    info = gpu.checkpoint_load(c, path, Bi=Bi, BiFT=BiFT, flags=gpu.CKPT_FROM_B)
    assert info.a == a
    # stored B = Bi0 / (a^2 N); loaded Bi = stored * a^2 / N^2
    want = (Bi0 / (a * a * N)) * (a * a / (N * N))
    assert np.array_equal(Bi.download(), want)
    scale = np.abs(BiFT0).max()
    assert np.abs(BiFT.download() - BiFT0).max() <= 1e-12 * scale
    # without the flag the stored spectrum comes back exactly
    gpu.checkpoint_load(c, path, BiFT=BiFT)
    assert np.array_equal(BiFT.download(), BiFT0)


def test_restart_from_B_matches_the_oracle(gpu, oracle, tmp_path):
    """The B-only restart against the oracle's restatement of hibernate's B / (a^2 N)
    (hibernation.hpp:529-538) and readIC's a^2 / N^2 rescale and forward transform
    (ic_read.hpp:307-318), then three more cycles on both from the restarted state:
    BiFT to the FFTs' rounding, positions within 1e-9 of a cell, fields within 1e-10."""
    N = 16
    path = str(tmp_path / "hib")
    o = oracle.Sim(N).ic(**oracle.default_icparams(N, 5.0 * N, seed=6))
    for _ in range(3):
        o.step()
    c = gpu.Context(N, gpu.PREC_FP64)
    s = gpu.Sim(c, N ** 3)
    from z0_common import load_sim
    load_sim(s, o)
    s.hibernate(path)
    a = o.s.a
    s2 = gpu.Sim(gpu.Context(N, gpu.PREC_FP64), N ** 3)
    s2.restart(path, flags=gpu.CKPT_FROM_B)
    # the oracle restarts from the same stored B
    want = oracle.restart_bift_from_b(oracle.hibernate_b(o.field("Bi"), a), a)
    got = s2.field("BiFT").download()
    assert np.abs(got - want).max() <= 2e-14 * np.abs(want).max()
    o.spectrum("BiFT")[:] = want
    for _ in range(3):
        o.step()
        s2.step()
    g = s2.particles().download()
    assert (g["ID"] == o.particles["ID"]).all()
    assert np.abs(g["pos"] - o.particles["pos"]).max() * N < 1e-9
    for name in ("phi", "chi", "Bi"):
        ref = o.field(name)
        assert np.abs(s2.field(name).download() - ref).max() <= 1e-10 * np.abs(ref).max(), name


def test_damaged_hibernation_files_are_refused(gpu, tmp_path):
    N = 8
    path = str(tmp_path / "hib")
    c = gpu.Context(N, gpu.PREC_FP64)
    s = gpu.Sim(c, N ** 3)
    s.ic_generate(**gpu.ic_params(5.0 * N, seed=2))
    s.step()
    s.hibernate(path)
    raw = bytearray(open(path, "rb").read())
    bad = str(tmp_path / "bad")
    flipped = bytearray(raw)
    flipped[4096 + 1000] ^= 0x10  # inside the particle section
    open(bad, "wb").write(flipped)
    s2 = gpu.Sim(gpu.Context(N, gpu.PREC_FP64), N ** 3)
    with pytest.raises(gpu.GevError):
        s2.restart(bad)
    open(bad, "wb").write(raw[:len(raw) - 100])  # truncated
    with pytest.raises(gpu.GevError):
        s2.restart(bad)
    hdr = bytearray(raw)
    hdr[60] ^= 0x01  # inside the header
    open(bad, "wb").write(hdr)
    with pytest.raises(gpu.GevError):
        s2.restart(bad)
    with pytest.raises(gpu.GevError):  # another grid size
        gpu.Sim(gpu.Context(16, gpu.PREC_FP64), 16 ** 3).restart(path)
    s2.restart(path)  # the intact file still loads
    assert os.path.getsize(path) == len(raw)
    # a refused load leaves the store and the fields as they were
    before = (s2.particles().download().tobytes(), s2.field("phi").download().tobytes())
    open(bad, "wb").write(flipped)
    with pytest.raises(gpu.GevError):
        s2.restart(bad)
    assert (s2.particles().download().tobytes(), s2.field("phi").download().tobytes()) == before


def pinned(gpu, n):
    """A pinned host buffer of n particle records (the direct host-access path of
    upload and download) and its numpy view."""
    torch = pytest.importorskip("torch")
    buf = torch.empty(max(n, 1) * gpu.PART.itemsize, dtype=torch.uint8, pin_memory=True)
    return buf, buf.numpy().view(gpu.PART)[:n]


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("n", [0, 1, 255, 257, 4097])
def test_pinned_upload_download_match_pageable(gpu, prec, n):
    """Upload and download through pinned memory (the kernels read and write the host
    buffer directly) give the same bits as through pageable memory (a device staging
    copy); odd counts exercise the last half vector of a block's tile.  An upload
    already in (cell, ID) order -- a download -- takes the order-preserving relink, and
    the next cycle is the same bits either way."""
    N = 16
    rng = np.random.default_rng(n)
    parts = np.zeros(n, gpu.PART)
    parts["pos"] = rng.random((n, 3))
    parts["vel"] = rng.standard_normal((n, 3)) * 1e-3
    parts["ID"] = rng.permutation(4 * n)[:n]
    ctx = gpu.Context(N, prec)
    a = gpu.Particles(ctx, n, 1.0).upload(parts)
    ref = a.download()
    _keep, hp = pinned(gpu, n)
    hp[:] = parts
    b = gpu.Particles(ctx, n, 1.0).upload(hp)
    _keep2, out = pinned(gpu, n)
    b.download(out=out)
    assert np.array_equal(out.view(np.uint8), ref.view(np.uint8))
    # ordered upload from pinned memory, then one update of both stores
    c = gpu.Particles(ctx, n, 1.0).upload(out)
    phi = ctx.real(1).upload(rng.standard_normal((N, N, N)) * 1e-5)
    for p in (a, c):
        gpu.update_pos(p, 0, 0.3, phi, None, None, 1, 1.0, float(N))
    _keep3, o2 = pinned(gpu, n)
    c.download(out=o2)
    assert np.array_equal(o2.view(np.uint8), a.download().view(np.uint8))
    # the cycle's fused kick + drift (mixed form: each cell's run left in atomic order);
    # a pinned download packs through the (cell, ID) permutation, a pageable one reorders
    # the store first: the same records
    chi = ctx.real(1).upload(rng.standard_normal((N, N, N)) * 1e-6)
    Bi = ctx.real(3).upload(rng.standard_normal((3, N, N, N)) * 1e-7)
    for p in (a, c):
        gpu.update_q_pos(p, 0.2, 1.0, 3, 0.3, 1.0, 3, phi, chi, Bi)
    _keep4, o3 = pinned(gpu, n)
    c.download(out=o3)
    assert np.array_equal(o3.view(np.uint8), a.download().view(np.uint8))
    c.download(out=o3)  # twice: the pinned download leaves the store usable
    assert np.array_equal(o3.view(np.uint8), a.download().view(np.uint8))


@pytest.mark.parametrize("prec", [0, 1])
def test_drift_without_fields(gpu, prec):
    """moveParticles(update_pos) in GR with nfield = 0: no field is read, each particle
    moves by dtau q / sqrt(q^2 + a^2) (wrapped into the box)."""
    N, n, dtau, a = 16, 1000, 0.5, 0.8
    rng = np.random.default_rng(5)
    parts = np.zeros(n, gpu.PART)
    parts["pos"] = rng.random((n, 3))
    parts["vel"] = rng.standard_normal((n, 3)) * 1e-2
    parts["ID"] = np.arange(n)
    ctx = gpu.Context(N, prec)
    p = gpu.Particles(ctx, n, 1.0).upload(parts)
    gpu.update_pos(p, 0, dtau, None, None, None, 0, a, a * a * N)
    got = p.download()
    got = got[np.argsort(got["ID"])]
    q = parts["vel"]
    want = (parts["pos"] + dtau * q / np.sqrt((q * q).sum(1) + a * a)[:, None]) % 1.0
    d = np.abs(got["pos"] - want)
    d = np.minimum(d, 1.0 - d)
    assert d.max() < (1e-12 if prec == 0 else 1e-6)
