"""ctypes front end of the CPU restatement (oracle/libgevoracle.so) and, where it
was built, of the reference's own gevolution.hpp compiled against the LATfield2
shim (oracle/_ref/libgevref.so).

TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg use this module as the checker; the CUDA product path never
imports it.

Array conventions follow oracle/gev_oracle.h: real fields are float64 arrays of
shape (ncomp, N, N, N) indexed [c, z, y, x]; half spectra are complex128 arrays
of shape (ncomp, N, N, N//2+1) indexed [c, kz, ky, kx]; symmetric tensors use
the component order 00, 01, 02, 11, 12, 22; particles are records of PART.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PART = np.dtype([("pos", "<f8", (3,)), ("vel", "<f8", (3,)), ("ID", "<i8")])
assert PART.itemsize == 56

_dp = ctypes.POINTER(ctypes.c_double)
_lp = ctypes.POINTER(ctypes.c_long)
_vp = ctypes.c_void_p


class Cosmo(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("Omega_cdm", "Omega_b", "Omega_m", "Omega_Lambda", "Omega_rad")]


class ICParams(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in
                ("h", "Omega_cdm", "Omega_b", "n_s", "sigma8", "z_in", "boxsize", "Cf", "steplimit")] + [
                    ("seed", ctypes.c_uint64), ("ksphere", ctypes.c_int), ("correct_displacement", ctypes.c_int)]


class SimStruct(ctypes.Structure):
    _fields_ = [("N", ctypes.c_int), ("np", ctypes.c_long), ("p", _vp), ("cell_start", _lp), ("mass", ctypes.c_double)] + [
        (n, _dp) for n in ("phi", "chi", "source", "Sij", "Bi", "scalarFT", "SijFT", "BiFT")] + [
        (n, ctypes.c_double) for n in ("a", "tau", "dtau", "dtau_old", "fourpiG", "Cf", "steplimit", "z_relax",
                                       "maxvel", "T00hom", "phik0")] + [
        ("cosmo", Cosmo), ("vector_elliptic", ctypes.c_int), ("cycle", ctypes.c_int),
        ("t_phase", ctypes.c_double * 5), ("fft_count", ctypes.c_long)]

# the phases of main.cpp's BENCHMARK breakdown (main.cpp:907-922), in t_phase order
PHASES = ("projections", "gravity solver", "thereof FFTs", "update momenta", "move particles")


def build(force=False):
    so = os.path.join(HERE, "libgevoracle.so")
    subprocess.run(["make", "-s", "-C", HERE, "libgevoracle.so"] + (["-B"] if force else []), check=True)
    return so


def build_ref(src=None):
    """Builds oracle/_ref/ from the gevolution-1.2 source tree: `src`, else the
    GEV_REFERENCE_SRC environment variable.  Returns None when neither names a tree
    holding gevolution.hpp (the libraries already built under _ref/ stay usable)."""
    src = src or os.environ.get("GEV_REFERENCE_SRC")
    if not src or not os.path.exists(os.path.join(src, "gevolution.hpp")):
        return None
    subprocess.run(["make", "-s", "-C", HERE, "ref", "REF_SRC=" + src], check=True)
    return os.path.join(HERE, "_ref", "libgevref.so")


def _load(path):
    lib = ctypes.CDLL(path)
    return lib


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        _lib = _load(build())
        L = _lib
        L.gevo_kick.restype = ctypes.c_double
        L.gevo_hconf.restype = ctypes.c_double
        L.gevo_next_dtau.restype = ctypes.c_double
        L.gevo_ic_pk.restype = ctypes.c_double
        L.gevo_ic_pk_amplitude.restype = ctypes.c_double
        L.gevo_bbks_T.restype = ctypes.c_double
        for f in ("gevo_poisson", "gevo_project_vector"):
            getattr(L, f).argtypes = [ctypes.c_int, _vp, _vp, ctypes.c_double, ctypes.c_double]
        L.gevo_evolve_vector.argtypes = [ctypes.c_int, _vp, _vp, ctypes.c_double]
        L.gevo_project_scalar.argtypes = [ctypes.c_int, _vp, _vp, ctypes.c_int]
        L.gevo_prepare_source_tensor.argtypes = [ctypes.c_int, _vp, _vp, _vp, ctypes.c_double]
        L.gevo_prepare_source_scalar.argtypes = [ctypes.c_int, _vp, _vp, _vp, ctypes.c_double, _vp] + [ctypes.c_double] * 3
        L.gevo_deposit_T00.argtypes = [ctypes.c_int, ctypes.c_long, _vp, _vp, ctypes.c_double, ctypes.c_double, _vp,
                                       ctypes.c_double, _vp]
        L.gevo_deposit_T0i.argtypes = [ctypes.c_int, ctypes.c_long, _vp, _vp, ctypes.c_double, _vp, ctypes.c_double, _vp]
        L.gevo_deposit_Tij.argtypes = L.gevo_deposit_T00.argtypes
        L.gevo_deposit_mass.argtypes = [ctypes.c_int, ctypes.c_long, _vp, _vp, ctypes.c_double, _vp]
        L.gevo_kick.argtypes = [ctypes.c_int, ctypes.c_long, _vp, ctypes.c_int, ctypes.c_double, _vp, _vp, _vp, ctypes.c_int,
                                ctypes.c_double, ctypes.c_double]
        L.gevo_drift.argtypes = L.gevo_kick.argtypes + [_vp]
        L.gevo_sort.argtypes = [ctypes.c_int, ctypes.c_long, _vp, _vp]
        L.gevo_hconf.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.POINTER(Cosmo)]
        L.gevo_rk4bg.argtypes = [_dp, ctypes.c_double, ctypes.POINTER(Cosmo), ctypes.c_double]
        L.gevo_ic_pk.argtypes = [ctypes.POINTER(ICParams), ctypes.c_double]
        L.gevo_ic_pk_amplitude.argtypes = [ctypes.POINTER(ICParams)]
        L.gevo_ic_potential_k.argtypes = [ctypes.c_int, ctypes.POINTER(ICParams), _vp]
        L.gevo_power_spectrum.argtypes = [ctypes.c_int, _vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          _vp, _vp, _vp, _vp, _vp]
    return _lib


def ref():
    """The reference's own functions (None where the sources are not present)."""
    global _ref
    if _ref is None:
        path = os.path.join(HERE, "_ref", "libgevref.so")
        if not os.path.exists(path):
            path = build_ref()
            if path is None:
                return None
        R = _load(path)
        R.gevref_kick.restype = ctypes.c_double
        R.gevref_hconf.restype = ctypes.c_double
        R.gevref_rk4bg.restype = ctypes.c_double
        for f in ("gevref_poisson", "gevref_project_vector"):
            getattr(R, f).argtypes = [ctypes.c_int, _vp, _vp, ctypes.c_double, ctypes.c_double]
        R.gevref_evolve_vector.argtypes = [ctypes.c_int, _vp, _vp, ctypes.c_double]
        R.gevref_project_scalar.argtypes = [ctypes.c_int, _vp, _vp, ctypes.c_int]
        R.gevref_project_tensor.argtypes = [ctypes.c_int, _vp, _vp]
        R.gevref_prepare_source_tensor.argtypes = [ctypes.c_int, _vp, _vp, _vp, ctypes.c_double]
        R.gevref_prepare_source_scalar.argtypes = [ctypes.c_int, _vp, _vp, _vp, ctypes.c_double, _vp] + [ctypes.c_double] * 3
        R.gevref_deposit.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_long, _vp, ctypes.c_double, ctypes.c_double, _vp,
                                     ctypes.c_double, _vp]
        R.gevref_kick.argtypes = [ctypes.c_int, ctypes.c_long, _vp, ctypes.c_int, ctypes.c_double, _vp, _vp, _vp,
                                  ctypes.c_int, ctypes.c_double, ctypes.c_double]
        R.gevref_drift.argtypes = R.gevref_kick.argtypes
        R.gevref_hconf.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.POINTER(Cosmo)]
        R.gevref_rk4bg.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.POINTER(Cosmo), ctypes.c_double]
        R.gevref_sim_step.argtypes = [ctypes.POINTER(SimStruct)]
        _ref = R
    return _ref


def _p(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def _c(a, dtype):
    a = np.ascontiguousarray(a, dtype=dtype)
    return a


# ---------------------------------------------------------------- FFT ----
def fft_r2c(x):
    x = _c(x, np.float64)
    N = x.shape[-1]
    lead = x.shape[:-3]
    xs = x.reshape((-1, N, N, N))
    out = np.zeros((xs.shape[0], N, N, N // 2 + 1), np.complex128)
    for c in range(xs.shape[0]):
        lib().gevo_fft_r2c(N, _p(xs[c]), _p(out[c]))
    return out.reshape(lead + (N, N, N // 2 + 1))


def fft_c2r(F):
    F = _c(F, np.complex128)
    N = F.shape[-2]
    lead = F.shape[:-3]
    Fs = F.reshape((-1, N, N, N // 2 + 1))
    out = np.zeros((Fs.shape[0], N, N, N), np.float64)
    for c in range(Fs.shape[0]):
        lib().gevo_fft_c2r(N, _p(Fs[c]), _p(out[c]))
    return out.reshape(lead + (N, N, N))


# ---------------------------------------------------------- k-space ops ----
def kspace_tables(N):
    g = np.zeros(N)
    ks = np.zeros(N, np.complex128)
    lib().gevo_kspace_tables(N, _p(g), _p(ks))
    return g, ks


def poisson(src, coeff, modif=0.0, impl=None):
    src = _c(src, np.complex128)
    N = src.shape[-2]
    out = np.zeros_like(src)
    _call("poisson", impl)(N, _p(src), _p(out), coeff, modif)
    return out


def _call(name, impl):
    if impl is None:
        return getattr(lib(), "gevo_" + name)
    return getattr(impl, "gevref_" + name)


def project_scalar(S, chi=None, add=0, impl=None):
    S = _c(S, np.complex128)
    N = S.shape[-2]
    chi = np.zeros(S.shape[1:], np.complex128) if chi is None else _c(chi, np.complex128).copy()
    _call("project_scalar", impl)(N, _p(S), _p(chi), add)
    return chi


def evolve_vector(S, B, a2dtau, impl=None):
    S = _c(S, np.complex128)
    B = _c(B, np.complex128).copy()
    _call("evolve_vector", impl)(S.shape[-2], _p(S), _p(B), a2dtau)
    return B


def project_vector(S, coeff=1.0, modif=0.0, impl=None):
    S = _c(S, np.complex128)
    out = np.zeros_like(S)
    _call("project_vector", impl)(S.shape[-2], _p(S), _p(out), coeff, modif)
    return out


def project_tensor(S, impl=None):
    S = _c(S, np.complex128)
    out = np.zeros_like(S)
    fn = _call("project_tensor", impl)
    if impl is None:
        lib().gevo_project_tensor.argtypes = [ctypes.c_int, _vp, _vp]
    fn(S.shape[-2], _p(S), _p(out))
    return out


def prepare_source_tensor(phi, T, coeff, impl=None):
    phi = _c(phi, np.float64)
    T = _c(T, np.float64)
    out = np.zeros_like(T)
    _call("prepare_source_tensor", impl)(phi.shape[-1], _p(phi), _p(T), _p(out), coeff)
    return out


def prepare_source_scalar(phi, chi, source, bg, coeff, coeff2, coeff3, impl=None):
    phi, chi, source = (_c(a, np.float64) for a in (phi, chi, source))
    out = np.zeros_like(source)
    _call("prepare_source_scalar", impl)(phi.shape[-1], _p(phi), _p(chi), _p(source), bg, _p(out), coeff, coeff2, coeff3)
    return out


# ------------------------------------------------------------ particles ----
def sort(N, parts):
    parts = np.ascontiguousarray(parts, dtype=PART).copy()
    cs = np.zeros(N ** 3 + 1, np.int64)
    lib().gevo_sort(N, len(parts), _p(parts), _p(cs))
    return parts, cs


def deposit(which, N, parts, mass, a=1.0, phi=None, coeff=1.0, out=None, impl=None):
    """which in ('T00', 'T0i', 'Tij', 'mass'); parts need not be sorted."""
    nc = {"T00": 1, "T0i": 3, "Tij": 6, "mass": 1}[which]
    out = np.zeros((nc, N, N, N)) if out is None else _c(out, np.float64).reshape(nc, N, N, N).copy()
    phi = None if phi is None else _c(phi, np.float64)
    if impl is not None:
        p = np.ascontiguousarray(parts, dtype=PART)
        impl.gevref_deposit({"T00": 0, "T0i": 1, "Tij": 2}[which], N, len(p), _p(p), mass, a, _p(phi), coeff, _p(out))
        return out
    p, cs = sort(N, parts)
    L = lib()
    if which == "T00":
        L.gevo_deposit_T00(N, len(p), _p(p), _p(cs), mass, a, _p(phi), coeff, _p(out))
    elif which == "T0i":
        L.gevo_deposit_T0i(N, len(p), _p(p), _p(cs), mass, _p(phi), coeff, _p(out))
    elif which == "Tij":
        L.gevo_deposit_Tij(N, len(p), _p(p), _p(cs), mass, a, _p(phi), coeff, _p(out))
    else:
        L.gevo_deposit_mass(N, len(p), _p(p), _p(cs), mass, _p(out))
    return out


def kick(N, parts, kind, dtau, phi, chi, Bi, nfield, a, a2N, impl=None):
    """update_q / update_q_Newton over all particles; returns (parts sorted by
    (cell, ID), updateVel value)."""
    p, _ = sort(N, parts)
    args = [_p(None if f is None else _c(f, np.float64)) for f in (phi, chi, Bi)]
    if impl is not None:
        v = impl.gevref_kick(N, len(p), _p(p), kind, dtau, *args, nfield, a, a2N)
    else:
        v = lib().gevo_kick(N, len(p), _p(p), kind, dtau, *args, nfield, a, a2N)
    return p, v


def drift(N, parts, kind, dtau, phi, chi, Bi, nfield, a, a2N, impl=None):
    p, _ = sort(N, parts)
    args = [_p(None if f is None else _c(f, np.float64)) for f in (phi, chi, Bi)]
    if impl is not None:
        impl.gevref_drift(N, len(p), _p(p), kind, dtau, *args, nfield, a, a2N)
    else:
        cs = np.zeros(N ** 3 + 1, np.int64)
        lib().gevo_drift(N, len(p), _p(p), kind, dtau, *args, nfield, a, a2N, _p(cs))
    return p


def hconf(a, fourpiG, cosmo, impl=None):
    c = Cosmo(**cosmo)
    if impl is not None:
        return impl.gevref_hconf(a, fourpiG, ctypes.byref(c))
    return lib().gevo_hconf(a, fourpiG, ctypes.byref(c))


def rk4bg(a, fourpiG, cosmo, dtau, impl=None):
    c = Cosmo(**cosmo)
    if impl is not None:
        return impl.gevref_rk4bg(a, fourpiG, ctypes.byref(c), dtau)
    x = ctypes.c_double(a)
    lib().gevo_rk4bg(ctypes.byref(x), fourpiG, ctypes.byref(c), dtau)
    return x.value


def power_spectrum(F, numbins, symmetric=False, deconvolve=True):
    F = _c(F, np.complex128)
    if F.ndim == 3:
        F = F[None]
    N = F.shape[-2]
    kb, pw, ks, ps = (np.zeros(numbins) for _ in range(4))
    occ = np.zeros(numbins, np.int32)
    lib().gevo_power_spectrum(N, _p(F), F.shape[0], int(symmetric), numbins, int(deconvolve), _p(kb), _p(pw), _p(ks),
                              _p(ps), _p(occ))
    return kb, pw, ks, ps, occ


# ------------------------------------------------------------ simulation ----
def default_icparams(N, boxsize, seed=1, z_in=100.0, Cf=48.0, steplimit=0.04, Omega_cdm=0.27, Omega_b=0.05,
                     sigma8=0.81, n_s=0.96, h=0.67, ksphere=1, correct_displacement=1):
    return dict(h=h, Omega_cdm=Omega_cdm, Omega_b=Omega_b, n_s=n_s, sigma8=sigma8, z_in=z_in, boxsize=boxsize, Cf=Cf,
                steplimit=steplimit, seed=seed, ksphere=ksphere, correct_displacement=correct_displacement)


class Sim:
    """One simulation state (gevo_sim) driven by the restatement, or, step by step,
    by the reference's own functions (step(impl=ref()))."""

    def __init__(self, N):
        self.N = N
        self.s = SimStruct()
        if lib().gevo_sim_alloc(ctypes.byref(self.s), N, ctypes.c_long(N ** 3)) != 0:
            raise MemoryError("gevo_sim_alloc")

    def __del__(self):
        try:
            lib().gevo_sim_free(ctypes.byref(self.s))
        except Exception:
            pass

    def ic(self, **params):
        icp = ICParams(**params)
        rc = lib().gevo_ic_generate(ctypes.byref(self.s), ctypes.byref(icp))
        if rc != 0:
            raise ValueError("gevo_ic_generate failed: %d" % rc)
        return self

    def step(self, impl=None):
        if impl is None:
            lib().gevo_sim_step(ctypes.byref(self.s))
        else:
            impl.gevref_sim_step(ctypes.byref(self.s))

    def step_fields(self):
        """main.cpp:372-598: deposits and the phi, chi, B solves."""
        lib().gevo_sim_step_fields(ctypes.byref(self.s))

    def step_particles(self):
        """main.cpp:743-872: kick, background, drift, next dtau."""
        lib().gevo_sim_step_particles(ctypes.byref(self.s))

    def phase_seconds(self):
        """Wall seconds per phase of main.cpp's BENCHMARK breakdown, summed over cycles."""
        out = {k: float(self.s.t_phase[i]) for i, k in enumerate(PHASES)}
        out["fft_count"] = int(self.s.fft_count)
        return out

    # views onto the state
    def _arr(self, name, shape, dtype):
        ptr = getattr(self.s, name)
        n = int(np.prod(shape))
        buf = (ctypes.c_double * (n * (2 if dtype == np.complex128 else 1))).from_address(ctypes.addressof(ptr.contents))
        return np.frombuffer(buf, dtype=dtype).reshape(shape)

    @property
    def particles(self):
        n = self.s.np
        buf = (ctypes.c_char * (n * 56)).from_address(self.s.p)
        return np.frombuffer(buf, dtype=PART)

    @property
    def cell_start(self):
        n = self.N ** 3 + 1
        return np.ctypeslib.as_array(self.s.cell_start, shape=(n,))

    def field(self, name):
        N = self.N
        nc = {"phi": 1, "chi": 1, "source": 1, "Sij": 6, "Bi": 3}[name]
        return self._arr(name, (nc, N, N, N), np.float64)

    def spectrum(self, name):
        N = self.N
        nc = {"scalarFT": 1, "SijFT": 6, "BiFT": 3}[name]
        return self._arr(name, (nc, N, N, N // 2 + 1), np.complex128)

    def scalars(self):
        return {k: getattr(self.s, k) for k in ("a", "tau", "dtau", "dtau_old", "fourpiG", "Cf", "steplimit", "z_relax",
                                                 "maxvel", "T00hom", "phik0", "mass", "cycle", "vector_elliptic")}

    @property
    def cosmo(self):
        c = self.s.cosmo
        return {k: getattr(c, k) for k, _ in Cosmo._fields_}


# ------------------------------------------------------ hibernation of B --
def hibernate_b(Bi, a):
    """B as hibernate writes it: B / (a^2 N) (hibernation.hpp:529-538)."""
    B = np.ascontiguousarray(Bi, np.float64).copy()
    N = B.shape[-1]
    L = lib()
    L.gevo_hibernate_b.argtypes = [ctypes.c_int, _vp, ctypes.c_double]
    L.gevo_hibernate_b(N, _p(B), a)
    return B


def restart_bift_from_b(B_stored, a):
    """readIC's restart of BiFT from the stored B (ic_read.hpp:307-318)."""
    B = np.ascontiguousarray(B_stored, np.float64).copy()
    N = B.shape[-1]
    F = np.zeros((3, N, N, N // 2 + 1), np.complex128)
    L = lib()
    L.gevo_restart_bift_from_b.argtypes = [ctypes.c_int, _vp, ctypes.c_double, _vp]
    L.gevo_restart_bift_from_b(N, _p(B), a, _p(F))
    return F


# ------------------------------------------------------ Gadget-2 snapshots --
_GADGET_REF = None


def _gadget_ref():
    """The reference's own Gadget-2 writer and reader (oracle/_ref/libgevref_gadget.so)."""
    global _GADGET_REF
    if _GADGET_REF is None:
        path = os.path.join(HERE, "_ref", "libgevref_gadget.so")
        if not os.path.exists(path):
            if build_ref() is None:
                return None
        R = _load(path)
        for tag in ("plain", "exact", "id4"):
            f = getattr(R, "gevref_gadget2_save_" + tag)
            f.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_long, _vp, _vp, _vp, ctypes.c_int, ctypes.c_double,
                          ctypes.c_double]
            f = getattr(R, "gevref_gadget2_load_" + tag)
            f.argtypes = [ctypes.c_char_p, ctypes.c_int, _vp, ctypes.c_long, _vp]
            f.restype = ctypes.c_long
        _GADGET_REF = R
    return _GADGET_REF


def _gadget_tag(exact, id_bytes):
    if exact and id_bytes == 8:
        return "exact"
    if not exact and id_bytes == 8:
        return "plain"
    if not exact and id_bytes == 4:
        return "id4"
    raise ValueError("the reference is built in three variants: default, EXACT_OUTPUT_REDSHIFTS, GADGET_ID_BYTES=4")


def gadget2_save(fname, N, parts, hdr, tracer_factor=1, dtau_pos=0.0, dtau_vel=0.0, phi=None, exact=False, id_bytes=8,
                 impl=None):
    """saveGadget2 of one rank into fname.  hdr: 256 header bytes.  impl='ref' runs
    the reference's own code (oracle/_ref)."""
    p = np.ascontiguousarray(parts, dtype=PART)
    hb = np.frombuffer(bytes(hdr), np.uint8).copy()
    assert hb.size == 256
    ph = None if phi is None else np.ascontiguousarray(phi, np.float64).reshape(-1)
    fn = os.fsencode(fname)
    if impl == "ref":
        R = _gadget_ref()
        rc = getattr(R, "gevref_gadget2_save_" + _gadget_tag(exact, id_bytes))(
            fn, N, len(p), _p(p), None if ph is None else _p(ph), _p(hb), tracer_factor, dtau_pos, dtau_vel)
    else:
        L = lib()
        L.gevo_gadget2_save.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_long, _vp, _vp, _vp, ctypes.c_int,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int]
        rc = L.gevo_gadget2_save(fn, N, len(p), _p(p), None if ph is None else _p(ph), _p(hb), tracer_factor, dtau_pos,
                                 dtau_vel, 1 if exact else 0, id_bytes)
    if rc != 0:
        raise RuntimeError("gadget2_save failed")


def gadget2_load(fname, N, cap, id_bytes=8, impl=None):
    """loadGadget2 of one file: (particles in (cell, ID) order, 256 header bytes)."""
    out = np.zeros(max(cap, 1), PART)
    hb = np.zeros(256, np.uint8)
    fn = os.fsencode(fname)
    if impl == "ref":
        R = _gadget_ref()
        n = getattr(R, "gevref_gadget2_load_" + _gadget_tag(False, id_bytes))(fn, N, _p(out), cap, _p(hb))
    else:
        L = lib()
        L.gevo_gadget2_load.argtypes = [ctypes.c_char_p, ctypes.c_int, _vp, ctypes.c_long, _vp, ctypes.c_int]
        L.gevo_gadget2_load.restype = ctypes.c_long
        n = L.gevo_gadget2_load(fn, N, _p(out), cap, _p(hb), id_bytes)
    if n < 0 or n > cap:
        raise RuntimeError("gadget2_load failed")
    return out[:n], hb.tobytes()


# ------------------------------------------------------- spectrum tables --
_TOOLS_REF = None


def _tools_ref():
    """The reference's own tools.hpp spectra and writer (oracle/_ref/libgevref_tools.so)."""
    global _TOOLS_REF
    if _TOOLS_REF is None:
        path = os.path.join(HERE, "_ref", "libgevref_tools.so")
        if not os.path.exists(path):
            if build_ref() is None:
                return None
        R = _load(path)
        R.gevref_cross_spectrum.argtypes = [ctypes.c_int, _vp, _vp] + [ctypes.c_int] * 6 + [_vp] * 5
        for tag in ("plain", "exact"):
            getattr(R, "gevref_write_power_spectrum_" + tag).argtypes = [_vp] * 5 + [
                ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_double,
                ctypes.c_double]
        _TOOLS_REF = R
    return _TOOLS_REF


def cross_spectrum_ref(F1, F2, numbins, deconvolve=True, ktype=1, comp1=-1, comp2=-1):
    """extractCrossSpectrum of the reference itself (spectra (ncomp, N, N, N/2+1))."""
    F1 = _c(F1, np.complex128)
    F2 = _c(F2, np.complex128)
    if F1.ndim == 3:
        F1, F2 = F1[None], F2[None]
    N = F1.shape[-2]
    out = [np.zeros(numbins) for _ in range(4)] + [np.zeros(numbins, np.int32)]
    _tools_ref().gevref_cross_spectrum(N, _p(F1), _p(F2), F1.shape[0], numbins, int(deconvolve), ktype, comp1, comp2,
                                       *[_p(o) for o in out])
    return tuple(out)


def write_power_spectrum(kbin, power, kscatter, pscatter, occupation, rescalek, rescalep, filename, description, a,
                         z_target=-1.0, exact=False, impl=None):
    """writePowerSpectrum: the restatement, or (impl='ref') the reference's own."""
    arrs = [np.ascontiguousarray(x, np.float64) for x in (kbin, power, kscatter, pscatter)]
    occ = np.ascontiguousarray(occupation, np.int32)
    args = [_p(x) for x in arrs] + [_p(occ), len(occ), rescalek, rescalep, os.fsencode(filename), description.encode(),
                                      a, z_target]
    if impl == "ref":
        getattr(_tools_ref(), "gevref_write_power_spectrum_" + ("exact" if exact else "plain"))(*args)
    else:
        L = lib()
        L.gevo_write_power_spectrum.argtypes = [_vp] * 5 + [ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                                           ctypes.c_char_p, ctypes.c_char_p, ctypes.c_double,
                                                           ctypes.c_double, ctypes.c_int]
        if L.gevo_write_power_spectrum(*args, 1 if exact else 0) != 0:
            raise RuntimeError("write_power_spectrum failed")


# ------------------------------------------------------ initial conditions --
_IC_REF = None


def _ic_ref():
    """The reference's sitmo engine, generateCICKernel and generateDisplacementField
    (oracle/_ref/libgevref_ic.so)."""
    global _IC_REF
    if _IC_REF is None:
        path = os.path.join(HERE, "_ref", "libgevref_ic.so")
        if not os.path.exists(path):
            if build_ref() is None:
                return None
        R = _load(path)
        R.gevref_sitmo_draws.argtypes = [ctypes.c_uint, ctypes.c_ulonglong, ctypes.c_long, _vp]
        R.gevref_displacement_field.argtypes = [ctypes.c_int, _vp, ctypes.c_double, ctypes.c_int, _vp, _vp,
                                                ctypes.c_uint, ctypes.c_int]
        R.gevref_cic_kernel.argtypes = [ctypes.c_int, ctypes.c_long, _vp, ctypes.c_int, _vp]
        _IC_REF = R
    return _IC_REF


def sitmo_draws(seed, d0, n, impl=None):
    """Draws [d0, d0 + n) of sitmo::prng_engine seeded with seed."""
    out = np.zeros(n, np.uint32)
    if impl == "ref":
        _ic_ref().gevref_sitmo_draws(seed, d0, n, _p(out))
    else:
        L = lib()
        L.gevo_sitmo_draw.argtypes = [ctypes.c_uint32, ctypes.c_uint64]
        L.gevo_sitmo_draw.restype = ctypes.c_uint32
        for i in range(n):
            out[i] = L.gevo_sitmo_draw(seed, d0 + i)
    return out


def displacement_field(K, coeff, x, y, seed, ksphere, impl=None):
    """generateDisplacementField<0> on the kernel spectrum K (N, N, N/2+1)."""
    F = np.ascontiguousarray(K, np.complex128).copy()
    N = F.shape[0]
    x = np.ascontiguousarray(x, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    if impl == "ref":
        _ic_ref().gevref_displacement_field(N, _p(F), coeff, len(x), _p(x), _p(y), seed, ksphere)
    else:
        L = lib()
        L.gevo_displacement_field.argtypes = [ctypes.c_int, _vp, ctypes.c_double, ctypes.c_int, _vp, _vp,
                                              ctypes.c_uint32, ctypes.c_int]
        L.gevo_displacement_field(N, _p(F), coeff, len(x), _p(x), _p(y), seed, ksphere)
    return F


def cic_kernel(N, pcldata=None, numtile=1, impl=None):
    """generateCICKernel as an N^3 field (pcldata None: the standard kernel)."""
    pc = None if pcldata is None else np.ascontiguousarray(pcldata, np.float32).reshape(-1)
    npcl = 0 if pc is None else len(pc) // 3
    if impl == "ref":
        out = np.zeros(N ** 3)
        _ic_ref().gevref_cic_kernel(N, npcl, None if pc is None else _p(pc), numtile, _p(out))
        return out.reshape(N, N, N)
    L = lib()
    L.gevo_cic_kernel.argtypes = [ctypes.c_int, ctypes.c_long, _vp, ctypes.c_int, _vp]
    K = np.zeros(27)
    L.gevo_cic_kernel(N, npcl, None if pc is None else _p(pc), numtile, _p(K))
    out = np.zeros((N, N, N))
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                out[dz % N, dy % N, dx % N] += K[(dx + 1) + 3 * (dy + 1) + 9 * (dz + 1)]
    return out


SC1_DIGITS = [0, 16, 20, 4, 5, 21, 17, 1, 32, 48, 52, 36, 37, 53, 49, 33, 40, 56, 60, 44, 45, 61, 57, 41, 8, 24, 28,
              12, 13, 29, 25, 9, 10, 26, 30, 14, 15, 31, 27, 11, 42, 58, 62, 46, 47, 63, 59, 43, 34, 50, 54, 38, 39,
              55, 51, 35, 2, 18, 22, 6, 7, 23, 19, 3]


def sc1_pcldata():
    """The sc1 template (64 particles of a 4^3 cell-centred lattice) in file order."""
    return np.array([[0.125 + 0.25 * ((d >> (2 * c)) & 3) for c in range(3)] for d in SC1_DIGITS], np.float32)


def ic_spline_knots(N, **params):
    icp = ICParams(**params)
    x, y = np.zeros(512), np.zeros(512)
    L = lib()
    L.gevo_ic_spline_knots.argtypes = [ctypes.c_int, ctypes.POINTER(ICParams), _vp, _vp]
    L.gevo_ic_spline_knots(N, ctypes.byref(icp), _p(x), _p(y))
    return x, y
