"""Python front end of libgev_gb300.so over its C-ABI (include/gev_gb300.h).

This is the binding the tests and bench.py use; it mirrors the reference's
objects -- Field<Real>, Field<Cplx>, Particles -- as device-resident handles
and calls the GPU kernels through ctypes.  There is no CPU fallback: if the
library or a GPU is missing every call raises GevError.

Host arrays use the oracle's layouts: real fields (ncomp, N, N, N) float64
indexed [c, z, y, x]; spectra (ncomp, N, N, N//2+1) complex128 indexed
[c, kz, ky, kx]; particles are records of PART.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgev_gb300.so")
PART = np.dtype([("pos", "<f8", (3,)), ("vel", "<f8", (3,)), ("ID", "<i8")])

OK, EINVAL, ENOMEM, ECUDA, ETIMEOUT, ENODEV = 0, -1, -2, -3, -4, -5
PREC_FP64, PREC_MIXED = 0, 1
FIELD_REAL, FIELD_SPECTRUM = 0, 1
GR, NEWTON = 0, 1

_vp = ctypes.c_void_p
_d = ctypes.c_double
_i = ctypes.c_int
_l = ctypes.c_long


class GevError(RuntimeError):
    pass


_lib = None

_SIGS = {
    "gev_ctx_create": [_i, _i, _i, ctypes.POINTER(_vp)],
    "gev_ctx_destroy": [_vp],
    "gev_ctx_sync": [_vp],
    "gev_ctx_stream": [_vp, ctypes.POINTER(_vp)],
    "gev_ctx_info": [_vp, ctypes.POINTER(_i), ctypes.POINTER(_i), ctypes.POINTER(ctypes.c_size_t)],
    "gev_ctx_launch_count": [_vp, ctypes.POINTER(ctypes.c_longlong)],
    "gev_ctx_set_timing": [_vp, _i],
    "gev_ctx_timing_report": [_vp, ctypes.c_char_p, ctypes.c_size_t, _i],
    "gev_ctx_fft_tiles": [_vp, ctypes.POINTER(_i)],
    "gev_ctx_set_fft_tiles": [_vp, ctypes.POINTER(_i)],
    "gev_ctx_stencil_shapes": [_vp, ctypes.POINTER(_i), ctypes.POINTER(_i)],
    "gev_ctx_set_stencil_shapes": [_vp, ctypes.POINTER(_i), ctypes.POINTER(_i)],
    "gev_field_create": [_vp, _i, _i, ctypes.POINTER(_vp)],
    "gev_field_destroy": [_vp],
    "gev_field_upload": [_vp, _vp],
    "gev_field_download": [_vp, _vp],
    "gev_field_zero": [_vp],
    "gev_field_device_ptr": [_vp, ctypes.POINTER(_vp), ctypes.POINTER(ctypes.c_size_t)],
    "gev_pcls_create": [_vp, _l, _d, ctypes.POINTER(_vp)],
    "gev_pcls_destroy": [_vp],
    "gev_pcls_upload": [_vp, _vp, _l],
    "gev_pcls_download": [_vp, _vp, ctypes.POINTER(_l)],
    "gev_pcls_count": [_vp, ctypes.POINTER(_l)],
    "gev_projection_T00": [_vp, _vp, _vp, _d, _vp, _d],
    "gev_projection_T0i": [_vp, _vp, _vp, _vp, _d],
    "gev_projection_Tij": [_vp, _vp, _vp, _d, _vp, _d],
    "gev_projection_mass": [_vp, _vp, _vp],
    "gev_prepare_source_tensor": [_vp, _vp, _vp, _vp, _d],
    "gev_prepare_source_scalar": [_vp, _vp, _vp, _vp, _d, _vp, _d, _d, _d],
    "gev_fft_r2c": [_vp, _vp, _vp],
    "gev_fft_c2r": [_vp, _vp, _vp],
    "gev_fft_c2r_poisson": [_vp, _vp, _vp, _d, _d],
    "gev_fft_axis": [_vp, _vp, _i, _i],
    "gev_solve_poisson": [_vp, _vp, _vp, _d, _d],
    "gev_project_scalar": [_vp, _vp, _vp, _i],
    "gev_evolve_vector": [_vp, _vp, _vp, _d],
    "gev_project_scalar_evolve_vector": [_vp, _vp, _vp, _vp, _d],
    "gev_project_vector": [_vp, _vp, _vp, _d, _d],
    "gev_project_tensor": [_vp, _vp, _vp],
    "gev_update_q": [_vp, _vp, _i, _d, _vp, _vp, _vp, _i, _d, _d, ctypes.POINTER(_d)],
    "gev_update_pos": [_vp, _vp, _i, _d, _vp, _vp, _vp, _i, _d, _d],
    "gev_update_q_pos": [_vp, _vp, _d, _d, _i, _d, _d, _i, _vp, _vp, _vp, _vp],
    "gev_projection_T00_Tij": [_vp, _vp, _vp, _vp, _d, _vp],
    "gev_field_sum": [_vp, _vp, _i, ctypes.POINTER(_d)],
    "gev_cross_spectrum": [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _i, _i, _i, _i],
}


def lib():
    """Loads libgev_gb300.so (building it first if the sources are newer)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise GevError("libgev_gb300.so is not built: run __graft_entry__.build() or "
                           "python gevolution-1.2_gb300/build.py")
        L = ctypes.CDLL(LIB_PATH)
        for name, args in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        L.gev_strerror.restype = ctypes.c_char_p
        L.gev_strerror.argtypes = [_i]
        L.gev_ctx_last_error.restype = ctypes.c_char_p
        L.gev_ctx_last_error.argtypes = [_vp]
        _lib = L
    return _lib


def _check(rc, ctx=None, what=""):
    if rc != OK:
        msg = lib().gev_strerror(rc).decode()
        if ctx is not None and ctx.handle:
            detail = lib().gev_ctx_last_error(ctx.handle)
            if detail:
                msg += ": " + detail.decode()
        raise GevError("%s failed (%d): %s" % (what, rc, msg))


def _h(obj):
    return None if obj is None else obj.handle


class Context:
    """One grid of N^3 cells on one GPU (the Lattice / latFT pair of main.cpp:213-215)."""

    def __init__(self, N, precision=PREC_FP64, device=0):
        self.handle = None
        h = _vp()
        _check(lib().gev_ctx_create(device, N, precision, ctypes.byref(h)), None, "gev_ctx_create(N=%d)" % N)
        self.handle = h.value
        self.N = N
        self.precision = precision

    def close(self):
        if self.handle:
            lib().gev_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sync(self):
        _check(lib().gev_ctx_sync(self.handle), self, "gev_ctx_sync")

    def stream(self):
        s = _vp()
        _check(lib().gev_ctx_stream(self.handle, ctypes.byref(s)), self, "gev_ctx_stream")
        return s.value

    def launches(self):
        n = ctypes.c_longlong()
        _check(lib().gev_ctx_launch_count(self.handle, ctypes.byref(n)), self, "gev_ctx_launch_count")
        return n.value

    def set_timing(self, on=True):
        """Brackets the library's kernels and cycle phases with CUDA events (see timing())."""
        _check(lib().gev_ctx_set_timing(self.handle, 1 if on else 0), self, "gev_ctx_set_timing")

    def timing(self, reset=True):
        """Device time per kernel / phase since the last reset: {name: (count, total_ms)}."""
        buf = ctypes.create_string_buffer(1 << 16)
        _check(lib().gev_ctx_timing_report(self.handle, buf, len(buf), 1 if reset else 0), self,
               "gev_ctx_timing_report")
        out = {}
        for ln in buf.value.decode().splitlines():
            name, cnt, ms = ln.split("\t")
            out[name] = (int(cnt), float(ms))
        return out

    def fft_tiles(self):
        """log2 of the lines a tile of the r2c rows, y, z and c2r rows FFT passes."""
        lg = (_i * 4)()
        _check(lib().gev_ctx_fft_tiles(self.handle, lg), self, "gev_ctx_fft_tiles")
        return {"r2c_rows": lg[0], "y": lg[1], "z": lg[2], "c2r_rows": lg[3]}

    def set_fft_tiles(self, r2c_rows, y, z, c2r_rows):
        """Pins the mixed form's FFT tile widths instead of timing them."""
        lg = (_i * 4)(r2c_rows, y, z, c2r_rows)
        _check(lib().gev_ctx_set_fft_tiles(self.handle, lg), self, "gev_ctx_set_fft_tiles")

    def stencil_shapes(self):
        """(threads a block, cap on blocks a SM) of the scalar and tensor source stencils."""
        th, ps = (_i * 2)(), (_i * 2)()
        _check(lib().gev_ctx_stencil_shapes(self.handle, th, ps), self, "gev_ctx_stencil_shapes")
        return {"scalar": (th[0], ps[0]), "tensor": (th[1], ps[1])}

    def set_stencil_shapes(self, scalar, tensor):
        """Pins the source stencils' (threads, blocks a SM) instead of timing them."""
        th, ps = (_i * 2)(scalar[0], tensor[0]), (_i * 2)(scalar[1], tensor[1])
        _check(lib().gev_ctx_set_stencil_shapes(self.handle, th, ps), self, "gev_ctx_set_stencil_shapes")

    def bytes_in_use(self):
        b = ctypes.c_size_t()
        _check(lib().gev_ctx_info(self.handle, None, None, ctypes.byref(b)), self, "gev_ctx_info")
        return b.value

    # factories
    def real(self, ncomp=1):
        return Field(self, FIELD_REAL, ncomp)

    def spectrum(self, ncomp=1):
        return Field(self, FIELD_SPECTRUM, ncomp)

    def particles(self, capacity, mass):
        return Particles(self, capacity, mass)


class Field:
    def __init__(self, ctx, kind, ncomp):
        self.ctx = ctx
        self.kind = kind
        self.ncomp = ncomp
        self.handle = None
        h = _vp()
        _check(lib().gev_field_create(ctx.handle, kind, ncomp, ctypes.byref(h)), ctx, "gev_field_create")
        self.handle = h.value

    def __del__(self):
        try:
            if self.handle:
                lib().gev_field_destroy(self.handle)
                self.handle = None
        except Exception:
            pass

    @property
    def shape(self):
        N = self.ctx.N
        return (self.ncomp, N, N, N) if self.kind == FIELD_REAL else (self.ncomp, N, N, N // 2 + 1)

    def upload(self, arr):
        dt = np.float64 if self.kind == FIELD_REAL else np.complex128
        a = np.ascontiguousarray(np.asarray(arr, dtype=dt).reshape(self.shape))
        _check(lib().gev_field_upload(self.handle, a.ctypes.data), self.ctx, "gev_field_upload")
        return self

    def download(self):
        dt = np.float64 if self.kind == FIELD_REAL else np.complex128
        out = np.empty(self.shape, dt)
        _check(lib().gev_field_download(self.handle, out.ctypes.data), self.ctx, "gev_field_download")
        return out

    def zero(self):
        _check(lib().gev_field_zero(self.handle), self.ctx, "gev_field_zero")
        return self

    def device_ptr(self):
        p = _vp()
        n = ctypes.c_size_t()
        _check(lib().gev_field_device_ptr(self.handle, ctypes.byref(p), ctypes.byref(n)), self.ctx,
               "gev_field_device_ptr")
        return p.value, n.value

    def sum(self, comp=0):
        out = _d()
        _check(lib().gev_field_sum(self.ctx.handle, self.handle, comp, ctypes.byref(out)), self.ctx, "gev_field_sum")
        return out.value


class Particles:
    def __init__(self, ctx, capacity, mass):
        self.ctx = ctx
        self.handle = None
        h = _vp()
        _check(lib().gev_pcls_create(ctx.handle, capacity, mass, ctypes.byref(h)), ctx, "gev_pcls_create")
        self.handle = h.value
        self.mass = mass

    def __del__(self):
        try:
            if self.handle:
                lib().gev_pcls_destroy(self.handle)
                self.handle = None
        except Exception:
            pass

    def upload(self, parts):
        p = np.ascontiguousarray(parts, dtype=PART)
        _check(lib().gev_pcls_upload(self.handle, p.ctypes.data if len(p) else None, len(p)), self.ctx,
               "gev_pcls_upload")
        return self

    def count(self):
        n = _l()
        _check(lib().gev_pcls_count(self.handle, ctypes.byref(n)), self.ctx, "gev_pcls_count")
        return n.value

    def download(self, out=None):
        """Particle records in (cell, ID) order, into `out` (e.g. pinned memory) when given."""
        if out is None:
            out = np.empty(self.count(), PART)
        n = _l()
        _check(lib().gev_pcls_download(self.handle, out.ctypes.data if len(out) else None, ctypes.byref(n)),
               self.ctx, "gev_pcls_download")
        return out


# ------------------------------------------------- reference-named operations --
def projection_T00(pcls, T00, a=1.0, phi=None, coeff=1.0):
    _check(lib().gev_projection_T00(pcls.ctx.handle, pcls.handle, T00.handle, a, _h(phi), coeff), pcls.ctx,
           "gev_projection_T00")


def projection_T0i(pcls, T0i, phi=None, coeff=1.0):
    _check(lib().gev_projection_T0i(pcls.ctx.handle, pcls.handle, T0i.handle, _h(phi), coeff), pcls.ctx,
           "gev_projection_T0i")


def projection_Tij(pcls, Tij, a=1.0, phi=None, coeff=1.0):
    _check(lib().gev_projection_Tij(pcls.ctx.handle, pcls.handle, Tij.handle, a, _h(phi), coeff), pcls.ctx,
           "gev_projection_Tij")


def projection_mass(pcls, rho):
    _check(lib().gev_projection_mass(pcls.ctx.handle, pcls.handle, rho.handle), pcls.ctx, "gev_projection_mass")


def prepare_source_tensor(phi, Tij, Sij, coeff):
    _check(lib().gev_prepare_source_tensor(phi.ctx.handle, phi.handle, Tij.handle, Sij.handle, coeff), phi.ctx,
           "gev_prepare_source_tensor")


def prepare_source_scalar(phi, chi, source, bgmodel, result, coeff, coeff2, coeff3):
    _check(lib().gev_prepare_source_scalar(phi.ctx.handle, phi.handle, chi.handle, source.handle, bgmodel,
                                           result.handle, coeff, coeff2, coeff3), phi.ctx, "gev_prepare_source_scalar")


def fft_r2c(real, spec):
    _check(lib().gev_fft_r2c(real.ctx.handle, real.handle, spec.handle), real.ctx, "gev_fft_r2c")


def fft_c2r(spec, real):
    _check(lib().gev_fft_c2r(spec.ctx.handle, spec.handle, real.handle), spec.ctx, "gev_fft_c2r")


def fft_c2r_poisson(srcFT, real, coeff, modif=0.0):
    """solveModifiedPoissonFT then c2r, srcFT kept (the potential spectrum is not written)."""
    _check(lib().gev_fft_c2r_poisson(srcFT.ctx.handle, srcFT.handle, real.handle, coeff, modif), srcFT.ctx,
           "gev_fft_c2r_poisson")


def fft_axis(spec, axis, sign):
    """One pass of the 3-D transform: 1-D FFT along y (axis 1) or z (axis 2), in place."""
    _check(lib().gev_fft_axis(spec.ctx.handle, spec.handle, axis, sign), spec.ctx, "gev_fft_axis")


def cross_spectrum(f1, f2=None, numbins=32, deconvolve=True, ktype=1, symmetric=False, comp1=-1, comp2=-1):
    """extractCrossSpectrum / extractPowerSpectrum (tools.hpp:53-240) on the device:
    returns (kbin, power, kscatter, pscatter, occupation), numbins entries each."""
    import numpy as np
    f2 = f1 if f2 is None else f2
    out = [np.zeros(numbins) for _ in range(4)]
    occ = np.zeros(numbins, np.int32)
    _check(lib().gev_cross_spectrum(f1.ctx.handle, f1.handle, f2.handle, *(o.ctypes.data for o in out), occ.ctypes.data,
                                    numbins, int(bool(deconvolve)), ktype, int(bool(symmetric)), comp1, comp2), f1.ctx,
           "gev_cross_spectrum")
    return out[0], out[1], out[2], out[3], occ


def solve_poisson(srcFT, potFT, coeff, modif=0.0):
    _check(lib().gev_solve_poisson(srcFT.ctx.handle, srcFT.handle, potFT.handle, coeff, modif), srcFT.ctx,
           "gev_solve_poisson")


def project_scalar(SijFT, chiFT, add=0):
    _check(lib().gev_project_scalar(SijFT.ctx.handle, SijFT.handle, chiFT.handle, add), SijFT.ctx,
           "gev_project_scalar")


def evolve_vector(SijFT, BiFT, a2dtau):
    _check(lib().gev_evolve_vector(SijFT.ctx.handle, SijFT.handle, BiFT.handle, a2dtau), SijFT.ctx,
           "gev_evolve_vector")

def project_scalar_evolve_vector(SijFT, chiFT, BiFT, a2dtau):
    """projectFTscalar(SijFT, chiFT) and evolveFTvector(SijFT, BiFT, a2dtau) in one pass."""
    _check(lib().gev_project_scalar_evolve_vector(SijFT.ctx.handle, SijFT.handle, chiFT.handle, BiFT.handle,
                                                  a2dtau), SijFT.ctx, "gev_project_scalar_evolve_vector")


def project_vector(SiFT, BiFT, coeff=1.0, modif=0.0):
    _check(lib().gev_project_vector(SiFT.ctx.handle, SiFT.handle, BiFT.handle, coeff, modif), SiFT.ctx,
           "gev_project_vector")


def project_tensor(SijFT, hijFT):
    _check(lib().gev_project_tensor(SijFT.ctx.handle, SijFT.handle, hijFT.handle), SijFT.ctx, "gev_project_tensor")


def projection_T00_Tij(pcls, T00, Tij, a, phi=None):
    """projection_init + projection_T00 and projection_init + projection_Tij in one sweep."""
    _check(lib().gev_projection_T00_Tij(pcls.ctx.handle, pcls.handle, T00.handle, Tij.handle, _d(a),
                                        phi.handle if phi is not None else None), pcls.ctx, "gev_projection_T00_Tij")


def update_q_pos(pcls, dtau_kick, a_kick, nfield_kick, dtau_drift, a_drift, nfield_drift, phi, chi, Bi, wait=True):
    """updateVel(update_q) then moveParticles(update_pos) in one pass (GR); returns maxvel."""
    out = _d()
    _check(lib().gev_update_q_pos(pcls.ctx.handle, pcls.handle, _d(dtau_kick), _d(a_kick), nfield_kick,
                                  _d(dtau_drift), _d(a_drift), nfield_drift, phi.handle, chi.handle, Bi.handle,
                                  ctypes.byref(out) if wait else None), pcls.ctx, "gev_update_q_pos")
    return out.value if wait else None


def update_q(pcls, kind, dtau, phi, chi, Bi, nfield, a, a2N):
    out = _d()
    _check(lib().gev_update_q(pcls.ctx.handle, pcls.handle, kind, dtau, _h(phi), _h(chi), _h(Bi), nfield, a, a2N,
                              ctypes.byref(out)), pcls.ctx, "gev_update_q")
    return out.value


def update_pos(pcls, kind, dtau, phi, chi, Bi, nfield, a, a2N):
    _check(lib().gev_update_pos(pcls.ctx.handle, pcls.handle, kind, dtau, _h(phi), _h(chi), _h(Bi), nfield, a, a2N),
           pcls.ctx, "gev_update_pos")


# ------------------------------------------------------------- simulation --
class Cosmology(ctypes.Structure):
    _fields_ = [(n, _d) for n in ("Omega_cdm", "Omega_b", "Omega_m", "Omega_Lambda", "Omega_rad")]


class SimState(ctypes.Structure):
    _fields_ = [(n, _d) for n in ("a", "tau", "dtau", "dtau_old", "fourpiG", "Cf", "steplimit", "z_relax", "maxvel",
                                  "T00hom", "phik0", "mass")] + [
        ("cosmo", Cosmology), ("vector_elliptic", _i), ("cycle", _i)]


_SIM_SIGS = {
    "gev_sim_create": [_vp, _l, ctypes.POINTER(_vp)],
    "gev_sim_destroy": [_vp],
    "gev_sim_set_state": [_vp, ctypes.POINTER(SimState)],
    "gev_sim_get_state": [_vp, ctypes.POINTER(SimState)],
    "gev_sim_field": [_vp, _i, ctypes.POINTER(_vp)],
    "gev_sim_particles": [_vp, ctypes.POINTER(_vp)],
    "gev_sim_step": [_vp],
    "gev_sim_step_graph": [_vp],
    "gev_sim_graph_info": [_vp, ctypes.POINTER(_l), ctypes.POINTER(_l), ctypes.POINTER(_l)],
}

SIM_FIELDS = {"phi": (0, FIELD_REAL, 1), "chi": (1, FIELD_REAL, 1), "source": (2, FIELD_REAL, 1),
              "Sij": (3, FIELD_REAL, 6), "Bi": (4, FIELD_REAL, 3), "scalarFT": (5, FIELD_SPECTRUM, 1),
              "SijFT": (6, FIELD_SPECTRUM, 6), "BiFT": (7, FIELD_SPECTRUM, 3)}


def _sim_lib():
    L = lib()
    if not getattr(L, "_sim_ready", False):
        for name, args in _SIM_SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        L._sim_ready = True
    return L


class _View:
    """Non-owning handle onto an object that a Sim owns."""

    def __del__(self):
        pass


class Sim:
    """Device state of one simulation and the main-loop cycle (include/gev_sim.h)."""

    def __init__(self, ctx, npart):
        self.ctx = ctx
        self.handle = None
        h = _vp()
        _check(_sim_lib().gev_sim_create(ctx.handle, npart, ctypes.byref(h)), ctx, "gev_sim_create")
        self.handle = h.value
        self._views = {}

    def __del__(self):
        try:
            if self.handle:
                _sim_lib().gev_sim_destroy(self.handle)
                self.handle = None
        except Exception:
            pass

    def field(self, name):
        if name not in self._views:
            which, kind, ncomp = SIM_FIELDS[name]
            h = _vp()
            _check(_sim_lib().gev_sim_field(self.handle, which, ctypes.byref(h)), self.ctx, "gev_sim_field")
            f = Field.__new__(Field)
            f.ctx, f.kind, f.ncomp, f.handle = self.ctx, kind, ncomp, None
            f._borrowed = h.value
            self._views[name] = f
        f = self._views[name]
        return _Borrowed(f)

    def particles(self):
        h = _vp()
        _check(_sim_lib().gev_sim_particles(self.handle, ctypes.byref(h)), self.ctx, "gev_sim_particles")
        p = _BorrowedParticles(self.ctx, h.value)
        return p

    def set_state(self, **kw):
        st = self.get_state_struct()
        for k, v in kw.items():
            if k == "cosmo":
                for ck, cv in v.items():
                    setattr(st.cosmo, ck, cv)
            else:
                setattr(st, k, v)
        _check(_sim_lib().gev_sim_set_state(self.handle, ctypes.byref(st)), self.ctx, "gev_sim_set_state")

    def get_state_struct(self):
        st = SimState()
        _check(_sim_lib().gev_sim_get_state(self.handle, ctypes.byref(st)), self.ctx, "gev_sim_get_state")
        return st

    def state(self):
        st = self.get_state_struct()
        d = {k: getattr(st, k) for k, _ in SimState._fields_ if k != "cosmo"}
        d["cosmo"] = {k: getattr(st.cosmo, k) for k, _ in Cosmology._fields_}
        return d

    def step(self):
        _check(_sim_lib().gev_sim_step(self.handle), self.ctx, "gev_sim_step")

    def step_graph(self):
        """The same cycle enqueued as one CUDA graph (gev_sim_step_graph)."""
        _check(_sim_lib().gev_sim_step_graph(self.handle), self.ctx, "gev_sim_step_graph")

    def graph_info(self):
        """(cycles launched as a graph, instantiations, cycles enqueued directly)."""
        v = [_l(), _l(), _l()]
        _check(_sim_lib().gev_sim_graph_info(self.handle, *[ctypes.byref(x) for x in v]), self.ctx,
               "gev_sim_graph_info")
        return tuple(x.value for x in v)


_BATCH_SIGS = {
    "gev_batch_create": [_i, ctypes.POINTER(_vp)],
    "gev_batch_destroy": [_vp],
    "gev_batch_step": [_vp, ctypes.POINTER(_vp), _i],
    "gev_batch_info": [_vp, ctypes.POINTER(_l), ctypes.POINTER(_l), ctypes.POINTER(_l)],
    "gev_batch_run": [_vp, ctypes.POINTER(_vp), _i, ctypes.POINTER(_d), ctypes.POINTER(_i)],
}


def _batch_lib():
    L = lib()
    if not getattr(L, "_batch_ready", False):
        for name, args in _BATCH_SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        L._batch_ready = True
    return L


class Batch:
    """One cycle of many simulations with one launch per kernel for each cohort of
    simulations of one grid size (gev_batch_step, include/gev_sim.h)."""

    def __init__(self, device=0):
        self.handle = None
        h = _vp()
        rc = _batch_lib().gev_batch_create(device, ctypes.byref(h))
        if rc != OK:
            raise GevError("gev_batch_create failed (%d)" % rc)
        self.handle = h.value

    def __del__(self):
        try:
            if self.handle:
                _batch_lib().gev_batch_destroy(self.handle)
                self.handle = None
        except Exception:
            pass

    def close(self):
        self.__del__()

    def step(self, sims):
        arr = (_vp * max(1, len(sims)))(*[s.handle for s in sims])
        rc = _batch_lib().gev_batch_step(self.handle, arr, len(sims))
        if rc != OK:
            _check(rc, sims[0].ctx if sims else None, "gev_batch_step")

    def run(self, sims, a_targets):
        """main.cpp's loop for each simulation in batched steps, each until the cycle that
        passes its target scale factor; returns the cycles each ran (waits at the end)."""
        n = len(sims)
        arr = (_vp * max(1, n))(*[s.handle for s in sims])
        at = (_d * max(1, n))(*a_targets)
        cyc = (_i * max(1, n))()
        rc = _batch_lib().gev_batch_run(self.handle, arr, n, at, cyc)
        if rc != OK:
            _check(rc, sims[0].ctx if sims else None, "gev_batch_run")
        return [cyc[k] for k in range(n)]

    def info(self):
        """(cycles run batched, cycles run directly, batched kernel launches)."""
        v = [_l(), _l(), _l()]
        _check(_batch_lib().gev_batch_info(self.handle, *[ctypes.byref(x) for x in v]), None, "gev_batch_info")
        return tuple(x.value for x in v)


class _Borrowed(Field):
    def __init__(self, f):
        self.ctx, self.kind, self.ncomp = f.ctx, f.kind, f.ncomp
        self.handle = f._borrowed

    def __del__(self):
        pass


class _BorrowedParticles(Particles):
    def __init__(self, ctx, handle):
        self.ctx = ctx
        self.handle = handle
        self.mass = None

    def __del__(self):
        pass


class ICParams(ctypes.Structure):
    _fields_ = [(n, _d) for n in ("h", "Omega_cdm", "Omega_b", "n_s", "sigma8", "z_in", "boxsize", "Cf",
                                  "steplimit")] + [("seed", ctypes.c_uint64), ("ksphere", _i),
                                                   ("correct_displacement", _i)]


def ic_params(boxsize, seed=1, z_in=100.0, Cf=48.0, steplimit=0.04, Omega_cdm=0.27, Omega_b=0.05, sigma8=0.81,
              n_s=0.96, h=0.67, ksphere=1, correct_displacement=1):
    """The initial-condition settings of the benchmark configurations (BBKS, z_in = 100,
    k-domain = sphere, correct displacement = yes)."""
    return dict(h=h, Omega_cdm=Omega_cdm, Omega_b=Omega_b, n_s=n_s, sigma8=sigma8, z_in=z_in, boxsize=boxsize, Cf=Cf,
                steplimit=steplimit, seed=seed, ksphere=ksphere, correct_displacement=correct_displacement)


def sim_ic_generate(sim, **params):
    L = _sim_lib()
    if not getattr(L, "_ic_ready", False):
        L.gev_sim_ic_generate.argtypes = [_vp, ctypes.POINTER(ICParams)]
        L.gev_sim_ic_generate.restype = ctypes.c_int
        L._ic_ready = True
    p = ICParams(**params)
    _check(L.gev_sim_ic_generate(sim.handle, ctypes.byref(p)), sim.ctx, "gev_sim_ic_generate")
    return sim


Sim.ic_generate = sim_ic_generate


# ------------------------------------------------ snapshots and restarts --
class Gadget2Header(ctypes.Structure):
    """gadget2_header (metadata.hpp:152-171), 256 bytes."""
    _fields_ = [("npart", ctypes.c_uint32 * 6), ("mass", _d * 6), ("time", _d), ("redshift", _d),
                ("flag_sfr", ctypes.c_int32), ("flag_feedback", ctypes.c_int32),
                ("npartTotal", ctypes.c_uint32 * 6), ("flag_cooling", ctypes.c_int32),
                ("num_files", ctypes.c_int32), ("BoxSize", _d), ("Omega0", _d), ("OmegaLambda", _d),
                ("HubbleParam", _d), ("flag_age", ctypes.c_int32), ("flag_metals", ctypes.c_int32),
                ("npartTotalHW", ctypes.c_uint32 * 6), ("fill", ctypes.c_char * 64)]


assert ctypes.sizeof(Gadget2Header) == 256

GADGET_LENGTH_CONVERSION = 0.001
GADGET_MASS_CONVERSION = 1.0e10
GADGET_VELOCITY_CONVERSION = 3.335640952e-6
CKPT_FROM_B = 1


class CheckpointInfo(ctypes.Structure):
    _fields_ = [("a", _d), ("tau", _d), ("dtau", _d), ("cycle", _i), ("has_state", _i), ("state", SimState),
                ("numpcl", _l), ("N", _i), ("prec", _i)]


_IO_SIGS = {
    "gev_gadget2_save": [_vp, _vp, ctypes.c_char_p, ctypes.POINTER(Gadget2Header), _i, _d, _d, _vp, _i, _i],
    "gev_gadget2_load": [_vp, _vp, ctypes.c_char_p, ctypes.POINTER(Gadget2Header), _i],
    "gev_checkpoint_save": [_vp, ctypes.c_char_p, _vp, _vp, _vp, _vp, _vp, _d, _d, _d, _i, ctypes.POINTER(SimState)],
    "gev_checkpoint_load": [_vp, ctypes.c_char_p, _vp, _vp, _vp, _vp, _vp, _i, ctypes.POINTER(CheckpointInfo)],
    "gev_checkpoint_info_read": [ctypes.c_char_p, ctypes.POINTER(CheckpointInfo)],
    "gev_sim_hibernate": [_vp, ctypes.c_char_p],
    "gev_sim_restart": [_vp, ctypes.c_char_p, _i],
}


def _io_lib():
    L = _sim_lib()
    if not getattr(L, "_io_ready", False):
        for name, args in _IO_SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        L._io_ready = True
    return L


def gadget2_header(npart, time, boxsize_mpc_h, mass=0.0, Omega0=0.32, OmegaLambda=0.68, h=0.67, redshift=None):
    """A header filled as writeSnapshots does (output.hpp:362-403) for one CDM species."""
    hdr = Gadget2Header()
    hdr.num_files = 1
    hdr.Omega0, hdr.OmegaLambda, hdr.HubbleParam = Omega0, OmegaLambda, h
    hdr.BoxSize = boxsize_mpc_h / GADGET_LENGTH_CONVERSION
    hdr.time = time
    hdr.redshift = (1.0 / time) - 1.0 if redshift is None else redshift
    hdr.npart[1] = npart % (1 << 32)
    hdr.npartTotal[1] = hdr.npart[1]
    hdr.npartTotalHW[1] = npart >> 32
    hdr.mass[1] = mass
    return hdr


def gadget2_save(pcls, filename, hdr, tracer_factor=1, dtau_pos=0.0, dtau_vel=0.0, phi=None, exact_output=False,
                 id_bytes=8):
    _check(_io_lib().gev_gadget2_save(pcls.ctx.handle, pcls.handle, os.fsencode(filename), ctypes.byref(hdr),
                                      tracer_factor, dtau_pos, dtau_vel, _h(phi) if phi is not None else None,
                                      1 if exact_output else 0, id_bytes), pcls.ctx, "gev_gadget2_save")


def gadget2_load(pcls, filename, id_bytes=8):
    hdr = Gadget2Header()
    _check(_io_lib().gev_gadget2_load(pcls.ctx.handle, pcls.handle, os.fsencode(filename), ctypes.byref(hdr),
                                      id_bytes), pcls.ctx, "gev_gadget2_load")
    return hdr


def checkpoint_save(ctx, path, pcls, phi, chi, Bi, BiFT, a, tau, dtau, cycle):
    _check(_io_lib().gev_checkpoint_save(ctx.handle, os.fsencode(path), pcls.handle, _h(phi), _h(chi),
                                         _h(Bi) if Bi is not None else None,
                                         _h(BiFT) if BiFT is not None else None, a, tau, dtau, cycle, None),
           ctx, "gev_checkpoint_save")


def checkpoint_load(ctx, path, pcls=None, phi=None, chi=None, Bi=None, BiFT=None, flags=0):
    info = CheckpointInfo()
    hv = [_h(x) for x in (pcls, phi, chi, Bi, BiFT)]
    _check(_io_lib().gev_checkpoint_load(ctx.handle, os.fsencode(path), *hv, flags, ctypes.byref(info)), ctx,
           "gev_checkpoint_load")
    return info


def checkpoint_info(path):
    info = CheckpointInfo()
    rc = _io_lib().gev_checkpoint_info_read(os.fsencode(path), ctypes.byref(info))
    if rc != OK:
        raise GevError("gev_checkpoint_info_read: not a readable hibernation file")
    return info


def _sim_hibernate(sim, path):
    _check(_io_lib().gev_sim_hibernate(sim.handle, os.fsencode(path)), sim.ctx, "gev_sim_hibernate")


def _sim_restart(sim, path, flags=0):
    _check(_io_lib().gev_sim_restart(sim.handle, os.fsencode(path), flags), sim.ctx, "gev_sim_restart")
    return sim


Sim.hibernate = _sim_hibernate
Sim.restart = _sim_restart


# ------------------------------------------------------- spectrum outputs --
MASK_PHI, MASK_CHI, MASK_POT, MASK_B, MASK_T00, MASK_RBARE, MASK_HIJ, MASK_DELTA, MASK_DBARE = (
    1, 2, 4, 8, 16, 64, 128, 4096, 8192)


class PkSettings(ctypes.Structure):
    _fields_ = [("out_pk", _i), ("numbins", _i), ("boxsize", _d), ("z_target", _d), ("exact_output", _i),
                ("output_path", ctypes.c_char_p), ("basename_pk", ctypes.c_char_p)]


_PK_SIGS = {
    "gev_write_power_spectrum": [_vp, _vp, _vp, _vp, _vp, _i, _d, _d, ctypes.c_char_p, ctypes.c_char_p, _d, _d, _i],
    "gev_sim_write_spectra": [_vp, ctypes.POINTER(PkSettings), _i],
    "gev_sim_step_fields": [_vp],
    "gev_sim_step_particles": [_vp],
}


def _pk_lib():
    L = _io_lib()
    if not getattr(L, "_pk_ready", False):
        for name, args in _PK_SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        L._pk_ready = True
    return L


def write_power_spectrum(kbin, power, kscatter, pscatter, occupation, rescalek, rescalep, filename, description, a,
                         z_target=-1.0, exact_output=False):
    """writePowerSpectrum (tools.hpp:268-345): host code, no GPU needed."""
    arrs = [np.ascontiguousarray(x, np.float64) for x in (kbin, power, kscatter, pscatter)]
    occ = np.ascontiguousarray(occupation, np.int32)
    rc = _pk_lib().gev_write_power_spectrum(*[x.ctypes.data for x in arrs], occ.ctypes.data, len(occ), rescalek,
                                            rescalep, os.fsencode(filename), description.encode(), a, z_target,
                                            1 if exact_output else 0)
    if rc != OK:
        raise GevError("gev_write_power_spectrum failed (%d)" % rc)


def _sim_write_spectra(sim, out_pk, numbins, boxsize, pkcount, output_path="", basename_pk="pk_", z_target=-1.0,
                       exact_output=False):
    cfg = PkSettings(out_pk, numbins, boxsize, z_target, 1 if exact_output else 0, os.fsencode(output_path),
                     os.fsencode(basename_pk))
    _check(_pk_lib().gev_sim_write_spectra(sim.handle, ctypes.byref(cfg), pkcount), sim.ctx, "gev_sim_write_spectra")


def _sim_step_fields(sim):
    _check(_pk_lib().gev_sim_step_fields(sim.handle), sim.ctx, "gev_sim_step_fields")


def _sim_step_particles(sim):
    _check(_pk_lib().gev_sim_step_particles(sim.handle), sim.ctx, "gev_sim_step_particles")


Sim.write_spectra = _sim_write_spectra
Sim.step_fields = _sim_step_fields
Sim.step_particles = _sim_step_particles


# ------------------------------------------------------------------ serving --
SERVE_MAX_BINS = 64


class Request(ctypes.Structure):
    _fields_ = [("N", _i), ("prec", _i), ("boxsize", _d), ("Omega_cdm", _d), ("Omega_b", _d), ("sigma8", _d),
                ("n_s", _d), ("h", _d), ("z_in", _d), ("z_target", _d), ("seed", ctypes.c_uint64), ("numbins", _i)]


class Result(ctypes.Structure):
    _fields_ = [("id", _l), ("N", _i), ("prec", _i), ("cycles", _i), ("status", _i), ("a", _d), ("tau", _d),
                ("t_submit", _d), ("t_admit", _d), ("t_done", _d), ("kbin", _d * SERVE_MAX_BINS),
                ("power", _d * SERVE_MAX_BINS), ("occupation", _i * SERVE_MAX_BINS), ("numbins", _i)]


class ServerStats(ctypes.Structure):
    _fields_ = [(n, _l) for n in ("submitted", "admitted", "completed", "failed", "active", "pending",
                                  "max_active_seen")] + [("particle_steps", _d), ("busy_seconds", _d)] + [
        (n, ctypes.c_size_t) for n in ("bytes_budget", "bytes_in_use", "bytes_peak")] + [("workers", _l),
                                                                                         ("graph_cycles", _l)]


_SERVE_SIGS = {
    "gev_server_create": [_i, ctypes.c_size_t, _i, _i, ctypes.POINTER(_vp)],
    "gev_server_create_workers": [_i, ctypes.c_size_t, _i, _i, _i, ctypes.POINTER(_vp)],
    "gev_server_set_graphs": [_vp, _i],
    "gev_server_submit": [_vp, ctypes.POINTER(Request), ctypes.POINTER(_l)],
    "gev_server_poll": [_vp, ctypes.POINTER(Result), _i, ctypes.POINTER(_i)],
    "gev_server_drain": [_vp, _d],
    "gev_server_stats_get": [_vp, ctypes.POINTER(ServerStats)],
    "gev_server_footprint": [_i, _i, _i, ctypes.POINTER(ctypes.c_size_t)],
    "gev_server_destroy": [_vp],
}


def _serve_lib():
    L = _pk_lib()
    if not getattr(L, "_serve_ready", False):
        for name, args in _SERVE_SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        L._serve_ready = True
    return L


def request(N, seed, z_target=0.0, prec=PREC_MIXED, boxsize=None, Omega_cdm=0.27, Omega_b=0.05, sigma8=0.81,
            n_s=0.96, h=0.67, z_in=100.0, numbins=32):
    """A simulation request: grid N (= particles per side), cosmology, seed, target redshift."""
    return Request(N, prec, 2.5 * N if boxsize is None else boxsize, Omega_cdm, Omega_b, sigma8, n_s, h, z_in, z_target,
                   seed, numbins)


def result_dict(r):
    nb = r.numbins
    return {"id": r.id, "N": r.N, "prec": r.prec, "cycles": r.cycles, "status": r.status, "a": r.a, "tau": r.tau,
            "t_submit": r.t_submit, "t_admit": r.t_admit, "t_done": r.t_done,
            "kbin": np.array(r.kbin[:nb]), "power": np.array(r.power[:nb]), "occupation": np.array(r.occupation[:nb])}


class Server:
    """Continuous batching of simulations on one GPU (include/gev_serve.h)."""

    def __init__(self, device=0, bytes_budget=0, max_active=0, inflight=0, workers=0, graphs=False):
        """workers: host threads that enqueue the simulations' cycles (0: chosen from
        the host's hardware threads); graphs: each cycle enqueued as one CUDA graph."""
        self.handle = None
        h = _vp()
        rc = _serve_lib().gev_server_create_workers(device, bytes_budget, max_active, inflight, workers,
                                                    ctypes.byref(h))
        if rc != OK:
            raise GevError("gev_server_create failed (%d)" % rc)
        self.handle = h.value
        if graphs:
            rc = _serve_lib().gev_server_set_graphs(self.handle, 1)
            if rc != OK:
                raise GevError("gev_server_set_graphs failed (%d)" % rc)

    def __del__(self):
        try:
            if self.handle:
                _serve_lib().gev_server_destroy(self.handle)
                self.handle = None
        except Exception:
            pass

    def close(self):
        self.__del__()

    def submit(self, req):
        i = _l()
        rc = _serve_lib().gev_server_submit(self.handle, ctypes.byref(req), ctypes.byref(i))
        if rc != OK:
            raise GevError("gev_server_submit failed (%d)" % rc)
        return i.value

    def poll(self, max_results=256):
        buf = (Result * max_results)()
        n = _i()
        _serve_lib().gev_server_poll(self.handle, buf, max_results, ctypes.byref(n))
        return [result_dict(buf[k]) for k in range(n.value)]

    def drain(self, timeout=0.0):
        rc = _serve_lib().gev_server_drain(self.handle, timeout)
        if rc != OK:
            raise GevError("gev_server_drain: %d" % rc)

    def stats(self):
        st = ServerStats()
        _serve_lib().gev_server_stats_get(self.handle, ctypes.byref(st))
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}


def footprint(N, prec=PREC_MIXED, device=0):
    b = ctypes.c_size_t()
    rc = _serve_lib().gev_server_footprint(device, N, prec, ctypes.byref(b))
    if rc != OK:
        raise GevError("gev_server_footprint failed (%d)" % rc)
    return b.value
