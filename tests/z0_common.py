"""Runs of gevolution's main loop from z_in to z = 0 with power spectra taken where
main.cpp writes them, for the oracle (CPU restatement) and for the CUDA path.

main.cpp:639-656 writes the spectra after the field solves of the first cycle
whose a has passed the next Pk redshift, before that cycle's kick and drift, and
main.cpp:685-692 ends the loop right after the last one.  The tables compared
are those of the FP64 parity criterion (writeSpectra, output.hpp:1762-2204, CDM
in GR mode):
    phi    extractPowerSpectrum of phi's r2c, no deconvolution
    chi    the same for chi
    B      extractPowerSpectrum of BiFT, no deconvolution
    delta  projection_T00_project(particles, a, phi), r2c, CIC deconvolution
Powers are compared bin by bin before writeSpectra's constant rescaling, which
cancels in a relative comparison.
"""
import numpy as np

PK_REDSHIFTS = (10.0, 3.0, 1.0, 0.5, 0.0)
NUMBINS = 64
SPECTRA = ("phi", "chi", "B", "delta")


def _oracle_spectra(O, o, nb):
    N = o.N
    a = o.s.a
    out = {}
    for name in ("phi", "chi"):
        out[name] = O.power_spectrum(O.fft_r2c(o.field(name)), nb, deconvolve=False)
    out["B"] = O.power_spectrum(o.spectrum("BiFT"), nb, deconvolve=False)
    T00 = O.deposit("T00", N, o.particles, o.s.mass, a, o.field("phi"), 1.0)
    out["delta"] = O.power_spectrum(O.fft_r2c(T00), nb, deconvolve=True)
    return out


def oracle_run(O, o, zpk=PK_REDSHIFTS, nb=NUMBINS, on_output=None):
    """Advances oracle simulation o to the last Pk redshift; returns one record per
    output: {"z", "a", "cycle", name: (kbin, power, kscatter, pscatter, occupation)}."""
    out = []
    k = 0
    while True:
        o.step_fields()
        a = o.s.a
        if 1.0 / a < zpk[k] + 1.0:
            rec = dict(z=zpk[k], a=a, cycle=o.s.cycle)
            rec.update(_oracle_spectra(O, o, nb))
            out.append(rec)
            if on_output:
                on_output(rec)
            k += 1
            if k == len(zpk):
                return out
        o.step_particles()


def _gpu_spectra(G, ctx, s, nb):
    st = s.state()
    out = {}
    for name in ("phi", "chi"):
        sp = ctx.spectrum(1)
        G.fft_r2c(s.field(name), sp)
        out[name] = G.cross_spectrum(sp, numbins=nb, deconvolve=False)
    out["B"] = G.cross_spectrum(s.field("BiFT"), numbins=nb, deconvolve=False)
    T = ctx.real(1)
    G.projection_T00(s.particles(), T, st["a"], s.field("phi"))
    sp = ctx.spectrum(1)
    G.fft_r2c(T, sp)
    out["delta"] = G.cross_spectrum(sp, numbins=nb, deconvolve=True)
    return out


def gpu_run(G, ctx, s, zpk=PK_REDSHIFTS, nb=NUMBINS, on_output=None):
    """The same loop through the C-ABI (gev_sim_step_fields / gev_sim_step_particles)."""
    out = []
    k = 0
    while True:
        s.step_fields()
        st = s.state()
        a = st["a"]
        if 1.0 / a < zpk[k] + 1.0:
            rec = dict(z=zpk[k], a=a, cycle=st["cycle"])
            rec.update(_gpu_spectra(G, ctx, s, nb))
            out.append(rec)
            if on_output:
                on_output(rec)
            k += 1
            if k == len(zpk):
                return out
        s.step_particles()


def load_sim(s, o):
    """Copies an oracle simulation state into a device simulation (both forms)."""
    s.particles().upload(o.particles)
    for name in ("phi", "chi", "Bi", "source", "Sij"):
        s.field(name).upload(o.field(name))
    for name in ("scalarFT", "SijFT", "BiFT"):
        s.field(name).upload(o.spectrum(name))
    sc = o.scalars()
    s.set_state(a=sc["a"], tau=sc["tau"], dtau=sc["dtau"], dtau_old=sc["dtau_old"], fourpiG=sc["fourpiG"],
                Cf=sc["Cf"], steplimit=sc["steplimit"], z_relax=sc["z_relax"], mass=sc["mass"], cycle=sc["cycle"],
                vector_elliptic=sc["vector_elliptic"], cosmo=o.cosmo)


def pk_max_rel(got, ref, kmax=None):
    """Largest per-bin relative deviation of power, over occupied bins (k <= kmax)."""
    kb, p, occ = ref[0], ref[1], ref[4]
    m = occ > 0
    if kmax is not None:
        m &= kb <= kmax
    assert (np.asarray(got[4]) == np.asarray(occ)).all(), "bin occupations differ"
    return float(np.max(np.abs(got[1][m] - p[m]) / np.abs(p[m])))


def by_id(parts):
    """Positions ordered by particle ID (IDs are 0 .. n-1 in the generated IC)."""
    out = np.empty((len(parts), 3))
    out[parts["ID"]] = parts["pos"]
    return out


def periodic_delta(x, y):
    d = np.asarray(x) - np.asarray(y)
    return d - np.round(d)
