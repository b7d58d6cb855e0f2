// gevolution_gpu.hpp -- drop-in C++ surface for gevolution 1.2's per-step
// particle-mesh path, over device-resident fields and particles.
//
// The names, argument order and meanings are those of gevolution.hpp and of
// the LATfield2 calls main.cpp makes on this path, so that the body of the main
// loop (main.cpp:372-879) compiles against this header with its own text:
//
//   projection_init(&source);
//   projection_T00_project(&pcls_cdm, &source, a, &phi);
//   projection_T00_comm(&source);
//   prepareFTsource<Real>(phi, chi, source, bg, source, c1, c2, c3);
//   plan_source.execute(FFT_FORWARD);
//   solveModifiedPoissonFT(scalarFT, scalarFT, 1. / (dx * dx), 3. * Hc / dtau_old);
//   plan_phi.execute(FFT_BACKWARD);
//   maxvel = pcls_cdm.updateVel(update_q, (dtau + dtau_old) / 2., update_cdm_fields, nf, f_params);
//   pcls_cdm.moveParticles(update_pos, dtau, update_cdm_fields, nf, f_params);
//
// Differences a caller sees: Field<T> and Particles<...> here live on the GPU
// (one gev_ctx per lattice); updateHalo() and the *_comm folds are no-ops
// because every kernel wraps indices periodically and the deposits fold their
// own halo; update_q / update_pos / update_q_Newton / update_pos_Newton are
// markers recognised by updateVel / moveParticles (the per-particle callbacks
// run on the device).  Errors abort the process like the reference's exit(-1) /
// parallel.abortForce() (gevolution.hpp:929-933, main.cpp:177), after printing
// the library's message; define GEV_GPU_THROW to get std::runtime_error instead.
#ifndef GEVOLUTION_GPU_HPP
#define GEVOLUTION_GPU_HPP

#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/gev_gb300.h"
#include "../../include/gev_io.h"

#ifndef FFT_FORWARD
#define FFT_FORWARD 1
#define FFT_BACKWARD -1
#endif

namespace gevgpu {

typedef double Real;
struct Cplx {
  double re, im;
};
enum { symmetric = 1 };

inline void check(int rc, gev_ctx *ctx, const char *what) {
  if (rc == GEV_OK) return;
  std::string msg = std::string(what) + ": " + gev_strerror(rc);
  if (ctx) msg += std::string(" (") + gev_ctx_last_error(ctx) + ")";
#ifdef GEV_GPU_THROW
  throw std::runtime_error(msg);
#else
  std::fprintf(stderr, "%s\n", msg.c_str());
  std::exit(-1);
#endif
}

// Lattice(3, box, halo) of main.cpp:213; initializeRealFFT gives the k-space lattice
class Lattice {
 public:
  gev_ctx *ctx = nullptr;
  int N = 0, halo_ = 0;
  bool fourier = false;
  Lattice() {}
  Lattice(int dim, const int *size, int halo, int device = 0, int precision = GEV_PREC_FP64) {
    initialize(dim, size, halo, device, precision);
  }
  Lattice(const Lattice &) = delete;
  Lattice &operator=(const Lattice &) = delete;
  // the real-space lattice owns the context handle; fields and particle stores
  // hold their own references, so they may be destroyed after it
  ~Lattice() {
    if (ctx && !fourier) gev_ctx_destroy(ctx);
  }
  void initialize(int, const int *size, int halo, int device = 0, int precision = GEV_PREC_FP64) {
    N = size[0];
    halo_ = halo;
    check(gev_ctx_create(device, N, precision, &ctx), nullptr, "Lattice");
  }
  void initializeRealFFT(Lattice &lat, int) {
    ctx = lat.ctx;
    N = lat.N;
    fourier = true;
  }
  int size(int i) const { return i == 0 && fourier ? N / 2 + 1 : N; }
  int halo() const { return halo_; }
};

template <class T>
class Field {
 public:
  Lattice *lat = nullptr;
  gev_field *f = nullptr;
  int ncomp = 0;
  bool sym = false;  // a symmetric rank-2 tensor (components 00 01 02 11 12 22)
  ~Field() {
    if (f) gev_field_destroy(f);
  }
  void initialize(Lattice &l, int nc = 1) { alloc(l, nc); }
  void initialize(Lattice &l, int rows, int cols, int symm) {
    sym = symm == symmetric;
    alloc(l, sym ? rows * (rows + 1) / 2 : rows * cols);
  }
  Lattice &lattice() { return *lat; }
  int components() const { return ncomp; }
  void updateHalo() {}  // periodic indexing inside every kernel
  void upload(const double *host) { check(gev_field_upload(f, host), lat->ctx, "Field::upload"); }
  void download(double *host) { check(gev_field_download(f, host), lat->ctx, "Field::download"); }

 private:
  void alloc(Lattice &l, int nc) {
    lat = &l;
    ncomp = nc;
    check(gev_field_create(l.ctx, l.fourier ? GEV_FIELD_SPECTRUM : GEV_FIELD_REAL, nc, &f), l.ctx, "Field::initialize");
  }
};

template <class F>
void projection_init(Field<F> *f) {
  check(gev_field_zero(f->f), f->lat->ctx, "projection_init");
}
// the deposits fold their own upper halo (periodic); the *_comm calls stay for source compatibility
inline void projection_T00_comm(Field<Real> *) {}
inline void projection_T0i_comm(Field<Real> *) {}
inline void projection_Tij_comm(Field<Real> *) {}
inline void scalarProjectionCIC_comm(Field<Real> *) {}

template <class C>
class PlanFFT {
 public:
  Field<Real> *r;
  Field<C> *k;
  PlanFFT(Field<Real> *rf, Field<C> *kf) : r(rf), k(kf) {}
  void execute(int dir) {
    gev_ctx *ctx = r->lat->ctx;
    if (dir == FFT_FORWARD)
      check(gev_fft_r2c(ctx, r->f, k->f), ctx, "PlanFFT::execute(FFT_FORWARD)");
    else
      check(gev_fft_c2r(ctx, k->f, r->f), ctx, "PlanFFT::execute(FFT_BACKWARD)");
  }
};

// per-particle callbacks of gevolution.hpp:570, 709, 810, 900 as markers
struct part_simple;
struct part_simple_info {
  double mass;
};
struct part_simple_dataType {};
typedef Real (*vel_cb)(double, double, part_simple *, double *, part_simple_info, Field<Real> **, void *, int, double *,
                       double *, int);
typedef void (*pos_cb)(double, double, part_simple *, double *, part_simple_info, Field<Real> **, void *, int, double *,
                       double *, int);
inline Real update_q(double, double, part_simple *, double *, part_simple_info, Field<Real> **, void *, int, double *,
                     double *, int) {
  return 0;
}
inline Real update_q_Newton(double, double, part_simple *, double *, part_simple_info, Field<Real> **, void *, int,
                            double *, double *, int) {
  return 0;
}
inline void update_pos(double, double, part_simple *, double *, part_simple_info, Field<Real> **, void *, int, double *,
                       double *, int) {}
inline void update_pos_Newton(double, double, part_simple *, double *, part_simple_info, Field<Real> **, void *, int,
                              double *, double *, int) {}

// Gadget-2 snapshots (metadata.hpp:111-171)
typedef gev_gadget2_header gadget2_header;
#ifndef GADGET_LENGTH_CONVERSION
#define GADGET_LENGTH_CONVERSION GEV_GADGET_LENGTH_CONVERSION
#endif
#ifndef GADGET_MASS_CONVERSION
#define GADGET_MASS_CONVERSION GEV_GADGET_MASS_CONVERSION
#endif
#ifndef GADGET_VELOCITY_CONVERSION
#define GADGET_VELOCITY_CONVERSION GEV_GADGET_VELOCITY_CONVERSION
#endif
#ifndef GADGET_ID_BYTES
#define GADGET_ID_BYTES 8
#endif

template <class part = part_simple, class part_info = part_simple_info, class part_dataType = part_simple_dataType>
class Particles {
 public:
  Lattice *lat = nullptr;
  gev_pcls *p = nullptr;
  ~Particles() {
    if (p) gev_pcls_destroy(p);
  }
  void initialize(part_info info, part_dataType, Lattice *l, Real *, long capacity) {
    lat = l;
    check(gev_pcls_create(l->ctx, capacity, info.mass, &p), l->ctx, "Particles::initialize");
  }
  void upload(const gev_part *host, long n) { check(gev_pcls_upload(p, host, n), lat->ctx, "Particles::upload"); }
  long download(gev_part *host) {
    long n = 0;
    check(gev_pcls_download(p, host, &n), lat->ctx, "Particles::download");
    return n;
  }
  // Particles::updateVel (main.cpp:775): returns the reduction of the callback's value
  Real updateVel(vel_cb fn, double dtau, Field<Real> **fields, int nfield, double *params) {
    const int kind = fn == update_q ? GEV_GR : (fn == update_q_Newton ? GEV_NEWTON : -1);
    if (kind < 0) check(GEV_EINVAL, lat->ctx, "updateVel: callback has no device implementation");
    double maxvel = 0.;
    check(gev_update_q(lat->ctx, p, kind, dtau, fields[0]->f, nfield > 1 ? fields[1]->f : nullptr,
                       nfield > 2 ? fields[2]->f : nullptr, nfield, params[0], kind == GEV_GR ? params[1] : 1., &maxvel),
          lat->ctx, "updateVel");
    return maxvel;
  }
  // Particles_gevolution::saveGadget2 (Particles_gevolution.hpp:30-251); built with
  // EXACT_OUTPUT_REDSHIFTS, the drift by dtau_pos and kick by dtau_vel with phi apply
  void saveGadget2(std::string filename, gadget2_header &hdr, const int tracer_factor = 1, double dtau_pos = 0.,
                   double dtau_vel = 0., Field<Real> *phi = NULL) {
#ifdef EXACT_OUTPUT_REDSHIFTS
    const int exact = 1;
#else
    const int exact = 0;
#endif
    check(gev_gadget2_save(lat->ctx, p, filename.c_str(), &hdr, tracer_factor, dtau_pos, dtau_vel,
                           (exact && phi) ? phi->f : nullptr, exact, GADGET_ID_BYTES),
          lat->ctx, "saveGadget2");
  }
  // Particles_gevolution::loadGadget2 (Particles_gevolution.hpp:574-665): adds the file's particles
  void loadGadget2(std::string filename, gadget2_header &hdr) {
    check(gev_gadget2_load(lat->ctx, p, filename.c_str(), &hdr, GADGET_ID_BYTES), lat->ctx, "loadGadget2");
  }
  // Particles::moveParticles (main.cpp:798): drift, periodic wrap, relink
  void moveParticles(pos_cb fn, double dtau, Field<Real> **fields, int nfield, double *params) {
    const int kind = fn == update_pos ? GEV_GR : (fn == update_pos_Newton ? GEV_NEWTON : -1);
    if (kind < 0) check(GEV_EINVAL, lat->ctx, "moveParticles: callback has no device implementation");
    check(gev_update_pos(lat->ctx, p, kind, dtau, (fields && nfield > 0) ? fields[0]->f : nullptr,
                         (fields && nfield > 1) ? fields[1]->f : nullptr, (fields && nfield > 2) ? fields[2]->f : nullptr,
                         kind == GEV_GR ? nfield : 0, params[0], kind == GEV_GR ? params[1] : 1.),
          lat->ctx, "moveParticles");
  }
};

// ---- gevolution.hpp functions with the reference signatures ----
template <class FieldType>
void prepareFTsource(Field<FieldType> &phi, Field<FieldType> &Tij, Field<FieldType> &Sij, const double coeff) {
  check(gev_prepare_source_tensor(phi.lat->ctx, phi.f, Tij.f, Sij.f, coeff), phi.lat->ctx, "prepareFTsource");
}
template <class FieldType>
void prepareFTsource(Field<FieldType> &phi, Field<FieldType> &chi, Field<FieldType> &source, const FieldType bgmodel,
                     Field<FieldType> &result, const double coeff, const double coeff2, const double coeff3) {
  check(gev_prepare_source_scalar(phi.lat->ctx, phi.f, chi.f, source.f, bgmodel, result.f, coeff, coeff2, coeff3),
        phi.lat->ctx, "prepareFTsource");
}
inline void projectFTscalar(Field<Cplx> &SijFT, Field<Cplx> &chiFT, const int add = 0) {
  check(gev_project_scalar(SijFT.lat->ctx, SijFT.f, chiFT.f, add), SijFT.lat->ctx, "projectFTscalar");
}
inline void evolveFTvector(Field<Cplx> &SijFT, Field<Cplx> &BiFT, const Real a2dtau) {
  check(gev_evolve_vector(SijFT.lat->ctx, SijFT.f, BiFT.f, a2dtau), SijFT.lat->ctx, "evolveFTvector");
}
inline void projectFTvector(Field<Cplx> &SiFT, Field<Cplx> &BiFT, const Real coeff = 1., const Real modif = 0.) {
  check(gev_project_vector(SiFT.lat->ctx, SiFT.f, BiFT.f, coeff, modif), SiFT.lat->ctx, "projectFTvector");
}
inline void projectFTtensor(Field<Cplx> &SijFT, Field<Cplx> &hijFT) {
  check(gev_project_tensor(SijFT.lat->ctx, SijFT.f, hijFT.f), SijFT.lat->ctx, "projectFTtensor");
}
inline void solveModifiedPoissonFT(Field<Cplx> &sourceFT, Field<Cplx> &potFT, Real coeff, const Real modif = 0.) {
  check(gev_solve_poisson(sourceFT.lat->ctx, sourceFT.f, potFT.f, coeff, modif), sourceFT.lat->ctx,
        "solveModifiedPoissonFT");
}
template <typename part, typename part_info, typename part_dataType>
void projection_T00_project(Particles<part, part_info, part_dataType> *pcls, Field<Real> *T00, double a = 1.,
                            Field<Real> *phi = NULL, double coeff = 1.) {
  check(gev_projection_T00(T00->lat->ctx, pcls->p, T00->f, a, phi ? phi->f : nullptr, coeff), T00->lat->ctx,
        "projection_T00_project");
}
template <typename part, typename part_info, typename part_dataType>
void projection_T0i_project(Particles<part, part_info, part_dataType> *pcls, Field<Real> *T0i, Field<Real> *phi = NULL,
                            double coeff = 1.) {
  check(gev_projection_T0i(T0i->lat->ctx, pcls->p, T0i->f, phi ? phi->f : nullptr, coeff), T0i->lat->ctx,
        "projection_T0i_project");
}
template <typename part, typename part_info, typename part_dataType>
void projection_Tij_project(Particles<part, part_info, part_dataType> *pcls, Field<Real> *Tij, double a = 1.,
                            Field<Real> *phi = NULL, double coeff = 1.) {
  check(gev_projection_Tij(Tij->lat->ctx, pcls->p, Tij->f, a, phi ? phi->f : nullptr, coeff), Tij->lat->ctx,
        "projection_Tij_project");
}
#ifndef KTYPE_GRID
#define KTYPE_GRID 0
#define KTYPE_LINEAR 1
#endif
// extractCrossSpectrum (tools.hpp:53-212) on device spectra; the per-bin sums are exact
// integer sums on the GPU, the averages and scatters formed as the reference forms them
inline void extractCrossSpectrum(Field<Cplx> &fld1FT, Field<Cplx> &fld2FT, Real *kbin, Real *power, Real *kscatter,
                                 Real *pscatter, int *occupation, const int numbins, const bool deconvolve = true,
                                 const int ktype = KTYPE_LINEAR, const int comp1 = -1, const int comp2 = -1) {
  check(gev_cross_spectrum(fld1FT.lat->ctx, fld1FT.f, fld2FT.f, kbin, power, kscatter, pscatter, occupation, numbins,
                           deconvolve ? 1 : 0, ktype, fld1FT.sym ? 1 : 0, comp1, comp2),
        fld1FT.lat->ctx, "extractCrossSpectrum");
}
// extractPowerSpectrum (tools.hpp:237-240)
inline void extractPowerSpectrum(Field<Cplx> &fldFT, Real *kbin, Real *power, Real *kscatter, Real *pscatter,
                                 int *occupation, const int numbins, const bool deconvolve = true,
                                 const int ktype = KTYPE_LINEAR) {
  extractCrossSpectrum(fldFT, fldFT, kbin, power, kscatter, pscatter, occupation, numbins, deconvolve, ktype);
}

template <typename part, typename part_info, typename part_dataType>
void scalarProjectionCIC_project(Particles<part, part_info, part_dataType> *pcls, Field<Real> *rho) {
  check(gev_projection_mass(rho->lat->ctx, pcls->p, rho->f), rho->lat->ctx, "scalarProjectionCIC_project");
}

// hibernate (hibernation.hpp:513-611): one binary file at path in place of the
// reference's HDF5 set -- the particles, phi, chi, B / (a^2 N) and, when given,
// the spectrum BiFT, which makes a restart exact
template <typename part, typename part_info, typename part_dataType>
void hibernate(const std::string &path, Particles<part, part_info, part_dataType> *pcls_cdm, Field<Real> &phi,
               Field<Real> &chi, Field<Real> &Bi, const double a, const double tau, const double dtau, const int cycle,
               Field<Cplx> *BiFT = NULL) {
  check(gev_checkpoint_save(phi.lat->ctx, path.c_str(), pcls_cdm->p, phi.f, chi.f, Bi.f, BiFT ? BiFT->f : nullptr, a,
                            tau, dtau, cycle, nullptr),
        phi.lat->ctx, "hibernate");
}
// the restart branch of readIC (ic_read.hpp:58-716): particles, phi, chi, B * a^2 / N^2
// and BiFT (the stored spectrum, or the forward transform of B as readIC makes it);
// a, tau, dtau_old = the hibernated dtau, cycle = the hibernated cycle + 1
template <typename part, typename part_info, typename part_dataType>
void readIC_restart(const std::string &path, Particles<part, part_info, part_dataType> *pcls_cdm, Field<Real> *phi,
                    Field<Real> *chi, Field<Real> *Bi, Field<Cplx> *BiFT, double &a, double &tau, double &dtau_old,
                    int &cycle) {
  gev_checkpoint_info info;
  check(gev_checkpoint_load(phi->lat->ctx, path.c_str(), pcls_cdm->p, phi->f, chi->f, Bi ? Bi->f : nullptr,
                            BiFT ? BiFT->f : nullptr, 0, &info),
        phi->lat->ctx, "readIC");
  a = info.a;
  tau = info.tau;
  dtau_old = info.dtau;
  cycle = info.cycle + 1;
}

}  // namespace gevgpu

#endif
