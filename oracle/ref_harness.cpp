// ref_harness.cpp -- compiles gevolution 1.2's own gevolution.hpp and
// background.hpp (unmodified, from the reference source tree) against the
// single-rank LATfield2 shim, and exposes each hot-path function over the flat
// arrays of gev_oracle.h.  Built by `make ref` into oracle/_ref/ only where the
// reference sources exist.  TEST INFRASTRUCTURE ONLY: it checks the CPU
// restatement and produces the golden vectors under tests/golden/.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <set>
#include <vector>

#include "LATfield2.hpp"
using namespace LATfield2;
#include "metadata.hpp"
#include "background.hpp"
#include "gevolution.hpp"

namespace {

typedef Particles<part_simple, part_simple_info, part_simple_dataType> Pcls;

struct Grid {
  Lattice lat, latFT;
  int N;
  explicit Grid(int n) : N(n) {
    int box[3] = {n, n, n};
    lat.initialize(3, box, 1);
    latFT.initializeRealFFT(lat, 0);
  }
};

void load_real(Field<Real> &f, const double *src, int N) {
  Site x(f.lattice());
  const size_t V = (size_t)N * N * N;
  for (int c = 0; c < f.components(); c++)
    for (x.first(); x.test(); x.next())
      f(x, c) = src[c * V + x.coord(0) + (size_t)N * (x.coord(1) + (size_t)N * x.coord(2))];
  f.updateHalo();
}
void store_real(Field<Real> &f, double *dst, int N) {
  Site x(f.lattice());
  const size_t V = (size_t)N * N * N;
  for (int c = 0; c < f.components(); c++)
    for (x.first(); x.test(); x.next())
      dst[c * V + x.coord(0) + (size_t)N * (x.coord(1) + (size_t)N * x.coord(2))] = f(x, c);
}
void load_cplx(Field<Cplx> &f, const double *src) { memcpy(f.data_.data(), src, sizeof(Cplx) * f.data_.size()); }
void store_cplx(Field<Cplx> &f, double *dst) { memcpy(dst, f.data_.data(), sizeof(Cplx) * f.data_.size()); }

void load_pcls(Pcls &p, Grid &g, const gevo_part *src, long np, double mass) {
  part_simple_info info;
  memset(&info, 0, sizeof(info));
  info.mass = mass;
  part_simple_dataType dt;
  Real box[3] = {1., 1., 1.};
  p.initialize(info, dt, &g.lat, box);
  for (long i = 0; i < np; i++) {
    part_simple q;
    for (int l = 0; l < 3; l++) {
      q.pos[l] = src[i].pos[l];
      q.vel[l] = src[i].vel[l];
    }
    q.ID = (long)src[i].ID;
    p.addParticle_global(q);
  }
}
long store_pcls(Pcls &p, gevo_part *dst) {
  long n = 0;
  for (size_t c = 0; c < p.field_.cells_.size(); c++)
    for (std::list<part_simple>::iterator it = p.field_.cells_[c].parts.begin(); it != p.field_.cells_[c].parts.end(); ++it) {
      for (int l = 0; l < 3; l++) {
        dst[n].pos[l] = it->pos[l];
        dst[n].vel[l] = it->vel[l];
      }
      dst[n].ID = it->ID;
      n++;
    }
  return n;
}

cosmology make_cosmo(const gevo_cosmo *c) {
  cosmology cm;
  memset(&cm, 0, sizeof(cm));
  cm.Omega_cdm = c->Omega_cdm;
  cm.Omega_b = c->Omega_b;
  cm.Omega_m = c->Omega_m;
  cm.Omega_Lambda = c->Omega_Lambda;
  cm.Omega_rad = c->Omega_rad;
  cm.Omega_fld = 0.;
  cm.w0_fld = -1.;
  cm.wa_fld = 0.;
  cm.num_ncdm = 0;
  return cm;
}

}  // namespace

extern "C" {

void gevref_prepare_source_tensor(int N, const double *phi, const double *T, double *S, double coeff) {
  Grid g(N);
  Field<Real> fphi, fT;
  fphi.initialize(g.lat, 1);
  fT.initialize(g.lat, 3, 3, symmetric);
  load_real(fphi, phi, N);
  load_real(fT, T, N);
  prepareFTsource<Real>(fphi, fT, fT, coeff);
  store_real(fT, S, N);
}

void gevref_prepare_source_scalar(int N, const double *phi, const double *chi, const double *source, double bg,
                                  double *result, double coeff, double coeff2, double coeff3) {
  Grid g(N);
  Field<Real> fphi, fchi, fs;
  fphi.initialize(g.lat, 1);
  fchi.initialize(g.lat, 1);
  fs.initialize(g.lat, 1);
  load_real(fphi, phi, N);
  load_real(fchi, chi, N);
  load_real(fs, source, N);
  prepareFTsource<Real>(fphi, fchi, fs, bg, fs, coeff, coeff2, coeff3);
  store_real(fs, result, N);
}

void gevref_poisson(int N, const double *src, double *pot, double coeff, double modif) {
  Grid g(N);
  Field<Cplx> f;
  f.initialize(g.latFT, 1);
  load_cplx(f, src);
  solveModifiedPoissonFT(f, f, coeff, modif);
  store_cplx(f, pot);
}

void gevref_project_scalar(int N, const double *S, double *chi, int add) {
  Grid g(N);
  Field<Cplx> fS, fc;
  fS.initialize(g.latFT, 3, 3, symmetric);
  fc.initialize(g.latFT, 1);
  load_cplx(fS, S);
  load_cplx(fc, chi);
  projectFTscalar(fS, fc, add);
  store_cplx(fc, chi);
}

void gevref_evolve_vector(int N, const double *S, double *B, double a2dtau) {
  Grid g(N);
  Field<Cplx> fS, fB;
  fS.initialize(g.latFT, 3, 3, symmetric);
  fB.initialize(g.latFT, 3);
  load_cplx(fS, S);
  load_cplx(fB, B);
  evolveFTvector(fS, fB, a2dtau);
  store_cplx(fB, B);
}

void gevref_project_vector(int N, const double *S, double *B, double coeff, double modif) {
  Grid g(N);
  Field<Cplx> fB;
  fB.initialize(g.latFT, 3);
  load_cplx(fB, S);
  projectFTvector(fB, fB, coeff, modif);
  store_cplx(fB, B);
}

void gevref_project_tensor(int N, const double *S, double *h) {
  Grid g(N);
  Field<Cplx> fS, fh;
  fS.initialize(g.latFT, 3, 3, symmetric);
  fh.initialize(g.latFT, 3, 3, symmetric);
  load_cplx(fS, S);
  projectFTtensor(fS, fh);
  store_cplx(fh, h);
}

/* which: 0 = T00, 1 = T0i, 2 = Tij; accumulates into out (interior values kept,
 * halo cleared), then the *_comm fold */
void gevref_deposit(int which, int N, long np, const gevo_part *p, double mass, double a, const double *phi,
                    double coeff, double *out) {
  Grid g(N);
  Pcls pc;
  load_pcls(pc, g, p, np, mass);
  Field<Real> fphi, fo;
  fphi.initialize(g.lat, 1);
  if (phi) load_real(fphi, phi, N);
  if (which == 0) fo.initialize(g.lat, 1);
  if (which == 1) fo.initialize(g.lat, 3);
  if (which == 2) fo.initialize(g.lat, 3, 3, symmetric);
  {
    Site x(fo.lattice());
    const size_t V = (size_t)N * N * N;
    for (int c = 0; c < fo.components(); c++)
      for (x.first(); x.test(); x.next())
        fo(x, c) = out[c * V + x.coord(0) + (size_t)N * (x.coord(1) + (size_t)N * x.coord(2))];
  }
  Field<Real> *pphi = phi ? &fphi : NULL;
  if (which == 0) { projection_T00_project(&pc, &fo, a, pphi, coeff); projection_T00_comm(&fo); }
  if (which == 1) { projection_T0i_project(&pc, &fo, pphi, coeff); projection_T0i_comm(&fo); }
  if (which == 2) { projection_Tij_project(&pc, &fo, a, pphi, coeff); projection_Tij_comm(&fo); }
  store_real(fo, out, N);
}

/* kind 0 = update_q (GR), 1 = update_q_Newton; returns the updateVel value */
double gevref_kick(int N, long np, gevo_part *p, int kind, double dtau, const double *phi, const double *chi,
                   const double *Bi, int nfield, double a, double a2N) {
  Grid g(N);
  Pcls pc;
  load_pcls(pc, g, p, np, 1.);
  Field<Real> fphi, fchi, fB;
  fphi.initialize(g.lat, 1);
  fchi.initialize(g.lat, 1);
  fB.initialize(g.lat, 3);
  if (phi) load_real(fphi, phi, N);
  if (chi) load_real(fchi, chi, N);
  if (Bi) load_real(fB, Bi, N);
  Field<Real> *fields[3] = {&fphi, &fchi, &fB};
  double params[2] = {a, a2N};
  double r = pc.updateVel(kind == 0 ? update_q : update_q_Newton, dtau, fields, nfield, params);
  store_pcls(pc, p);
  return r;
}

/* kind 0 = update_pos (GR), 1 = update_pos_Newton; relinks */
void gevref_drift(int N, long np, gevo_part *p, int kind, double dtau, const double *phi, const double *chi,
                  const double *Bi, int nfield, double a, double a2N) {
  Grid g(N);
  Pcls pc;
  load_pcls(pc, g, p, np, 1.);
  Field<Real> fphi, fchi, fB;
  fphi.initialize(g.lat, 1);
  fchi.initialize(g.lat, 1);
  fB.initialize(g.lat, 3);
  if (phi) load_real(fphi, phi, N);
  if (chi) load_real(fchi, chi, N);
  if (Bi) load_real(fB, Bi, N);
  Field<Real> *fields[3] = {&fphi, &fchi, &fB};
  double params[2] = {a, a2N};
  if (kind == 0)
    pc.moveParticles(update_pos, dtau, fields, nfield, params);
  else
    pc.moveParticles(update_pos_Newton, dtau, NULL, 0, params);
  store_pcls(pc, p);
}

double gevref_hconf(double a, double fourpiG, const gevo_cosmo *c) { return Hconf(a, fourpiG, make_cosmo(c)); }

double gevref_rk4bg(double a, double fourpiG, const gevo_cosmo *c, double dtau) {
  rungekutta4bg(a, fourpiG, make_cosmo(c), dtau);
  return a;
}

/* one cycle of main.cpp:372-879 (GR, CDM only, no outputs) over the state in s,
 * calling the reference's own functions */
int gevref_sim_step(gevo_sim *s) {
  const int N = s->N;
  Grid g(N);
  const double dx = 1.0 / (double)N;
  cosmology cosmo = make_cosmo(&s->cosmo);
  const double fourpiG = s->fourpiG;
  double a = s->a;
  Pcls pcls_cdm;
  load_pcls(pcls_cdm, g, s->p, s->np, s->mass);
  Field<Real> phi, source, chi, Sij, Bi;
  Field<Cplx> scalarFT, SijFT, BiFT;
  source.initialize(g.lat, 1);
  phi.initialize(g.lat, 1);
  chi.initialize(g.lat, 1);
  scalarFT.initialize(g.latFT, 1);
  PlanFFT<Cplx> plan_source(&source, &scalarFT);
  PlanFFT<Cplx> plan_phi(&phi, &scalarFT);
  PlanFFT<Cplx> plan_chi(&chi, &scalarFT);
  Sij.initialize(g.lat, 3, 3, symmetric);
  SijFT.initialize(g.latFT, 3, 3, symmetric);
  PlanFFT<Cplx> plan_Sij(&Sij, &SijFT);
  Bi.initialize(g.lat, 3);
  BiFT.initialize(g.latFT, 3);
  PlanFFT<Cplx> plan_Bi(&Bi, &BiFT);
  load_real(phi, s->phi, N);
  load_real(chi, s->chi, N);
  load_real(Bi, s->Bi, N);
  load_cplx(scalarFT, s->scalarFT);
  load_cplx(BiFT, s->BiFT);
  Field<Real> *update_cdm_fields[3] = {&phi, &chi, &Bi};
  double f_params[5];
  const long numpts3d = (long)N * N * N;

  projection_init(&source);
  projection_T00_project(&pcls_cdm, &source, a, &phi);
  projection_T00_comm(&source);
  if (s->vector_elliptic) {
    projection_init(&Bi);
    projection_T0i_project(&pcls_cdm, &Bi, &phi);
    projection_T0i_comm(&Bi);
  }
  projection_init(&Sij);
  projection_Tij_project(&pcls_cdm, &Sij, a, &phi);
  projection_Tij_comm(&Sij);

  double T00hom = 0.;
  Site x(g.lat);
  for (x.first(); x.test(); x.next()) T00hom += source(x);
  T00hom /= (double)numpts3d;
  s->T00hom = T00hom;

  if (s->dtau_old > 0.) {
    prepareFTsource<Real>(phi, chi, source, cosmo.Omega_cdm + cosmo.Omega_b + bg_ncdm(a, cosmo), source,
                          3. * Hconf(a, fourpiG, cosmo) * dx * dx / s->dtau_old, fourpiG * dx * dx / a,
                          3. * Hconf(a, fourpiG, cosmo) * Hconf(a, fourpiG, cosmo) * dx * dx);
    plan_source.execute(FFT_FORWARD);
    solveModifiedPoissonFT(scalarFT, scalarFT, 1. / (dx * dx), 3. * Hconf(a, fourpiG, cosmo) / s->dtau_old);
    plan_phi.execute(FFT_BACKWARD);
  }
  phi.updateHalo();
  s->phik0 = scalarFT.data_[0].real();

  prepareFTsource<Real>(phi, Sij, Sij, 2. * fourpiG * dx * dx / a);
  plan_Sij.execute(FFT_FORWARD);
  projectFTscalar(SijFT, scalarFT);
  plan_chi.execute(FFT_BACKWARD);
  chi.updateHalo();
  if (s->vector_elliptic) {
    plan_Bi.execute(FFT_FORWARD);
    projectFTvector(BiFT, BiFT, fourpiG * dx * dx);
  } else
    evolveFTvector(SijFT, BiFT, a * a * s->dtau_old);
  plan_Bi.execute(FFT_BACKWARD);
  Bi.updateHalo();

  const double dtau = s->dtau, dtau_old = s->dtau_old;
  f_params[0] = a;
  f_params[1] = a * a * N;
  double maxvel = pcls_cdm.updateVel(update_q, (dtau + dtau_old) / 2., update_cdm_fields,
                                     (1. / a < s->z_relax + 1. ? 3 : 2), f_params);
  rungekutta4bg(a, fourpiG, cosmo, 0.5 * dtau);
  f_params[0] = a;
  f_params[1] = a * a * N;
  pcls_cdm.moveParticles(update_pos, dtau, update_cdm_fields, (1. / a < s->z_relax + 1. ? 3 : 0), f_params);
  rungekutta4bg(a, fourpiG, cosmo, 0.5 * dtau);
  maxvel /= sqrt(maxvel * maxvel + 1.0);

  s->maxvel = maxvel;
  s->a = a;
  s->tau += dtau;
  s->dtau_old = dtau;
  if (s->Cf * dx < s->steplimit / Hconf(a, fourpiG, cosmo))
    s->dtau = s->Cf * dx;
  else
    s->dtau = s->steplimit / Hconf(a, fourpiG, cosmo);
  s->cycle++;

  store_pcls(pcls_cdm, s->p);
  gevo_sort(N, s->np, s->p, s->cell_start);
  store_real(phi, s->phi, N);
  store_real(chi, s->chi, N);
  store_real(source, s->source, N);
  store_real(Sij, s->Sij, N);
  store_real(Bi, s->Bi, N);
  store_cplx(scalarFT, s->scalarFT);
  store_cplx(SijFT, s->SijFT);
  store_cplx(BiFT, s->BiFT);
  return 0;
}

}  // extern "C"
