/*
 * gev_ic.c -- initial conditions and power spectrum for the CPU restatement.
 * TEST INFRASTRUCTURE ONLY (the checker for the CUDA path).
 *
 * Initial conditions restate the mPk branch of generateIC_basic
 * (ic_basic.hpp:1626-2259) for CDM with baryons folded in, GR, no ncdm:
 *   1. a Gaussian displacement potential in k-space (generateDisplacementField,
 *      ic_basic.hpp:1089-1379) with the standard lattice-Laplacian kernel
 *      (generateCICKernel without a template, ic_basic.hpp:748-771) -- the modes
 *      come from a counter-based hash instead of the sitmo stream, and P(k) is
 *      evaluated from the BBKS formula instead of a cspline of an mPk file;
 *   2. particles on the sc1 template lattice tiled N/4 times
 *      (initializeParticlePositions, ic_basic.hpp:1400-1434), displaced by
 *      displace_pcls_ic_basic (ic_basic.hpp:60-91);
 *   3. phi from the CIC mass deposit and solveModifiedPoissonFT
 *      (ic_basic.hpp:2176-2195), velocities by initialize_q_ic_basic with the
 *      linear rescale (ic_basic.hpp:2199-2206), B and chi from the T0i / Tij
 *      deposits (ic_basic.hpp:2232-2252).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "gev_oracle.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

#define C_SPEED_OF_LIGHT 2997.92458 /* metadata.hpp:98, units of 100 km/s */

/* sc1_crystal.dat: the 64 template particles as lattice digits x + 4y + 16z of
 * offsets (0.125 + 0.25 * digit), in file order (decoded from the Gadget-2
 * template shipped with gevolution 1.2). */
static const int SC1_ORDER[64] = {0,  16, 20, 4,  5,  21, 17, 1,  32, 48, 52, 36, 37, 53, 49, 33,
                                  40, 56, 60, 44, 45, 61, 57, 41, 8,  24, 28, 12, 13, 29, 25, 9,
                                  10, 26, 30, 14, 15, 31, 27, 11, 42, 58, 62, 46, 47, 63, 59, 43,
                                  34, 50, 54, 38, 39, 55, 51, 35, 2,  18, 22, 6,  7,  23, 19, 3};

uint64_t gevo_hash64(uint64_t seed, uint64_t c) {
  uint64_t z = seed * 0x9E3779B97F4A7C15ull + c * 0xD1B54A32D192ED03ull + 0x632BE59BD9B4E019ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static double u01(uint64_t h) { return (double)((h >> 11) + 1) * (1.0 / 9007199254740992.0); }

/* BBKS transfer function (Bardeen, Bond, Kaiser & Szalay 1986, eq. G3), shape Gamma */
double gevo_bbks_T(double k, double Gamma) {
  const double q = k / Gamma;
  if (q < 1e-12) return 1.0;
  const double t = 1. + 3.89 * q + pow(16.1 * q, 2) + pow(5.46 * q, 3) + pow(6.71 * q, 4);
  return log(1. + 2.34 * q) / (2.34 * q) * pow(t, -0.25);
}

static double tophat(double x) {
  if (x < 1e-4) return 1. - x * x / 10.;
  return 3. * (sin(x) - x * cos(x)) / (x * x * x);
}

/* linear growth factor D(a) of a flat LCDM background (Heath 1977):
 * D ~ H(a) int_0^a da' / (a' H(a'))^3, Simpson in a */
static double growth(double a, double Om, double OL) {
  const int n = 4000;
  double s = 0.;
  for (int i = 0; i <= n; i++) {
    double x = a * (double)i / n;
    double f = 0.;
    if (x > 0.) {
      double E = sqrt(Om / (x * x * x) + OL);
      f = 1. / pow(x * E, 3);
    }
    s += f * ((i == 0 || i == n) ? 1. : (i % 2 ? 4. : 2.));
  }
  s *= a / n / 3.;
  return sqrt(Om / (a * a * a) + OL) * s;
}

double gevo_ic_pk_amplitude(const gevo_icparams *ic) {
  const double Om = ic->Omega_cdm + ic->Omega_b, OL = 1. - Om;
  const double Gamma = Om * ic->h;
  /* sigma_8^2 = 1/(2 pi^2) int k^3 P(k) W(8k)^2 dln k, Simpson in ln k */
  const int n = 20000;
  const double lk0 = log(1e-5), lk1 = log(1e3);
  double s = 0.;
  for (int i = 0; i <= n; i++) {
    double lk = lk0 + (lk1 - lk0) * i / n, k = exp(lk);
    double T = gevo_bbks_T(k, Gamma), W = tophat(8. * k);
    double f = k * k * k * pow(k, ic->n_s) * T * T * W * W;
    s += f * ((i == 0 || i == n) ? 1. : (i % 2 ? 4. : 2.));
  }
  s *= (lk1 - lk0) / n / 3. / (2. * M_PI * M_PI);
  const double A = ic->sigma8 * ic->sigma8 / s;
  const double a_in = 1. / (1. + ic->z_in);
  const double g = growth(a_in, Om, OL) / growth(1., Om, OL);
  return A * g * g;
}

double gevo_ic_pk(const gevo_icparams *ic, double k) {
  const double Om = ic->Omega_cdm + ic->Omega_b;
  const double T = gevo_bbks_T(k, Om * ic->h);
  return gevo_ic_pk_amplitude(ic) * pow(k, ic->n_s) * T * T;
}

static void cosmo_of(const gevo_icparams *ic, gevo_cosmo *c) {
  c->Omega_cdm = ic->Omega_cdm;
  c->Omega_b = ic->Omega_b;
  c->Omega_m = ic->Omega_cdm + ic->Omega_b;
  c->Omega_rad = 0.;
  c->Omega_Lambda = 1. - c->Omega_m - c->Omega_rad;
}

/* the displacement potential in k-space, generateDisplacementField
 * (ic_basic.hpp:1089-1379) with coeff = H_conf^2 and the standard kernel */
void gevo_ic_potential_k(int N, const gevo_icparams *ic, double *potd) {
  const int NH = N / 2 + 1;
  const int kmax = N / 2 - 1;
  const double L = ic->boxsize;
  gevo_cosmo cm;
  cosmo_of(ic, &cm);
  const double fourpiG = 1.5 * L * L / C_SPEED_OF_LIGHT / C_SPEED_OF_LIGHT;
  const double a = 1. / (1. + ic->z_in);
  const double H = gevo_hconf(a, fourpiG, &cm);
  const double coeff = H * H;
  const double amp = gevo_ic_pk_amplitude(ic);
  const double Gamma = cm.Omega_m * ic->h;
  double *gk2 = (double *)malloc(sizeof(double) * N), *ks = (double *)malloc(sizeof(double) * 2 * N);
  double *sinc = (double *)malloc(sizeof(double) * N);
  gevo_kspace_tables(N, gk2, ks);
  sinc[0] = 1.;
  for (int i = 1; i < N; i++) sinc[i] = sin(M_PI * (double)i / (double)N) * (double)N / (M_PI * (double)i);
  for (long kz = 0; kz < N; kz++)
    for (long ky = 0; ky < N; ky++)
      for (long kx = 0; kx < NH; kx++) {
        const size_t id = kx + NH * (ky + (size_t)N * kz);
        const long sy = ky <= N / 2 ? ky : N - ky, sz = kz <= N / 2 ? kz : N - kz;
        const double n2 = (double)(kx * kx + sy * sy + sz * sz);
        double re = 0., im = 0.;
        if (id != 0 && kx < kmax && sy < kmax && sz < kmax && !(ic->ksphere && n2 >= (double)kmax * kmax)) {
          const double k2 = n2 * 4. * M_PI * M_PI;
          const double kphys = sqrt(k2) / L; /* h/Mpc */
          const double T = gevo_bbks_T(kphys, Gamma);
          const double P = amp * pow(kphys, ic->n_s) * T * T;
          const double spl = sqrt(0.5 * P * L) / L / L; /* loadPowerSpectrum, ic_basic.hpp:436-437, 1681-1685 */
          const double s = sinc[kx] * sinc[sy] * sinc[sz];
          const double kern = gk2[kx] + gk2[ky] + gk2[kz];
          const double r1 = u01(gevo_hash64(ic->seed, 2 * (uint64_t)id));
          const double r2 = u01(gevo_hash64(ic->seed, 2 * (uint64_t)id + 1));
          const double m = (1. + 7.5 * coeff / k2) / kern * sqrt(-2. * log(r1)) * spl * s;
          re = cos(2. * M_PI * r2) * m;
          im = sin(2. * M_PI * r2) * m;
        }
        potd[2 * id] = re;
        potd[2 * id + 1] = im;
      }
  free(gk2);
  free(ks);
  free(sinc);
}

#define FLD(f, dx_, dy_, dz_) \
  (f)[(size_t)((c[0] + (dx_)) % N) + (size_t)N * ((size_t)((c[1] + (dy_)) % N) + (size_t)N * (size_t)((c[2] + (dz_)) % N))]

/* CIC-weighted forward-difference gradient / dx, ic_basic.hpp:71-86 and 137-152 */
static void cic_grad(int N, const double *f, const int *c, const double *r, double *g) {
  const double dx = 1.0 / (double)N;
  g[0] = (1. - r[1]) * (1. - r[2]) * (FLD(f, 1, 0, 0) - FLD(f, 0, 0, 0));
  g[1] = (1. - r[0]) * (1. - r[2]) * (FLD(f, 0, 1, 0) - FLD(f, 0, 0, 0));
  g[2] = (1. - r[0]) * (1. - r[1]) * (FLD(f, 0, 0, 1) - FLD(f, 0, 0, 0));
  g[0] += r[1] * (1. - r[2]) * (FLD(f, 1, 1, 0) - FLD(f, 0, 1, 0));
  g[1] += r[0] * (1. - r[2]) * (FLD(f, 1, 1, 0) - FLD(f, 1, 0, 0));
  g[2] += r[0] * (1. - r[1]) * (FLD(f, 1, 0, 1) - FLD(f, 1, 0, 0));
  g[0] += (1. - r[1]) * r[2] * (FLD(f, 1, 0, 1) - FLD(f, 0, 0, 1));
  g[1] += (1. - r[0]) * r[2] * (FLD(f, 0, 1, 1) - FLD(f, 0, 0, 1));
  g[2] += (1. - r[0]) * r[1] * (FLD(f, 0, 1, 1) - FLD(f, 0, 1, 0));
  g[0] += r[1] * r[2] * (FLD(f, 1, 1, 1) - FLD(f, 0, 1, 1));
  g[1] += r[0] * r[2] * (FLD(f, 1, 1, 1) - FLD(f, 1, 0, 1));
  g[2] += r[0] * r[1] * (FLD(f, 1, 1, 1) - FLD(f, 1, 1, 0));
  g[0] /= dx;
  g[1] /= dx;
  g[2] /= dx;
}
#undef FLD

static void cell_ref(int N, const gevo_part *p, int *c, double *r) {
  const double dx = 1.0 / (double)N;
  for (int i = 0; i < 3; i++) {
    c[i] = gevo_cell_of(N, p->pos[i]);
    r[i] = p->pos[i] / dx - (double)c[i];
  }
}

/* particleHorizon (background.hpp:200-212): tau = int 2 ds / (s Hconf(s^2)),
 * s = sqrt(a), from 1e-7 sqrt(a) to sqrt(a), divided by sqrt(4 pi G); Simpson */
static double particle_horizon(double a, double fourpiG, const gevo_cosmo *c) {
  const int n = 20000;
  const double s0 = sqrt(a) * 1.0e-7, s1 = sqrt(a);
  double s = 0.;
  for (int i = 0; i <= n; i++) {
    double x = s0 + (s1 - s0) * i / n;
    double f = 2. / (x * gevo_hconf(x * x, 1., c));
    s += f * ((i == 0 || i == n) ? 1. : (i % 2 ? 4. : 2.));
  }
  s *= (s1 - s0) / n / 3.;
  return s / sqrt(fourpiG);
}

int gevo_ic_generate(gevo_sim *s, const gevo_icparams *ic) {
  const int N = s->N;
  if (N % 4 != 0) return -1;
  const size_t V = (size_t)N * N * N;
  const size_t K = (size_t)N * N * (N / 2 + 1) * 2;
  const double dx = 1.0 / (double)N;
  const int numtile = N / 4;
  const double L = ic->boxsize;
  if (s->np != (long)V) return -2;

  cosmo_of(ic, &s->cosmo);
  const gevo_cosmo *cm = &s->cosmo;
  s->fourpiG = 1.5 * L * L / C_SPEED_OF_LIGHT / C_SPEED_OF_LIGHT; /* main.cpp:286 */
  const double fourpiG = s->fourpiG;
  const double a = 1. / (1. + ic->z_in);
  s->a = a;
  s->Cf = ic->Cf;
  s->steplimit = ic->steplimit;
  s->z_relax = ic->z_in;
  s->tau = particle_horizon(a, fourpiG, cm);
  s->dtau = gevo_next_dtau(s);
  s->dtau_old = 0.;
  s->cycle = 0;
  const double H = gevo_hconf(a, fourpiG, cm);

  /* displacement potential -> chi */
  gevo_ic_potential_k(N, ic, s->scalarFT);
  gevo_fft_c2r(N, s->scalarFT, s->chi);

  /* sc1 template particles, ic_basic.hpp:1400-1434 */
  s->mass = (cm->Omega_cdm + cm->Omega_b) / (double)(64L * numtile * numtile * numtile);
  long n = 0;
  for (long zt = 0; zt < numtile; zt++)
    for (long yt = 0; yt < numtile; yt++)
      for (long xt = 0; xt < numtile; xt++)
        for (long i = 0; i < 64; i++) {
          const int d = SC1_ORDER[i];
          const float off[3] = {0.125f + 0.25f * (float)(d & 3), 0.125f + 0.25f * (float)((d >> 2) & 3),
                                0.125f + 0.25f * (float)(d >> 4)};
          gevo_part *pt = s->p + n++;
          pt->pos[0] = ((double)xt + (double)off[0]) / (double)numtile;
          pt->pos[1] = ((double)yt + (double)off[1]) / (double)numtile;
          pt->pos[2] = ((double)zt + (double)off[2]) / (double)numtile;
          pt->vel[0] = pt->vel[1] = pt->vel[2] = 0.;
          pt->ID = i + 64L * (xt + (long)numtile * (yt + (long)numtile * zt));
        }
  gevo_sort(N, s->np, s->p, s->cell_start);

  /* displace_pcls_ic_basic with coeff 1 (ic_basic.hpp:1997) */
  for (long j = 0; j < s->np; j++) {
    int c[3];
    double r[3], g[3];
    cell_ref(N, s->p + j, c, r);
    cic_grad(N, s->chi, c, r, g);
    for (int i = 0; i < 3; i++) s->p[j].pos[i] += 1. * g[i];
  }
  for (long j = 0; j < s->np; j++)
    for (int i = 0; i < 3; i++) gevo_wrap(&s->p[j].pos[i]);
  gevo_sort(N, s->np, s->p, s->cell_start);

  /* phi (ic_basic.hpp:2176-2196) */
  memset(s->source, 0, V * sizeof(double));
  gevo_deposit_mass(N, s->np, s->p, s->cell_start, s->mass, s->source);
  gevo_fft_r2c(N, s->source, s->scalarFT);
  s->scalarFT[0] = 0.;
  s->scalarFT[1] = 0.;
  gevo_poisson(N, s->scalarFT, s->scalarFT, fourpiG / a, 3. * 1 * (H * H + fourpiG * cm->Omega_m / a));
  gevo_fft_c2r(N, s->scalarFT, s->phi);

  /* velocities: initialize_q_ic_basic with the linear rescale (ic_basic.hpp:2199-2206),
   * Omega_m(a), Omega_rad(a) from background.hpp:143-145 */
  const double Om_a = cm->Omega_m / ((cm->Omega_cdm + cm->Omega_b) + cm->Omega_Lambda * a * a * a + cm->Omega_rad / a);
  const double Or_a = (cm->Omega_rad + (cm->Omega_cdm + cm->Omega_b - cm->Omega_m) * a) /
                      ((cm->Omega_cdm + cm->Omega_b) * a + cm->Omega_Lambda * a * a * a * a + cm->Omega_rad);
  const double rescale = a / H / (1.5 * Om_a + 2. * Or_a);
  double vmax = 0.;
  for (long j = 0; j < s->np; j++) {
    int c[3];
    double r[3], g[3], v2 = 0.;
    cell_ref(N, s->p + j, c, r);
    cic_grad(N, s->phi, c, r, g);
    for (int i = 0; i < 3; i++) {
      s->p[j].vel[i] = -g[i] * rescale;
      v2 += s->p[j].vel[i] * s->p[j].vel[i];
    }
    if (v2 > vmax) vmax = v2;
  }
  double maxvel = sqrt(vmax) / a;

  /* B (ic_basic.hpp:2232-2240) */
  memset(s->Bi, 0, 3 * V * sizeof(double));
  gevo_deposit_T0i(N, s->np, s->p, s->cell_start, s->mass, s->phi, 1., s->Bi);
  for (int c = 0; c < 3; c++) gevo_fft_r2c(N, s->Bi + c * V, s->BiFT + c * K);
  gevo_project_vector(N, s->BiFT, s->BiFT, fourpiG / (double)N / (double)N, 0.);
  for (int c = 0; c < 3; c++) gevo_fft_c2r(N, s->BiFT + c * K, s->Bi + c * V);

  /* chi (ic_basic.hpp:2242-2252) */
  memset(s->Sij, 0, 6 * V * sizeof(double));
  gevo_deposit_Tij(N, s->np, s->p, s->cell_start, s->mass, a, s->phi, 1., s->Sij);
  gevo_prepare_source_tensor(N, s->phi, s->Sij, s->Sij, 2. * fourpiG / a / (double)N / (double)N);
  for (int c = 0; c < 6; c++) gevo_fft_r2c(N, s->Sij + c * V, s->SijFT + c * K);
  gevo_project_scalar(N, s->SijFT, s->scalarFT, 0);
  gevo_fft_c2r(N, s->scalarFT, s->chi);

  /* main.cpp:324-330 */
  maxvel /= sqrt(maxvel * maxvel + 1.0);
  s->maxvel = maxvel;
  (void)dx;
  return 0;
}

/* extractCrossSpectrum of a field with itself (tools.hpp:53-212), linear k,
 * single rank.  symmetric != 0 treats the 6 components as a symmetric tensor. */
void gevo_power_spectrum(int N, const double *FTd, int ncomp, int symmetric, int numbins, int deconvolve,
                         double *kbin, double *power, double *kscatter, double *pscatter, int *occupation) {
  const int NH = N / 2 + 1;
  if (N < 2) return;
  const size_t NK = (size_t)N * N * NH;
  double *typek2 = (double *)malloc(sizeof(double) * N), *sinc = (double *)malloc(sizeof(double) * N);
  int i;
  for (i = 0; i <= N / 2; i++) {
    typek2[i] = 2. * M_PI * (double)i;
    typek2[i] *= typek2[i];
  }
  for (; i < N; i++) {
    typek2[i] = 2. * M_PI * (double)(N - i);
    typek2[i] *= typek2[i];
  }
  sinc[0] = 1.;
  for (i = 1; i <= N / 2; i++)
    sinc[i] = deconvolve ? sin(M_PI * (float)i / (float)N) * (float)N / (M_PI * (float)i) : 1.;
  for (; i < N; i++) sinc[i] = sinc[N - i];
  const double k2max = 3. * typek2[N / 2];
  for (i = 0; i < numbins; i++) {
    kbin[i] = power[i] = kscatter[i] = pscatter[i] = 0.;
    occupation[i] = 0;
  }
  for (long kz = 0; kz < N; kz++)
    for (long ky = 0; ky < N; ky++)
      for (long kx = 0; kx < NH; kx++) {
        int weight;
        if (kx == 0 && ky == 0 && kz == 0) continue;
        else if (kx == 0) weight = 1;
        else if (kx == N / 2 && N % 2 == 0) weight = 1;
        else weight = 2;
        const size_t id = kx + NH * (ky + (size_t)N * kz);
        const double k2 = typek2[kx] + typek2[ky] + typek2[kz];
        double s = sinc[kx] * sinc[ky] * sinc[kz];
        s *= s;
        double p = 0.;
        if (symmetric) {
          for (int c = 1; c <= 4; c += (c == 2 ? 2 : 1)) /* 01, 02, 12 */
            p += FTd[2 * (c * NK + id)] * FTd[2 * (c * NK + id)] + FTd[2 * (c * NK + id) + 1] * FTd[2 * (c * NK + id) + 1];
          p *= 2.;
          const int dg[3] = {0, 3, 5};
          for (int c = 0; c < 3; c++)
            p += FTd[2 * (dg[c] * NK + id)] * FTd[2 * (dg[c] * NK + id)] +
                 FTd[2 * (dg[c] * NK + id) + 1] * FTd[2 * (dg[c] * NK + id) + 1];
        } else {
          for (int c = 0; c < ncomp; c++)
            p += FTd[2 * (c * NK + id)] * FTd[2 * (c * NK + id)] + FTd[2 * (c * NK + id) + 1] * FTd[2 * (c * NK + id) + 1];
        }
        int b = (int)floor((double)((double)numbins * sqrt(k2 / k2max)));
        if (b < numbins) {
          kbin[b] += weight * sqrt(k2);
          kscatter[b] += weight * k2;
          power[b] += weight * p * k2 * sqrt(k2) / s;
          pscatter[b] += weight * p * p * k2 * k2 * k2 / s / s;
          occupation[b] += weight;
        }
      }
  for (i = 0; i < numbins; i++) {
    if (occupation[i] > 0) {
      kscatter[i] = sqrt(kscatter[i] * occupation[i] - kbin[i] * kbin[i]) / occupation[i];
      if (!isfinite(kscatter[i])) kscatter[i] = 0.;
      kbin[i] = kbin[i] / occupation[i];
      power[i] /= occupation[i];
      pscatter[i] = sqrt(pscatter[i] / occupation[i] - power[i] * power[i]);
      if (!isfinite(pscatter[i])) pscatter[i] = 0.;
    }
  }
  free(typek2);
  free(sinc);
}
