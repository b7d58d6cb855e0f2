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

/* the tabulated spectrum the mPk branch reads (ic_basic.hpp:343-471, 1679-1700):
 * the BBKS P(k) [(Mpc/h)^3] at z_in on NPK log-spaced k [h/Mpc] covering every
 * mode of the grid, as spline knots x = k L and values sqrt(P L / 2) / L^2 */
#define GEVO_NPK 512
void gevo_ic_spline_knots(int N, const gevo_icparams *ic, double *x, double *y) {
  const double L = ic->boxsize;
  const double lk0 = log(M_PI / L), lk1 = log(4. * M_PI * (double)N / L);
  for (int i = 0; i < GEVO_NPK; i++) {
    const double k = exp(lk0 + (lk1 - lk0) * (double)i / (double)(GEVO_NPK - 1));
    const double P = gevo_ic_pk(ic, k);
    x[i] = k * L;
    y[i] = sqrt(0.5 * P * L);
    y[i] = y[i] / L / L;
  }
}

/* the sc1 template as loadHomogeneousTemplate leaves it: positions / BoxSize */
static void sc1_pcldata(float *d) {
  for (int i = 0; i < 64; i++) {
    const int g = SC1_ORDER[i];
    d[3 * i] = 0.125f + 0.25f * (float)(g & 3);
    d[3 * i + 1] = 0.125f + 0.25f * (float)((g >> 2) & 3);
    d[3 * i + 2] = 0.125f + 0.25f * (float)(g >> 4);
  }
}

/* the displacement potential in k-space (generateIC_basic, ic_basic.hpp:1670-1700):
 * the CIC kernel (of the sc1 template with `correct displacement`, else the
 * lattice Laplacian) transformed forward, then generateDisplacementField with
 * coeff = H_conf^2 (GR), the sitmo stream of seed and the spline of the BBKS table */
void gevo_ic_potential_k(int N, const gevo_icparams *ic, double *potd) {
  const double L = ic->boxsize;
  gevo_cosmo cm;
  cosmo_of(ic, &cm);
  const double fourpiG = 1.5 * L * L / C_SPEED_OF_LIGHT / C_SPEED_OF_LIGHT;
  const double a = 1. / (1. + ic->z_in);
  const double H = gevo_hconf(a, fourpiG, &cm);
  double K[27];
  float pcl[192];
  sc1_pcldata(pcl);
  if (ic->correct_displacement)
    gevo_cic_kernel(N, 64, pcl, N / 4, K);
  else
    gevo_cic_kernel(N, 0, NULL, 1, K);
  double *ker = (double *)calloc((size_t)N * N * N, sizeof(double));
  for (int dz = -1; dz <= 1; dz++)
    for (int dy = -1; dy <= 1; dy++)
      for (int dx = -1; dx <= 1; dx++)
        ker[(size_t)((dx + N) % N) + (size_t)N * ((size_t)((dy + N) % N) + (size_t)N * (size_t)((dz + N) % N))] +=
            K[(dx + 1) + 3 * (dy + 1) + 9 * (dz + 1)];
  gevo_fft_r2c(N, ker, potd);
  free(ker);
  double x[GEVO_NPK], y[GEVO_NPK];
  gevo_ic_spline_knots(N, ic, x, y);
  gevo_displacement_field(N, potd, H * H, GEVO_NPK, x, y, (uint32_t)ic->seed, ic->ksphere);
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

/* ===================================================================== */
/* the sitmo stream and generateDisplacementField's layout               */
/* ===================================================================== */

/* sitmo::prng_engine (prng_engine.hpp:88-230), restated: draw d of the engine
 * seeded with s is 32-bit half (d & 1: high) of word (d & 7) / 2 of block d / 8,
 * a block being the Threefish-256 encryption (20 rounds, 5 key injections; Skein
 * 1.3 rotation constants) of the counter (d / 8, 0, 0, 0) under the key
 * (s, 0, 0, 0), plus the final key injection. */
static uint64_t rotl64(uint64_t x, int r) { return (x << r) | (x >> (64 - r)); }
void gevo_sitmo_block(uint32_t seed, uint64_t block, uint64_t out[4]) {
  static const int R[8][2] = {{14, 16}, {52, 57}, {23, 40}, {5, 37}, {25, 33}, {46, 12}, {58, 22}, {32, 32}};
  uint64_t k[5] = {seed, 0, 0, 0, 0};
  k[4] = 0x1BD11BDAA9FC1A22ull ^ k[0] ^ k[1] ^ k[2] ^ k[3];
  uint64_t b[4] = {block, 0, 0, 0};
  for (int r = 0; r < 20; r++) {
    if (r % 4 == 0) { /* key injection s = r / 4 */
      const int s = r / 4;
      b[0] += k[s % 5];
      b[1] += k[(s + 1) % 5];
      b[2] += k[(s + 2) % 5];
      b[3] += k[(s + 3) % 5] + (uint64_t)s;
    }
    const int *rr = R[r % 8];
    if (r % 2 == 0) { /* pairs (0,1) and (2,3) */
      b[0] += b[1];
      b[1] = rotl64(b[1], rr[0]) ^ b[0];
      b[2] += b[3];
      b[3] = rotl64(b[3], rr[1]) ^ b[2];
    } else { /* pairs (0,3) and (2,1) */
      b[0] += b[3];
      b[3] = rotl64(b[3], rr[0]) ^ b[0];
      b[2] += b[1];
      b[1] = rotl64(b[1], rr[1]) ^ b[2];
    }
  }
  for (int i = 0; i < 4; i++) out[i] = b[i] + k[(5 + i) % 5];
  out[3] += 5;
}
uint32_t gevo_sitmo_draw(uint32_t seed, uint64_t d) {
  uint64_t o[4];
  gevo_sitmo_block(seed, d >> 3, o);
  const uint64_t w = o[(d & 7) >> 1];
  return (d & 1) ? (uint32_t)(w >> 32) : (uint32_t)(w & 0xFFFFFFFFull);
}

/* gsl_interp_cspline restated (natural cubic spline; see oracle/ref_shim/gsl/gsl_spline.h) */
void gevo_spline_init(int n, const double *x, const double *y, double *c) {
  for (int i = 0; i < n; i++) c[i] = 0.;
  if (n < 3) return;
  const int m = n - 2;
  double *dg = (double *)malloc(sizeof(double) * m), *of = (double *)malloc(sizeof(double) * m);
  double *rh = (double *)malloc(sizeof(double) * m);
  for (int i = 0; i < m; i++) {
    const double h0 = x[i + 1] - x[i], h1 = x[i + 2] - x[i + 1];
    dg[i] = 2.0 * (h0 + h1);
    of[i] = h1;
    rh[i] = 3.0 * ((y[i + 2] - y[i + 1]) / h1 - (y[i + 1] - y[i]) / h0);
  }
  for (int i = 1; i < m; i++) {
    const double w = of[i - 1] / dg[i - 1];
    dg[i] = dg[i] - w * of[i - 1];
    rh[i] = rh[i] - w * rh[i - 1];
  }
  c[m] = rh[m - 1] / dg[m - 1];
  for (int i = m - 1; i > 0; i--) c[i] = (rh[i - 1] - of[i - 1] * c[i + 1]) / dg[i - 1];
  free(dg);
  free(of);
  free(rh);
}
double gevo_spline_eval(int n, const double *x, const double *y, const double *c, double v) {
  int lo = 0, hi = n - 1;
  while (hi > lo + 1) {
    const int mid = (lo + hi) / 2;
    if (x[mid] > v)
      hi = mid;
    else
      lo = mid;
  }
  const double h = x[lo + 1] - x[lo], t = v - x[lo];
  const double ci = c[lo], cn = c[lo + 1];
  const double b = (y[lo + 1] - y[lo]) / h - h * (cn + 2.0 * ci) / 3.0;
  const double d = (cn - ci) / (3.0 * h);
  return y[lo] + t * (b + t * (ci + t * d));
}

/* one mode of generateDisplacementField: the kernel value K in, the mode out
 * (ic_basic.hpp:1147-1167, LATfield2 Imag arithmetic as the shim defines it) */
static void gdf_mode(double *f, float k2, float s, uint32_t u1, uint32_t u2, double coeff, int conj, int n,
                     const double *x, const double *y, const double *c) {
  const float r1 = (float)u1 / (float)4294967295u, r2 = (float)u2 / (float)4294967295u;
  const double d1 = 1. + 7.5 * coeff / k2;
  const double tr = cos(2. * M_PI * r2) * d1, ti = (conj ? -sin(2. * M_PI * r2) : sin(2. * M_PI * r2)) * d1;
  const double Kr = f[0], Ki = f[1], nn = Kr * Kr + Ki * Ki;
  double qr = (tr * Kr + ti * Ki) / nn, qi = (ti * Kr - tr * Ki) / nn;
  /* log(r1) and sqrt(k2) of float arguments are the float overloads of <cmath> in
   * the reference (C++, using namespace std): logf and sqrtf */
  const double g = sqrt(-2. * logf(r1)), sp = gevo_spline_eval(n, x, y, c, sqrtf(k2));
  qr = qr * g;
  qi = qi * g;
  qr = qr * sp;
  qi = qi * sp;
  f[0] = qr * s;
  f[1] = qi * s;
}

/* generateDisplacementField<0> (ic_basic.hpp:1089-1379) on one rank: F holds the
 * kernel spectrum on entry and the modes on return (N^2 (N/2+1) complex, kx
 * fastest); the stream of each (ky, kz) line of each quadrant starts at its own
 * multiple of 65536^2 and 65536 draws, as the reference's discards place it */
void gevo_displacement_field(int N, double *F, double coeff, int n, const double *x, const double *y, uint32_t seed,
                             int ksphere) {
  const int NH = N / 2 + 1, kmax = N / 2 - 1;
  const uint64_t H = 65536;
  double *c = (double *)malloc(sizeof(double) * n);
  gevo_spline_init(n, x, y, c);
  float *sinc = (float *)malloc(sizeof(float) * N);
  sinc[0] = 1.;
  for (int i = 1; i < N; i++) sinc[i] = sin(M_PI * (float)i / (float)N) * (float)N / (M_PI * (float)i);
  /* pass 0: A (ky, kz <= N/2), 1: B (ky > N/2), 2: C (kz > N/2, kx >= 1), 3: D (both, kx >= 1),
   * 4: kx = 0 of C from A's lines, conjugated, 5: kx = 0 of D from C's lines, conjugated */
  for (int pass = 0; pass < 6; pass++)
    for (int kz = 0; kz < N; kz++)
      for (int ky = 0; ky < N; ky++) {
        const int ylo = ky <= N / 2, zlo = kz <= N / 2;
        const int sy = ylo ? ky : N - ky, sz = zlo ? kz : N - kz;
        uint64_t line;
        int kx0, kx1 = N / 2, conj = 0;
        if (pass == 0 && ylo && zlo) {
          line = (uint64_t)kz * H + (uint64_t)ky;
          kx0 = (ky == 0 && kz == 0) ? 1 : 0;
        } else if (pass == 1 && !ylo && zlo) {
          line = (H + (uint64_t)kz) * H + (uint64_t)(N - ky);
          kx0 = 0;
        } else if (pass == 2 && ylo && !zlo) {
          line = (2 * H + (uint64_t)(N - kz)) * H + (uint64_t)ky;
          kx0 = 1;
        } else if (pass == 3 && !ylo && !zlo) {
          line = (3 * H + (uint64_t)(N - kz)) * H + (uint64_t)(N - ky);
          kx0 = 1;
        } else if (pass == 4 && ylo && !zlo) {
          line = (uint64_t)(N - kz) * H + (uint64_t)ky;
          kx0 = 0;
          kx1 = 0;
          conj = 1;
        } else if (pass == 5 && !ylo && !zlo) {
          line = (2 * H + (uint64_t)(N - kz)) * H + (uint64_t)(N - ky);
          kx0 = 0;
          kx1 = 0;
          conj = 1;
        } else {
          continue;
        }
        uint64_t d = line * H;
        for (int kx = kx0; kx <= kx1; kx++) {
          double *f = F + 2 * ((size_t)kx + (size_t)NH * ((size_t)ky + (size_t)N * kz));
          const float k2 = (float)(kx * kx) + (float)(sy * sy) + (float)(sz * sz);
          if (kx >= kmax || sy >= kmax || sz >= kmax || (k2 >= kmax * kmax && ksphere > 0)) {
            f[0] = f[1] = 0.;
            continue;
          }
          const float s = sinc[kx] * sinc[sy] * sinc[sz];
          float k2s = k2;
          k2s *= 4. * M_PI * M_PI;
          uint32_t u1;
          do u1 = gevo_sitmo_draw(seed, d++);
          while ((float)u1 / (float)4294967295u == 0.);
          const uint32_t u2 = gevo_sitmo_draw(seed, d++);
          gdf_mode(f, k2s, s, u1, u2, coeff, conj, n, x, y, c);
        }
      }
  F[0] = F[1] = 0.; /* the origin */
  free(c);
  free(sinc);
}

/* generateCICKernel (ic_basic.hpp:737-1052) restated: the real-space kernel that
 * the displacement field divides by, as the 27 values around the origin,
 * K[(dx + 1) + 3 (dy + 1) + 9 (dz + 1)].  numpcl = 0: the standard lattice
 * Laplacian; otherwise the kernel of the template particles (pcldata: numpcl
 * float triples in [0, 1) of the template box, tiled numtile times), written
 * with the reference's own float / double types term by term. */
void gevo_cic_kernel(int N, long numpcl, const float *pcldata, int numtile, double K[27]) {
  const long linesize = N;
  double renorm = (double)(linesize * linesize);
  for (int i = 0; i < 27; i++) K[i] = 0.;
#define KER(dx, dy, dz) K[((dx) + 1) + 3 * ((dy) + 1) + 9 * ((dz) + 1)]
  if (numpcl == 0 || pcldata == NULL) {
    KER(0, 0, 0) = 6. * renorm;
    KER(1, 0, 0) = -renorm;
    KER(-1, 0, 0) = -renorm;
    KER(0, 1, 0) = -renorm;
    KER(0, 0, 1) = -renorm;
    KER(0, -1, 0) = -renorm;
    KER(0, 0, -1) = -renorm;
    return;
  }
  renorm /= (double)(numpcl * (long)numtile * (long)numtile * (long)numtile) / (double)(linesize * linesize * linesize);
  /* octant o: per axis, whether the particle is measured from the far side
   * (1 - p, stepping -1) or the near side (p, stepping +1) */
  static const int FAR[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
  for (long i = 0; i < numpcl; i++)
    for (int oct = 0; oct < 8; oct++) {
      float w[3];
      int sgn[3], skip = 0;
      for (int c = 0; c < 3; c++) {
        const float p = pcldata[3 * i + c];
        if (FAR[oct][c]) { /* linesize * (1. - p) / numtile: double */
          const double t = linesize * (1. - p) / numtile;
          if (t >= 1.) skip = 1;
          w[c] = 1. - t;
          sgn[c] = -1;
        } else { /* linesize * p / numtile: float */
          const float t = linesize * p / numtile;
          if (t >= 1.) skip = 1;
          w[c] = 1. - t;
          sgn[c] = 1;
        }
      }
      if (skip) continue;
      const float wx = w[0], wy = w[1], wz = w[2];
      const int sx = sgn[0], sy = sgn[1], sz = sgn[2];
      float ww, q1;
      /* 0-direction */
      ww = wy * wz * renorm;
      q1 = (wx > 0.9) ? 2. : 1.;
      KER(0, 0, 0) += ww * wy * wz * q1;
      KER(sx, 0, 0) -= ww * wy * wz;
      if (wx > 0.9) KER(-sx, 0, 0) -= ww * wy * wz;
      KER(0, 0, sz) += ww * wy * (1. - wz) * q1;
      KER(sx, 0, sz) -= ww * wy * (1. - wz);
      if (wx > 0.9) KER(-sx, 0, sz) -= ww * wy * (1. - wz);
      KER(0, sy, 0) += ww * (1. - wy) * wz * q1;
      KER(sx, sy, 0) -= ww * (1. - wy) * wz;
      if (wx > 0.9) KER(-sx, sy, 0) -= ww * (1. - wy) * wz;
      KER(0, sy, sz) += ww * (1. - wy) * (1. - wz) * q1;
      KER(sx, sy, sz) -= ww * (1. - wy) * (1. - wz);
      if (wx > 0.9) KER(-sx, sy, sz) -= ww * (1. - wy) * (1. - wz);
      /* 1-direction */
      ww = wx * wz * renorm;
      q1 = (wy > 0.9) ? 2. : 1.;
      KER(0, 0, 0) += ww * wx * wz * q1;
      KER(sx, 0, 0) += ww * (1. - wx) * wz * q1;
      KER(0, 0, sz) += ww * wx * (1. - wz) * q1;
      KER(sx, 0, sz) += ww * (1. - wx) * (1. - wz) * q1;
      KER(0, sy, 0) -= ww * wx * wz;
      KER(sx, sy, 0) -= ww * (1. - wx) * wz;
      KER(0, sy, sz) -= ww * wx * (1. - wz);
      KER(sx, sy, sz) -= ww * (1. - wx) * (1. - wz);
      if (wy > 0.9) {
        KER(0, -sy, 0) -= ww * wx * wz;
        KER(sx, -sy, 0) -= ww * (1. - wx) * wz;
        KER(0, -sy, sz) -= ww * wx * (1. - wz);
        KER(sx, -sy, sz) -= ww * (1. - wx) * (1. - wz);
      }
      /* 2-direction */
      ww = wx * wy * renorm;
      q1 = (wz > 0.9) ? 2. : 1.;
      KER(0, 0, 0) += ww * wx * wy * q1;
      KER(sx, 0, 0) += ww * (1. - wx) * wy * q1;
      KER(0, sy, 0) += ww * wx * (1. - wy) * q1;
      KER(sx, sy, 0) += ww * (1. - wx) * (1. - wy) * q1;
      KER(0, 0, sz) -= ww * wx * wy;
      KER(sx, 0, sz) -= ww * (1. - wx) * wy;
      KER(0, sy, sz) -= ww * wx * (1. - wy);
      KER(sx, sy, sz) -= ww * (1. - wx) * (1. - wy);
      if (wz > 0.9) {
        KER(0, 0, -sz) -= ww * wx * wy;
        KER(sx, 0, -sz) -= ww * (1. - wx) * wy;
        KER(0, sy, -sz) -= ww * wx * (1. - wy);
        KER(sx, sy, -sz) -= ww * (1. - wx) * (1. - wy);
      }
    }
#undef KER
}
