/*
 * gev_oracle.c -- CPU restatement (FP64) of gevolution 1.2's per-step
 * particle-mesh path.  TEST INFRASTRUCTURE ONLY (the checker for the CUDA
 * path); see gev_oracle.h for the layout conventions.
 *
 * Build with -ffp-contract=off so that every expression rounds the way it is
 * written: the restatement keeps the reference's evaluation order operation by
 * operation, which makes it bit-identical to gevolution.hpp compiled against the
 * single-rank LATfield2 shim under oracle/ref_shim (checked in tests/).
 */
#define _POSIX_C_SOURCE 199309L
#include "gev_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

typedef struct {
  double re, im;
} cx;

/* complex arithmetic with the semantics of LATfield2's Imag as restated in
 * oracle/ref_shim/LATfield2.hpp */
static inline cx C(double r, double i) { cx z = {r, i}; return z; }
static inline cx cadd(cx a, cx b) { return C(a.re + b.re, a.im + b.im); }
static inline cx csub(cx a, cx b) { return C(a.re - b.re, a.im - b.im); }
static inline cx cmul(cx a, cx b) { return C(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
static inline cx rmul(double d, cx a) { return C(d * a.re, d * a.im); }
static inline cx cdivr(cx a, double d) { return C(a.re / d, a.im / d); }
static inline cx cconj(cx a) { return C(a.re, -a.im); }

/* ===================================================================== */
/* FFT: recursive mixed-radix decimation in time, twiddles in long double */
/* ===================================================================== */

#define TWCACHE 16
static struct {
  int L;
  cx *tw;
} g_tw[TWCACHE];

static const cx *twiddles_locked(int L);
/* the cache is shared by the threads of the parallel FFT loops below */
static const cx *twiddles(int L) {
  const cx *t;
#pragma omp critical(gevo_twiddles)
  t = twiddles_locked(L);
  return t;
}
static const cx *twiddles_locked(int L) {
  for (int i = 0; i < TWCACHE; i++)
    if (g_tw[i].L == L) return g_tw[i].tw;
  int slot = -1;
  for (int i = 0; i < TWCACHE; i++)
    if (g_tw[i].L == 0) { slot = i; break; }
  if (slot < 0) { slot = 0; free(g_tw[0].tw); }
  cx *t = (cx *)malloc(sizeof(cx) * (size_t)L);
  for (int j = 0; j < L; j++) {
    long double ang = 2.0L * 3.14159265358979323846264338327950288L * (long double)j / (long double)L;
    t[j].re = (double)cosl(ang);
    t[j].im = (double)-sinl(ang);
  }
  g_tw[slot].L = L;
  g_tw[slot].tw = t;
  return t;
}

static int smallest_factor(int L) {
  for (int p = 2; p * p <= L; p++)
    if (L % p == 0) return p;
  return L;
}

/* out[k] = sum_n in[n*is] W^{nk}, W = e^{sign 2 pi i / L}; tw is the table of the
 * top-level length L0 */
static void fft_rec(int L, int L0, const cx *in, long is, cx *out, const cx *tw, int sign) {
  if (L == 1) { out[0] = in[0]; return; }
  int p = smallest_factor(L);
  int m = L / p;
  for (int r = 0; r < p; r++) fft_rec(m, L0, in + r * is, is * p, out + (long)r * m, tw, sign);
  long s = L0 / L;
  cx t[64], y[64];
  for (int k = 0; k < m; k++) {
    for (int r = 0; r < p; r++) {
      cx w = tw[((long)r * k * s) % L0];
      if (sign > 0) w.im = -w.im;
      t[r] = cmul(out[(long)r * m + k], w);
    }
    for (int q = 0; q < p; q++) {
      cx acc = t[0];
      for (int r = 1; r < p; r++) {
        cx w = tw[(((long)r * q) % p) * (L0 / p)];
        if (sign > 0) w.im = -w.im;
        acc = cadd(acc, cmul(t[r], w));
      }
      y[q] = acc;
    }
    for (int q = 0; q < p; q++) out[(long)q * m + k] = y[q];
  }
}

/* one line with a given twiddle table and a caller-owned scratch of L values */
static void fft1d_tw(int L, cx *data, int sign, const cx *tw, cx *scratch) {
  memcpy(scratch, data, sizeof(cx) * (size_t)L);
  fft_rec(L, L, scratch, 1, data, tw, sign);
}

void gevo_fft1d(int L, double *data, int sign) {
  const cx *tw = twiddles(L);
  cx *in = (cx *)malloc(sizeof(cx) * (size_t)L);
  fft1d_tw(L, (cx *)data, sign, tw, in);
  free(in);
}

/* The 3-D transforms run their independent lines on OpenMP threads (when built
 * with -fopenmp).  Each line is transformed by the same code on the same values
 * whichever thread takes it, so the result does not depend on the thread count. */

/* r2c along x, then c2c along y and z (unnormalised, FFTW sign). */
void gevo_fft_r2c(int N, const double *in, double *outd) {
  const int NH = N / 2 + 1;
  cx *out = (cx *)outd;
  const cx *tw = twiddles(N);
#pragma omp parallel
  {
    cx *line = (cx *)malloc(sizeof(cx) * (size_t)N);
    cx *scr = (cx *)malloc(sizeof(cx) * (size_t)N);
#pragma omp for schedule(static)
    for (long zy = 0; zy < (long)N * N; zy++) {
      const long z = zy / N, y = zy % N;
      const double *src = in + (size_t)N * (y + (size_t)N * z);
      for (int x = 0; x < N; x++) line[x] = C(src[x], 0.0);
      fft1d_tw(N, line, -1, tw, scr);
      cx *dst = out + (size_t)NH * (y + (size_t)N * z);
      for (int k = 0; k < NH; k++) dst[k] = line[k];
    }
#pragma omp for schedule(static)
    for (long z = 0; z < N; z++)
      for (long kx = 0; kx < NH; kx++) {
        for (long y = 0; y < N; y++) line[y] = out[kx + NH * (y + (size_t)N * z)];
        fft1d_tw(N, line, -1, tw, scr);
        for (long y = 0; y < N; y++) out[kx + NH * (y + (size_t)N * z)] = line[y];
      }
#pragma omp for schedule(static)
    for (long y = 0; y < N; y++)
      for (long kx = 0; kx < NH; kx++) {
        for (long z = 0; z < N; z++) line[z] = out[kx + NH * (y + (size_t)N * z)];
        fft1d_tw(N, line, -1, tw, scr);
        for (long z = 0; z < N; z++) out[kx + NH * (y + (size_t)N * z)] = line[z];
      }
    free(scr);
    free(line);
  }
}

/* c2c along z and y (inverse) into a copy, then c2r along x; input untouched.
 * The c2r uses kx in [0, N/2] and the Hermitian images of 1..N/2-1; the
 * imaginary parts at kx = 0 and kx = N/2 do not contribute. */
void gevo_fft_c2r(int N, const double *ind, double *out) {
  const int NH = N / 2 + 1;
  const size_t n = (size_t)N * N * NH;
  cx *tmp = (cx *)malloc(sizeof(cx) * n);
  memcpy(tmp, ind, sizeof(cx) * n);
  const cx *tw = twiddles(N);
#pragma omp parallel
  {
    cx *line = (cx *)malloc(sizeof(cx) * (size_t)N);
    cx *scr = (cx *)malloc(sizeof(cx) * (size_t)N);
#pragma omp for schedule(static)
    for (long y = 0; y < N; y++)
      for (long kx = 0; kx < NH; kx++) {
        for (long z = 0; z < N; z++) line[z] = tmp[kx + NH * (y + (size_t)N * z)];
        fft1d_tw(N, line, +1, tw, scr);
        for (long z = 0; z < N; z++) tmp[kx + NH * (y + (size_t)N * z)] = line[z];
      }
#pragma omp for schedule(static)
    for (long z = 0; z < N; z++)
      for (long kx = 0; kx < NH; kx++) {
        for (long y = 0; y < N; y++) line[y] = tmp[kx + NH * (y + (size_t)N * z)];
        fft1d_tw(N, line, +1, tw, scr);
        for (long y = 0; y < N; y++) tmp[kx + NH * (y + (size_t)N * z)] = line[y];
      }
#pragma omp for schedule(static)
    for (long zy = 0; zy < (long)N * N; zy++) {
      const long z = zy / N, y = zy % N;
      const cx *src = tmp + (size_t)NH * (y + (size_t)N * z);
      for (int k = 0; k < NH; k++) line[k] = src[k];
      line[0].im = 0.0;
      line[N / 2].im = 0.0;
      for (int k = 1; k < N / 2; k++) line[N - k] = cconj(src[k]);
      fft1d_tw(N, line, +1, tw, scr);
      double *dst = out + (size_t)N * (y + (size_t)N * z);
      for (int x = 0; x < N; x++) dst[x] = line[x].re;
    }
    free(scr);
    free(line);
  }
  free(tmp);
}

/* ===================================================================== */
/* k-space operators                                                      */
/* ===================================================================== */

/* gridk2 / kshift tables, gevolution.hpp:222-227 */
void gevo_kspace_tables(int N, double *gridk2, double *kshift) {
  for (int i = 0; i < N; i++) {
    double g = 2. * (double)N * sin(M_PI * (double)i / (double)N);
    kshift[2 * i] = g * cos(M_PI * (double)i / (double)N);
    kshift[2 * i + 1] = g * -sin(M_PI * (double)i / (double)N);
    gridk2[i] = g * g;
  }
}

#define KLOOP_BEGIN                                                   \
  const int NH = N / 2 + 1;                                           \
  const size_t NK = (size_t)N * N * NH;                               \
  double *gk2 = (double *)malloc(sizeof(double) * N);                 \
  cx *ks = (cx *)malloc(sizeof(cx) * N);                              \
  gevo_kspace_tables(N, gk2, (double *)ks);                           \
  _Pragma("omp parallel for schedule(static)")                        \
  for (long kz = 0; kz < N; kz++)                                     \
    for (long ky = 0; ky < N; ky++)                                   \
      for (long kx = 0; kx < NH; kx++) {                              \
        const size_t id = kx + NH * (ky + (size_t)N * kz);            \
        const double g0 = gk2[kx], g1 = gk2[ky], g2 = gk2[kz];        \
        const cx k0 = ks[kx], k1 = ks[ky], k2s = ks[kz];              \
        (void)g0; (void)g1; (void)g2; (void)k0; (void)k1; (void)k2s;
#define KLOOP_END \
  }               \
  free(gk2);      \
  free(ks);

/* solveModifiedPoissonFT, gevolution.hpp:501-535 */
void gevo_poisson(int N, const double *srcd, double *potd, double coeff, double modif) {
  const cx *src = (const cx *)srcd;
  cx *pot = (cx *)potd;
  coeff /= -((long)N * (long)N * (long)N);
  KLOOP_BEGIN
  (void)NK;
  if (id == 0) {
    if (modif == 0.)
      pot[0] = C(0., 0.);
    else
      pot[0] = cdivr(rmul(coeff, src[0]), modif);
  } else {
    pot[id] = cdivr(rmul(coeff, src[id]), g0 + g1 + g2 + modif);
  }
  KLOOP_END
}

/* projectFTscalar, gevolution.hpp:211-265 */
void gevo_project_scalar(int N, const double *Sd, double *chid, int add) {
  const cx *S = (const cx *)Sd;
  cx *chi = (cx *)chid;
  KLOOP_BEGIN
  if (id == 0) {
    chi[0] = C(0., 0.);
  } else {
    const cx S00 = S[id], S01 = S[NK + id], S02 = S[2 * NK + id];
    const cx S11 = S[3 * NK + id], S12 = S[4 * NK + id], S22 = S[5 * NK + id];
    cx t = rmul(g1 + g2 - 2. * g0, S00);
    t = cadd(t, rmul(g0 + g2 - 2. * g1, S11));
    t = cadd(t, rmul(g0 + g1 - 2. * g2, S22));
    t = csub(t, cmul(cmul(rmul(6., k0), k1), S01));
    t = csub(t, cmul(cmul(rmul(6., k0), k2s), S02));
    t = csub(t, cmul(cmul(rmul(6., k1), k2s), S12));
    t = cdivr(t, 2. * (g0 + g1 + g2) * (g0 + g1 + g2) * N);
    chi[id] = add ? cadd(chi[id], t) : t;
  }
  KLOOP_END
}

/* evolveFTvector, gevolution.hpp:284-330 */
void gevo_evolve_vector(int N, const double *Sd, double *Bd, double a2dtau) {
  const cx *S = (const cx *)Sd;
  cx *B = (cx *)Bd;
  KLOOP_BEGIN
  if (id == 0) {
    B[0] = C(0., 0.);
    B[NK] = C(0., 0.);
    B[2 * NK] = C(0., 0.);
  } else {
    const cx S00 = S[id], S01 = S[NK + id], S02 = S[2 * NK + id];
    const cx S11 = S[3 * NK + id], S12 = S[4 * NK + id], S22 = S[5 * NK + id];
    double k4 = g0 + g1 + g2;
    k4 *= k4;
    const cx pre = C(0., -2. * a2dtau / k4);
    cx x, u;
    x = csub(csub(csub(rmul(g1 + g2, S00), rmul(g1, S11)), rmul(g2, S22)), cmul(cmul(rmul(2., k1), k2s), S12));
    u = cadd(cmul(cconj(k0), x), rmul(g1 + g2 - g0, cadd(cmul(k1, S01), cmul(k2s, S02))));
    B[id] = cadd(B[id], cmul(pre, u));
    x = csub(csub(csub(rmul(g0 + g2, S11), rmul(g0, S00)), rmul(g2, S22)), cmul(cmul(rmul(2., k0), k2s), S02));
    u = cadd(cmul(cconj(k1), x), rmul(g0 + g2 - g1, cadd(cmul(k0, S01), cmul(k2s, S12))));
    B[NK + id] = cadd(B[NK + id], cmul(pre, u));
    x = csub(csub(csub(rmul(g0 + g1, S22), rmul(g0, S00)), rmul(g1, S11)), cmul(cmul(rmul(2., k0), k1), S01));
    u = cadd(cmul(cconj(k2s), x), rmul(g0 + g1 - g2, cadd(cmul(k0, S02), cmul(k1, S12))));
    B[2 * NK + id] = cadd(B[2 * NK + id], cmul(pre, u));
  }
  KLOOP_END
}

/* projectFTvector, gevolution.hpp:350-392 (input and output may alias) */
void gevo_project_vector(int N, const double *Sd, double *Bd, double coeff, double modif) {
  const cx *S = (const cx *)Sd;
  cx *B = (cx *)Bd;
  KLOOP_BEGIN
  if (id == 0) {
    B[0] = C(0., 0.);
    B[NK] = C(0., 0.);
    B[2 * NK] = C(0., 0.);
  } else {
    const cx S0 = S[id], S1 = S[NK + id], S2 = S[2 * NK + id];
    double kk = g0 + g1 + g2;
    cx tmp = cdivr(cadd(cadd(cmul(k0, S0), cmul(k1, S1)), cmul(k2s, S2)), kk);
    B[id] = cdivr(rmul(coeff, rmul(4., csub(S0, cmul(cconj(k0), tmp)))), kk + modif);
    B[NK + id] = cdivr(rmul(coeff, rmul(4., csub(S1, cmul(cconj(k1), tmp)))), kk + modif);
    B[2 * NK + id] = cdivr(rmul(coeff, rmul(4., csub(S2, cmul(cconj(k2s), tmp)))), kk + modif);
  }
  KLOOP_END
}

/* projectFTtensor, gevolution.hpp:411-482 (input and output may alias) */
void gevo_project_tensor(int N, const double *Sd, double *hd) {
  const cx *S = (const cx *)Sd;
  cx *h = (cx *)hd;
  KLOOP_BEGIN
  if (id == 0) {
    for (int c = 0; c < 6; c++) h[c * NK] = C(0., 0.);
  } else {
    const cx Sxx = S[id], Sxy = S[NK + id], Sxz = S[2 * NK + id];
    const cx Syy = S[3 * NK + id], Syz = S[4 * NK + id], Szz = S[5 * NK + id];
    const double kk = g0 + g1 + g2;
    const double k6 = kk * kk * kk * N;
    cx t;
    /* 00 */
    t = rmul(g0 - kk, cadd(rmul(g0 - kk, Sxx), cmul(rmul(2., k0), cadd(cmul(k1, Sxy), cmul(k2s, Sxz)))));
    t = cadd(t, rmul((g0 + kk) * (g1 + kk) - 2. * kk * kk, Syy));
    t = cadd(t, rmul((g0 + kk) * (g2 + kk) - 2. * kk * kk, Szz));
    t = cadd(t, cmul(cmul(rmul(2. * (g0 + kk), k1), k2s), Syz));
    const cx h00 = cdivr(t, k6);
    /* 01 */
    t = rmul(2. * (g0 - kk) * (g1 - kk), Sxy);
    t = cadd(t, cmul(cmul(rmul(g2 + kk, cconj(k0)), cconj(k1)), Szz));
    t = cadd(t, cmul(rmul(g0 - kk, cconj(k1)), cadd(cmul(cconj(k0), Sxx), cmul(rmul(2., k2s), Sxz))));
    t = cadd(t, cmul(rmul(g1 - kk, cconj(k0)), cadd(cmul(cconj(k1), Syy), cmul(rmul(2., k2s), Syz))));
    const cx h01 = cdivr(t, k6);
    /* 02 */
    t = rmul(2. * (g0 - kk) * (g2 - kk), Sxz);
    t = cadd(t, cmul(cmul(rmul(g1 + kk, cconj(k0)), cconj(k2s)), Syy));
    t = cadd(t, cmul(rmul(g0 - kk, cconj(k2s)), cadd(cmul(cconj(k0), Sxx), cmul(rmul(2., k1), Sxy))));
    t = cadd(t, cmul(rmul(g2 - kk, cconj(k0)), cadd(cmul(cconj(k2s), Szz), cmul(rmul(2., k1), Syz))));
    const cx h02 = cdivr(t, k6);
    /* 11 */
    t = rmul(g1 - kk, cadd(rmul(g1 - kk, Syy), cmul(rmul(2., k1), cadd(cmul(k0, Sxy), cmul(k2s, Syz)))));
    t = cadd(t, rmul((g1 + kk) * (g0 + kk) - 2. * kk * kk, Sxx));
    t = cadd(t, rmul((g1 + kk) * (g2 + kk) - 2. * kk * kk, Szz));
    t = cadd(t, cmul(cmul(rmul(2. * (g1 + kk), k0), k2s), Sxz));
    const cx h11 = cdivr(t, k6);
    /* 12 */
    t = rmul(2. * (g1 - kk) * (g2 - kk), Syz);
    t = cadd(t, cmul(cmul(rmul(g0 + kk, cconj(k1)), cconj(k2s)), Sxx));
    t = cadd(t, cmul(rmul(g1 - kk, cconj(k2s)), cadd(cmul(cconj(k1), Syy), cmul(rmul(2., k0), Sxy))));
    t = cadd(t, cmul(rmul(g2 - kk, cconj(k1)), cadd(cmul(cconj(k2s), Szz), cmul(rmul(2., k0), Sxz))));
    const cx h12 = cdivr(t, k6);
    /* 22 */
    t = rmul(g2 - kk, cadd(rmul(g2 - kk, Szz), cmul(rmul(2., k2s), cadd(cmul(k0, Sxz), cmul(k1, Syz)))));
    t = cadd(t, rmul((g2 + kk) * (g0 + kk) - 2. * kk * kk, Sxx));
    t = cadd(t, rmul((g2 + kk) * (g1 + kk) - 2. * kk * kk, Syy));
    t = cadd(t, cmul(cmul(rmul(2. * (g2 + kk), k0), k1), Sxy));
    const cx h22 = cdivr(t, k6);
    h[id] = h00;
    h[NK + id] = h01;
    h[2 * NK + id] = h02;
    h[3 * NK + id] = h11;
    h[4 * NK + id] = h12;
    h[5 * NK + id] = h22;
  }
  KLOOP_END
}

/* ===================================================================== */
/* real-space sources                                                    */
/* ===================================================================== */

static inline size_t SI(int N, int x, int y, int z) {
  x = (x + N) % N;
  y = (y + N) % N;
  z = (z + N) % N;
  return (size_t)x + (size_t)N * ((size_t)y + (size_t)N * (size_t)z);
}

/* prepareFTsource (tensor), gevolution.hpp:56-147 (PHINONLINEAR, not ORIGINALMETRIC).
 * Sij may be the same array as Tij. */
void gevo_prepare_source_tensor(int N, const double *phi, const double *T, double *S, double coeff) {
  const size_t V = (size_t)N * N * N;
#pragma omp parallel for schedule(static)
  for (int z = 0; z < N; z++)
    for (int y = 0; y < N; y++)
      for (int x = 0; x < N; x++) {
        const size_t i = SI(N, x, y, z);
        const double p = phi[i];
        const double pxp = phi[SI(N, x + 1, y, z)], pxm = phi[SI(N, x - 1, y, z)];
        const double pyp = phi[SI(N, x, y + 1, z)], pym = phi[SI(N, x, y - 1, z)];
        const double pzp = phi[SI(N, x, y, z + 1)], pzm = phi[SI(N, x, y, z - 1)];
        const double pxy = phi[SI(N, x + 1, y + 1, z)], pxz = phi[SI(N, x + 1, y, z + 1)];
        const double pyz = phi[SI(N, x, y + 1, z + 1)];
        double s;
        s = coeff * T[i];
        s += 0.5 * (pxp - pxm) * (pxp - pxm);
        S[i] = s;
        s = coeff * T[3 * V + i];
        s += 0.5 * (pyp - pym) * (pyp - pym);
        S[3 * V + i] = s;
        s = coeff * T[5 * V + i];
        s += 0.5 * (pzp - pzm) * (pzp - pzm);
        S[5 * V + i] = s;
        s = coeff * T[V + i];
        s += pxp * pyp - p * pxy;
        s += 0.5 * p * p;
        s -= 0.5 * pxp * pxp;
        s -= 0.5 * pyp * pyp;
        s += 0.5 * pxy * pxy;
        S[V + i] = s;
        s = coeff * T[2 * V + i];
        s += pxp * pzp - p * pxz;
        s += 0.5 * p * p;
        s -= 0.5 * pxp * pxp;
        s -= 0.5 * pzp * pzp;
        s += 0.5 * pxz * pxz;
        S[2 * V + i] = s;
        s = coeff * T[4 * V + i];
        s += pyp * pzp - p * pyz;
        s += 0.5 * p * p;
        s -= 0.5 * pyp * pyp;
        s -= 0.5 * pzp * pzp;
        s += 0.5 * pyz * pyz;
        S[4 * V + i] = s;
      }
}

/* prepareFTsource (scalar), gevolution.hpp:169-192 (PHINONLINEAR, not ORIGINALMETRIC).
 * result may be the same array as source. */
void gevo_prepare_source_scalar(int N, const double *phi, const double *chi, const double *source,
                                double bgmodel, double *result, double coeff, double coeff2,
                                double coeff3) {
#pragma omp parallel for schedule(static)
  for (int z = 0; z < N; z++)
    for (int y = 0; y < N; y++)
      for (int x = 0; x < N; x++) {
        const size_t i = SI(N, x, y, z);
        const double p = phi[i];
        const double dxp = phi[SI(N, x - 1, y, z)] - phi[SI(N, x + 1, y, z)];
        const double dyp = phi[SI(N, x, y - 1, z)] - phi[SI(N, x, y + 1, z)];
        const double dzp = phi[SI(N, x, y, z - 1)] - phi[SI(N, x, y, z + 1)];
        double r = coeff2 * (source[i] - bgmodel);
        r *= 1. - 2. * p;
        r += 0.125 * dxp * dxp;
        r += 0.125 * dyp * dyp;
        r += 0.125 * dzp * dzp;
        r += (coeff3 - coeff) * p - coeff3 * chi[i];
        result[i] = r;
      }
}

/* ===================================================================== */
/* particle store                                                         */
/* ===================================================================== */

int gevo_cell_of(int N, double p) {
  const double dx = 1.0 / (double)N;
  int c = (int)(p / dx);
  if (c >= N) c = N - 1;
  if (c < 0) c = 0;
  return c;
}

void gevo_wrap(double *p) {
  if (*p >= 1.0)
    *p -= 1.0;
  else if (*p < 0.0) {
    *p += 1.0;
    if (*p >= 1.0) *p -= 1.0;
  }
}

static long cell_index(int N, const gevo_part *q) {
  return (long)gevo_cell_of(N, q->pos[0]) +
         (long)N * ((long)gevo_cell_of(N, q->pos[1]) + (long)N * (long)gevo_cell_of(N, q->pos[2]));
}
static int cmp_id(const void *a, const void *b) {
  const gevo_part *p = (const gevo_part *)a, *q = (const gevo_part *)b;
  return p->ID < q->ID ? -1 : (p->ID > q->ID ? 1 : 0);
}

/* (cell, ID) order: a stable counting sort by cell, then each cell's run sorted
 * by ID (insertion sort; qsort for long runs).  IDs are unique, so the order is
 * a total order and does not depend on how it is reached. */
void gevo_sort(int N, long np, gevo_part *p, long *cell_start) {
  const long V = (long)N * N * N;
  long *cs = cell_start ? cell_start : (long *)malloc(sizeof(long) * (size_t)(V + 1));
  long *key = (long *)malloc(sizeof(long) * (size_t)(np > 0 ? np : 1));
  long *fill = (long *)malloc(sizeof(long) * (size_t)V);
  gevo_part *tmp = (gevo_part *)malloc(sizeof(gevo_part) * (size_t)(np > 0 ? np : 1));
#pragma omp parallel for schedule(static)
  for (long i = 0; i < np; i++) key[i] = cell_index(N, p + i);
  for (long c = 0; c <= V; c++) cs[c] = 0;
  for (long i = 0; i < np; i++) cs[key[i] + 1]++;
  for (long c = 0; c < V; c++) cs[c + 1] += cs[c];
  memcpy(fill, cs, sizeof(long) * (size_t)V);
  for (long i = 0; i < np; i++) tmp[fill[key[i]]++] = p[i];
#pragma omp parallel for schedule(dynamic, 4096)
  for (long c = 0; c < V; c++) {
    const long b = cs[c], e = cs[c + 1];
    if (e - b > 64) {
      qsort(tmp + b, (size_t)(e - b), sizeof(gevo_part), cmp_id);
      continue;
    }
    for (long i = b + 1; i < e; i++) {
      const gevo_part t = tmp[i];
      long j = i - 1;
      while (j >= b && tmp[j].ID > t.ID) {
        tmp[j + 1] = tmp[j];
        j--;
      }
      tmp[j + 1] = t;
    }
  }
  memcpy(p, tmp, sizeof(gevo_part) * (size_t)np);
  free(tmp);
  free(fill);
  free(key);
  if (!cell_start) free(cs);
}

/* ===================================================================== */
/* deposits: accumulate into a field with an upper halo, then fold        */
/* ===================================================================== */

typedef struct {
  int N, M; /* M = N + 1 */
  double *e;
} ext_t;

static void ext_open(ext_t *E, int N, const double *f) {
  E->N = N;
  E->M = N + 1;
  const size_t M = (size_t)E->M;
  E->e = (double *)calloc(M * M * M, sizeof(double));
#pragma omp parallel for schedule(static)
  for (int z = 0; z < N; z++)
    for (int y = 0; y < N; y++)
      for (int x = 0; x < N; x++) E->e[x + M * (y + M * z)] = f[SI(N, x, y, z)];
}
static inline double *EX(ext_t *E, int x, int y, int z) {
  const size_t M = (size_t)E->M;
  return E->e + x + M * (y + M * (size_t)z);
}
/* the *_comm halo fold (x, then y, then z) and write-back; within one fold every
 * statement adds one halo value into one interior value */
static void ext_close(ext_t *E, double *f) {
  const int N = E->N;
#pragma omp parallel for schedule(static)
  for (int z = 0; z <= N; z++)
    for (int y = 0; y <= N; y++) *EX(E, 0, y, z) += *EX(E, N, y, z);
#pragma omp parallel for schedule(static)
  for (int z = 0; z <= N; z++)
    for (int x = 0; x < N; x++) *EX(E, x, 0, z) += *EX(E, x, N, z);
#pragma omp parallel for schedule(static)
  for (int y = 0; y < N; y++)
    for (int x = 0; x < N; x++) *EX(E, x, y, 0) += *EX(E, x, y, N);
#pragma omp parallel for schedule(static)
  for (int z = 0; z < N; z++)
    for (int y = 0; y < N; y++)
      for (int x = 0; x < N; x++) f[SI(N, x, y, z)] = *EX(E, x, y, z);
  free(E->e);
}

/* phi at the 8 corners in the order 000 001 010 011 100 101 110 111 (XYZ) */
static void local_cube_phi(int N, const double *phi, int x, int y, int z, double *l) {
  if (!phi) {
    for (int i = 0; i < 8; i++) l[i] = 0.0;
    return;
  }
  l[0] = phi[SI(N, x, y, z)];
  l[1] = phi[SI(N, x, y, z + 1)];
  l[2] = phi[SI(N, x, y + 1, z)];
  l[3] = phi[SI(N, x, y + 1, z + 1)];
  l[4] = phi[SI(N, x + 1, y, z)];
  l[5] = phi[SI(N, x + 1, y, z + 1)];
  l[6] = phi[SI(N, x + 1, y + 1, z)];
  l[7] = phi[SI(N, x + 1, y + 1, z + 1)];
}

/* The deposits run over chunks of z planes on OpenMP threads, in two phases per
 * chunk.  (1) Each nonempty cell's sums over its particles (the reference's
 * local cube) are formed into a buffer, one cell per iteration.  (2) Each
 * target plane t of the field with the upper halo is owned by one thread, which
 * adds to it first the upper halves (corners at z + 1) of the cells of plane
 * t - 1 and then the lower halves of the cells of plane t, each in site order.
 * One loop over all cells in site order adds to every field value in exactly
 * that order (a cell adds at most once to any one value), so the sums do not
 * depend on the thread count. */
typedef struct {
  int N;
  double dx, a, mass;
  const gevo_part *p;
  const long *cs;
  const double *phi;
  ext_t *E;
} dep_t;
typedef void (*dep_cell_fn)(const dep_t *D, long c, int x, int y, int z, double *out);
typedef void (*dep_half_fn)(const dep_t *D, const double *v, int x, int y, int t);

static void dep_run(const dep_t *D, int nv, dep_cell_fn cell, dep_half_fn lower, dep_half_fn upper) {
  const int N = D->N;
  const long P = (long)N * N;
  long pl = (1L << 20) / P;
  const int zc = pl < 1 ? 1 : (pl > N ? N : (int)pl);
  /* slot s holds cell plane z0 - 1 + s */
  double *buf = (double *)malloc(sizeof(double) * (size_t)nv * (size_t)P * (size_t)(zc + 1));
  for (int z0 = 0; z0 < N; z0 += zc) {
    const int z1 = z0 + zc < N ? z0 + zc : N;
#pragma omp parallel for schedule(dynamic, 1024)
    for (long k = 0; k < P * (z1 - z0); k++) {
      const long c = P * z0 + k;
      if (D->cs[c + 1] == D->cs[c]) continue;
      cell(D, c, (int)(c % N), (int)((c / N) % N), (int)(c / P), buf + (size_t)nv * (size_t)(P + k));
    }
    const int tend = z1 == N ? N + 1 : z1;
#pragma omp parallel for schedule(static, 1)
    for (int t = z0; t < tend; t++) {
      if (t >= 1) {
        const int zc_ = t - 1;
        const double *slot = buf + (size_t)nv * (size_t)P * (size_t)(zc_ - (z0 - 1));
        for (long k = 0; k < P; k++) {
          const long c = P * zc_ + k;
          if (D->cs[c + 1] == D->cs[c]) continue;
          upper(D, slot + (size_t)nv * k, (int)(k % N), (int)(k / N), t);
        }
      }
      if (t < N) {
        const double *slot = buf + (size_t)nv * (size_t)P * (size_t)(t - (z0 - 1));
        for (long k = 0; k < P; k++) {
          const long c = P * t + k;
          if (D->cs[c + 1] == D->cs[c]) continue;
          lower(D, slot + (size_t)nv * k, (int)(k % N), (int)(k / N), t);
        }
      }
    }
    /* the last plane of the chunk feeds the next chunk's first target plane */
    memcpy(buf, buf + (size_t)nv * (size_t)P * (size_t)(z1 - z0), sizeof(double) * (size_t)nv * (size_t)P);
  }
  free(buf);
}

/* ---- projection_T00_project, gevolution.hpp:926-1022, + scalarProjectionCIC_comm ---- */
static void t00_cell(const dep_t *D, long c, int x, int y, int z, double *lc) {
  const int N = D->N;
  const double dx = D->dx, a = D->a;
  const gevo_part *p = D->p;
  const double ref[3] = {x * dx, y * dx, z * dx};
  double e = a, f = 0., l[8];
  for (int i = 0; i < 8; i++) lc[i] = 0.;
  local_cube_phi(N, D->phi, x, y, z, l);
  for (long j = D->cs[c]; j < D->cs[c + 1]; j++) {
    double up[3], dn[3];
    for (int i = 0; i < 3; i++) {
      up[i] = (p[j].pos[i] - ref[i]) / dx;
      dn[i] = 1.0 - up[i];
    }
    if (D->phi) {
      const double *q = p[j].vel;
      f = q[0] * q[0] + q[1] * q[1] + q[2] * q[2];
      e = sqrt(f + a * a);
      f = 3. * e + f / e;
    }
    lc[0] += dn[0] * dn[1] * dn[2] * (e + f * l[0]);
    lc[1] += dn[0] * dn[1] * up[2] * (e + f * l[1]);
    lc[2] += dn[0] * up[1] * dn[2] * (e + f * l[2]);
    lc[3] += dn[0] * up[1] * up[2] * (e + f * l[3]);
    lc[4] += up[0] * dn[1] * dn[2] * (e + f * l[4]);
    lc[5] += up[0] * dn[1] * up[2] * (e + f * l[5]);
    lc[6] += up[0] * up[1] * dn[2] * (e + f * l[6]);
    lc[7] += up[0] * up[1] * up[2] * (e + f * l[7]);
  }
}
/* the eight corner sums times the mass factor; lower: corners 0 2 4 6 at z = t */
static void cic8_lower(const dep_t *D, const double *lc, int x, int y, int t) {
  ext_t *E = D->E;
  const double mass = D->mass;
  *EX(E, x, y, t) += lc[0] * mass;
  *EX(E, x, y + 1, t) += lc[2] * mass;
  *EX(E, x + 1, y, t) += lc[4] * mass;
  *EX(E, x + 1, y + 1, t) += lc[6] * mass;
}
static void cic8_upper(const dep_t *D, const double *lc, int x, int y, int t) {
  ext_t *E = D->E;
  const double mass = D->mass;
  *EX(E, x, y, t) += lc[1] * mass;
  *EX(E, x, y + 1, t) += lc[3] * mass;
  *EX(E, x + 1, y, t) += lc[5] * mass;
  *EX(E, x + 1, y + 1, t) += lc[7] * mass;
}

void gevo_deposit_T00(int N, long np, const gevo_part *p, const long *cs, double m, double a,
                      const double *phi, double coeff, double *T00) {
  (void)np;
  const double dx = 1.0 / (double)N;
  double mass = coeff / (dx * dx * dx);
  mass *= m;
  mass /= a;
  ext_t E;
  ext_open(&E, N, T00);
  const dep_t D = {N, dx, a, mass, p, cs, phi, &E};
  dep_run(&D, 8, t00_cell, cic8_lower, cic8_upper);
  ext_close(&E, T00);
}

/* ---- scalarProjectionCIC_project (LATfield2, used by main.cpp:402 and
 * ic_basic.hpp:2180): plain CIC mass deposit m/dx^3 * w, + comm fold ---- */
static void mass_cell(const dep_t *D, long c, int x, int y, int z, double *lc) {
  const double dx = D->dx;
  const gevo_part *p = D->p;
  const double ref[3] = {x * dx, y * dx, z * dx};
  for (int i = 0; i < 8; i++) lc[i] = 0.;
  for (long j = D->cs[c]; j < D->cs[c + 1]; j++) {
    double up[3], dn[3];
    for (int i = 0; i < 3; i++) {
      up[i] = (p[j].pos[i] - ref[i]) / dx;
      dn[i] = 1.0 - up[i];
    }
    lc[0] += dn[0] * dn[1] * dn[2];
    lc[1] += dn[0] * dn[1] * up[2];
    lc[2] += dn[0] * up[1] * dn[2];
    lc[3] += dn[0] * up[1] * up[2];
    lc[4] += up[0] * dn[1] * dn[2];
    lc[5] += up[0] * dn[1] * up[2];
    lc[6] += up[0] * up[1] * dn[2];
    lc[7] += up[0] * up[1] * up[2];
  }
}

void gevo_deposit_mass(int N, long np, const gevo_part *p, const long *cs, double m, double *rho) {
  (void)np;
  const double dx = 1.0 / (double)N;
  const double mass = m / (dx * dx * dx);
  ext_t E;
  ext_open(&E, N, rho);
  const dep_t D = {N, dx, 1., mass, p, cs, NULL, &E};
  dep_run(&D, 8, mass_cell, cic8_lower, cic8_upper);
  ext_close(&E, rho);
}

/* ---- projection_T0i_project, gevolution.hpp:1045-1147, + vectorProjectionCICNGP_comm ----
 * per cell: the 12 link sums, then the 8 corner values of phi */
static void t0i_cell(const dep_t *D, long c, int x, int y, int z, double *qi) {
  const double dx = D->dx, mass = D->mass;
  const gevo_part *p = D->p;
  const double ref[3] = {x * dx, y * dx, z * dx};
  for (int i = 0; i < 12; i++) qi[i] = 0.;
  local_cube_phi(D->N, D->phi, x, y, z, qi + 12);
  for (long j = D->cs[c]; j < D->cs[c + 1]; j++) {
    double up[3], dn[3];
    for (int i = 0; i < 3; i++) {
      up[i] = (p[j].pos[i] - ref[i]) / dx;
      dn[i] = 1.0 - up[i];
    }
    const double *q = p[j].vel;
    double w = mass * q[0];
    qi[0] += w * dn[1] * dn[2];
    qi[1] += w * up[1] * dn[2];
    qi[2] += w * dn[1] * up[2];
    qi[3] += w * up[1] * up[2];
    w = mass * q[1];
    qi[4] += w * dn[0] * dn[2];
    qi[5] += w * up[0] * dn[2];
    qi[6] += w * dn[0] * up[2];
    qi[7] += w * up[0] * up[2];
    w = mass * q[2];
    qi[8] += w * dn[0] * dn[1];
    qi[9] += w * up[0] * dn[1];
    qi[10] += w * dn[0] * up[1];
    qi[11] += w * up[0] * up[1];
  }
}
static void t0i_lower(const dep_t *D, const double *qi, int x, int y, int t) {
  ext_t *E = D->E;
  const double *l = qi + 12;
  *EX(&E[0], x, y, t) += qi[0] * (1. + l[0] + l[4]);
  *EX(&E[1], x, y, t) += qi[4] * (1. + l[0] + l[2]);
  *EX(&E[2], x, y, t) += qi[8] * (1. + l[0] + l[1]);
  *EX(&E[1], x + 1, y, t) += qi[5] * (1. + l[4] + l[6]);
  *EX(&E[2], x + 1, y, t) += qi[9] * (1. + l[4] + l[5]);
  *EX(&E[0], x, y + 1, t) += qi[1] * (1. + l[2] + l[6]);
  *EX(&E[2], x, y + 1, t) += qi[10] * (1. + l[2] + l[3]);
  *EX(&E[2], x + 1, y + 1, t) += qi[11] * (1. + l[6] + l[7]);
}
static void t0i_upper(const dep_t *D, const double *qi, int x, int y, int t) {
  ext_t *E = D->E;
  const double *l = qi + 12;
  *EX(&E[0], x, y, t) += qi[2] * (1. + l[1] + l[5]);
  *EX(&E[1], x, y, t) += qi[6] * (1. + l[1] + l[3]);
  *EX(&E[0], x, y + 1, t) += qi[3] * (1. + l[3] + l[7]);
  *EX(&E[1], x + 1, y, t) += qi[7] * (1. + l[5] + l[7]);
}

void gevo_deposit_T0i(int N, long np, const gevo_part *p, const long *cs, double m,
                      const double *phi, double coeff, double *T0i) {
  (void)np;
  const size_t V = (size_t)N * N * N;
  const double dx = 1.0 / (double)N;
  double mass = coeff / (dx * dx * dx);
  mass *= m;
  ext_t E[3];
  for (int c = 0; c < 3; c++) ext_open(&E[c], N, T0i + c * V);
  const dep_t D = {N, dx, 1., mass, p, cs, phi, E};
  dep_run(&D, 20, t0i_cell, t0i_lower, t0i_upper);
  for (int c = 0; c < 3; c++) ext_close(&E[c], T0i + c * V);
}

/* ---- projection_Tij_project, gevolution.hpp:1172-1297, + symtensorProjectionCICNGP_comm ----
 * component slots: 0=00 1=01 2=02 3=11 4=12 5=22; per cell: the 6 plaquette
 * sums, then the 24 diagonal corner sums */
static const int tij_diag[3] = {0, 3, 5};
static void tij_cell(const dep_t *D, long c, int x, int y, int z, double *tij) {
  const double dx = D->dx, a = D->a, mass = D->mass;
  const gevo_part *p = D->p;
  const double ref[3] = {(double)x * dx, (double)y * dx, (double)z * dx};
  double *tii = tij + 6, l[8];
  for (int i = 0; i < 30; i++) tij[i] = 0.;
  local_cube_phi(D->N, D->phi, x, y, z, l);
  for (long j = D->cs[c]; j < D->cs[c + 1]; j++) {
    double up[3], dn[3];
    for (int i = 0; i < 3; i++) {
      up[i] = (p[j].pos[i] - ref[i]) / dx;
      dn[i] = 1.0 - up[i];
    }
    const double *q = p[j].vel;
    double f = q[0] * q[0] + q[1] * q[1] + q[2] * q[2];
    const double e = sqrt(f + a * a);
    f = 4. + a * a / (f + a * a);
    for (int i = 0; i < 3; i++) {
      const double w = mass * q[i] * q[i] / e;
      tii[0 + i * 8] += w * dn[0] * dn[1] * dn[2] * (1. + f * l[0]);
      tii[1 + i * 8] += w * dn[0] * dn[1] * up[2] * (1. + f * l[1]);
      tii[2 + i * 8] += w * dn[0] * up[1] * dn[2] * (1. + f * l[2]);
      tii[3 + i * 8] += w * dn[0] * up[1] * up[2] * (1. + f * l[3]);
      tii[4 + i * 8] += w * up[0] * dn[1] * dn[2] * (1. + f * l[4]);
      tii[5 + i * 8] += w * up[0] * dn[1] * up[2] * (1. + f * l[5]);
      tii[6 + i * 8] += w * up[0] * up[1] * dn[2] * (1. + f * l[6]);
      tii[7 + i * 8] += w * up[0] * up[1] * up[2] * (1. + f * l[7]);
    }
    double w = mass * q[0] * q[1] / e;
    tij[0] += w * dn[2] * (1. + f * 0.25 * (l[0] + l[2] + l[4] + l[6]));
    tij[1] += w * up[2] * (1. + f * 0.25 * (l[1] + l[3] + l[5] + l[7]));
    w = mass * q[0] * q[2] / e;
    tij[2] += w * dn[1] * (1. + f * 0.25 * (l[0] + l[1] + l[4] + l[5]));
    tij[3] += w * up[1] * (1. + f * 0.25 * (l[2] + l[3] + l[6] + l[7]));
    w = mass * q[1] * q[2] / e;
    tij[4] += w * dn[0] * (1. + f * 0.25 * (l[0] + l[1] + l[2] + l[3]));
    tij[5] += w * up[0] * (1. + f * 0.25 * (l[4] + l[5] + l[6] + l[7]));
  }
}
static void tij_lower(const dep_t *D, const double *tij, int x, int y, int t) {
  ext_t *E = D->E;
  const double *tii = tij + 6;
  for (int i = 0; i < 3; i++) *EX(&E[tij_diag[i]], x, y, t) += tii[8 * i];
  *EX(&E[1], x, y, t) += tij[0];
  *EX(&E[2], x, y, t) += tij[2];
  *EX(&E[4], x, y, t) += tij[4];
  for (int i = 0; i < 3; i++) *EX(&E[tij_diag[i]], x + 1, y, t) += tii[4 + 8 * i];
  *EX(&E[4], x + 1, y, t) += tij[5];
  for (int i = 0; i < 3; i++) *EX(&E[tij_diag[i]], x, y + 1, t) += tii[2 + 8 * i];
  *EX(&E[2], x, y + 1, t) += tij[3];
  for (int i = 0; i < 3; i++) *EX(&E[tij_diag[i]], x + 1, y + 1, t) += tii[6 + 8 * i];
}
static void tij_upper(const dep_t *D, const double *tij, int x, int y, int t) {
  ext_t *E = D->E;
  const double *tii = tij + 6;
  for (int i = 0; i < 3; i++) *EX(&E[tij_diag[i]], x, y, t) += tii[1 + 8 * i];
  *EX(&E[1], x, y, t) += tij[1];
  for (int i = 0; i < 3; i++) *EX(&E[tij_diag[i]], x + 1, y, t) += tii[5 + 8 * i];
  for (int i = 0; i < 3; i++) *EX(&E[tij_diag[i]], x, y + 1, t) += tii[3 + 8 * i];
  for (int i = 0; i < 3; i++) *EX(&E[tij_diag[i]], x + 1, y + 1, t) += tii[7 + 8 * i];
}

void gevo_deposit_Tij(int N, long np, const gevo_part *p, const long *cs, double m, double a,
                      const double *phi, double coeff, double *Tij) {
  (void)np;
  const size_t V = (size_t)N * N * N;
  const double dx = 1.0 / (double)N;
  double mass = coeff / (dx * dx * dx);
  mass *= m;
  mass /= a;
  ext_t E[6];
  for (int c = 0; c < 6; c++) ext_open(&E[c], N, Tij + c * V);
  const dep_t D = {N, dx, a, mass, p, cs, phi, E};
  dep_run(&D, 30, tij_cell, tij_lower, tij_upper);
  for (int c = 0; c < 6; c++) ext_close(&E[c], Tij + c * V);
}

/* ===================================================================== */
/* particle updates                                                      */
/* ===================================================================== */

#define F(fld, dx_, dy_, dz_) (fld)[SI(N, cx_ + (dx_), cy_ + (dy_), cz_ + (dz_))]

/* update_q, gevolution.hpp:570-678 (GRADIENT_ORDER 1) */
static double update_q_one(int N, gevo_part *pt, const double *r, int cx_, int cy_, int cz_,
                           double dtau, const double *phi, const double *chi, const double *Bi,
                           int nfield, const double *params) {
  const size_t V = (size_t)N * N * N;
  const double dx = 1.0 / (double)N;
  double gradphi[3] = {0, 0, 0};
  double pgradB[3] = {0, 0, 0};
  double *q = pt->vel;
  double v2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2];
  double e2 = v2 + params[0] * params[0];

  gradphi[0] = (1. - r[1]) * (1. - r[2]) * (F(phi, 1, 0, 0) - F(phi, 0, 0, 0));
  gradphi[1] = (1. - r[0]) * (1. - r[2]) * (F(phi, 0, 1, 0) - F(phi, 0, 0, 0));
  gradphi[2] = (1. - r[0]) * (1. - r[1]) * (F(phi, 0, 0, 1) - F(phi, 0, 0, 0));
  gradphi[0] += r[1] * (1. - r[2]) * (F(phi, 1, 1, 0) - F(phi, 0, 1, 0));
  gradphi[1] += r[0] * (1. - r[2]) * (F(phi, 1, 1, 0) - F(phi, 1, 0, 0));
  gradphi[2] += r[0] * (1. - r[1]) * (F(phi, 1, 0, 1) - F(phi, 1, 0, 0));
  gradphi[0] += (1. - r[1]) * r[2] * (F(phi, 1, 0, 1) - F(phi, 0, 0, 1));
  gradphi[1] += (1. - r[0]) * r[2] * (F(phi, 0, 1, 1) - F(phi, 0, 0, 1));
  gradphi[2] += (1. - r[0]) * r[1] * (F(phi, 0, 1, 1) - F(phi, 0, 1, 0));
  gradphi[0] += r[1] * r[2] * (F(phi, 1, 1, 1) - F(phi, 0, 1, 1));
  gradphi[1] += r[0] * r[2] * (F(phi, 1, 1, 1) - F(phi, 1, 0, 1));
  gradphi[2] += r[0] * r[1] * (F(phi, 1, 1, 1) - F(phi, 1, 1, 0));

  gradphi[0] *= (v2 + e2) / e2;
  gradphi[1] *= (v2 + e2) / e2;
  gradphi[2] *= (v2 + e2) / e2;

  if (nfield >= 2 && chi != NULL) {
    gradphi[0] -= (1. - r[1]) * (1. - r[2]) * (F(chi, 1, 0, 0) - F(chi, 0, 0, 0));
    gradphi[1] -= (1. - r[0]) * (1. - r[2]) * (F(chi, 0, 1, 0) - F(chi, 0, 0, 0));
    gradphi[2] -= (1. - r[0]) * (1. - r[1]) * (F(chi, 0, 0, 1) - F(chi, 0, 0, 0));
    gradphi[0] -= r[1] * (1. - r[2]) * (F(chi, 1, 1, 0) - F(chi, 0, 1, 0));
    gradphi[1] -= r[0] * (1. - r[2]) * (F(chi, 1, 1, 0) - F(chi, 1, 0, 0));
    gradphi[2] -= r[0] * (1. - r[1]) * (F(chi, 1, 0, 1) - F(chi, 1, 0, 0));
    gradphi[0] -= (1. - r[1]) * r[2] * (F(chi, 1, 0, 1) - F(chi, 0, 0, 1));
    gradphi[1] -= (1. - r[0]) * r[2] * (F(chi, 0, 1, 1) - F(chi, 0, 0, 1));
    gradphi[2] -= (1. - r[0]) * r[1] * (F(chi, 0, 1, 1) - F(chi, 0, 1, 0));
    gradphi[0] -= r[1] * r[2] * (F(chi, 1, 1, 1) - F(chi, 0, 1, 1));
    gradphi[1] -= r[0] * r[2] * (F(chi, 1, 1, 1) - F(chi, 1, 0, 1));
    gradphi[2] -= r[0] * r[1] * (F(chi, 1, 1, 1) - F(chi, 1, 1, 0));
  }

  e2 = sqrt(e2);

  if (nfield >= 3 && Bi != NULL) {
    const double *B0 = Bi, *B1 = Bi + V, *B2 = Bi + 2 * V;
    pgradB[0] = ((1. - r[2]) * (F(B1, 1, 0, 0) - F(B1, 0, 0, 0)) + r[2] * (F(B1, 1, 0, 1) - F(B1, 0, 0, 1))) * q[1];
    pgradB[0] += ((1. - r[1]) * (F(B2, 1, 0, 0) - F(B2, 0, 0, 0)) + r[1] * (F(B2, 1, 1, 0) - F(B2, 0, 1, 0))) * q[2];
    pgradB[0] += (1. - r[1]) * (1. - r[2]) * ((r[0] - 1.) * F(B0, -1, 0, 0) + (1. - 2. * r[0]) * F(B0, 0, 0, 0) + r[0] * F(B0, 1, 0, 0)) * q[0];
    pgradB[0] += r[1] * (1. - r[2]) * ((r[0] - 1.) * F(B0, -1, 1, 0) + (1. - 2. * r[0]) * F(B0, 0, 1, 0) + r[0] * F(B0, 1, 1, 0)) * q[0];
    pgradB[0] += (1. - r[1]) * r[2] * ((r[0] - 1.) * F(B0, -1, 0, 1) + (1. - 2. * r[0]) * F(B0, 0, 0, 1) + r[0] * F(B0, 1, 0, 1)) * q[0];
    pgradB[0] += r[1] * r[2] * ((r[0] - 1.) * F(B0, -1, 1, 1) + (1. - 2. * r[0]) * F(B0, 0, 1, 1) + r[0] * F(B0, 1, 1, 1)) * q[0];

    pgradB[1] = ((1. - r[0]) * (F(B2, 0, 1, 0) - F(B2, 0, 0, 0)) + r[0] * (F(B2, 1, 1, 0) - F(B2, 1, 0, 0))) * q[2];
    pgradB[1] += ((1. - r[2]) * (F(B0, 0, 1, 0) - F(B0, 0, 0, 0)) + r[2] * (F(B0, 0, 1, 1) - F(B0, 0, 0, 1))) * q[0];
    pgradB[1] += (1. - r[0]) * (1. - r[2]) * ((r[1] - 1.) * F(B1, 0, -1, 0) + (1. - 2. * r[1]) * F(B1, 0, 0, 0) + r[1] * F(B1, 0, 1, 0)) * q[1];
    pgradB[1] += r[0] * (1. - r[2]) * ((r[1] - 1.) * F(B1, 1, -1, 0) + (1. - 2. * r[1]) * F(B1, 1, 0, 0) + r[1] * F(B1, 1, 1, 0)) * q[1];
    pgradB[1] += (1. - r[0]) * r[2] * ((r[1] - 1.) * F(B1, 0, -1, 1) + (1. - 2. * r[1]) * F(B1, 0, 0, 1) + r[1] * F(B1, 0, 1, 1)) * q[1];
    pgradB[1] += r[0] * r[2] * ((r[1] - 1.) * F(B1, 1, -1, 1) + (1. - 2. * r[1]) * F(B1, 1, 0, 1) + r[1] * F(B1, 1, 1, 1)) * q[1];

    pgradB[2] = ((1. - r[1]) * (F(B0, 0, 0, 1) - F(B0, 0, 0, 0)) + r[1] * (F(B0, 0, 1, 1) - F(B0, 0, 1, 0))) * q[0];
    pgradB[2] += ((1. - r[0]) * (F(B1, 0, 0, 1) - F(B1, 0, 0, 0)) + r[0] * (F(B1, 1, 0, 1) - F(B1, 1, 0, 0))) * q[1];
    pgradB[2] += (1. - r[0]) * (1. - r[1]) * ((r[2] - 1.) * F(B2, 0, 0, -1) + (1. - 2. * r[2]) * F(B2, 0, 0, 0) + r[2] * F(B2, 0, 0, 1)) * q[2];
    pgradB[2] += r[0] * (1. - r[1]) * ((r[2] - 1.) * F(B2, 1, 0, -1) + (1. - 2. * r[2]) * F(B2, 1, 0, 0) + r[2] * F(B2, 1, 0, 1)) * q[2];
    pgradB[2] += (1. - r[0]) * r[1] * ((r[2] - 1.) * F(B2, 0, 1, -1) + (1. - 2. * r[2]) * F(B2, 0, 1, 0) + r[2] * F(B2, 0, 1, 1)) * q[2];
    pgradB[2] += r[0] * r[1] * ((r[2] - 1.) * F(B2, 1, 1, -1) + (1. - 2. * r[2]) * F(B2, 1, 1, 0) + r[2] * F(B2, 1, 1, 1)) * q[2];

    gradphi[0] += pgradB[0] / params[1] / e2;
    gradphi[1] += pgradB[1] / params[1] / e2;
    gradphi[2] += pgradB[2] / params[1] / e2;
  }

  v2 = 0.;
  for (int i = 0; i < 3; i++) {
    q[i] -= dtau * e2 * gradphi[i] / dx;
    v2 += q[i] * q[i];
  }
  return v2 / params[0] / params[0];
}

/* update_q_Newton, gevolution.hpp:709-776 */
static double update_q_newton_one(int N, gevo_part *pt, const double *r, int cx_, int cy_, int cz_,
                                  double dtau, const double *psi, const double *chi, int nfield,
                                  const double *params) {
  const double dx = 1.0 / (double)N;
  double g[3] = {0, 0, 0};
  g[0] = (1. - r[1]) * (1. - r[2]) * (F(psi, 1, 0, 0) - F(psi, 0, 0, 0));
  g[1] = (1. - r[0]) * (1. - r[2]) * (F(psi, 0, 1, 0) - F(psi, 0, 0, 0));
  g[2] = (1. - r[0]) * (1. - r[1]) * (F(psi, 0, 0, 1) - F(psi, 0, 0, 0));
  g[0] += r[1] * (1. - r[2]) * (F(psi, 1, 1, 0) - F(psi, 0, 1, 0));
  g[1] += r[0] * (1. - r[2]) * (F(psi, 1, 1, 0) - F(psi, 1, 0, 0));
  g[2] += r[0] * (1. - r[1]) * (F(psi, 1, 0, 1) - F(psi, 1, 0, 0));
  g[0] += (1. - r[1]) * r[2] * (F(psi, 1, 0, 1) - F(psi, 0, 0, 1));
  g[1] += (1. - r[0]) * r[2] * (F(psi, 0, 1, 1) - F(psi, 0, 0, 1));
  g[2] += (1. - r[0]) * r[1] * (F(psi, 0, 1, 1) - F(psi, 0, 1, 0));
  g[0] += r[1] * r[2] * (F(psi, 1, 1, 1) - F(psi, 0, 1, 1));
  g[1] += r[0] * r[2] * (F(psi, 1, 1, 1) - F(psi, 1, 0, 1));
  g[2] += r[0] * r[1] * (F(psi, 1, 1, 1) - F(psi, 1, 1, 0));
  if (nfield >= 2 && chi != NULL) {
    g[0] -= (1. - r[1]) * (1. - r[2]) * (F(chi, 1, 0, 0) - F(chi, 0, 0, 0));
    g[1] -= (1. - r[0]) * (1. - r[2]) * (F(chi, 0, 1, 0) - F(chi, 0, 0, 0));
    g[2] -= (1. - r[0]) * (1. - r[1]) * (F(chi, 0, 0, 1) - F(chi, 0, 0, 0));
    g[0] -= r[1] * (1. - r[2]) * (F(chi, 1, 1, 0) - F(chi, 0, 1, 0));
    g[1] -= r[0] * (1. - r[2]) * (F(chi, 1, 1, 0) - F(chi, 1, 0, 0));
    g[2] -= r[0] * (1. - r[1]) * (F(chi, 1, 0, 1) - F(chi, 1, 0, 0));
    g[0] -= (1. - r[1]) * r[2] * (F(chi, 1, 0, 1) - F(chi, 0, 0, 1));
    g[1] -= (1. - r[0]) * r[2] * (F(chi, 0, 1, 1) - F(chi, 0, 0, 1));
    g[2] -= (1. - r[0]) * r[1] * (F(chi, 0, 1, 1) - F(chi, 0, 1, 0));
    g[0] -= r[1] * r[2] * (F(chi, 1, 1, 1) - F(chi, 0, 1, 1));
    g[1] -= r[0] * r[2] * (F(chi, 1, 1, 1) - F(chi, 1, 0, 1));
    g[2] -= r[0] * r[1] * (F(chi, 1, 1, 1) - F(chi, 1, 1, 0));
  }
  double v2 = 0.;
  double *q = pt->vel;
  for (int i = 0; i < 3; i++) {
    q[i] -= dtau * params[0] * g[i] / dx;
    v2 += q[i] * q[i];
  }
  return v2 / params[0] / params[0];
}

/* update_pos, gevolution.hpp:810-871 */
static void update_pos_one(int N, gevo_part *pt, const double *r, int cx_, int cy_, int cz_, double dtau,
                           const double *phi_f, const double *chi_f, const double *Bi, int nfield,
                           const double *params) {
  const size_t V = (size_t)N * N * N;
  double v[3];
  const double *q = pt->vel;
  double v2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2];
  double e2 = v2 + params[0] * params[0];
  double phi = 0, chi = 0;
  if (nfield >= 1) {
    phi = F(phi_f, 0, 0, 0) * (1. - r[0]) * (1. - r[1]) * (1. - r[2]);
    phi += F(phi_f, 1, 0, 0) * r[0] * (1. - r[1]) * (1. - r[2]);
    phi += F(phi_f, 0, 1, 0) * (1. - r[0]) * r[1] * (1. - r[2]);
    phi += F(phi_f, 1, 1, 0) * r[0] * r[1] * (1. - r[2]);
    phi += F(phi_f, 0, 0, 1) * (1. - r[0]) * (1. - r[1]) * r[2];
    phi += F(phi_f, 1, 0, 1) * r[0] * (1. - r[1]) * r[2];
    phi += F(phi_f, 0, 1, 1) * (1. - r[0]) * r[1] * r[2];
    phi += F(phi_f, 1, 1, 1) * r[0] * r[1] * r[2];
  }
  if (nfield >= 2) {
    chi = F(chi_f, 0, 0, 0) * (1. - r[0]) * (1. - r[1]) * (1. - r[2]);
    chi += F(chi_f, 1, 0, 0) * r[0] * (1. - r[1]) * (1. - r[2]);
    chi += F(chi_f, 0, 1, 0) * (1. - r[0]) * r[1] * (1. - r[2]);
    chi += F(chi_f, 1, 1, 0) * r[0] * r[1] * (1. - r[2]);
    chi += F(chi_f, 0, 0, 1) * (1. - r[0]) * (1. - r[1]) * r[2];
    chi += F(chi_f, 1, 0, 1) * r[0] * (1. - r[1]) * r[2];
    chi += F(chi_f, 0, 1, 1) * (1. - r[0]) * r[1] * r[2];
    chi += F(chi_f, 1, 1, 1) * r[0] * r[1] * r[2];
  }
  v2 = (1. + (3. - v2 / e2) * phi - chi) / sqrt(e2);
  v[0] = q[0] * v2;
  v[1] = q[1] * v2;
  v[2] = q[2] * v2;
  if (nfield >= 3) {
    const double *B0 = Bi, *B1 = Bi + V, *B2 = Bi + 2 * V;
    double b[3];
    b[0] = F(B0, 0, 0, 0) * (1. - r[1]) * (1. - r[2]);
    b[1] = F(B1, 0, 0, 0) * (1. - r[0]) * (1. - r[2]);
    b[2] = F(B2, 0, 0, 0) * (1. - r[0]) * (1. - r[1]);
    b[1] += F(B1, 1, 0, 0) * r[0] * (1. - r[2]);
    b[2] += F(B2, 1, 0, 0) * r[0] * (1. - r[1]);
    b[0] += F(B0, 0, 1, 0) * r[1] * (1. - r[2]);
    b[2] += F(B2, 0, 1, 0) * (1. - r[0]) * r[1];
    b[0] += F(B0, 0, 0, 1) * (1. - r[1]) * r[2];
    b[1] += F(B1, 0, 0, 1) * (1. - r[0]) * r[2];
    b[1] += F(B1, 1, 0, 1) * r[0] * r[2];
    b[0] += F(B0, 0, 1, 1) * r[1] * r[2];
    b[2] += F(B2, 1, 1, 0) * r[0] * r[1];
    for (int l = 0; l < 3; l++) pt->pos[l] += dtau * (v[l] + b[l] / params[1]);
  } else {
    for (int l = 0; l < 3; l++) pt->pos[l] += dtau * v[l];
  }
}
#undef F

/* the callback arguments of Particles::updateVel / moveParticles: the linked
 * cell and ref_dist = pos/dx - cell */
static void cell_and_ref(int N, const gevo_part *pt, int *c, double *r) {
  const double dx = 1.0 / (double)N;
  for (int i = 0; i < 3; i++) {
    c[i] = gevo_cell_of(N, pt->pos[i]);
    r[i] = pt->pos[i] / dx - (double)c[i];
  }
}

double gevo_kick(int N, long np, gevo_part *p, int kind, double dtau, const double *phi,
                 const double *chi, const double *Bi, int nfield, double a, double a2N) {
  const double params[2] = {a, a2N};
  double vmax = 0.;
  /* particles are independent and the maximum does not depend on the order */
#pragma omp parallel for schedule(static) reduction(max : vmax)
  for (long j = 0; j < np; j++) {
    int c[3];
    double r[3];
    cell_and_ref(N, p + j, c, r);
    double v = (kind == 0)
                   ? update_q_one(N, p + j, r, c[0], c[1], c[2], dtau, phi, chi, Bi, nfield, params)
                   : update_q_newton_one(N, p + j, r, c[0], c[1], c[2], dtau, phi, chi, nfield, params);
    if (v > vmax) vmax = v;
  }
  return sqrt(vmax);
}

void gevo_drift(int N, long np, gevo_part *p, int kind, double dtau, const double *phi,
                const double *chi, const double *Bi, int nfield, double a, double a2N,
                long *cell_start) {
  const double params[2] = {a, a2N};
#pragma omp parallel for schedule(static)
  for (long j = 0; j < np; j++) {
    if (kind == 0) {
      int c[3];
      double r[3];
      cell_and_ref(N, p + j, c, r);
      update_pos_one(N, p + j, r, c[0], c[1], c[2], dtau, phi, chi, Bi, nfield, params);
    } else {
      /* update_pos_Newton, gevolution.hpp:900-903 */
      for (int l = 0; l < 3; l++) p[j].pos[l] += dtau * p[j].vel[l] / params[0];
    }
  }
#pragma omp parallel for schedule(static)
  for (long j = 0; j < np; j++)
    for (int l = 0; l < 3; l++) gevo_wrap(&p[j].pos[l]);
  gevo_sort(N, np, p, cell_start);
}

/* ===================================================================== */
/* background                                                            */
/* ===================================================================== */

/* Hconf, background.hpp:137-140, without ncdm and fluid terms */
double gevo_hconf(double a, double fourpiG, const gevo_cosmo *c) {
  return sqrt((2. * fourpiG / 3.) *
              (((c->Omega_cdm + c->Omega_b) / a) + (c->Omega_Lambda * a * a) + (c->Omega_rad / a / a)));
}

/* rungekutta4bg, background.hpp:167-177 */
void gevo_rk4bg(double *a_, double fourpiG, const gevo_cosmo *c, double dtau) {
  double a = *a_;
  double k1a, k2a, k3a, k4a;
  k1a = a * gevo_hconf(a, fourpiG, c);
  k2a = (a + k1a * dtau / 2.) * gevo_hconf(a + k1a * dtau / 2., fourpiG, c);
  k3a = (a + k2a * dtau / 2.) * gevo_hconf(a + k2a * dtau / 2., fourpiG, c);
  k4a = (a + k3a * dtau) * gevo_hconf(a + k3a * dtau, fourpiG, c);
  a += dtau * (k1a + 2. * k2a + 2. * k3a + k4a) / 6.;
  *a_ = a;
}

/* ===================================================================== */
/* simulation state and one cycle of the main loop                        */
/* ===================================================================== */

int gevo_sim_alloc(gevo_sim *s, int N, long np) {
  memset(s, 0, sizeof(*s));
  const size_t V = (size_t)N * N * N;
  const size_t K = (size_t)N * N * (N / 2 + 1) * 2;
  s->N = N;
  s->np = np;
  s->p = (gevo_part *)calloc((size_t)np, sizeof(gevo_part));
  s->cell_start = (long *)calloc(V + 1, sizeof(long));
  s->phi = (double *)calloc(V, sizeof(double));
  s->chi = (double *)calloc(V, sizeof(double));
  s->source = (double *)calloc(V, sizeof(double));
  s->Sij = (double *)calloc(6 * V, sizeof(double));
  s->Bi = (double *)calloc(3 * V, sizeof(double));
  s->scalarFT = (double *)calloc(K, sizeof(double));
  s->SijFT = (double *)calloc(6 * K, sizeof(double));
  s->BiFT = (double *)calloc(3 * K, sizeof(double));
  return (s->p && s->cell_start && s->phi && s->chi && s->source && s->Sij && s->Bi && s->scalarFT &&
          s->SijFT && s->BiFT)
             ? 0
             : -1;
}

void gevo_sim_free(gevo_sim *s) {
  free(s->p);
  free(s->cell_start);
  free(s->phi);
  free(s->chi);
  free(s->source);
  free(s->Sij);
  free(s->Bi);
  free(s->scalarFT);
  free(s->SijFT);
  free(s->BiFT);
  memset(s, 0, sizeof(*s));
}

/* dtau rule, main.cpp:292-295 and 869-872 */
double gevo_next_dtau(const gevo_sim *s) {
  const double dx = 1.0 / (double)s->N;
  const double H = gevo_hconf(s->a, s->fourpiG, &s->cosmo);
  if (s->Cf * dx < s->steplimit / H) return s->Cf * dx;
  return s->steplimit / H;
}

static double wall_s(void) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

/* main.cpp:372-598 for CDM only, GR: the stress-energy deposits and the phi, chi
 * and B solves.  Timed into t_phase as main.cpp's BENCHMARK build times them
 * (projection_time 372-453, gravity_solver_time 454-602 with fft_time and
 * fft_count for the transforms). */
int gevo_sim_step_fields(gevo_sim *s) {
  const int N = s->N;
  const size_t V = (size_t)N * N * N;
  const size_t K = (size_t)N * N * (N / 2 + 1) * 2;
  const double dx = 1.0 / (double)N;
  const gevo_cosmo *cm = &s->cosmo;
  const double fourpiG = s->fourpiG;
  const double a = s->a;
  double t0 = wall_s(), t1;

  memset(s->source, 0, V * sizeof(double));
  gevo_deposit_T00(N, s->np, s->p, s->cell_start, s->mass, a, s->phi, 1., s->source);
  if (s->vector_elliptic) {
    memset(s->Bi, 0, 3 * V * sizeof(double));
    gevo_deposit_T0i(N, s->np, s->p, s->cell_start, s->mass, s->phi, 1., s->Bi);
  }
  memset(s->Sij, 0, 6 * V * sizeof(double));
  gevo_deposit_Tij(N, s->np, s->p, s->cell_start, s->mass, a, s->phi, 1., s->Sij);
  t1 = wall_s();
  s->t_phase[0] += t1 - t0;
  t0 = t1;

  double T00hom = 0.;
  for (size_t i = 0; i < V; i++) T00hom += s->source[i];
  T00hom /= (double)V;
  s->T00hom = T00hom;

  double tf = 0.;
#define GEVO_FFT(call)      \
  do {                      \
    const double f0 = wall_s(); \
    call;                   \
    tf += wall_s() - f0;    \
  } while (0)
  if (s->dtau_old > 0.) {
    const double H = gevo_hconf(a, fourpiG, cm);
    gevo_prepare_source_scalar(N, s->phi, s->chi, s->source, cm->Omega_cdm + cm->Omega_b, s->source,
                               3. * H * dx * dx / s->dtau_old, fourpiG * dx * dx / a,
                               3. * H * H * dx * dx);
    GEVO_FFT(gevo_fft_r2c(N, s->source, s->scalarFT));
    gevo_poisson(N, s->scalarFT, s->scalarFT, 1. / (dx * dx), 3. * H / s->dtau_old);
    GEVO_FFT(gevo_fft_c2r(N, s->scalarFT, s->phi));
    s->fft_count += 2;
  }
  s->phik0 = s->scalarFT[0];

  gevo_prepare_source_tensor(N, s->phi, s->Sij, s->Sij, 2. * fourpiG * dx * dx / a);
  GEVO_FFT(for (int c = 0; c < 6; c++) gevo_fft_r2c(N, s->Sij + c * V, s->SijFT + c * K));
  gevo_project_scalar(N, s->SijFT, s->scalarFT, 0);
  GEVO_FFT(gevo_fft_c2r(N, s->scalarFT, s->chi));
  s->fft_count += 7;

  if (s->vector_elliptic) {
    GEVO_FFT(for (int c = 0; c < 3; c++) gevo_fft_r2c(N, s->Bi + c * V, s->BiFT + c * K));
    gevo_project_vector(N, s->BiFT, s->BiFT, fourpiG * dx * dx, 0.);
    s->fft_count += 1;
  } else {
    gevo_evolve_vector(N, s->SijFT, s->BiFT, a * a * s->dtau_old);
  }
  GEVO_FFT(for (int c = 0; c < 3; c++) gevo_fft_c2r(N, s->BiFT + c * K, s->Bi + c * V));
  s->fft_count += 3;
#undef GEVO_FFT
  t1 = wall_s();
  s->t_phase[1] += t1 - t0;
  s->t_phase[2] += tf;
  return 0;
}

/* main.cpp:743-872: the kick (update_q_time), the background half step, the
 * drift with the relink (moveParts_time), the second half step and the next dtau */
int gevo_sim_step_particles(gevo_sim *s) {
  const int N = s->N;
  const gevo_cosmo *cm = &s->cosmo;
  const double fourpiG = s->fourpiG;
  double a = s->a;
  const double dtau = s->dtau;
  double t0 = wall_s(), t1;
  double maxvel = gevo_kick(N, s->np, s->p, 0, (dtau + s->dtau_old) / 2., s->phi, s->chi, s->Bi,
                            (1. / a < s->z_relax + 1. ? 3 : 2), a, a * a * N);
  t1 = wall_s();
  s->t_phase[3] += t1 - t0;
  gevo_rk4bg(&a, fourpiG, cm, 0.5 * dtau);
  t0 = wall_s();
  gevo_drift(N, s->np, s->p, 0, dtau, s->phi, s->chi, s->Bi, (1. / a < s->z_relax + 1. ? 3 : 0), a,
             a * a * N, s->cell_start);
  s->t_phase[4] += wall_s() - t0;
  gevo_rk4bg(&a, fourpiG, cm, 0.5 * dtau);
  maxvel /= sqrt(maxvel * maxvel + 1.0);
  s->maxvel = maxvel;
  s->a = a;
  s->tau += dtau;
  s->dtau_old = dtau;
  s->dtau = gevo_next_dtau(s);
  s->cycle++;
  return 0;
}

/* main.cpp:372-879 for CDM only, GR, no outputs */
int gevo_sim_step(gevo_sim *s) {
  gevo_sim_step_fields(s);
  return gevo_sim_step_particles(s);
}
