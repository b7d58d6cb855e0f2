// gev_spectrum.cu -- binned power and cross spectra of device spectra:
// extractCrossSpectrum / extractPowerSpectrum (tools.hpp:53-240), without copying
// the half spectrum to the host.
//
// Per mode (kx, ky, kz) of the half spectrum, as the reference: weight 1 on the
// kx = 0 and kx = N/2 planes and 2 elsewhere, the k = 0 mode skipped; k2 from the
// grid or the linear k table; s = (sinc_x sinc_y sinc_z)^2, the CIC window being
// deconvolved; p = Re sum_c f1_c conj(f2_c) (a symmetric tensor: twice the
// off-diagonal terms plus the diagonal ones); bin = floor(numbins sqrt(k2/k2max)).
// Per bin the sums of w sqrt(k2), w k2, w p k2^(3/2) / s, w p^2 k2^3 / s^2 and w;
// the host then forms averages and scatters exactly as the reference does.
//
// The sums are exact integer sums, so the result does not depend on the order of
// the modes: pass 1 finds each bin's largest |contribution| per quantity (integer
// max of the FP64 bit pattern), which with the bin's occupation fixes a
// power-of-two scale; pass 2 adds every contribution times its scale, rounded to
// an int64.  A thread walks a run of consecutive kx, along which the bin never
// decreases, and issues one atomic per bin it leaves.  Results are
// bit-reproducible and agree with the reference's sequential FP64 sums to
// rounding (about 1e-15 relative).
#include <cmath>
#include <cstring>
#include <vector>

#include "gev_internal.cuh"

namespace {

constexpr int PK_SEG = 32;      // kx values per thread run
constexpr int PK_MAXBINS = 65536;

struct PkArgs {
  const double *typek2, *sinc;
  double k2max;
  int N, NH, numbins;
  long NK;           // complex elements per component
  int ncomp;         // components summed (ignored when sym)
  int sym;           // symmetric tensor 00 01 02 11 12 22
  int c1, c2;        // single components of f1, f2 (>= 0), else -1
};

// round(c * 2^k) for |c| 2^k < 2^62, with integer instructions only
__device__ __forceinline__ long long fixed_of_double(double c, int k) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(c);
  const int e = (int)((b >> 52) & 0x7ff);
  if (e == 0) return 0;  // zero or subnormal: far below every scale used here
  const long long m = (long long)((b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull);
  const int sh = e - 1075 + k;
  long long q;
  if (sh >= 0)
    q = sh < 11 ? m << sh : 0x3FFFFFFFFFFFFFFFll;  // the bound keeps sh <= 9
  else if (sh >= -53)
    q = (m + (1ll << (-sh - 1))) >> (-sh);
  else
    q = 0;
  return (b >> 63) ? -q : q;
}

template <typename T>
__device__ __forceinline__ double mode_power(const typename CT<T>::C *f1, const typename CT<T>::C *f2,
                                             const PkArgs &a, long id) {
  double p = 0.;
  if (a.c1 >= 0) {
    const auto u = f1[a.c1 * a.NK + id], v = f2[a.c2 * a.NK + id];
    return (double)u.x * (double)v.x + (double)u.y * (double)v.y;
  }
  if (a.sym) {
    const int off[3] = {1, 2, 4}, dg[3] = {0, 3, 5};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const auto u = f1[off[c] * a.NK + id], v = f2[off[c] * a.NK + id];
      p += (double)u.x * (double)v.x + (double)u.y * (double)v.y;
    }
    p *= 2.;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const auto u = f1[dg[c] * a.NK + id], v = f2[dg[c] * a.NK + id];
      p += (double)u.x * (double)v.x + (double)u.y * (double)v.y;
    }
    return p;
  }
  for (int c = 0; c < a.ncomp; ++c) {
    const auto u = f1[c * a.NK + id], v = f2[c * a.NK + id];
    p += (double)u.x * (double)v.x + (double)u.y * (double)v.y;
  }
  return p;
}

// PASS 0: per-bin max |contribution| (4 quantities) and occupation.
// PASS 1: per-bin fixed-point sums with the scales kshift[q * numbins + bin].
template <typename T, int PASS>
__global__ void __launch_bounds__(256) k_spectrum(const typename CT<T>::C *__restrict__ f1,
                                                  const typename CT<T>::C *__restrict__ f2, PkArgs a,
                                                  unsigned long long *maxbits, int *occ, unsigned long long *sums,
                                                  const int *__restrict__ kshift) {
  const int N = a.N, NH = a.NH, nb = a.numbins;
  const int nseg = (NH + PK_SEG - 1) / PK_SEG;
  const long items = (long)N * N * nseg;
  for (long it = blockIdx.x * (long)blockDim.x + threadIdx.x; it < items; it += (long)gridDim.x * blockDim.x) {
    const long row = it / nseg;
    const int seg = (int)(it - row * nseg);
    const int ky = (int)(row % N), kz = (int)(row / N);
    const int kx0 = seg * PK_SEG, kx1 = min(kx0 + PK_SEG, NH);
    const double ty = a.typek2[ky], tz = a.typek2[kz], sy = a.sinc[ky], sz = a.sinc[kz];
    int cur = -1, wsum = 0;
    double m[4] = {0., 0., 0., 0.};
    long long acc[4] = {0, 0, 0, 0};
    int ks[4] = {0, 0, 0, 0};
    for (int kx = kx0; kx < kx1; ++kx) {
      if (kx == 0 && ky == 0 && kz == 0) continue;
      const int w = (kx == 0 || (kx == N / 2 && (N % 2) == 0)) ? 1 : 2;
      const double k2 = (a.typek2[kx] + ty) + tz;  // the reference's order: the bin edges match it exactly
      double s = (a.sinc[kx] * sy) * sz;
      s *= s;
      const int b = (int)floor((double)nb * sqrt(k2 / a.k2max));
      if (b >= nb) continue;
      const long id = kx + (long)NH * row;
      const double p = mode_power<T>(f1, f2, a, id);
      const double sk = sqrt(k2);
      const double c[4] = {w * sk, w * k2, w * p * k2 * sk / s, w * p * p * k2 * k2 * k2 / s / s};
      if (b != cur) {
        if (cur >= 0) {
          if (PASS == 0) {
#pragma unroll
            for (int q = 0; q < 4; ++q) atomicMax(&maxbits[q * nb + cur], (unsigned long long)__double_as_longlong(m[q]));
            atomicAdd(&occ[cur], wsum);
          } else {
#pragma unroll
            for (int q = 0; q < 4; ++q)
              if (acc[q] != 0) atomicAdd(&sums[q * nb + cur], (unsigned long long)acc[q]);
          }
        }
        cur = b;
        wsum = 0;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          m[q] = 0.;
          acc[q] = 0;
          if (PASS == 1) ks[q] = kshift[q * nb + b];
        }
      }
      if (PASS == 0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) m[q] = fmax(m[q], fabs(c[q]));
        wsum += w;
      } else {
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[q] += fixed_of_double(c[q], ks[q]);
      }
    }
    if (cur >= 0) {
      if (PASS == 0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) atomicMax(&maxbits[q * nb + cur], (unsigned long long)__double_as_longlong(m[q]));
        atomicAdd(&occ[cur], wsum);
      } else {
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (acc[q] != 0) atomicAdd(&sums[q * nb + cur], (unsigned long long)acc[q]);
      }
    }
  }
}

bool spec_ok(gev_ctx *ctx, const gev_field *f) { return f && f->ctx == ctx && f->kind == GEV_FIELD_SPECTRUM; }

}  // namespace

extern "C" int gev_cross_spectrum(gev_ctx *ctx, const gev_field *f1, const gev_field *f2, double *kbin, double *power,
                                  double *kscatter, double *pscatter, int *occupation, int numbins, int deconvolve,
                                  int ktype, int symmetric, int comp1, int comp2) {
  if (!ctx || !spec_ok(ctx, f1) || !spec_ok(ctx, f2) || !kbin || !power || !kscatter || !pscatter || !occupation ||
      numbins < 1 || numbins > PK_MAXBINS || (ktype != 0 && ktype != 1))
    return gev_fail(ctx, GEV_EINVAL, "cross_spectrum: two spectra of the context, host arrays, 1 <= numbins <= 65536, ktype 0/1");
  const bool single = comp1 >= 0 && comp2 >= 0 && comp1 < f1->ncomp && comp2 < f2->ncomp;
  if (!single && f1->ncomp != f2->ncomp)
    return gev_fail(ctx, GEV_EINVAL, "cross_spectrum: component counts differ");
  if (!single && symmetric && f1->ncomp != 6)
    return gev_fail(ctx, GEV_EINVAL, "cross_spectrum: a symmetric tensor has 6 components");
  const int N = ctx->N, NH = N / 2 + 1, nb = numbins;
  // k and window tables, computed as tools.hpp:66-106 does
  std::vector<double> typek2(N), sinc(N);
  if (ktype == 0) {
    for (int i = 0; i < N; i++) {
      typek2[i] = 2. * (double)N * sin(M_PI * (double)i / (double)N);
      typek2[i] *= typek2[i];
    }
  } else {
    int i;
    for (i = 0; i <= N / 2; i++) {
      typek2[i] = 2. * M_PI * (double)i;
      typek2[i] *= typek2[i];
    }
    for (; i < N; i++) {
      typek2[i] = 2. * M_PI * (double)(N - i);
      typek2[i] *= typek2[i];
    }
  }
  {
    int i;
    sinc[0] = 1.;
    for (i = 1; i <= N / 2; i++)
      sinc[i] = deconvolve ? sin(M_PI * (float)i / (float)N) * (float)N / (M_PI * (float)i) : 1.;
    for (; i < N; i++) sinc[i] = sinc[N - i];
  }
  // device scratch (8-byte words): tables 2N, max bits 4 nb, sums 4 nb, then
  // occupation nb ints and scales 4 nb ints
  const size_t off_tab = 0, off_max = 2 * (size_t)N, off_sum = off_max + 4 * (size_t)nb,
               off_int = off_sum + 4 * (size_t)nb, words = off_int + (5 * (size_t)nb + 1) / 2;
  int rc = ctx_ensure_red(ctx, words);
  if (rc) return rc;
  double *d = ctx->d_red;
  GEV_CHECK_CUDA(ctx, cudaMemcpyAsync(d + off_tab, typek2.data(), N * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  GEV_CHECK_CUDA(ctx, cudaMemcpyAsync(d + off_tab + N, sinc.data(), N * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  GEV_CHECK_CUDA(ctx, cudaMemsetAsync(d + off_max, 0, (words - off_max) * sizeof(double), ctx->stream));
  PkArgs a;
  a.typek2 = d + off_tab;
  a.sinc = d + off_tab + N;
  a.k2max = 3. * typek2[N / 2];
  a.N = N;
  a.NH = NH;
  a.numbins = nb;
  a.NK = (long)N * N * NH;
  a.ncomp = f1->ncomp;
  a.sym = (!single && symmetric) ? 1 : 0;
  a.c1 = single ? comp1 : -1;
  a.c2 = single ? comp2 : -1;
  unsigned long long *maxbits = (unsigned long long *)(d + off_max);
  unsigned long long *sums = (unsigned long long *)(d + off_sum);
  int *occ = (int *)(d + off_int);
  int *kshift = occ + nb;
  const long items = (long)N * N * ((NH + PK_SEG - 1) / PK_SEG);
  const int blocks = grid_for(ctx, (size_t)items, 256, 8);
  if (ctx->prec == GEV_PREC_FP64)
    k_spectrum<double, 0><<<blocks, 256, 0, ctx->stream>>>((const double2 *)f1->d, (const double2 *)f2->d, a, maxbits,
                                                           occ, sums, kshift);
  else
    k_spectrum<float, 0><<<blocks, 256, 0, ctx->stream>>>((const float2 *)f1->d, (const float2 *)f2->d, a, maxbits, occ,
                                                          sums, kshift);
  GEV_LAUNCH_CHECK(ctx);
  std::vector<unsigned long long> mx(4 * (size_t)nb), sm(4 * (size_t)nb);
  std::vector<int> oc(nb), ksh(4 * (size_t)nb);
  GEV_CHECK_CUDA(ctx, cudaMemcpyAsync(mx.data(), maxbits, mx.size() * 8, cudaMemcpyDeviceToHost, ctx->stream));
  GEV_CHECK_CUDA(ctx, cudaMemcpyAsync(oc.data(), occ, nb * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  GEV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  for (int q = 0; q < 4; ++q)
    for (int b = 0; b < nb; ++b) {
      double m;
      memcpy(&m, &mx[q * nb + b], 8);
      const double bound = m * (double)(oc[b] > 0 ? oc[b] : 1);
      int e2 = 0;
      if (bound > 0.) frexp(bound, &e2);  // bound < 2^e2
      ksh[q * nb + b] = bound > 0. ? 62 - e2 : 0;
    }
  GEV_CHECK_CUDA(ctx, cudaMemcpyAsync(kshift, ksh.data(), ksh.size() * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  if (ctx->prec == GEV_PREC_FP64)
    k_spectrum<double, 1><<<blocks, 256, 0, ctx->stream>>>((const double2 *)f1->d, (const double2 *)f2->d, a, maxbits,
                                                           occ, sums, kshift);
  else
    k_spectrum<float, 1><<<blocks, 256, 0, ctx->stream>>>((const float2 *)f1->d, (const float2 *)f2->d, a, maxbits, occ,
                                                          sums, kshift);
  GEV_LAUNCH_CHECK(ctx);
  GEV_CHECK_CUDA(ctx, cudaMemcpyAsync(sm.data(), sums, sm.size() * 8, cudaMemcpyDeviceToHost, ctx->stream));
  GEV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  // averages and scatters as tools.hpp:185-197
  for (int b = 0; b < nb; ++b) {
    kbin[b] = ldexp((double)(long long)sm[0 * nb + b], -ksh[0 * nb + b]);
    kscatter[b] = ldexp((double)(long long)sm[1 * nb + b], -ksh[1 * nb + b]);
    power[b] = ldexp((double)(long long)sm[2 * nb + b], -ksh[2 * nb + b]);
    pscatter[b] = ldexp((double)(long long)sm[3 * nb + b], -ksh[3 * nb + b]);
    occupation[b] = oc[b];
    if (occupation[b] > 0) {
      kscatter[b] = sqrt(kscatter[b] * occupation[b] - kbin[b] * kbin[b]) / occupation[b];
      if (!std::isfinite(kscatter[b])) kscatter[b] = 0.;
      kbin[b] = kbin[b] / occupation[b];
      power[b] /= occupation[b];
      pscatter[b] = sqrt(pscatter[b] / occupation[b] - power[b] * power[b]);
      if (!std::isfinite(pscatter[b])) pscatter[b] = 0.;
    }
  }
  return GEV_OK;
}
