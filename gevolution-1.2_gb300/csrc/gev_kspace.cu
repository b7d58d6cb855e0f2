// gev_kspace.cu -- the k-space operators of gevolution's field solver,
// one thread per half-spectrum point (kx fastest, coalesced).
//
// Each kernel evaluates the same expression as the reference function it
// replaces (gevolution.hpp:211-535) with the same gridk2 / kshift tables
// (built on the host exactly as gevolution.hpp:222-227 builds them); divisions
// by a per-k denominator are done once as a reciprocal.  The k = 0 point gets
// the reference's special value.  Streaming: HBM-bound in the FP32 form,
// FP64-pipe-bound in the FP64 form.
#include "gev_batch.cuh"

namespace {

template <typename T>
struct KIdx {
  int kx, ky, kz;
  size_t id;
};

// grid sizes and their invariant divisors (N^2 (N/2+1) < 2^32)
struct KDim {
  int N, NH;
  Div32 dNH, dN;
};
inline KDim make_kdim(int N) {
  KDim d;
  d.N = N;
  d.NH = N / 2 + 1;
  d.dNH = make_div32((unsigned)d.NH);
  d.dN = make_div32((unsigned)N);
  return d;
}

template <typename T>
__device__ __forceinline__ bool kidx(size_t id, const KDim &kd, KIdx<T> &k) {
  k.id = id;
  const unsigned i = (unsigned)id, r = div32(i, kd.dNH), q = div32(r, kd.dN);
  k.kx = (int)(i - r * (unsigned)kd.NH);
  k.ky = (int)(r - q * (unsigned)kd.N);
  k.kz = (int)q;
  return true;
}

// solveModifiedPoissonFT, gevolution.hpp:501-535; coeff already divided by -N^3
template <typename T>
__device__ __forceinline__ void k_poisson_body(const typename CT<T>::C *src, typename CT<T>::C *pot,
                                               const T *__restrict__ gk2, T coeff, T modif, KDim kd, size_t n) {
  const int N = kd.N, NH = kd.NH;
  typedef typename CT<T>::C C;
  for (size_t id = blockIdx.x * (size_t)blockDim.x + threadIdx.x; id < n; id += (size_t)gridDim.x * blockDim.x) {
    KIdx<T> k;
    kidx<T>(id, kd, k);
    const C s = src[id];
    C out;
    if (id == 0) {
      out = (modif == (T)0) ? cmk<C>(0, 0) : cscale(coeff / modif, s);
    } else {
      const T f = coeff / (gk2[k.kx] + gk2[k.ky] + gk2[k.kz] + modif);
      out = cscale(f, s);
    }
    pot[id] = out;
  }
}
template <typename T>
__global__ void k_poisson(const typename CT<T>::C *src, typename CT<T>::C *pot, const T *__restrict__ gk2, T coeff,
                          T modif, KDim kd, size_t n) {
  k_poisson_body<T>(src, pot, gk2, coeff, modif, kd, n);
}

// projectFTscalar, gevolution.hpp:211-265: chi at one k != 0
template <typename T, typename C>
__device__ __forceinline__ C chi_at(C S00, C S01, C S02, C S11, C S12, C S22, T g0, T g1, T g2, C k0, C k1, C k2,
                                    int N) {
  C t = cscale(g1 + g2 - (T)2 * g0, S00);
  t = cadd(t, cscale(g0 + g2 - (T)2 * g1, S11));
  t = cadd(t, cscale(g0 + g1 - (T)2 * g2, S22));
  t = csub(t, cmul(cscale((T)6, cmul(k0, k1)), S01));
  t = csub(t, cmul(cscale((T)6, cmul(k0, k2)), S02));
  t = csub(t, cmul(cscale((T)6, cmul(k1, k2)), S12));
  const T kk = g0 + g1 + g2;
  return cscale((T)1 / ((T)2 * kk * kk * (T)N), t);
}
// evolveFTvector, gevolution.hpp:284-330: the increments of B_0, B_1, B_2 at one k != 0
template <typename T, typename C>
__device__ __forceinline__ void evolve_at(C S00, C S01, C S02, C S11, C S12, C S22, T g0, T g1, T g2, C k0, C k1,
                                          C k2, T a2dtau, C &d0, C &d1, C &d2) {
  T k4 = g0 + g1 + g2;
  k4 *= k4;
  const T pre = (T)-2 * a2dtau / k4;  // multiplies by i * pre
  C x, u;
  x = csub(csub(csub(cscale(g1 + g2, S00), cscale(g1, S11)), cscale(g2, S22)), cmul(cscale((T)2, cmul(k1, k2)), S12));
  u = cadd(cmul(cconj(k0), x), cscale(g1 + g2 - g0, cadd(cmul(k1, S01), cmul(k2, S02))));
  d0 = cmk<C>(-pre * u.y, pre * u.x);
  x = csub(csub(csub(cscale(g0 + g2, S11), cscale(g0, S00)), cscale(g2, S22)), cmul(cscale((T)2, cmul(k0, k2)), S02));
  u = cadd(cmul(cconj(k1), x), cscale(g0 + g2 - g1, cadd(cmul(k0, S01), cmul(k2, S12))));
  d1 = cmk<C>(-pre * u.y, pre * u.x);
  x = csub(csub(csub(cscale(g0 + g1, S22), cscale(g0, S00)), cscale(g1, S11)), cmul(cscale((T)2, cmul(k0, k1)), S01));
  u = cadd(cmul(cconj(k2), x), cscale(g0 + g1 - g2, cadd(cmul(k0, S02), cmul(k1, S12))));
  d2 = cmk<C>(-pre * u.y, pre * u.x);
}

// projectFTscalar, gevolution.hpp:211-265
template <typename T>
__global__ void k_project_scalar(const typename CT<T>::C *__restrict__ S, typename CT<T>::C *chi,
                                 const T *__restrict__ gk2, const typename CT<T>::C *__restrict__ ks, int add, KDim kd,
                                 size_t n) {
  const int N = kd.N, NH = kd.NH;
  typedef typename CT<T>::C C;
  for (size_t id = blockIdx.x * (size_t)blockDim.x + threadIdx.x; id < n; id += (size_t)gridDim.x * blockDim.x) {
    if (id == 0) {
      chi[0] = cmk<C>(0, 0);
      continue;
    }
    KIdx<T> k;
    kidx<T>(id, kd, k);
    const T g0 = gk2[k.kx], g1 = gk2[k.ky], g2 = gk2[k.kz];
    const C k0 = ks[k.kx], k1 = ks[k.ky], k2 = ks[k.kz];
    const C S00 = S[id], S01 = S[n + id], S02 = S[2 * n + id], S11 = S[3 * n + id], S12 = S[4 * n + id],
            S22 = S[5 * n + id];
    const C t = chi_at<T>(S00, S01, S02, S11, S12, S22, g0, g1, g2, k0, k1, k2, N);
    chi[id] = add ? cadd(chi[id], t) : t;
  }
}

// evolveFTvector, gevolution.hpp:284-330 (B += ...)
template <typename T>
__global__ void k_evolve_vector(const typename CT<T>::C *__restrict__ S, typename CT<T>::C *B,
                                const T *__restrict__ gk2, const typename CT<T>::C *__restrict__ ks, T a2dtau, KDim kd,
                                size_t n) {
  const int N = kd.N, NH = kd.NH;
  typedef typename CT<T>::C C;
  for (size_t id = blockIdx.x * (size_t)blockDim.x + threadIdx.x; id < n; id += (size_t)gridDim.x * blockDim.x) {
    if (id == 0) {
      B[0] = B[n] = B[2 * n] = cmk<C>(0, 0);
      continue;
    }
    KIdx<T> k;
    kidx<T>(id, kd, k);
    const T g0 = gk2[k.kx], g1 = gk2[k.ky], g2 = gk2[k.kz];
    const C k0 = ks[k.kx], k1 = ks[k.ky], k2 = ks[k.kz];
    const C S00 = S[id], S01 = S[n + id], S02 = S[2 * n + id], S11 = S[3 * n + id], S12 = S[4 * n + id],
            S22 = S[5 * n + id];
    C d0, d1, d2;
    evolve_at<T>(S00, S01, S02, S11, S12, S22, g0, g1, g2, k0, k1, k2, a2dtau, d0, d1, d2);
    B[id] = cadd(B[id], d0);
    B[n + id] = cadd(B[n + id], d1);
    B[2 * n + id] = cadd(B[2 * n + id], d2);
  }
}

// projectFTscalar (add = 0) and evolveFTvector in one pass: the six SijFT components
// read once for both, the same arithmetic as the two kernels
template <typename T>
__device__ __forceinline__ void k_project_evolve_body(const typename CT<T>::C *__restrict__ S, typename CT<T>::C *chi,
                                                      typename CT<T>::C *B, const T *__restrict__ gk2,
                                                      const typename CT<T>::C *__restrict__ ks, T a2dtau, KDim kd,
                                                      size_t n) {
  const int N = kd.N;
  typedef typename CT<T>::C C;
  for (size_t id = blockIdx.x * (size_t)blockDim.x + threadIdx.x; id < n; id += (size_t)gridDim.x * blockDim.x) {
    if (id == 0) {
      chi[0] = cmk<C>(0, 0);
      B[0] = B[n] = B[2 * n] = cmk<C>(0, 0);
      continue;
    }
    KIdx<T> k;
    kidx<T>(id, kd, k);
    const T g0 = gk2[k.kx], g1 = gk2[k.ky], g2 = gk2[k.kz];
    const C k0 = ks[k.kx], k1 = ks[k.ky], k2 = ks[k.kz];
    const C S00 = S[id], S01 = S[n + id], S02 = S[2 * n + id], S11 = S[3 * n + id], S12 = S[4 * n + id],
            S22 = S[5 * n + id];
    chi[id] = chi_at<T>(S00, S01, S02, S11, S12, S22, g0, g1, g2, k0, k1, k2, N);
    C d0, d1, d2;
    evolve_at<T>(S00, S01, S02, S11, S12, S22, g0, g1, g2, k0, k1, k2, a2dtau, d0, d1, d2);
    B[id] = cadd(B[id], d0);
    B[n + id] = cadd(B[n + id], d1);
    B[2 * n + id] = cadd(B[2 * n + id], d2);
  }
}
template <typename T>
__global__ void k_project_evolve(const typename CT<T>::C *__restrict__ S, typename CT<T>::C *chi,
                                 typename CT<T>::C *B, const T *__restrict__ gk2,
                                 const typename CT<T>::C *__restrict__ ks, T a2dtau, KDim kd, size_t n) {
  k_project_evolve_body<T>(S, chi, B, gk2, ks, a2dtau, kd, n);
}

// projectFTvector, gevolution.hpp:350-392 (S may equal B)
template <typename T>
__global__ void k_project_vector(const typename CT<T>::C *S, typename CT<T>::C *B, const T *__restrict__ gk2,
                                 const typename CT<T>::C *__restrict__ ks, T coeff, T modif, KDim kd, size_t n) {
  const int N = kd.N, NH = kd.NH;
  typedef typename CT<T>::C C;
  for (size_t id = blockIdx.x * (size_t)blockDim.x + threadIdx.x; id < n; id += (size_t)gridDim.x * blockDim.x) {
    if (id == 0) {
      B[0] = B[n] = B[2 * n] = cmk<C>(0, 0);
      continue;
    }
    KIdx<T> k;
    kidx<T>(id, kd, k);
    const T g0 = gk2[k.kx], g1 = gk2[k.ky], g2 = gk2[k.kz];
    const C k0 = ks[k.kx], k1 = ks[k.ky], k2 = ks[k.kz];
    const C S0 = S[id], S1 = S[n + id], S2 = S[2 * n + id];
    const T kk = g0 + g1 + g2;
    const C tmp = cscale((T)1 / kk, cadd(cadd(cmul(k0, S0), cmul(k1, S1)), cmul(k2, S2)));
    const T f = (T)4 * coeff / (kk + modif);
    B[id] = cscale(f, csub(S0, cmul(cconj(k0), tmp)));
    B[n + id] = cscale(f, csub(S1, cmul(cconj(k1), tmp)));
    B[2 * n + id] = cscale(f, csub(S2, cmul(cconj(k2), tmp)));
  }
}

// projectFTtensor, gevolution.hpp:411-482 (S may equal h)
template <typename T>
__global__ void k_project_tensor(const typename CT<T>::C *S, typename CT<T>::C *h, const T *__restrict__ gk2,
                                 const typename CT<T>::C *__restrict__ ks, KDim kd, size_t n) {
  const int N = kd.N, NH = kd.NH;
  typedef typename CT<T>::C C;
  for (size_t id = blockIdx.x * (size_t)blockDim.x + threadIdx.x; id < n; id += (size_t)gridDim.x * blockDim.x) {
    if (id == 0) {
      for (int c = 0; c < 6; c++) h[c * n] = cmk<C>(0, 0);
      continue;
    }
    KIdx<T> k;
    kidx<T>(id, kd, k);
    const T g0 = gk2[k.kx], g1 = gk2[k.ky], g2 = gk2[k.kz];
    const C k0 = ks[k.kx], k1 = ks[k.ky], k2 = ks[k.kz];
    const C c0 = cconj(k0), c1 = cconj(k1), c2 = cconj(k2);
    const C Sxx = S[id], Sxy = S[n + id], Sxz = S[2 * n + id], Syy = S[3 * n + id], Syz = S[4 * n + id],
            Szz = S[5 * n + id];
    const T kk = g0 + g1 + g2;
    const T r6 = (T)1 / (kk * kk * kk * (T)N);
    const T two = (T)2;
    C t, h00, h01, h02, h11, h12, h22;
    t = cscale(g0 - kk, cadd(cscale(g0 - kk, Sxx), cmul(cscale(two, k0), cadd(cmul(k1, Sxy), cmul(k2, Sxz)))));
    t = cadd(t, cscale((g0 + kk) * (g1 + kk) - two * kk * kk, Syy));
    t = cadd(t, cscale((g0 + kk) * (g2 + kk) - two * kk * kk, Szz));
    t = cadd(t, cmul(cscale(two * (g0 + kk), cmul(k1, k2)), Syz));
    h00 = cscale(r6, t);
    t = cscale(two * (g0 - kk) * (g1 - kk), Sxy);
    t = cadd(t, cmul(cscale(g2 + kk, cmul(c0, c1)), Szz));
    t = cadd(t, cmul(cscale(g0 - kk, c1), cadd(cmul(c0, Sxx), cmul(cscale(two, k2), Sxz))));
    t = cadd(t, cmul(cscale(g1 - kk, c0), cadd(cmul(c1, Syy), cmul(cscale(two, k2), Syz))));
    h01 = cscale(r6, t);
    t = cscale(two * (g0 - kk) * (g2 - kk), Sxz);
    t = cadd(t, cmul(cscale(g1 + kk, cmul(c0, c2)), Syy));
    t = cadd(t, cmul(cscale(g0 - kk, c2), cadd(cmul(c0, Sxx), cmul(cscale(two, k1), Sxy))));
    t = cadd(t, cmul(cscale(g2 - kk, c0), cadd(cmul(c2, Szz), cmul(cscale(two, k1), Syz))));
    h02 = cscale(r6, t);
    t = cscale(g1 - kk, cadd(cscale(g1 - kk, Syy), cmul(cscale(two, k1), cadd(cmul(k0, Sxy), cmul(k2, Syz)))));
    t = cadd(t, cscale((g1 + kk) * (g0 + kk) - two * kk * kk, Sxx));
    t = cadd(t, cscale((g1 + kk) * (g2 + kk) - two * kk * kk, Szz));
    t = cadd(t, cmul(cscale(two * (g1 + kk), cmul(k0, k2)), Sxz));
    h11 = cscale(r6, t);
    t = cscale(two * (g1 - kk) * (g2 - kk), Syz);
    t = cadd(t, cmul(cscale(g0 + kk, cmul(c1, c2)), Sxx));
    t = cadd(t, cmul(cscale(g1 - kk, c2), cadd(cmul(c1, Syy), cmul(cscale(two, k0), Sxy))));
    t = cadd(t, cmul(cscale(g2 - kk, c1), cadd(cmul(c2, Szz), cmul(cscale(two, k0), Sxz))));
    h12 = cscale(r6, t);
    t = cscale(g2 - kk, cadd(cscale(g2 - kk, Szz), cmul(cscale(two, k2), cadd(cmul(k0, Sxz), cmul(k1, Syz)))));
    t = cadd(t, cscale((g2 + kk) * (g0 + kk) - two * kk * kk, Sxx));
    t = cadd(t, cscale((g2 + kk) * (g1 + kk) - two * kk * kk, Syy));
    t = cadd(t, cmul(cscale(two * (g2 + kk), cmul(k0, k1)), Sxy));
    h22 = cscale(r6, t);
    h[id] = h00;
    h[n + id] = h01;
    h[2 * n + id] = h02;
    h[3 * n + id] = h11;
    h[4 * n + id] = h12;
    h[5 * n + id] = h22;
  }
}

template <typename T>
int launch_kspace(gev_ctx *ctx, int op, const void *in, void *out, double p1, double p2, int add) {
  typedef typename CT<T>::C C;
  const int N = ctx->N, NH = N / 2 + 1;
  const size_t n = (size_t)N * N * NH;
  const int threads = 256, blocks = grid_for(ctx, n, threads, 16);
  const T *gk2 = (const T *)ctx->d_gridk2;
  const C *ks = (const C *)ctx->d_kshift;
  GevTimed tm_(ctx, op == 0 ? "k_poisson" : "k_kspace");
  switch (op) {
    case 0:
      gev_launch_if<sizeof(T) == 4, k_poisson_body<T>, 256, 1>(ctx, k_poisson<T>, dim3(blocks), dim3(threads), 0, (const C *)in, (C *)out,
                                            gk2, (T)p1, (T)p2, make_kdim(N), n);
      break;
    case 1:
      k_project_scalar<T><<<blocks, threads, 0, ctx->stream>>>((const C *)in, (C *)out, gk2, ks, add, make_kdim(N), n);
      break;
    case 2:
      k_evolve_vector<T><<<blocks, threads, 0, ctx->stream>>>((const C *)in, (C *)out, gk2, ks, (T)p1, make_kdim(N), n);
      break;
    case 3:
      k_project_vector<T><<<blocks, threads, 0, ctx->stream>>>((const C *)in, (C *)out, gk2, ks, (T)p1, (T)p2,
                                                               make_kdim(N), n);
      break;
    default:
      k_project_tensor<T><<<blocks, threads, 0, ctx->stream>>>((const C *)in, (C *)out, gk2, ks, make_kdim(N), n);
  }
  GEV_LAUNCH_CHECK(ctx);
  return GEV_OK;
}

int kspace(gev_ctx *ctx, int op, const gev_field *in, int nin, gev_field *out, int nout, double p1, double p2,
           int add) {
  if (!ctx || !in || !out || in->ctx != ctx || out->ctx != ctx) return gev_fail(ctx, GEV_EINVAL, "null or foreign field");
  if (in->kind != GEV_FIELD_SPECTRUM || out->kind != GEV_FIELD_SPECTRUM)
    return gev_fail(ctx, GEV_EINVAL, "k-space operators take spectra");
  if (in->ncomp != nin || out->ncomp != nout) return gev_fail(ctx, GEV_EINVAL, "wrong number of components");
  return ctx->prec == GEV_PREC_FP64 ? launch_kspace<double>(ctx, op, in->d, out->d, p1, p2, add)
                                    : launch_kspace<float>(ctx, op, in->d, out->d, p1, p2, add);
}

}  // namespace

// k_poisson over one component's raw device spectra (in may equal out); coeff as the
// kernel takes it, already divided by -N^3
int kspace_poisson_raw(gev_ctx *ctx, const void *in, void *out, double coeff, double modif) {
  return ctx->prec == GEV_PREC_FP64 ? launch_kspace<double>(ctx, 0, in, out, coeff, modif, 0)
                                    : launch_kspace<float>(ctx, 0, in, out, coeff, modif, 0);
}

extern "C" {

int gev_solve_poisson(gev_ctx *ctx, const gev_field *srcFT, gev_field *potFT, double coeff, double modif) {
  if (!ctx) return GEV_EINVAL;
  const double N3 = (double)((long)ctx->N * (long)ctx->N * (long)ctx->N);
  return kspace(ctx, 0, srcFT, 1, potFT, 1, coeff / -N3, modif, 0);
}
int gev_project_scalar(gev_ctx *ctx, const gev_field *SijFT, gev_field *chiFT, int add) {
  return kspace(ctx, 1, SijFT, 6, chiFT, 1, 0., 0., add);
}
int gev_evolve_vector(gev_ctx *ctx, const gev_field *SijFT, gev_field *BiFT, double a2dtau) {
  return kspace(ctx, 2, SijFT, 6, BiFT, 3, a2dtau, 0., 0);
}
int gev_project_scalar_evolve_vector(gev_ctx *ctx, const gev_field *SijFT, gev_field *chiFT, gev_field *BiFT,
                                     double a2dtau) {
  if (!ctx || !SijFT || !chiFT || !BiFT || SijFT->ctx != ctx || chiFT->ctx != ctx || BiFT->ctx != ctx ||
      SijFT->kind != GEV_FIELD_SPECTRUM || chiFT->kind != GEV_FIELD_SPECTRUM || BiFT->kind != GEV_FIELD_SPECTRUM ||
      SijFT->ncomp != 6 || chiFT->ncomp != 1 || BiFT->ncomp != 3 || chiFT == SijFT || BiFT == SijFT)
    return gev_fail(ctx, GEV_EINVAL, "project_scalar_evolve_vector: SijFT (6), chiFT (1), BiFT (3), distinct spectra");
  const int N = ctx->N, NH = N / 2 + 1;
  const size_t n = (size_t)N * N * NH;
  const int blocks = grid_for(ctx, n, 256, 16);
  GevTimed tm_(ctx, "k_project_evolve");
  if (ctx->prec == GEV_PREC_FP64)
    k_project_evolve<double><<<blocks, 256, 0, ctx->stream>>>(
        (const CT<double>::C *)SijFT->d, (CT<double>::C *)chiFT->d, (CT<double>::C *)BiFT->d,
        (const double *)ctx->d_gridk2, (const CT<double>::C *)ctx->d_kshift, a2dtau, make_kdim(N), n);
  else
    gev_launch<k_project_evolve_body<float>, 256, 5>(
        ctx, k_project_evolve<float>, dim3(blocks), dim3(256), 0, (const CT<float>::C *)SijFT->d,
        (CT<float>::C *)chiFT->d, (CT<float>::C *)BiFT->d, (const float *)ctx->d_gridk2,
        (const CT<float>::C *)ctx->d_kshift, (float)a2dtau, make_kdim(N), n);
  GEV_LAUNCH_CHECK(ctx);
  return GEV_OK;
}
int gev_project_vector(gev_ctx *ctx, const gev_field *SiFT, gev_field *BiFT, double coeff, double modif) {
  return kspace(ctx, 3, SiFT, 3, BiFT, 3, coeff, modif, 0);
}
int gev_project_tensor(gev_ctx *ctx, const gev_field *SijFT, gev_field *hijFT) {
  return kspace(ctx, 4, SijFT, 6, hijFT, 6, 0., 0., 0);
}

}  // extern "C"
