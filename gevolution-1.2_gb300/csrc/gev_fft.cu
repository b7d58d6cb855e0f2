// gev_fft.cu -- hand-written 3-D r2c / c2r FFT for sm_103a.
//
// Replaces PlanFFT<Cplx>::execute (LATfield2 over FFTW; main.cpp:477-596):
// unnormalised, FFTW sign convention, half spectrum with kx in [0, N/2] stored
// fastest.  The backward transform leaves its input spectrum untouched (the
// parabolic B update accumulates into BiFT across steps, gevolution.hpp:317-325,
// and main.cpp:521-533 reads scalarFT after the phi c2r), so it runs its first
// pass out of place into a context-owned scratch spectrum.
//
// Structure: three passes over HBM per transform.
//   x : rows of N reals viewed as N/2 complex, FFT of length N/2 in shared
//       memory, then the real-to-complex split (r2c) or merge (c2r);
//   y, z : batches of B consecutive kx columns (B * sizeof(complex) contiguous
//       bytes per row), FFT of length N along the strided axis.
// In shared memory a batch is stored element-major, X[i * LD + c] for element i
// of line c, so consecutive threads work on consecutive lines: global rows load
// and store coalesced and butterfly reads / writes hit consecutive banks.
// Each line FFT is an in-place mixed-radix decimation-in-frequency transform
// (a radix-3 stage first when the length has a factor 3, then radix 8, then
// one radix 4 or 2): every butterfly reads and writes the same R slots, so one
// shared buffer holds the batch and twice as many blocks fit on an SM as with
// a ping-pong buffer.  The output comes out in mixed-radix digit-reversed
// order, which the store phase undoes through a small permutation table.
// Twiddles and the permutation are staged in shared memory; the index
// arithmetic is shifts and masks (every sub-length after the first stage is a
// power of two) or an exact multiply-high division.
#include <vector>

#include "gev_fft_bfly.cuh"
#include "gev_batch.cuh"

namespace {

// exact q = t / d for t < 2^32 / d (d < 2^11 here): q = umulhi(t, ceil(2^32 / d))
struct FastDiv {
  unsigned d, m;
};
inline FastDiv make_div(unsigned d) {
  FastDiv f;
  f.d = d;
  f.m = (unsigned)((((unsigned long long)1 << 32) + d - 1) / d);
  return f;
}
__device__ __forceinline__ unsigned fdiv(unsigned t, const FastDiv &f) { return __umulhi(t, f.m); }

// One decimation-in-frequency stage of radix R over the B lines of a batch
// (element-major, element stride LD), in place.  span = current sub-transform
// length; sub = span / R is a power of two.  Butterfly (block bb, offset j)
// reads x[bb span + j + r sub], forms the R-point DFT, multiplies output q by
// W_span^{j q} and writes it back to bb span + j + q sub.
template <typename T, int SIGN, int R>
__device__ __forceinline__ void dif_stage(typename CT<T>::C *X, int L, int LD, int lgB, int span, int lgsub,
                                          const typename CT<T>::C *tw) {
  typedef typename CT<T>::C C;
  const int sub = 1 << lgsub;
  const int total = (L / R) << lgB;
  const int B1 = (1 << lgB) - 1;
  const int twstep = L / span;
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int c = t & B1, u = t >> lgB;
    const int j = u & (sub - 1);
    const int base = (u >> lgsub) * span + j;
    C v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = X[(base + r * sub) * LD + c];
    Bfly<T, SIGN>::template run<R>(v);
    if (j != 0) {
#pragma unroll
      for (int q = 1; q < R; ++q) {
        C w = tw[j * q * twstep];
        if (SIGN > 0) w.y = -w.y;
        v[q] = cmul(v[q], w);
      }
    }
#pragma unroll
    for (int q = 0; q < R; ++q) X[(base + q * sub) * LD + c] = v[q];
  }
}

// full line FFT of the batch, in place; the result sits at digit-reversed slots
template <typename T, int SIGN>
__device__ void fft_dif(typename CT<T>::C *X, int LD, int lgB, const FftPlan &pl, const typename CT<T>::C *tw) {
  int span = pl.L;
  for (int s = 0; s < pl.nst; ++s) {
    const int R = pl.R[s];
    const int sub = span / R;
    const int lgsub = 31 - __clz(sub);
    if (R == 8)
      dif_stage<T, SIGN, 8>(X, pl.L, LD, lgB, span, lgsub, tw);
    else if (R == 4)
      dif_stage<T, SIGN, 4>(X, pl.L, LD, lgB, span, lgsub, tw);
    else if (R == 2)
      dif_stage<T, SIGN, 2>(X, pl.L, LD, lgB, span, lgsub, tw);
    else
      dif_stage<T, SIGN, 3>(X, pl.L, LD, lgB, span, lgsub, tw);
    __syncthreads();
    span = sub;
  }
}

template <typename T>
__device__ __forceinline__ void stage_tables(typename CT<T>::C *sh, const typename CT<T>::C *__restrict__ g,
                                             unsigned short *shp, const unsigned short *__restrict__ gp, int L) {
  for (int i = threadIdx.x; i < L; i += blockDim.x) {
    sh[i] = __ldg(&g[i]);
    shp[i] = __ldg(&gp[i]);
  }
}

// y / z pass: one block = one plane x B consecutive kx columns.  in may equal out.
template <typename T, int SIGN>
__device__ __forceinline__ void k_fft_cols_body(const typename CT<T>::C *in, typename CT<T>::C *out, FftPlan pl,
                                                  const typename CT<T>::C *__restrict__ twg,
                                                  const unsigned short *__restrict__ permg, int NH, long line_stride,
                                                  long plane_stride, int lgB) {
  typedef typename CT<T>::C C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int L = pl.L, B = 1 << lgB;
  C *tw = reinterpret_cast<C *>(smem_raw);
  C *buf = tw + L;
  unsigned short *perm = reinterpret_cast<unsigned short *>(buf + (size_t)L * B);
  const int nchunks = (NH + B - 1) >> lgB;
  const long plane = blockIdx.x / nchunks;
  const int c0 = (int)(blockIdx.x - plane * nchunks) << lgB;
  const int nbv = min(B, NH - c0);
  stage_tables<T>(tw, twg, perm, permg, L);
  const C *src = in + plane * plane_stride + c0;
  for (int t = threadIdx.x; t < (L << lgB); t += blockDim.x) {
    const int c = t & (B - 1), i = t >> lgB;
    if (c < nbv) buf[i * B + c] = src[(long)i * line_stride + c];
  }
  __syncthreads();
  fft_dif<T, SIGN>(buf, B, lgB, pl, tw);
  C *dst = out + plane * plane_stride + c0;
  for (int t = threadIdx.x; t < (L << lgB); t += blockDim.x) {
    const int c = t & (B - 1), k = t >> lgB;
    if (c < nbv) dst[(long)k * line_stride + c] = buf[perm[k] * B + c];
  }
}
template <typename T, int SIGN>
__global__ void __launch_bounds__(256) k_fft_cols(const typename CT<T>::C *in, typename CT<T>::C *out, FftPlan pl,
                                                  const typename CT<T>::C *__restrict__ twg,
                                                  const unsigned short *__restrict__ permg, int NH, long line_stride,
                                                  long plane_stride, int lgB) {
  k_fft_cols_body<T, SIGN>(in, out, pl, twg, permg, NH, line_stride, plane_stride, lgB);
}

// x pass, forward: B rows of N reals -> N/2+1 complex each (row stride NH out)
template <typename T>
__device__ __forceinline__ void k_fft_r2c_rows_body(const T *__restrict__ in, typename CT<T>::C *__restrict__ out,
                                                      FftPlan pl, const typename CT<T>::C *__restrict__ twHg,
                                                      const unsigned short *__restrict__ permg,
                                                      const typename CT<T>::C *__restrict__ twN, int NH, long nrows,
                                                      int lgB, FastDiv divM, FastDiv divW) {
  typedef typename CT<T>::C C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int M = pl.L, B = 1 << lgB, LD = B + 1;
  C *tw = reinterpret_cast<C *>(smem_raw);
  C *buf = tw + M;
  unsigned short *perm = reinterpret_cast<unsigned short *>(buf + (size_t)M * LD);
  const long row0 = (long)blockIdx.x << lgB;
  const int nb = (int)min((long)B, nrows - row0);
  stage_tables<T>(tw, twHg, perm, permg, M);
  const C *src = reinterpret_cast<const C *>(in) + row0 * M;
  for (int t = threadIdx.x; t < nb * M; t += blockDim.x) {
    const int c = (int)fdiv((unsigned)t, divM), i = t - c * M;
    buf[i * LD + c] = src[t];
  }
  __syncthreads();
  fft_dif<T, -1>(buf, LD, lgB, pl, tw);
  C *dst = out + row0 * NH;
  const int W = M + 1;
  for (int t = threadIdx.x; t < nb * W; t += blockDim.x) {
    const int c = (int)fdiv((unsigned)t, divW), k = t - c * W;
    const C zk = buf[perm[k == M ? 0 : k] * LD + c];
    const C zc = cconj(buf[perm[k == 0 ? 0 : M - k] * LD + c]);
    const C E = cscale((T)0.5, cadd(zk, zc));
    const C d = csub(zk, zc);
    const C O = cmk<C>((T)0.5 * d.y, (T)-0.5 * d.x);  // -i/2 (zk - zc)
    const C w = __ldg(&twN[k]);
    dst[(long)c * NH + k] = cadd(E, cmul(w, O));
  }
}
template <typename T>
__global__ void __launch_bounds__(256) k_fft_r2c_rows(const T *__restrict__ in, typename CT<T>::C *__restrict__ out,
                                                      FftPlan pl, const typename CT<T>::C *__restrict__ twHg,
                                                      const unsigned short *__restrict__ permg,
                                                      const typename CT<T>::C *__restrict__ twN, int NH, long nrows,
                                                      int lgB, FastDiv divM, FastDiv divW) {
  k_fft_r2c_rows_body<T>(in, out, pl, twHg, permg, twN, NH, nrows, lgB, divM, divW);
}

// x pass, backward: N/2+1 complex -> N reals per row
template <typename T>
__device__ __forceinline__ void k_fft_c2r_rows_body(const typename CT<T>::C *__restrict__ in, T *__restrict__ out,
                                                      FftPlan pl, const typename CT<T>::C *__restrict__ twHg,
                                                      const unsigned short *__restrict__ permg,
                                                      const typename CT<T>::C *__restrict__ twN, int NH, long nrows,
                                                      int lgB, FastDiv divM, FastDiv divW) {
  typedef typename CT<T>::C C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int M = pl.L, B = 1 << lgB, LD = B + 1, W = M + 1;
  C *tw = reinterpret_cast<C *>(smem_raw);
  C *buf = tw + M;
  C *xin = buf + (size_t)M * LD;  // B rows of M+1, row-major
  unsigned short *perm = reinterpret_cast<unsigned short *>(xin + (size_t)B * W);
  const long row0 = (long)blockIdx.x << lgB;
  const int nb = (int)min((long)B, nrows - row0);
  stage_tables<T>(tw, twHg, perm, permg, M);
  const C *src = in + row0 * NH;
  for (int t = threadIdx.x; t < nb * W; t += blockDim.x) {
    const int c = (int)fdiv((unsigned)t, divW), k = t - c * W;
    xin[c * W + k] = src[(long)c * NH + k];
  }
  __syncthreads();
  for (int t = threadIdx.x; t < (M << lgB); t += blockDim.x) {
    const int c = t & (B - 1), k = t >> lgB;
    if (c >= nb) continue;
    C A = xin[c * W + k];
    C Bv = xin[c * W + (M - k)];
    if (k == 0) {
      A.y = (T)0;
      Bv.y = (T)0;
    }
    const C Bc = cconj(Bv);
    const C s = cadd(A, Bc), d = csub(A, Bc);
    const C w = cconj(__ldg(&twN[k]));  // e^{+2 pi i k / N}
    const C wd = cmul(w, d);
    buf[k * LD + c] = cmk<C>(s.x - wd.y, s.y + wd.x);  // s + i w d
  }
  __syncthreads();
  fft_dif<T, +1>(buf, LD, lgB, pl, tw);
  C *dst = reinterpret_cast<C *>(out) + row0 * M;
  for (int t = threadIdx.x; t < nb * M; t += blockDim.x) {
    const int c = (int)fdiv((unsigned)t, divM), i = t - c * M;
    dst[t] = buf[perm[i] * LD + c];
  }
}
template <typename T>
__global__ void __launch_bounds__(256) k_fft_c2r_rows(const typename CT<T>::C *__restrict__ in, T *__restrict__ out,
                                                      FftPlan pl, const typename CT<T>::C *__restrict__ twHg,
                                                      const unsigned short *__restrict__ permg,
                                                      const typename CT<T>::C *__restrict__ twN, int NH, long nrows,
                                                      int lgB, FastDiv divM, FastDiv divW) {
  k_fft_c2r_rows_body<T>(in, out, pl, twHg, permg, twN, NH, nrows, lgB, divM, divW);
}

inline int ilog2(int v) {
  int l = 0;
  while ((1 << (l + 1)) <= v) ++l;
  return l;
}
// lines per batch: about `target` bytes of batch data, a power of two in [lo, hi]
inline int batch_lg(int L, size_t csz, int lo, int hi, size_t target) {
  int B = (int)(target / ((size_t)L * csz));
  if (B < lo) B = lo;
  if (B > hi) B = hi;
  return ilog2(B);
}

template <typename T>
int set_smem_attrs() {
  const int big = 200 * 1024;
  cudaFuncSetAttribute(k_fft_cols<T, -1>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(k_fft_cols<T, +1>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(k_fft_r2c_rows<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(k_fft_c2r_rows<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  return cudaGetLastError() == cudaSuccess ? GEV_OK : GEV_ECUDA;
}

template <typename T, int SIGN>
int run_cols(gev_ctx *ctx, const void *in, void *out, long line_stride, long plane_stride) {
  typedef typename CT<T>::C C;
  const int N = ctx->N, NH = N / 2 + 1;
  if (fft_reg_ok(N)) return fft_cols_reg(ctx, in, out, line_stride, plane_stride, SIGN);
  int lgB = batch_lg(N, sizeof(C), 2, 16, 32768);
  while ((1 << lgB) > NH && lgB > 0) --lgB;
  const int B = 1 << lgB;
  const long nchunks = (NH + B - 1) / B;
  const long blocks = (long)N * nchunks;
  const size_t smem = ((size_t)N + (size_t)N * B) * sizeof(C) + (size_t)N * 2;
  GevTimed tm_(ctx, "k_fft_cols");
  gev_launch_if<sizeof(T) == 4, k_fft_cols_body<T, SIGN>, 256, 5>(
      ctx, k_fft_cols<T, SIGN>, dim3((unsigned)blocks), dim3(256), smem, (const C *)in, (C *)out, ctx->planN,
      (const C *)ctx->d_twN, (const unsigned short *)ctx->d_permN, NH, line_stride, plane_stride, lgB);
  GEV_LAUNCH_CHECK(ctx);
  return GEV_OK;
}

template <typename T>
int r2c_comp(gev_ctx *ctx, const void *real, void *spec) {
  typedef typename CT<T>::C C;
  const int N = ctx->N, NH = N / 2 + 1, M = N / 2;
  const long nrows = (long)N * N;
  if (fft_reg_ok(M)) {
    int rc = fft_r2c_rows_reg(ctx, real, spec);
    if (rc) return rc;
    rc = run_cols<T, -1>(ctx, spec, spec, NH, (long)N * NH);
    if (rc) return rc;
    return run_cols<T, -1>(ctx, spec, spec, (long)N * NH, NH);
  }
  const int lgB = batch_lg(M, sizeof(C), 1, 64, 32768), B = 1 << lgB;
  const size_t smem = ((size_t)M + (size_t)M * (B + 1)) * sizeof(C) + (size_t)M * 2;
  GevTimed tm_(ctx, "k_fft_r2c_rows");
  gev_launch_if<sizeof(T) == 4, k_fft_r2c_rows_body<T>, 256, 5>(
      ctx, k_fft_r2c_rows<T>, dim3((unsigned)((nrows + B - 1) / B)), dim3(256), smem, (const T *)real, (C *)spec,
      ctx->planH, (const C *)ctx->d_twH, (const unsigned short *)ctx->d_permH, (const C *)ctx->d_twN, NH, nrows,
      lgB, make_div(M), make_div(M + 1));
  GEV_LAUNCH_CHECK(ctx);
  int rc = run_cols<T, -1>(ctx, spec, spec, NH, (long)N * NH);  // y: lines along ky, planes kz
  if (rc) return rc;
  return run_cols<T, -1>(ctx, spec, spec, (long)N * NH, NH);  // z: lines along kz, planes ky
}

// pois: the FP32 power-of-two z pass applies solveModifiedPoissonFT's factor (coeff,
// already divided by -N^3, and modif) to its input as it loads it
template <typename T>
int c2r_comp(gev_ctx *ctx, const void *spec, void *real, void *scratch, const double *pois = nullptr) {
  typedef typename CT<T>::C C;
  const int N = ctx->N, NH = N / 2 + 1, M = N / 2;
  int rc = pois ? fft_cols_z_poisson(ctx, spec, scratch, pois[0], pois[1])
                : run_cols<T, +1>(ctx, spec, scratch, (long)N * NH, NH);  // z, out of place
  if (rc) return rc;
  rc = run_cols<T, +1>(ctx, scratch, scratch, NH, (long)N * NH);  // y, in place
  if (rc) return rc;
  if (fft_reg_ok(M)) return fft_c2r_rows_reg(ctx, scratch, real);
  const long nrows = (long)N * N;
  const int lgB = batch_lg(M, sizeof(C), 1, 64, 32768), B = 1 << lgB;
  const size_t smem = ((size_t)M + (size_t)M * (B + 1) + (size_t)B * (M + 1)) * sizeof(C) + (size_t)M * 2;
  GevTimed tm_(ctx, "k_fft_c2r_rows");
  gev_launch_if<sizeof(T) == 4, k_fft_c2r_rows_body<T>, 256, 5>(
      ctx, k_fft_c2r_rows<T>, dim3((unsigned)((nrows + B - 1) / B)), dim3(256), smem, (const C *)scratch,
      (T *)real, ctx->planH, (const C *)ctx->d_twH, (const unsigned short *)ctx->d_permH, (const C *)ctx->d_twN, NH,
      nrows, lgB, make_div(M), make_div(M + 1));
  GEV_LAUNCH_CHECK(ctx);
  return GEV_OK;
}

}  // namespace

// a radix-3 stage first (at most one), then radix 8, then one radix 4 or 2:
// every sub-length after the first stage is then a power of two
int fft_build_plan(int L, FftPlan *pl) {
  pl->L = L;
  pl->nst = 0;
  int n = L;
  if (n % 3 == 0) {
    pl->R[pl->nst++] = 3;
    n /= 3;
  }
  while (n % 8 == 0 && pl->nst < GEV_MAX_RADICES) {
    pl->R[pl->nst++] = 8;
    n /= 8;
  }
  while (n % 4 == 0 && pl->nst < GEV_MAX_RADICES) {
    pl->R[pl->nst++] = 4;
    n /= 4;
  }
  while (n % 2 == 0 && pl->nst < GEV_MAX_RADICES) {
    pl->R[pl->nst++] = 2;
    n /= 2;
  }
  return n == 1 ? GEV_OK : GEV_EINVAL;
}

// slot of frequency k after the in-place DIF stages: the mixed-radix digits of
// k (first stage's radix least significant) weighted by the sub-lengths
void fft_perm(const FftPlan &pl, std::vector<unsigned short> &perm) {
  perm.resize(pl.L);
  for (int k = 0; k < pl.L; ++k) {
    int rem = k, span = pl.L, p = 0;
    for (int s = 0; s < pl.nst; ++s) {
      const int R = pl.R[s], sub = span / R;
      p += (rem % R) * sub;
      rem /= R;
      span = sub;
    }
    perm[k] = (unsigned short)p;
  }
}

int fft_init_kernels(int prec) {
  return prec == GEV_PREC_FP64 ? set_smem_attrs<double>() : set_smem_attrs<float>();
}

int fft_r2c_comp(gev_ctx *ctx, const void *real, void *spec) {
  fft_autotune(ctx);
  return ctx->prec == GEV_PREC_FP64 ? r2c_comp<double>(ctx, real, spec) : r2c_comp<float>(ctx, real, spec);
}

// c2r of the solution of solveModifiedPoissonFT for the spectrum srcFT, which is kept.
// FP32 on power-of-two grids: the factor is applied in the first (z) pass as it loads
// its input; otherwise the solve writes the scratch spectrum and the c2r transforms it
// there in place.  Either way the bits of the two calls in place.
int fft_c2r_poisson_comp(gev_ctx *ctx, const void *srcFT, void *real, double coeff, double modif) {
  fft_autotune(ctx);
  const double N3 = (double)((long)ctx->N * (long)ctx->N * (long)ctx->N);
  if (ctx->prec != GEV_PREC_FP64 && fft_reg_ok(ctx->N)) {
    const double pois[2] = {coeff / -N3, modif};
    return c2r_comp<float>(ctx, srcFT, real, ctx->d_fft_scratch, pois);
  }
  int rc = kspace_poisson_raw(ctx, srcFT, ctx->d_fft_scratch, coeff / -N3, modif);
  if (rc) return rc;
  return ctx->prec == GEV_PREC_FP64 ? c2r_comp<double>(ctx, ctx->d_fft_scratch, real, ctx->d_fft_scratch)
                                    : c2r_comp<float>(ctx, ctx->d_fft_scratch, real, ctx->d_fft_scratch);
}

int fft_c2r_comp(gev_ctx *ctx, const void *spec, void *real, void *scratch) {
  fft_autotune(ctx);  // before the scratch holds this transform's z pass
  return ctx->prec == GEV_PREC_FP64 ? c2r_comp<double>(ctx, spec, real, scratch)
                                    : c2r_comp<float>(ctx, spec, real, scratch);
}

extern "C" int gev_fft_axis(gev_ctx *ctx, gev_field *spec, int axis, int sign) {
  if (!ctx || !spec || spec->ctx != ctx || spec->kind != GEV_FIELD_SPECTRUM || (axis != 1 && axis != 2) ||
      (sign != -1 && sign != 1))
    return gev_fail(ctx, GEV_EINVAL, "fft_axis: spectrum, axis 1 (y) or 2 (z), sign -1 or +1");
  const int N = ctx->N, NH = N / 2 + 1;
  const long ls = axis == 1 ? NH : (long)N * NH, ps = axis == 1 ? (long)N * NH : NH;
  fft_autotune(ctx);
  for (int c = 0; c < spec->ncomp; ++c) {
    void *d = (char *)spec->d + c * spec->comp_elems * spec->elem_bytes;
    int rc;
    if (ctx->prec == GEV_PREC_FP64)
      rc = sign < 0 ? run_cols<double, -1>(ctx, d, d, ls, ps) : run_cols<double, +1>(ctx, d, d, ls, ps);
    else
      rc = sign < 0 ? run_cols<float, -1>(ctx, d, d, ls, ps) : run_cols<float, +1>(ctx, d, d, ls, ps);
    if (rc) return rc;
  }
  return GEV_OK;
}
