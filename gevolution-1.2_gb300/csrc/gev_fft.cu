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
//   y, z : batches of B consecutive kx columns (coalesced B*sizeof(complex)
//       segments), FFT of length N along the strided axis in shared memory.
// Each line FFT is a Stockham self-sorting transform with radix-8/4/2/3
// stages ping-ponging between two shared-memory buffers; lengths 2^a 3^b.
#include "gev_internal.cuh"

namespace {

template <typename T, int SIGN>
struct Bfly {
  typedef typename CT<T>::C C;
  // multiply by SIGN * i
  static __device__ __forceinline__ C mi(C a) { return SIGN < 0 ? cmk<C>(a.y, -a.x) : cmk<C>(-a.y, a.x); }
  static __device__ __forceinline__ void r2(C *v) {
    C a = v[0];
    v[0] = cadd(a, v[1]);
    v[1] = csub(a, v[1]);
  }
  static __device__ __forceinline__ void r4(C *v) {
    C a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]), a2 = cadd(v[1], v[3]), a3 = mi(csub(v[1], v[3]));
    v[0] = cadd(a0, a2);
    v[2] = csub(a0, a2);
    v[1] = cadd(a1, a3);
    v[3] = csub(a1, a3);
  }
  static __device__ __forceinline__ void r8(C *v) {
    const T c = (T)0.707106781186547524400844362104849039;
    C b[4], d[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      b[r] = cadd(v[r], v[r + 4]);
      d[r] = csub(v[r], v[r + 4]);
    }
    // d[r] *= e^{SIGN 2 pi i r / 8}
    d[1] = cmk<C>(c * (d[1].x - (T)SIGN * d[1].y), c * (d[1].y + (T)SIGN * d[1].x));
    d[2] = mi(d[2]);
    d[3] = cmk<C>(c * (-d[3].x - (T)SIGN * d[3].y), c * ((T)SIGN * d[3].x - d[3].y));
    r4(b);
    r4(d);
    v[0] = b[0];
    v[2] = b[1];
    v[4] = b[2];
    v[6] = b[3];
    v[1] = d[0];
    v[3] = d[1];
    v[5] = d[2];
    v[7] = d[3];
  }
  static __device__ __forceinline__ void r3(C *v) {
    const T s = (T)0.866025403784438646763723170752936183;
    C t1 = cadd(v[1], v[2]);
    C t2 = csub(v[0], cscale((T)0.5, t1));
    C t3 = cscale(s, mi(csub(v[1], v[2])));
    v[0] = cadd(v[0], t1);
    v[1] = cadd(t2, t3);
    v[2] = csub(t2, t3);
  }
  template <int R>
  static __device__ __forceinline__ void run(C *v) {
    if (R == 2) r2(v);
    if (R == 3) r3(v);
    if (R == 4) r4(v);
    if (R == 8) r8(v);
  }
};

// one Stockham stage of radix R over nlines lines of length L (line stride ldl)
template <typename T, int SIGN, int R>
__device__ __forceinline__ void stage(const typename CT<T>::C *X, typename CT<T>::C *Y, int L, int ldl, int nlines,
                                      int Ns, const typename CT<T>::C *__restrict__ tw) {
  typedef typename CT<T>::C C;
  const int nb = L / R;
  const int total = nlines * nb;
  const int twstep = L / (Ns * R);
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int c = t / nb, j = t - c * nb;
    const int k = j % Ns;
    const C *xl = X + c * ldl;
    C *yl = Y + c * ldl;
    C v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = xl[j + r * nb];
    if (k != 0) {
#pragma unroll
      for (int r = 1; r < R; ++r) {
        C w = __ldg(&tw[r * k * twstep]);
        if (SIGN > 0) w.y = -w.y;
        v[r] = cmul(v[r], w);
      }
    }
    Bfly<T, SIGN>::template run<R>(v);
    const int base = (j - k) * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) yl[base + r * Ns] = v[r];
  }
}

// full line FFT; returns the buffer that holds the result
template <typename T, int SIGN>
__device__ typename CT<T>::C *fft_core(typename CT<T>::C *X, typename CT<T>::C *Y, int ldl, int nlines,
                                       const FftPlan &pl, const typename CT<T>::C *__restrict__ tw) {
  typedef typename CT<T>::C C;
  int Ns = 1;
  for (int s = 0; s < pl.nst; ++s) {
    const int R = pl.R[s];
    if (R == 8)
      stage<T, SIGN, 8>(X, Y, pl.L, ldl, nlines, Ns, tw);
    else if (R == 4)
      stage<T, SIGN, 4>(X, Y, pl.L, ldl, nlines, Ns, tw);
    else if (R == 2)
      stage<T, SIGN, 2>(X, Y, pl.L, ldl, nlines, Ns, tw);
    else
      stage<T, SIGN, 3>(X, Y, pl.L, ldl, nlines, Ns, tw);
    __syncthreads();
    C *t = X;
    X = Y;
    Y = t;
    Ns *= R;
  }
  return X;
}

// y / z pass: planes of lines; B consecutive kx columns per block.  in may equal out.
template <typename T, int SIGN>
__global__ void __launch_bounds__(256) k_fft_cols(const typename CT<T>::C *in, typename CT<T>::C *out, FftPlan pl,
                                                  const typename CT<T>::C *__restrict__ tw, int NH, long line_stride,
                                                  long plane_stride, int B) {
  typedef typename CT<T>::C C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int L = pl.L, ldl = L + 1;
  C *buf0 = reinterpret_cast<C *>(smem_raw);
  C *buf1 = buf0 + (size_t)B * ldl;
  const int nchunks = (NH + B - 1) / B;
  const long plane = blockIdx.x / nchunks;
  const int c0 = (int)(blockIdx.x - plane * nchunks) * B;
  const int nb = min(B, NH - c0);
  const C *src = in + plane * plane_stride + c0;
  for (int t = threadIdx.x; t < L * B; t += blockDim.x) {
    const int i = t / B, c = t - i * B;
    if (c < nb) buf0[c * ldl + i] = src[(long)i * line_stride + c];
  }
  __syncthreads();
  C *res = fft_core<T, SIGN>(buf0, buf1, ldl, nb, pl, tw);
  C *dst = out + plane * plane_stride + c0;
  for (int t = threadIdx.x; t < L * B; t += blockDim.x) {
    const int i = t / B, c = t - i * B;
    if (c < nb) dst[(long)i * line_stride + c] = res[c * ldl + i];
  }
}

// x pass, forward: rows of N reals -> N/2+1 complex (row stride NH in the output)
template <typename T>
__global__ void __launch_bounds__(256) k_fft_r2c_rows(const T *__restrict__ in, typename CT<T>::C *__restrict__ out,
                                                      FftPlan pl, const typename CT<T>::C *__restrict__ twH,
                                                      const typename CT<T>::C *__restrict__ twN, int NH, long nrows,
                                                      int B) {
  typedef typename CT<T>::C C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int M = pl.L, ldl = M + 1;
  C *buf0 = reinterpret_cast<C *>(smem_raw);
  C *buf1 = buf0 + (size_t)B * ldl;
  const long row0 = (long)blockIdx.x * B;
  const int nb = (int)min((long)B, nrows - row0);
  const C *src = reinterpret_cast<const C *>(in) + row0 * M;
  for (int t = threadIdx.x; t < nb * M; t += blockDim.x) {
    const int c = t / M, i = t - c * M;
    buf0[c * ldl + i] = src[t];
  }
  __syncthreads();
  C *Z = fft_core<T, -1>(buf0, buf1, ldl, nb, pl, twH);
  C *dst = out + row0 * NH;
  const int W = M + 1;
  for (int t = threadIdx.x; t < nb * W; t += blockDim.x) {
    const int c = t / W, k = t - c * W;
    const C zk = Z[c * ldl + (k == M ? 0 : k)];
    const C zc = cconj(Z[c * ldl + (k == 0 ? 0 : M - k)]);
    const C E = cscale((T)0.5, cadd(zk, zc));
    const C d = csub(zk, zc);
    const C O = cmk<C>((T)0.5 * d.y, (T)-0.5 * d.x);  // -i/2 (zk - zc)
    const C w = __ldg(&twN[k]);
    dst[(long)c * NH + k] = cadd(E, cmul(w, O));
  }
}

// x pass, backward: N/2+1 complex -> N reals per row
template <typename T>
__global__ void __launch_bounds__(256) k_fft_c2r_rows(const typename CT<T>::C *__restrict__ in, T *__restrict__ out,
                                                      FftPlan pl, const typename CT<T>::C *__restrict__ twH,
                                                      const typename CT<T>::C *__restrict__ twN, int NH, long nrows,
                                                      int B) {
  typedef typename CT<T>::C C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int M = pl.L, ldl = M + 1;
  C *buf0 = reinterpret_cast<C *>(smem_raw);
  C *buf1 = buf0 + (size_t)B * ldl;
  C *xin = buf1 + (size_t)B * ldl;  // B rows of M+1
  const long row0 = (long)blockIdx.x * B;
  const int nb = (int)min((long)B, nrows - row0);
  const C *src = in + row0 * NH;
  const int W = M + 1;
  for (int t = threadIdx.x; t < nb * W; t += blockDim.x) {
    const int c = t / W, k = t - c * W;
    xin[c * W + k] = src[(long)c * NH + k];
  }
  __syncthreads();
  for (int t = threadIdx.x; t < nb * M; t += blockDim.x) {
    const int c = t / M, k = t - c * M;
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
    buf0[c * ldl + k] = cmk<C>(s.x - wd.y, s.y + wd.x);  // s + i w d
  }
  __syncthreads();
  C *z = fft_core<T, +1>(buf0, buf1, ldl, nb, pl, twH);
  C *dst = reinterpret_cast<C *>(out) + row0 * M;
  for (int t = threadIdx.x; t < nb * M; t += blockDim.x) {
    const int c = t / M, i = t - c * M;
    dst[t] = z[c * ldl + i];
  }
}

template <typename T>
size_t cols_smem(int L, int B) {
  return 2 * (size_t)B * (L + 1) * sizeof(typename CT<T>::C);
}
inline int cols_B(int L, int NH) {
  int B = 2048 / L;
  if (B < 1) B = 1;
  if (B > 16) B = 16;
  if (B > NH) B = NH;
  return B;
}
inline int rows_B(int M) {
  int B = 2048 / M;
  if (B < 1) B = 1;
  if (B > 64) B = 64;
  return B;
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
  const int B = cols_B(N, NH);
  const long nchunks = (NH + B - 1) / B;
  const long blocks = (long)N * nchunks;
  k_fft_cols<T, SIGN><<<(unsigned)blocks, 256, cols_smem<T>(N, B), ctx->stream>>>(
      (const C *)in, (C *)out, ctx->planN, (const C *)ctx->d_twN, NH, line_stride, plane_stride, B);
  GEV_LAUNCH_CHECK(ctx);
  return GEV_OK;
}

template <typename T>
int r2c_comp(gev_ctx *ctx, const void *real, void *spec) {
  typedef typename CT<T>::C C;
  const int N = ctx->N, NH = N / 2 + 1, M = N / 2;
  const long nrows = (long)N * N;
  const int B = rows_B(M);
  const size_t smem = 2 * (size_t)B * (M + 1) * sizeof(C);
  k_fft_r2c_rows<T><<<(unsigned)((nrows + B - 1) / B), 256, smem, ctx->stream>>>(
      (const T *)real, (C *)spec, ctx->planH, (const C *)ctx->d_twH, (const C *)ctx->d_twN, NH, nrows, B);
  GEV_LAUNCH_CHECK(ctx);
  int rc = run_cols<T, -1>(ctx, spec, spec, NH, (long)N * NH);  // y: lines along ky, planes kz
  if (rc) return rc;
  return run_cols<T, -1>(ctx, spec, spec, (long)N * NH, NH);  // z: lines along kz, planes ky
}

template <typename T>
int c2r_comp(gev_ctx *ctx, const void *spec, void *real, void *scratch) {
  typedef typename CT<T>::C C;
  const int N = ctx->N, NH = N / 2 + 1, M = N / 2;
  int rc = run_cols<T, +1>(ctx, spec, scratch, (long)N * NH, NH);  // z, out of place
  if (rc) return rc;
  rc = run_cols<T, +1>(ctx, scratch, scratch, NH, (long)N * NH);  // y, in place
  if (rc) return rc;
  const long nrows = (long)N * N;
  const int B = rows_B(M);
  const size_t smem = 3 * (size_t)B * (M + 1) * sizeof(C);
  k_fft_c2r_rows<T><<<(unsigned)((nrows + B - 1) / B), 256, smem, ctx->stream>>>(
      (const C *)scratch, (T *)real, ctx->planH, (const C *)ctx->d_twH, (const C *)ctx->d_twN, NH, nrows, B);
  GEV_LAUNCH_CHECK(ctx);
  return GEV_OK;
}

}  // namespace

int fft_build_plan(int L, FftPlan *pl) {
  pl->L = L;
  pl->nst = 0;
  int n = L;
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
  while (n % 3 == 0 && pl->nst < GEV_MAX_RADICES) {
    pl->R[pl->nst++] = 3;
    n /= 3;
  }
  return n == 1 ? GEV_OK : GEV_EINVAL;
}

int fft_init_kernels(int prec) {
  return prec == GEV_PREC_FP64 ? set_smem_attrs<double>() : set_smem_attrs<float>();
}

int fft_r2c_comp(gev_ctx *ctx, const void *real, void *spec) {
  return ctx->prec == GEV_PREC_FP64 ? r2c_comp<double>(ctx, real, spec) : r2c_comp<float>(ctx, real, spec);
}

int fft_c2r_comp(gev_ctx *ctx, const void *spec, void *real, void *scratch) {
  return ctx->prec == GEV_PREC_FP64 ? c2r_comp<double>(ctx, spec, real, scratch)
                                    : c2r_comp<float>(ctx, spec, real, scratch);
}
