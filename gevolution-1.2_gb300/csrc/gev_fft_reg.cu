// gev_fft_reg.cu -- register-resident FFT passes for power-of-two lengths
// 8 <= L <= 1024: the y / z passes of grids N = 8 ... 1024 and the x pass of
// grids N = 16 ... 2048.  gev_fft.cu calls these whenever the length allows and
// its shared-memory staged kernels otherwise (lengths with a factor 3).
//
// Work layout.  A line of L elements is held by L/8 threads, 8 elements
// (registers) each.  A tile is B consecutive lines: column tiles take 8 lines for
// FP32 and 4 for FP64 (every row of a tile 64 contiguous bytes; 16 lines in the
// FP32 z pass), row tiles 4 lines; thread (m, c) = (tid / B, tid % B) holds
// elements of line c.
//
// Transform.  Decimation in frequency, in place: stages s = 0 .. N8-1 are
// radix 8 (span L / 8^s); when log2 L is not a multiple of 3 a last radix-4 or
// radix-2 stage follows.  A radix-8 stage runs in the registers of one thread
// (its 8 inputs lie span/8 apart).  Between stages the tile goes through shared
// memory, element-major (X[slot * B + c]) with bit 0 of the slot flipped by its
// bit 3, which keeps every exchange pattern free of bank conflicts.  In-place
// DIF leaves frequency freq(p) in slot p, where freq is a fixed bit permutation
// (the stage digits in reverse order): evaluated at compile time for the
// register index and once per thread for the rest, so no table is read.
//
// Blocks are persistent (resident blocks per SM x SMs, looping over the tiles)
// and stage the twiddle table in shared memory once.
#include "gev_fft_bfly.cuh"
#include "gev_internal.cuh"

namespace {

constexpr int ilog2c(int v) { return v <= 1 ? 0 : 1 + ilog2c(v >> 1); }

// lines per tile: 8 for FP32, 4 for FP64 (64 bytes of every column-tile row)
template <typename T>
__host__ __device__ constexpr int tile_lg() {
  return sizeof(T) == 4 ? 3 : 2;
}
// The column passes take 2^LGB lines per tile.  The z pass of an FP32 spectrum,
// whose rows lie a plane apart, reads 16 lines (a whole 128-byte line per row)
// up to L = 512 (1024 threads): fewer, longer DRAM bursts than 8 lines.  The y
// pass, whose rows are consecutive in a plane, is faster with the default 8.
// the x-pass (row) kernels take 4 rows a tile in both precisions: smaller blocks,
// more of them resident, measured faster than 8 or 16 (and than 2) for FP32
constexpr int row_tile_lg() { return 2; }
template <typename T, int L>
constexpr int reg_threads() {
  return (L / 8) << row_tile_lg();
}
constexpr int col_min_blocks(int esize, int threads) {
  return (esize == 4 ? 1024 : 512) / threads > 0 ? (esize == 4 ? 1024 : 512) / threads : 1;
}
// resident blocks asked of the compiler: 1024 threads per SM for FP32 (64
// registers), 512 for FP64, whose own pipe bounds it anyway
template <typename T, int L>
constexpr int reg_min_blocks() {
  return (sizeof(T) == 4 ? 1024 : 512) / reg_threads<T, L>() > 0 ? (sizeof(T) == 4 ? 1024 : 512) / reg_threads<T, L>()
                                                                 : 1;
}

template <typename T, int SIGN, int L>
struct RegFft {
  typedef typename CT<T>::C C;
  static constexpr int LG = ilog2c(L);
  static constexpr int N8 = LG / 3, REM = LG % 3;
  static constexpr int NST = N8 + (REM ? 1 : 0);
  static constexpr int TPL = L / 8;  // threads per line

  static __device__ __forceinline__ int phys(int p) { return p ^ ((p >> 3) & 1); }

  // slot of register r of thread m in stage S (inputs and outputs alike)
  template <int S>
  static __device__ __forceinline__ int slot(int m, int r) {
    if constexpr (S < N8) {
      constexpr int lgsub = LG - 3 * S - 3;
      return ((m >> lgsub) << (lgsub + 3)) | (m & ((1 << lgsub) - 1)) | (r << lgsub);
    } else {
      return (m << 3) | r;
    }
  }

  // frequency held by slot p after the last stage
  static __host__ __device__ constexpr int freq(int p) {
    int k = 0;
    for (int s = 0; s < N8; ++s) k |= ((p >> (LG - 3 * s - 3)) & 7) << (3 * s);
    if (REM) k |= (p & ((1 << REM) - 1)) << (3 * N8);
    return k;
  }

  template <int S>
  static __device__ __forceinline__ void stage(C (&v)[8], int m, const C *tw) {
    if constexpr (S < N8) {
      Bfly<T, SIGN>::r8(v);
      constexpr int lgsub = LG - 3 * S - 3;
      if constexpr (lgsub > 0) {  // output q times W_span^{j q}, W_span = W_L^{8^S}
        const int j = m & ((1 << lgsub) - 1);
#pragma unroll
        for (int q = 1; q < 8; ++q) {
          C w = tw[(j * q) << (3 * S)];
          if (SIGN > 0) w.y = -w.y;
          v[q] = cmul(v[q], w);
        }
      }
    } else if constexpr (REM == 2) {
      Bfly<T, SIGN>::r4(v);
      Bfly<T, SIGN>::r4(v + 4);
    } else {
#pragma unroll
      for (int u = 0; u < 8; u += 2) Bfly<T, SIGN>::r2(v + u);
    }
  }

  // stages S .. NST-1; v holds the inputs of stage S on entry and the outputs of
  // the last stage (slots 8m + q) on return.  Starts every exchange with a
  // barrier, so X may still be in use by the caller's previous reads.
  template <int S>
  static __device__ __forceinline__ void run_from(C (&v)[8], C *X, int B, int c, int m, const C *tw) {
    stage<S>(v, m, tw);
    if constexpr (S + 1 < NST) {
      __syncthreads();
#pragma unroll
      for (int r = 0; r < 8; ++r) X[phys(slot<S>(m, r)) * B + c] = v[r];
      __syncthreads();
#pragma unroll
      for (int r = 0; r < 8; ++r) v[r] = X[phys(slot<S + 1>(m, r)) * B + c];
      run_from<S + 1>(v, X, B, c, m, tw);
    }
  }
};

// row of natural-order element k in the tile the row kernels write after the last
// stage: bits 0-1 flipped by bits 4-5, so that the thread groups of a warp, whose
// outputs lie 16 elements apart, fall on all four quarters of the banks
__device__ __forceinline__ int nat(int k) { return k ^ ((k >> 4) & 3); }

template <typename C>
__device__ __forceinline__ void stage_tw(C *tw, const C *__restrict__ g, int L) {
  for (int i = threadIdx.x; i < L; i += blockDim.x) tw[i] = __ldg(&g[i]);
  __syncthreads();
}

// y / z pass over B columns (consecutive kx) of one plane per tile; in may equal out
template <typename T, int SIGN, int L, int LGB>
__global__ void __launch_bounds__((L / 8) << LGB, col_min_blocks(sizeof(T), (L / 8) << LGB))
    k_fft_cols_reg(const typename CT<T>::C *in, typename CT<T>::C *out, const typename CT<T>::C *__restrict__ twg,
                   int NH, long ES, long PS, int ntiles) {
  typedef RegFft<T, SIGN, L> R;
  typedef typename CT<T>::C C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *tw = reinterpret_cast<C *>(smem_raw);
  C *X = tw + L;
  constexpr int lgB = LGB, B = 1 << LGB;
  stage_tw(tw, twg, L);
  const int c = threadIdx.x & (B - 1), m = threadIdx.x >> lgB;
  const unsigned nchunks = (unsigned)(NH + B - 1) >> lgB;
  const int kb = R::freq(m << 3);
  const long rstep = (long)R::TPL * ES;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const unsigned plane = (unsigned)t / nchunks;
    const int col = (int)(((unsigned)t - plane * nchunks) << lgB) + c;
    const bool on = col < NH;
    const C *src = in + (long)plane * PS + col + (long)m * ES;
    C v[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) v[r] = on ? src[r * rstep] : cmk<C>(0, 0);
    R::template run_from<0>(v, X, B, c, m, tw);
    if (on) {
      C *dst = out + (long)plane * PS + col;
#pragma unroll
      for (int q = 0; q < 8; ++q) dst[(long)(kb | R::freq(q)) * ES] = v[q];
    }
  }
}

// x pass, forward: rows of N = 2L reals, each an L-point complex FFT followed by
// the real-to-complex split into N/2+1 outputs (row stride NH)
template <typename T, int L>
__global__ void __launch_bounds__(reg_threads<T, L>(), reg_min_blocks<T, L>()) k_fft_r2c_rows_reg(const T *__restrict__ in, typename CT<T>::C *__restrict__ out,
                                                           const typename CT<T>::C *__restrict__ twHg,
                                                           const typename CT<T>::C *__restrict__ twN, int NH,
                                                           long nrows, int ntiles) {
  typedef RegFft<T, -1, L> R;
  typedef typename CT<T>::C C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *tw = reinterpret_cast<C *>(smem_raw);
  C *X = tw + L;
  constexpr int lgB = row_tile_lg(), B = 1 << lgB;
  stage_tw(tw, twHg, L);
  const int c = threadIdx.x & (B - 1), m = threadIdx.x >> lgB;
  const int kb = R::freq(m << 3);
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const long row = ((long)t << lgB) + c;
    const bool on = row < nrows;
    const C *src = reinterpret_cast<const C *>(in) + row * L + m;
    C v[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) v[r] = on ? src[r * R::TPL] : cmk<C>(0, 0);
    R::template run_from<0>(v, X, B, c, m, tw);
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 8; ++q) X[nat(kb | R::freq(q)) * B + c] = v[q];  // Z[k], natural order
    __syncthreads();
    if (on) {
      C *dst = out + row * NH;
#pragma unroll
      for (int r = 0; r <= 8; ++r) {
        if (r == 8 && m != 0) break;
        const int k = r < 8 ? m + r * R::TPL : L;
        const C zk = X[nat(k & (L - 1)) * B + c];
        const C zc = cconj(X[nat((L - k) & (L - 1)) * B + c]);
        const C E = cscale((T)0.5, cadd(zk, zc));
        const C d = csub(zk, zc);
        const C O = cmk<C>((T)0.5 * d.y, (T)-0.5 * d.x);  // -i/2 (zk - zc)
        dst[k] = cadd(E, cmul(__ldg(&twN[k]), O));
      }
    }
  }
}

// x pass, backward: rows of N/2+1 complex -> N = 2L reals
template <typename T, int L>
__global__ void __launch_bounds__(reg_threads<T, L>(), reg_min_blocks<T, L>()) k_fft_c2r_rows_reg(const typename CT<T>::C *__restrict__ in, T *__restrict__ out,
                                                           const typename CT<T>::C *__restrict__ twHg,
                                                           const typename CT<T>::C *__restrict__ twN, int NH,
                                                           long nrows, int ntiles) {
  typedef RegFft<T, +1, L> R;
  typedef typename CT<T>::C C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *tw = reinterpret_cast<C *>(smem_raw);
  C *X = tw + L;  // (L + 1) * B
  constexpr int lgB = row_tile_lg(), B = 1 << lgB;
  stage_tw(tw, twHg, L);
  const int c = threadIdx.x & (B - 1), m = threadIdx.x >> lgB;
  const int kb = R::freq(m << 3);
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const long row = ((long)t << lgB) + c;
    const bool on = row < nrows;
    const C *src = in + row * NH;
    __syncthreads();
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int k = m + r * R::TPL;
      X[k * B + c] = on ? src[k] : cmk<C>(0, 0);
    }
    if (m == 0) X[L * B + c] = on ? src[L] : cmk<C>(0, 0);
    __syncthreads();
    C v[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int k = m + r * R::TPL;
      C A = X[k * B + c], Bv = X[(L - k) * B + c];
      if (k == 0) {  // the imaginary parts of the kx = 0 and N/2 modes do not enter a real transform
        A.y = (T)0;
        Bv.y = (T)0;
      }
      const C Bc = cconj(Bv);
      const C s = cadd(A, Bc), d = csub(A, Bc);
      const C wd = cmul(cconj(__ldg(&twN[k])), d);  // e^{+2 pi i k / N} d
      v[r] = cmk<C>(s.x - wd.y, s.y + wd.x);         // s + i w d
    }
    R::template run_from<0>(v, X, B, c, m, tw);
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 8; ++q) X[nat(kb | R::freq(q)) * B + c] = v[q];
    __syncthreads();
    if (on) {
      C *dst = reinterpret_cast<C *>(out) + row * L;
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        const int k = m + r * R::TPL;
        dst[k] = X[nat(k) * B + c];
      }
    }
  }
}

// ------------------------------------------------------------------ launch --
template <typename K>
int launch_cfg(gev_ctx *ctx, K kern, int threads, size_t smem, long ntiles, int &per_sm, int &grid) {
  if (per_sm <= 0) {
    if (smem > 48 * 1024 && cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
      return gev_fail(ctx, GEV_ECUDA, "fft: shared memory attribute");
    int per = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, threads, smem) != cudaSuccess || per < 1)
      return gev_fail(ctx, GEV_ECUDA, "fft: occupancy query");
    per_sm = per;
  }
  const long g = (long)ctx->sms * per_sm;
  grid = (int)(g < ntiles ? g : ntiles);
  return GEV_OK;
}

template <typename T, int SIGN, int L, int LGB>
int cols_LB(gev_ctx *ctx, const void *in, void *out, long ES, long PS) {
  typedef typename CT<T>::C C;
  static int per_sm = 0;
  constexpr int B = 1 << LGB, threads = (L / 8) * B;
  const int NH = ctx->N / 2 + 1;
  const long ntiles = (long)ctx->N * ((NH + B - 1) / B);
  const size_t smem = ((size_t)L + (size_t)L * B) * sizeof(C);
  int grid = 0;
  int rc = launch_cfg(ctx, k_fft_cols_reg<T, SIGN, L, LGB>, threads, smem, ntiles, per_sm, grid);
  if (rc) return rc;
  k_fft_cols_reg<T, SIGN, L, LGB><<<grid, threads, smem, ctx->stream>>>((const C *)in, (C *)out,
                                                                        (const C *)ctx->d_twN, NH, ES, PS, (int)ntiles);
  GEV_LAUNCH_CHECK(ctx);
  return GEV_OK;
}

// the wide tile for a pass whose rows are further apart than its tiles (ES > PS)
template <typename T, int SIGN, int L>
int cols_L(gev_ctx *ctx, const void *in, void *out, long ES, long PS) {
  if constexpr (sizeof(T) == 4 && L <= 512) {
    if (ES > PS) return cols_LB<T, SIGN, L, 4>(ctx, in, out, ES, PS);
  }
  return cols_LB<T, SIGN, L, tile_lg<T>()>(ctx, in, out, ES, PS);
}

template <typename T, int L>
int r2c_L(gev_ctx *ctx, const void *real, void *spec) {
  typedef typename CT<T>::C C;
  static int per_sm = 0;
  const int N = ctx->N, NH = N / 2 + 1, lgB = row_tile_lg(), B = 1 << lgB;
  const int threads = (L / 8) * B;
  const long nrows = (long)N * N, ntiles = (nrows + B - 1) / B;
  const size_t smem = ((size_t)L + (size_t)L * B) * sizeof(C);
  int grid = 0;
  int rc = launch_cfg(ctx, k_fft_r2c_rows_reg<T, L>, threads, smem, ntiles, per_sm, grid);
  if (rc) return rc;
  k_fft_r2c_rows_reg<T, L><<<grid, threads, smem, ctx->stream>>>((const T *)real, (C *)spec, (const C *)ctx->d_twH,
                                                                 (const C *)ctx->d_twN, NH, nrows, (int)ntiles);
  GEV_LAUNCH_CHECK(ctx);
  return GEV_OK;
}

template <typename T, int L>
int c2r_L(gev_ctx *ctx, const void *spec, void *real) {
  typedef typename CT<T>::C C;
  static int per_sm = 0;
  const int N = ctx->N, NH = N / 2 + 1, lgB = row_tile_lg(), B = 1 << lgB;
  const int threads = (L / 8) * B;
  const long nrows = (long)N * N, ntiles = (nrows + B - 1) / B;
  const size_t smem = ((size_t)L + (size_t)(L + 1) * B) * sizeof(C);
  int grid = 0;
  int rc = launch_cfg(ctx, k_fft_c2r_rows_reg<T, L>, threads, smem, ntiles, per_sm, grid);
  if (rc) return rc;
  k_fft_c2r_rows_reg<T, L><<<grid, threads, smem, ctx->stream>>>((const C *)spec, (T *)real, (const C *)ctx->d_twH,
                                                                 (const C *)ctx->d_twN, NH, nrows, (int)ntiles);
  GEV_LAUNCH_CHECK(ctx);
  return GEV_OK;
}

#define GEV_REG_SWITCH(L, CALL) \
  switch (L) {                  \
    case 8: return CALL(8);     \
    case 16: return CALL(16);   \
    case 32: return CALL(32);   \
    case 64: return CALL(64);   \
    case 128: return CALL(128); \
    case 256: return CALL(256); \
    case 512: return CALL(512); \
    case 1024: return CALL(1024); \
    default: return GEV_EINVAL; \
  }

}  // namespace

bool fft_reg_ok(int L) { return L >= 8 && L <= 1024 && (L & (L - 1)) == 0; }

int fft_cols_reg(gev_ctx *ctx, const void *in, void *out, long ES, long PS, int sign) {
  const int L = ctx->N;
  if (ctx->prec == GEV_PREC_FP64) {
    if (sign < 0) {
#define CALL(l) cols_L<double, -1, l>(ctx, in, out, ES, PS)
      GEV_REG_SWITCH(L, CALL)
#undef CALL
    } else {
#define CALL(l) cols_L<double, 1, l>(ctx, in, out, ES, PS)
      GEV_REG_SWITCH(L, CALL)
#undef CALL
    }
  } else {
    if (sign < 0) {
#define CALL(l) cols_L<float, -1, l>(ctx, in, out, ES, PS)
      GEV_REG_SWITCH(L, CALL)
#undef CALL
    } else {
#define CALL(l) cols_L<float, 1, l>(ctx, in, out, ES, PS)
      GEV_REG_SWITCH(L, CALL)
#undef CALL
    }
  }
}

int fft_r2c_rows_reg(gev_ctx *ctx, const void *real, void *spec) {
  const int L = ctx->N / 2;
  if (ctx->prec == GEV_PREC_FP64) {
#define CALL(l) r2c_L<double, l>(ctx, real, spec)
    GEV_REG_SWITCH(L, CALL)
#undef CALL
  } else {
#define CALL(l) r2c_L<float, l>(ctx, real, spec)
    GEV_REG_SWITCH(L, CALL)
#undef CALL
  }
}

int fft_c2r_rows_reg(gev_ctx *ctx, const void *spec, void *real) {
  const int L = ctx->N / 2;
  if (ctx->prec == GEV_PREC_FP64) {
#define CALL(l) c2r_L<double, l>(ctx, spec, real)
    GEV_REG_SWITCH(L, CALL)
#undef CALL
  } else {
#define CALL(l) c2r_L<float, l>(ctx, spec, real)
    GEV_REG_SWITCH(L, CALL)
#undef CALL
  }
}
