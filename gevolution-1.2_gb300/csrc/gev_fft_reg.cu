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
// memory, element-major (X[slot * B + c]) with low bits of the slot flipped by
// its bits 3 and up (SWZ): the column kernels flip bit 0 by bit 3; the row
// kernels, whose 2- and 4-line tiles put 4 or 8 slots of one line in a half-warp,
// flip bits 0-2 by bits 3-5, which removes the 2-way conflict of their last
// radix-4 read (18% extra shared wavefronts at L = 256 by an emulation of the
// bank pattern).  The wider flip measured faster for the rows (r2c rows 0.302 ->
// 0.262 ms at 512^3) and slower for the columns (y pass 0.245 -> 0.283 ms).  In-place
// DIF leaves frequency freq(p) in slot p, where freq is a fixed bit permutation
// (the stage digits in reverse order): evaluated at compile time for the
// register index and once per thread for the rest, so no table is read.
//
// Blocks are persistent (resident blocks per SM x SMs, looping over the tiles)
// and stage the twiddle table in shared memory once.
#include <array>
#include <atomic>
#include <map>
#include <mutex>
#include <utility>

#include "gev_fft_bfly.cuh"
#include "gev_batch.cuh"

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
// Tile widths (log2 of the lines a tile) are compile-time constants of each kernel
// instance.  The FP32 widths of a context's row, y and z passes are chosen by
// timing the candidates once on the context's scratch spectrum (fft_autotune); the
// defaults below hold until then and for FP64.  Every width gives the same bits.
constexpr int ROW_LG_DEFAULT = 2;
template <int L, int LG>
constexpr bool fits() {
  return ((L / 8) << LG) <= 1024;
}
// resident blocks asked of the compiler: 1024 threads per SM for FP32 (64
// registers), 512 for FP64, whose own pipe bounds it anyway
constexpr int col_min_blocks(int esize, int threads) {
  return (esize == 4 ? 1024 : 512) / threads > 0 ? (esize == 4 ? 1024 : 512) / threads : 1;
}

template <typename T, int SIGN, int L, int SWZ = 1>
struct RegFft {
  typedef typename CT<T>::C C;
  static constexpr int LG = ilog2c(L);
  static constexpr int N8 = LG / 3, REM = LG % 3;
  static constexpr int NST = N8 + (REM ? 1 : 0);
  static constexpr int TPL = L / 8;  // threads per line

  static __device__ __forceinline__ int phys(int p) { return p ^ ((p >> 3) & SWZ); }

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
// stage.  With 4 or 8 lines a tile, bits 0-1 are flipped by bits 4-5, so that the
// thread groups of a warp, whose outputs lie 16 elements apart, fall on all four
// quarters of the banks.  With 2 lines a half-warp holds 8 threads of a line, whose
// outputs differ in bit 0 and bits 4-5: bits 1-2 are flipped by bits 4-5 instead, so
// that all 8 land in different bank pairs (r2c 0.833 -> 0.820 ms and c2r 0.827 ->
// 0.818 ms for a 512^3 transform with 2-line row tiles; the same bits).
template <int LGB>
__device__ __forceinline__ int nat(int k) {
  if constexpr (LGB == 1) return k ^ ((k >> 3) & 6);
  return k ^ ((k >> 4) & 3);
}

template <typename C>
__device__ __forceinline__ void stage_tw(C *tw, const C *__restrict__ g, int L) {
  for (int i = threadIdx.x; i < L; i += blockDim.x) tw[i] = __ldg(&g[i]);
  __syncthreads();
}

// solveModifiedPoissonFT's factor at (kx, ky, kz), as k_poisson applies it (coeff
// already divided by -N^3)
struct PoisArgs {
  const float *gk2;
  float coeff, modif;
};
__device__ __forceinline__ float poisson_factor(const PoisArgs &p, int kx, int ky, int kz) {
  if ((kx | ky | kz) == 0) return p.modif == 0.f ? 0.f : p.coeff / p.modif;
  return p.coeff / (p.gk2[kx] + p.gk2[ky] + p.gk2[kz] + p.modif);
}

// y / z pass over B columns (consecutive kx) of one plane per tile; in may equal out.
// POIS (FP32 z pass, lines along kz, planes ky): each element is multiplied by its
// Poisson factor as it is loaded, the pass that follows the solve folded into it.
template <typename T, int SIGN, int L, int LGB, bool POIS>
__device__ __forceinline__ void k_fft_cols_reg_body(const typename CT<T>::C *in, typename CT<T>::C *out, const typename CT<T>::C *__restrict__ twg,
                   int NH, long ES, long PS, int ntiles, PoisArgs pois) {
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
    if constexpr (POIS) {
#pragma unroll
      for (int r = 0; r < 8; ++r)
        if (on) v[r] = cscale(poisson_factor(pois, col, (int)plane, m + r * R::TPL), v[r]);
    }
    R::template run_from<0>(v, X, B, c, m, tw);
    if (on) {
      C *dst = out + (long)plane * PS + col;
#pragma unroll
      for (int q = 0; q < 8; ++q) dst[(long)(kb | R::freq(q)) * ES] = v[q];
    }
  }
}
template <typename T, int SIGN, int L, int LGB, bool POIS = false>
__global__ void __launch_bounds__((L / 8) << LGB, col_min_blocks(sizeof(T), (L / 8) << LGB))
    k_fft_cols_reg(const typename CT<T>::C *in, typename CT<T>::C *out, const typename CT<T>::C *__restrict__ twg,
                   int NH, long ES, long PS, int ntiles, PoisArgs pois) {
  k_fft_cols_reg_body<T, SIGN, L, LGB, POIS>(in, out, twg, NH, ES, PS, ntiles, pois);
}

// x pass, forward: rows of N = 2L reals, each an L-point complex FFT followed by
// the real-to-complex split into N/2+1 outputs (row stride NH)
template <typename T, int L, int LGB>
__device__ __forceinline__ void k_fft_r2c_rows_reg_body(const T *__restrict__ in, typename CT<T>::C *__restrict__ out,
                                                           const typename CT<T>::C *__restrict__ twHg,
                                                           const typename CT<T>::C *__restrict__ twN, int NH,
                                                           long nrows, int ntiles) {
  typedef RegFft<T, -1, L, 7> R;
  typedef typename CT<T>::C C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *tw = reinterpret_cast<C *>(smem_raw);
  C *X = tw + L;
  constexpr int lgB = LGB, B = 1 << lgB;
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
    for (int q = 0; q < 8; ++q) X[nat<LGB>(kb | R::freq(q)) * B + c] = v[q];  // Z[k], natural order
    __syncthreads();
    if (on) {
      C *dst = out + row * NH;
#pragma unroll
      for (int r = 0; r <= 8; ++r) {
        if (r == 8 && m != 0) break;
        const int k = r < 8 ? m + r * R::TPL : L;
        const C zk = X[nat<LGB>(k & (L - 1)) * B + c];
        const C zc = cconj(X[nat<LGB>((L - k) & (L - 1)) * B + c]);
        const C E = cscale((T)0.5, cadd(zk, zc));
        const C d = csub(zk, zc);
        const C O = cmk<C>((T)0.5 * d.y, (T)-0.5 * d.x);  // -i/2 (zk - zc)
        dst[k] = cadd(E, cmul(__ldg(&twN[k]), O));
      }
    }
  }
}
template <typename T, int L, int LGB>
__global__ void __launch_bounds__((L / 8) << LGB, col_min_blocks(sizeof(T), (L / 8) << LGB)) k_fft_r2c_rows_reg(const T *__restrict__ in, typename CT<T>::C *__restrict__ out,
                                                           const typename CT<T>::C *__restrict__ twHg,
                                                           const typename CT<T>::C *__restrict__ twN, int NH,
                                                           long nrows, int ntiles) {
  k_fft_r2c_rows_reg_body<T, L, LGB>(in, out, twHg, twN, NH, nrows, ntiles);
}

// x pass, backward: rows of N/2+1 complex -> N = 2L reals
template <typename T, int L, int LGB>
__device__ __forceinline__ void k_fft_c2r_rows_reg_body(const typename CT<T>::C *__restrict__ in, T *__restrict__ out,
                                                           const typename CT<T>::C *__restrict__ twHg,
                                                           const typename CT<T>::C *__restrict__ twN, int NH,
                                                           long nrows, int ntiles) {
  typedef RegFft<T, +1, L, 7> R;
  typedef typename CT<T>::C C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *tw = reinterpret_cast<C *>(smem_raw);
  C *X = tw + L;  // (L + 1) * B
  constexpr int lgB = LGB, B = 1 << lgB;
  stage_tw(tw, twHg, L);
  const int c = threadIdx.x & (B - 1), m = threadIdx.x >> lgB;
  const int kb = R::freq(m << 3);
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const long row = ((long)t << lgB) + c;
    const bool on = row < nrows;
    // element k and its mirror L - k straight from the row (a warp's mirrored reads
    // are consecutive too, and the second read of each element hits L1); the first
    // exchange of run_from starts with the barrier that protects X
    const C *src = in + (on ? row : 0) * NH;
    C v[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int k = m + r * R::TPL;
      C A = on ? src[k] : cmk<C>(0, 0), Bv = on ? src[L - k] : cmk<C>(0, 0);
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
    for (int q = 0; q < 8; ++q) X[nat<LGB>(kb | R::freq(q)) * B + c] = v[q];
    __syncthreads();
    if (on) {
      C *dst = reinterpret_cast<C *>(out) + row * L;
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        const int k = m + r * R::TPL;
        dst[k] = X[nat<LGB>(k) * B + c];
      }
    }
  }
}
template <typename T, int L, int LGB>
__global__ void __launch_bounds__((L / 8) << LGB, col_min_blocks(sizeof(T), (L / 8) << LGB)) k_fft_c2r_rows_reg(const typename CT<T>::C *__restrict__ in, T *__restrict__ out,
                                                           const typename CT<T>::C *__restrict__ twHg,
                                                           const typename CT<T>::C *__restrict__ twN, int NH,
                                                           long nrows, int ntiles) {
  k_fft_c2r_rows_reg_body<T, L, LGB>(in, out, twHg, twN, NH, nrows, ntiles);
}

// ------------------------------------------------------------------ launch --
// grids up to this size have batched forms of the passes (gev_batch.cuh): a batch
// steps many small simulations; larger grids fill the GPU alone
constexpr int BATCH_MAX_L = 256;

// per_sm: the kernel's resident blocks per SM, queried on its first launch (a
// process-wide value; several host threads may launch it first at once)
template <typename K>
int launch_cfg(gev_ctx *ctx, K kern, int threads, size_t smem, long ntiles, std::atomic<int> &per_sm, int &grid) {
  int per = per_sm.load(std::memory_order_relaxed);
  if (per <= 0) {
    if (smem > 48 * 1024 && cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
      return gev_fail(ctx, GEV_ECUDA, "fft: shared memory attribute");
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, threads, smem) != cudaSuccess || per < 1)
      return gev_fail(ctx, GEV_ECUDA, "fft: occupancy query");
    per_sm.store(per, std::memory_order_relaxed);
  }
  const long g = (long)ctx->sms * per;
  grid = (int)(g < ntiles ? g : ntiles);
  return GEV_OK;
}

template <typename T, int SIGN, int L, int LGB, bool POIS = false>
int cols_LB(gev_ctx *ctx, const void *in, void *out, long ES, long PS, PoisArgs pois = PoisArgs{nullptr, 0.f, 0.f}) {
  static_assert(fits<L, LGB>(), "column tile too wide");
  typedef typename CT<T>::C C;
  static std::atomic<int> per_sm{0};
  constexpr int B = 1 << LGB, threads = (L / 8) * B;
  const int NH = ctx->N / 2 + 1;
  const long ntiles = (long)ctx->N * ((NH + B - 1) / B);
  const size_t smem = ((size_t)L + (size_t)L * B) * sizeof(C);
  int grid = 0;
  int rc = launch_cfg(ctx, k_fft_cols_reg<T, SIGN, L, LGB, POIS>, threads, smem, ntiles, per_sm, grid);
  if (rc) return rc;
  GevTimed tm_(ctx, "k_fft_cols_reg");
  gev_launch_if<sizeof(T) == 4 && L <= BATCH_MAX_L, k_fft_cols_reg_body<T, SIGN, L, LGB, POIS>, threads, col_min_blocks(sizeof(T), threads)>(
      ctx, k_fft_cols_reg<T, SIGN, L, LGB, POIS>, dim3(grid), dim3(threads), smem, (const C *)in, (C *)out,
      (const C *)ctx->d_twN, NH, ES, PS, (int)ntiles, pois);
  GEV_LAUNCH_CHECK(ctx);
  return GEV_OK;
}

// the width of a pass: tuned (FP32), else 16 lines for the FP32 z pass up to L = 512
// (rows a plane apart: ES > PS) and tile_lg otherwise
template <typename T, int L>
int col_lg(const gev_ctx *ctx, bool zpass) {
  if (sizeof(T) == 4 && ctx->fft_lg[zpass ? 2 : 1] >= 0) return ctx->fft_lg[zpass ? 2 : 1];
  return (sizeof(T) == 4 && L <= 512 && zpass) ? 4 : tile_lg<T>();
}
template <typename T, int SIGN, int L>
int cols_L(gev_ctx *ctx, const void *in, void *out, long ES, long PS) {
  if constexpr (sizeof(T) == 8) {
    return cols_LB<T, SIGN, L, tile_lg<T>()>(ctx, in, out, ES, PS);
  } else {
    switch (col_lg<T, L>(ctx, ES > PS)) {
      case 2: return cols_LB<T, SIGN, L, 2>(ctx, in, out, ES, PS);
      case 3:
        if constexpr (fits<L, 3>()) return cols_LB<T, SIGN, L, 3>(ctx, in, out, ES, PS);
        break;
      case 4:
        if constexpr (fits<L, 4>()) return cols_LB<T, SIGN, L, 4>(ctx, in, out, ES, PS);
        break;
    }
    return gev_fail(ctx, GEV_EINVAL, "fft: column tile width");
  }
}

// the FP32 backward z pass (spectrum -> out) with the Poisson factor applied to its input
template <int L>
int cols_z_poisson(gev_ctx *ctx, const void *in, void *out, PoisArgs pois) {
  const long N = ctx->N, NH = N / 2 + 1, ES = N * NH, PS = NH;
  switch (col_lg<float, L>(ctx, true)) {
    case 2: return cols_LB<float, 1, L, 2, true>(ctx, in, out, ES, PS, pois);
    case 3:
      if constexpr (fits<L, 3>()) return cols_LB<float, 1, L, 3, true>(ctx, in, out, ES, PS, pois);
      break;
    case 4:
      if constexpr (fits<L, 4>()) return cols_LB<float, 1, L, 4, true>(ctx, in, out, ES, PS, pois);
      break;
  }
  return gev_fail(ctx, GEV_EINVAL, "fft: column tile width");
}

// nrows: rows of the transform (N^2; fewer only while tuning)
template <typename T, int L, int LGB>
int r2c_LB(gev_ctx *ctx, const void *real, void *spec, long nrows) {
  static_assert(fits<L, LGB>(), "row tile too wide");
  typedef typename CT<T>::C C;
  static std::atomic<int> per_sm{0};
  constexpr int B = 1 << LGB, threads = (L / 8) * B;
  const int NH = ctx->N / 2 + 1;
  const long ntiles = (nrows + B - 1) / B;
  const size_t smem = ((size_t)L + (size_t)L * B) * sizeof(C);
  int grid = 0;
  int rc = launch_cfg(ctx, k_fft_r2c_rows_reg<T, L, LGB>, threads, smem, ntiles, per_sm, grid);
  if (rc) return rc;
  GevTimed tm_(ctx, "k_fft_r2c_rows_reg");
  gev_launch_if<sizeof(T) == 4 && 2 * L <= BATCH_MAX_L, k_fft_r2c_rows_reg_body<T, L, LGB>, threads, col_min_blocks(sizeof(T), threads)>(
      ctx, k_fft_r2c_rows_reg<T, L, LGB>, dim3(grid), dim3(threads), smem, (const T *)real, (C *)spec,
      (const C *)ctx->d_twH, (const C *)ctx->d_twN, NH, nrows, (int)ntiles);
  GEV_LAUNCH_CHECK(ctx);
  return GEV_OK;
}

template <typename T, int L, int LGB>
int c2r_LB(gev_ctx *ctx, const void *spec, void *real, long nrows) {
  static_assert(fits<L, LGB>(), "row tile too wide");
  typedef typename CT<T>::C C;
  static std::atomic<int> per_sm{0};
  constexpr int B = 1 << LGB, threads = (L / 8) * B;
  const int NH = ctx->N / 2 + 1;
  const long ntiles = (nrows + B - 1) / B;
  const size_t smem = ((size_t)L + (size_t)(L + 1) * B) * sizeof(C);
  int grid = 0;
  int rc = launch_cfg(ctx, k_fft_c2r_rows_reg<T, L, LGB>, threads, smem, ntiles, per_sm, grid);
  if (rc) return rc;
  GevTimed tm_(ctx, "k_fft_c2r_rows_reg");
  gev_launch_if<sizeof(T) == 4 && 2 * L <= BATCH_MAX_L, k_fft_c2r_rows_reg_body<T, L, LGB>, threads, col_min_blocks(sizeof(T), threads)>(
      ctx, k_fft_c2r_rows_reg<T, L, LGB>, dim3(grid), dim3(threads), smem, (const C *)spec, (T *)real,
      (const C *)ctx->d_twH, (const C *)ctx->d_twN, NH, nrows, (int)ntiles);
  GEV_LAUNCH_CHECK(ctx);
  return GEV_OK;
}

template <typename T, int L>
int row_lg(const gev_ctx *ctx, bool c2r) {
  if (sizeof(T) == 4 && ctx->fft_lg[c2r ? 3 : 0] >= 0) return ctx->fft_lg[c2r ? 3 : 0];
  return ROW_LG_DEFAULT;
}
template <typename T, int L>
int rows_L(gev_ctx *ctx, const void *in, void *out, bool c2r, long nrows, int lg) {
  if constexpr (sizeof(T) == 8) {
    return c2r ? c2r_LB<T, L, ROW_LG_DEFAULT>(ctx, in, out, nrows) : r2c_LB<T, L, ROW_LG_DEFAULT>(ctx, in, out, nrows);
  } else {
    switch (lg) {
      case 1: return c2r ? c2r_LB<T, L, 1>(ctx, in, out, nrows) : r2c_LB<T, L, 1>(ctx, in, out, nrows);
      case 2:
        if constexpr (fits<L, 2>())
          return c2r ? c2r_LB<T, L, 2>(ctx, in, out, nrows) : r2c_LB<T, L, 2>(ctx, in, out, nrows);
        break;
      case 3:
        if constexpr (fits<L, 3>())
          return c2r ? c2r_LB<T, L, 3>(ctx, in, out, nrows) : r2c_LB<T, L, 3>(ctx, in, out, nrows);
        break;
    }
    return gev_fail(ctx, GEV_EINVAL, "fft: row tile width");
  }
}
template <typename T, int L>
int r2c_L(gev_ctx *ctx, const void *real, void *spec) {
  return rows_L<T, L>(ctx, real, spec, false, (long)ctx->N * ctx->N, row_lg<T, L>(ctx, false));
}
template <typename T, int L>
int c2r_L(gev_ctx *ctx, const void *spec, void *real) {
  return rows_L<T, L>(ctx, spec, real, true, (long)ctx->N * ctx->N, row_lg<T, L>(ctx, true));
}

// ---------------------------------------------------------------- tuning --
// mean ms of 5 launches of fn after one warm-up launch, on the context's stream;
// a candidate that fails to launch gets +inf
template <typename F>
float time_ms(gev_ctx *ctx, F &&fn) {
  cudaEvent_t a = nullptr, b = nullptr;
  float ms = 3.4e38f;
  if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
    cudaGetLastError();
  } else if (fn() == GEV_OK) {
    cudaEventRecord(a, ctx->stream);
    int rc = GEV_OK;
    for (int k = 0; k < 5 && rc == GEV_OK; ++k) rc = fn();
    cudaEventRecord(b, ctx->stream);
    if (rc == GEV_OK && cudaEventSynchronize(b) == cudaSuccess && cudaEventElapsedTime(&ms, a, b) == cudaSuccess)
      ms /= 5.f;
    else
      ms = 3.4e38f;
  }
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  return ms;
}

// The candidates run on the context's scratch spectrum (filled with a bounded
// pattern first): the column passes in place over the whole component, the row
// passes over half the rows, reading one half of the scratch and writing the other.
// Three rounds over the candidates, each keeping its best time (the first rounds of
// a process may run before the clocks have settled); a candidate replaces the
// measured default only when it is more than 3% faster.
__global__ void k_tune_fill(float *s, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    s[i] = (float)((unsigned)(i * 2654435761u) >> 8) * (1.f / 16777216.f) - 0.5f;
}
inline int pick(const float *t, int lo, int hi, int def) {
  int best = def;
  for (int lg = lo; lg <= hi; ++lg)
    if (t[lg] < 0.97f * t[def] && t[lg] < t[best]) best = lg;
  return best;
}
template <int L>
void tune_cols(gev_ctx *ctx) {
  float2 *S = (float2 *)ctx->d_fft_scratch;
  const long N = ctx->N, NH = N / 2 + 1;
  for (int z = 0; z < 2; ++z) {
    const long ES = z ? N * NH : NH, PS = z ? NH : N * NH;
    float t[5] = {3.4e38f, 3.4e38f, 3.4e38f, 3.4e38f, 3.4e38f};
    for (int round = 0; round < 3; ++round) {
      t[2] = fminf(t[2], time_ms(ctx, [&] { return cols_LB<float, -1, L, 2>(ctx, S, S, ES, PS); }));
      if constexpr (fits<L, 3>())
        t[3] = fminf(t[3], time_ms(ctx, [&] { return cols_LB<float, -1, L, 3>(ctx, S, S, ES, PS); }));
      if constexpr (fits<L, 4>())
        t[4] = fminf(t[4], time_ms(ctx, [&] { return cols_LB<float, -1, L, 4>(ctx, S, S, ES, PS); }));
    }
    ctx->fft_lg[z ? 2 : 1] = pick(t, 2, 4, col_lg<float, L>(ctx, z != 0));
  }
}
template <int L>
void tune_rows(gev_ctx *ctx) {
  float2 *S = (float2 *)ctx->d_fft_scratch;
  const long N = ctx->N, NH = N / 2 + 1, half = N * N / 2;
  // r2c: half * N reals at S[0, half * L), half * NH complex after them; c2r: half * NH
  // complex at S[0, half * NH), half * N reals after them (both within N^2 NH complex)
  for (int c2r = 0; c2r < 2; ++c2r) {
    const void *in = S;
    void *out = c2r ? (void *)(S + half * NH) : (void *)(S + half * L);
    float t[4] = {3.4e38f, 3.4e38f, 3.4e38f, 3.4e38f};
    for (int round = 0; round < 3; ++round)
      for (int lg = 1; lg <= 3; ++lg)
        if (((L / 8) << lg) <= 1024)
          t[lg] = fminf(t[lg], time_ms(ctx, [&] { return rows_L<float, L>(ctx, in, out, c2r != 0, half, lg); }));
    ctx->fft_lg[c2r ? 3 : 0] = pick(t, 1, 3, ROW_LG_DEFAULT);
  }
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

extern "C" int gev_ctx_fft_tiles(gev_ctx *ctx, int *lg) {
  if (!ctx || !lg) return gev_fail(ctx, GEV_EINVAL, "ctx_fft_tiles: null argument");
  const bool f32 = ctx->prec != GEV_PREC_FP64;
  const int N = ctx->N;
  const int defaults[4] = {ROW_LG_DEFAULT, f32 ? 3 : 2, (f32 && N <= 512) ? 4 : (f32 ? 3 : 2), ROW_LG_DEFAULT};
  for (int p = 0; p < 4; ++p) lg[p] = (f32 && ctx->fft_lg[p] >= 0) ? ctx->fft_lg[p] : defaults[p];
  return GEV_OK;
}

extern "C" int gev_ctx_set_fft_tiles(gev_ctx *ctx, const int *lg) {
  if (!ctx || !lg) return gev_fail(ctx, GEV_EINVAL, "ctx_set_fft_tiles: null argument");
  const int N = ctx->N;
  if (ctx->prec == GEV_PREC_FP64 || !fft_reg_ok(N))
    return gev_fail(ctx, GEV_EINVAL, "ctx_set_fft_tiles: the FP64 form and non-power-of-two grids keep fixed tiles");
  const bool rows_ok = fft_reg_ok(N / 2);
  for (int p = 0; p < 4; ++p) {
    const bool row = p == 0 || p == 3;
    const int L = row ? N / 2 : N, lo = row ? 1 : 2, hi = row ? 3 : 4;
    if ((row && !rows_ok) ? lg[p] != ROW_LG_DEFAULT : (lg[p] < lo || lg[p] > hi || ((L / 8) << lg[p]) > 1024))
      return gev_fail(ctx, GEV_EINVAL, "ctx_set_fft_tiles: rows 1..3, columns 2..4, at most 1024 threads a tile");
  }
  for (int p = 0; p < 4; ++p) ctx->fft_lg[p] = lg[p];
  ctx->fft_tuned = true;
  return GEV_OK;
}

int fft_cols_z_poisson(gev_ctx *ctx, const void *spec, void *out, double coeff, double modif) {
  const PoisArgs pois{(const float *)ctx->d_gridk2, (float)coeff, (float)modif};
  switch (ctx->N) {
#define CALL(l) \
  case l: return cols_z_poisson<l>(ctx, spec, out, pois);
    CALL(8) CALL(16) CALL(32) CALL(64) CALL(128) CALL(256) CALL(512) CALL(1024)
#undef CALL
    default: return gev_fail(ctx, GEV_EINVAL, "fft_cols_z_poisson: power-of-two grids of 8 to 1024");
  }
}

// widths already timed in this process, per (device, N): a later context of a size
// seen before takes them instead of timing again (a server creates dozens of
// contexts of a few sizes)
static std::mutex g_tiles_mu;
static std::map<std::pair<int, int>, std::array<int, 4>> g_tiles;
static void fft_tune_all(gev_ctx *ctx);

void fft_autotune(gev_ctx *ctx) {
  if (ctx->fft_tuned) return;
  if (ctx->rec) {  // a recorded cycle cannot time anything: batch only tuned contexts
    ctx->rec->bad = true;
    return;
  }
  ctx->fft_tuned = true;
  const int N = ctx->N;
  if (ctx->prec == GEV_PREC_FP64 || !ctx->d_fft_scratch || !fft_reg_ok(N)) return;
  const auto key = std::make_pair(ctx->device, N);
  {
    std::lock_guard<std::mutex> lk(g_tiles_mu);
    const auto it = g_tiles.find(key);
    if (it != g_tiles.end()) {
      for (int p = 0; p < 4; ++p) ctx->fft_lg[p] = it->second[p];
      return;
    }
  }
  fft_tune_all(ctx);
  std::lock_guard<std::mutex> lk(g_tiles_mu);
  g_tiles[key] = {ctx->fft_lg[0], ctx->fft_lg[1], ctx->fft_lg[2], ctx->fft_lg[3]};
}

// times the candidate widths of the four passes on the context's scratch spectrum
static void fft_tune_all(gev_ctx *ctx) {
  const int N = ctx->N;
  k_tune_fill<<<grid_for(ctx, ctx->fft_scratch_bytes / 4, 256, 8), 256, 0, ctx->stream>>>(
      (float *)ctx->d_fft_scratch, ctx->fft_scratch_bytes / 4);
  if (cudaGetLastError() != cudaSuccess) return;
  switch (N) {
#define TUNE(l)         \
  case l:               \
    tune_cols<l>(ctx);  \
    break;
    TUNE(8) TUNE(16) TUNE(32) TUNE(64) TUNE(128) TUNE(256) TUNE(512) TUNE(1024)
#undef TUNE
    default: break;
  }
  if (!fft_reg_ok(N / 2)) return;
  switch (N / 2) {
#define TUNE(l)         \
  case l:               \
    tune_rows<l>(ctx);  \
    break;
    TUNE(8) TUNE(16) TUNE(32) TUNE(64) TUNE(128) TUNE(256) TUNE(512) TUNE(1024)
#undef TUNE
    default: break;
  }
}

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
