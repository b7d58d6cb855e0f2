// gev_internal.cuh -- shared definitions of the GB300 hot-path library:
// context / field / particle-store layouts, complex helpers, periodic indexing
// and error plumbing.
//
// Device layouts (chosen for coalescing on GB300, not copied from LATfield2):
//   real field  : ncomp planes of N^3 elements, x fastest, no halo; neighbours
//                 are addressed with periodic wrap inside the kernels.
//   spectrum    : ncomp planes of N*N*NH complex, NH = N/2+1, kx fastest.
//   particles   : structure of arrays (pos x/y/z FP64, vel x/y/z in the form's
//                 real type, int64 ID, uint32 cell key), kept in (cell, ID)
//                 order so that a cell's particles are contiguous and cells
//                 follow the field's memory order.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <string>
#include <vector>

#include "../../include/gev_gb300.h"
#include "../../include/gev_sim.h"

#define GEV_MAX_RADICES 12

struct FftPlan {
  int L;
  int nst;
  int R[GEV_MAX_RADICES];
};

struct GevRecorder;  // gev_batch.cuh

struct gev_ctx {
  int device = 0;
  int N = 0;
  int prec = GEV_PREC_FP64;
  int sms = 0;
  cudaStream_t stream = nullptr;
  // k-space tables (gridk2[N], kshift[N] complex), stored in the form's real type
  void *d_gridk2 = nullptr, *d_kshift = nullptr;
  // twiddles e^{-2 pi i t / L} for L = N and L = N/2
  void *d_twN = nullptr, *d_twH = nullptr;
  // output slot of each frequency after the in-place FFT stages (L = N, N/2)
  void *d_permN = nullptr, *d_permH = nullptr;
  FftPlan planN{}, planH{};
  // scratch: one spectrum component for the input-preserving c2r, deposit cubes,
  // reductions
  void *d_fft_scratch = nullptr;
  size_t fft_scratch_bytes = 0;
  void *d_cube = nullptr;
  size_t cube_bytes = 0;
  double *d_red = nullptr;  // partial sums / max
  size_t red_elems = 0;
  // FP32 FFT tile widths (log2 lines a tile) of the r2c rows, y, z and c2r rows
  // passes, chosen by timing on the first transform (-1: the default)
  int fft_lg[4] = {-1, -1, -1, -1};
  bool fft_tuned = false;
  // FP32 source stencils (scalar, tensor): threads a block and the cap on blocks a
  // SM of their grid-stride launches, chosen by timing on the first call
  int st_threads[2] = {256, 256};
  int st_per_sm[2] = {16, 16};
  bool st_tuned = false;
  long long launches = 0;
  // optional device timing of named regions (gev_ctx_set_timing): a CUDA event
  // pair on the stream around each region, summed per name when the report is read
  struct TimedRegion {
    const char *name;
    cudaEvent_t start, stop;
  };
  bool timing = false;
  std::vector<TimedRegion> timed;
  std::vector<cudaEvent_t> event_pool;
  std::vector<std::string> timed_names;
  std::vector<long> timed_count;
  std::vector<double> timed_ms;
  size_t bytes_in_use = 0;
  std::string err;
  // lifetime: the handle returned by gev_ctx_create holds one reference and
  // every field / particle store / simulation holds one more, so the context's
  // stream and buffers outlive all of them whatever order they are destroyed in
  int refs = 1;
  bool closed = false;
  // set while a cycle is recorded for a batched step (gev_batch.cuh): launches on the
  // batched path are recorded instead of enqueued
  GevRecorder *rec = nullptr;
};

void ctx_retain(gev_ctx *ctx);
void ctx_release(gev_ctx *ctx);

// Times the work a scope enqueues on the context's stream when the context's
// timing is on (an event before and after); costs nothing otherwise.  Names are
// string literals: a kernel's name, or "phase:..." for a phase of main.cpp's
// BENCHMARK breakdown (main.cpp:907-922).
struct GevTimed {
  gev_ctx *ctx;
  long idx = -1;
  GevTimed(gev_ctx *c, const char *name);
  ~GevTimed() { stop(); }
  void stop();  // ends the region before the scope does
  GevTimed(const GevTimed &) = delete;
  GevTimed &operator=(const GevTimed &) = delete;
};

struct gev_field {
  gev_ctx *ctx = nullptr;
  int kind = GEV_FIELD_REAL;
  int ncomp = 0;
  size_t comp_elems = 0;  // real elements or complex elements per component
  size_t elem_bytes = 0;  // sizeof(real) or sizeof(complex)
  void *d = nullptr;
};

struct PclsArrays {
  double *px = nullptr, *py = nullptr, *pz = nullptr;
  void *vx = nullptr, *vy = nullptr, *vz = nullptr;  // real type of the form
  int64_t *id = nullptr;
  uint32_t *cell = nullptr;
  // mixed form only: the position inside the linked cell, pos * N - cell, as
  // FP32.  The FP64 position stays the master state; the drift re-derives the
  // offset from it, and the kick and the deposits read only the offset, so they
  // issue no FP64 instructions (GB300 runs FP64 at 1/64 of the FP32 rate).
  float *rx = nullptr, *ry = nullptr, *rz = nullptr;
  // one allocation holds all the arrays of a set; the store's second set (alt) is
  // written only by a relink, so between relinks the mixed-form deposit keeps its
  // per-particle prefactor records there
  void *block = nullptr;
  size_t block_bytes = 0;
};

struct gev_pcls {
  gev_ctx *ctx = nullptr;
  long n = 0, cap = 0;
  double mass = 0.;
  PclsArrays cur, alt;
  uint32_t *count = nullptr;  // per cell, N^3
  uint32_t *start = nullptr;  // per cell, N^3 + 1
  uint32_t *rank = nullptr;   // per particle
  uint32_t *perm = nullptr;   // per particle
  uint32_t *scan_tmp = nullptr;
  size_t scan_tmp_elems = 0;
  // false after a mixed-form relink that left each cell's run in atomic order
  bool id_order = true;
  // mixed-form deposit scales (16 words): [0] max |q|^2 and [4] max |phi| (FP32 bits),
  // [1] max particles in a cell, [2], [3] the accumulator scale powers of the last
  // deposit's groups, [5..8] their prefactor and weight-factor powers; [15] set by an
  // upload whose particles are not in (cell, ID) order
  uint32_t *bounds = nullptr;
  // mixed-form T00 / Tij deposit: per-particle prefactor records (12 words a particle),
  // kept in the alt array set's block; an allocation of its own only if that is smaller
  void *prep = nullptr;
  // mixed-form gather deposit: the dense-cell tables (cell -> slot, slot -> cell, the
  // slots' corner sums), after the prefactor records in the alt block when it has room,
  // else an allocation of their own
  void *dense = nullptr;
  size_t bytes = 0;  // device bytes this store counts in its context's bytes_in_use
};

// one simulation (include/gev_sim.h)
struct gev_sim {
  gev_ctx *ctx = nullptr;
  gev_pcls *pcls = nullptr;
  gev_field *phi = nullptr, *chi = nullptr, *source = nullptr, *Sij = nullptr, *Bi = nullptr;
  gev_field *scalarFT = nullptr, *SijFT = nullptr, *BiFT = nullptr;
  gev_sim_state st{};
  double *host_words = nullptr;  // pinned: [0] T00 sum, [1] max bits, [2] phi(k=0).re
  double *dev_words = nullptr;
  // gev_sim_step_graph: the executable graph of the last captured cycle, and counts
  // of cycles launched as a graph, instantiations, and cycles enqueued directly
  cudaGraphExec_t gexec = nullptr;
  long graph_launches = 0, graph_builds = 0, graph_direct = 0;
};

// ----------------------------------------------------------------- errors --
#define GEV_CHECK_CUDA(ctx, call)                                                      \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess) {                                                           \
      if (ctx) (ctx)->err = std::string(#call) + ": " + cudaGetErrorString(e_);        \
      return GEV_ECUDA;                                                                \
    }                                                                                  \
  } while (0)

#define GEV_LAUNCH_CHECK(ctx)                                                          \
  do {                                                                                 \
    (ctx)->launches++;                                                                 \
    cudaError_t e_ = cudaGetLastError();                                               \
    if (e_ != cudaSuccess) {                                                           \
      (ctx)->err = std::string("kernel launch: ") + cudaGetErrorString(e_);            \
      return GEV_ECUDA;                                                                \
    }                                                                                  \
  } while (0)

inline int gev_fail(gev_ctx *ctx, int code, const char *msg) {
  if (ctx) ctx->err = msg;
  return code;
}

// ---------------------------------------------------------------- complex --
template <typename R>
struct CT;
template <>
struct CT<double> {
  typedef double2 C;
};
template <>
struct CT<float> {
  typedef float2 C;
};

template <typename C>
__device__ __forceinline__ C cmk(decltype(C::x) r, decltype(C::x) i) {
  C z;
  z.x = r;
  z.y = i;
  return z;
}
template <typename C>
__device__ __forceinline__ C cadd(C a, C b) { return cmk<C>(a.x + b.x, a.y + b.y); }
template <typename C>
__device__ __forceinline__ C csub(C a, C b) { return cmk<C>(a.x - b.x, a.y - b.y); }
template <typename C>
__device__ __forceinline__ C cmul(C a, C b) { return cmk<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
template <typename C>
__device__ __forceinline__ C cconj(C a) { return cmk<C>(a.x, -a.y); }
template <typename C>
__device__ __forceinline__ C cscale(decltype(C::x) d, C a) { return cmk<C>(d * a.x, d * a.y); }

// --------------------------------------------------------------- indexing --
__device__ __forceinline__ int wrapi(int i, int N) { return i < 0 ? i + N : (i >= N ? i - N : i); }
__device__ __forceinline__ size_t sidx(int x, int y, int z, int N) {
  return (size_t)x + (size_t)N * ((size_t)y + (size_t)N * (size_t)z);
}

// lg of N when N is a power of two, else -1
__host__ __device__ inline int lg_pow2(int N) {
  int l = 0;
  while ((1 << l) < N) ++l;
  return (1 << l) == N ? l : -1;
}

// f * 2^-24 for a 24-bit f, built from bits (an int -> float conversion issues on
// the FP64 pipe on GB300): (f >> 1) * 2^-23 = (1 + (f >> 1) 2^-23) - 1 exactly, plus
// the last bit; every step is exact, so the result equals (float)f * 2^-24.
__device__ __forceinline__ float frac24(unsigned f) {
  float r = __uint_as_float(0x3F800000u | (f >> 1)) - 1.0f;
  if (f & 1u) r += 5.9604644775390625e-8f;
  return r;
}

// (double)f from bits, without the float -> double conversion instruction
__device__ __forceinline__ double f2d_bits(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned e = (b >> 23) & 0xffu;
  const unsigned long long s = (unsigned long long)(b >> 31) << 63;
  unsigned long long m = b & 0x7fffffu;
  unsigned long long d;
  if (e == 0u) {
    if (m == 0ull) {
      d = s;
    } else {  // subnormal float: normalise (a normal double)
      const int sh = __clz((int)m) - 8;
      m = (m << sh) & 0x7fffffull;
      d = s | ((unsigned long long)(1023 - 126 - sh) << 52) | (m << 29);
    }
  } else if (e == 0xffu) {
    d = s | (0x7ffull << 52) | (m << 29);
  } else {
    d = s | ((unsigned long long)(e - 127u + 1023u) << 52) | (m << 29);
  }
  return __longlong_as_double((long long)d);
}

// cell = floor(x N) (clamped to N-1) and r = x N - cell as FP32, for x in [0, 1).
// With N = 2^lg the split reads the double's bits (x N is an exact exponent
// shift), so it issues no FP64 instruction; r keeps the leading 24 bits of the
// fraction.  Other N use FP64 arithmetic.
__device__ __forceinline__ void pos_split(double x, int N, int lg, int &c, float &r) {
  if (lg >= 0) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7ff);
    const int sh = 1075 - e - lg;  // x N = m * 2^-sh, m the 53-bit significand; x < 1 gives sh >= 53 - lg
    if (e == 0 || sh >= 88) {       // zero, denormal, or x N < 2^-35
      c = 0;
      r = 0.f;
      return;
    }
    const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
    if (sh >= 64) {
      c = 0;
      r = frac24((unsigned)(m >> (sh - 24)));
    } else {
      c = (int)(m >> sh);
      const unsigned long long frac = m & ((1ull << sh) - 1ull);
      r = frac24((unsigned)(frac >> (sh - 24)));
    }
    if (c >= N) {
      c = N - 1;
      r = 1.f;
    }
  } else {
    const double xn = x * (double)N;
    c = (int)xn;
    if (c >= N) c = N - 1;
    if (c < 0) c = 0;
    r = (float)(xn - (double)c);
  }
}

// periodic wrap into [0, 1), deciding on the bit pattern (integer compares) and
// with one FP64 add whose addend is selected (+1 below 0, -1 at 1 and above, 0
// otherwise: x + 0 is x), so that no predicated FP64 instructions are issued; a
// tiny negative x whose x + 1 rounds to 1 gives 0, as moveParticles' second test does
__device__ __forceinline__ double wrap01_bits(double x) {
  const long long b = __double_as_longlong(x);
  const bool neg = b < 0, big = b >= 0x3FF0000000000000ll;  // sign bit set (incl. -0) / x >= 1
  double y = x + (neg ? 1.0 : (big ? -1.0 : 0.0));
  if (neg && __double_as_longlong(y) >= 0x3FF0000000000000ll) y = 0.0;
  return y;
}

// v * 2^-k rounded once to the nearest FP32 (ties to even): the int64 -> FP32
// conversion rounds v, and the power-of-two factor is exact because the product
// stays normal -- |RN(v)| lies in [1, 2^63] for v != 0, so for -64 <= k <= 126 the
// result lies in [2^-126, 2^127].  The deposit scales keep k = kq + kg in [-64, 121]
// (fx_group in gev_deposit_fx.cu).  One conversion and one
// multiply; the same bits as building the float from v's leading bits with
// integer instructions (about twenty a value), and 0.36 ms less per 512^3 cycle,
// whose T00 + Tij gather converts seven sums a node.
__device__ __forceinline__ float float_of_fixed(long long v, int k) {
  return __fmul_rn(__ll2float_rn(v), __int_as_float((127 - k) << 23));
}

// n / d for every 32-bit n with one multiply-high (division by an invariant
// integer, round-up method): m = floor(2^32 (2^l - d) / d) + 1, l = ceil(log2 d)
struct Div32 {
  unsigned d = 1, m = 1;
  int s1 = 0, s2 = 0;
};
inline Div32 make_div32(unsigned d) {
  Div32 v;
  v.d = d;
  int l = 0;
  while ((1ull << l) < d) ++l;
  v.m = (unsigned)((((1ull << 32) * ((1ull << l) - d)) / d) + 1);
  v.s1 = l < 1 ? l : 1;
  v.s2 = l - 1 > 0 ? l - 1 : 0;
  return v;
}
__device__ __forceinline__ unsigned div32(unsigned n, const Div32 &v) {
  const unsigned t = __umulhi(v.m, n);
  return (t + ((n - t) >> v.s1)) >> v.s2;
}

// the periodic neighbours of cell i = x + N (y + N z) as index offsets modulo 2^32
// (N^3 < 2^32): f[i + xp] is f(x + 1, y, z) and so on
struct Nb3 {
  unsigned i, xm, xp, ym, yp, zm, zp;
};
__device__ __forceinline__ Nb3 nb3(unsigned i, int x, int y, int z, int N) {
  const unsigned n1 = (unsigned)N, n2 = n1 * n1, n3 = n2 * n1;
  Nb3 b;
  b.i = i;
  b.xm = x == 0 ? n1 - 1u : 0u - 1u;
  b.xp = x == N - 1 ? 1u - n1 : 1u;
  b.ym = y == 0 ? n2 - n1 : 0u - n1;
  b.yp = y == N - 1 ? n1 - n2 : n1;
  b.zm = z == 0 ? n3 - n2 : 0u - n2;
  b.zp = z == N - 1 ? n2 - n3 : n2;
  return b;
}
// x, y, z of cell i: shifts for a power-of-two N, else two invariant divisions
__device__ __forceinline__ void cell_xyz(unsigned i, int N, int lg, const Div32 &dN, int &x, int &y, int &z) {
  if (lg >= 0) {
    x = (int)(i & (unsigned)(N - 1));
    y = (int)((i >> lg) & (unsigned)(N - 1));
    z = (int)(i >> (2 * lg));
  } else {
    const unsigned r = div32(i, dN), q = div32(r, dN);
    x = (int)(i - r * (unsigned)N);
    y = (int)(r - q * (unsigned)N);
    z = (int)q;
  }
}

inline int grid_for(const gev_ctx *ctx, size_t work, int threads, int per_sm = 8) {
  size_t blocks = (work + threads - 1) / threads;
  size_t cap = (size_t)ctx->sms * per_sm;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  return (int)blocks;
}

// ---------------------------------------------------------- internal API --
// (implemented in the .cu files; all enqueue on ctx->stream)
int fft_build_plan(int L, FftPlan *pl);
int fft_r2c_comp(gev_ctx *ctx, const void *real, void *spec);
int fft_c2r_comp(gev_ctx *ctx, const void *spec, void *real, void *scratch);
// register-resident passes for power-of-two lengths 8..1024 (gev_fft_reg.cu)
bool fft_reg_ok(int L);
int fft_cols_reg(gev_ctx *ctx, const void *in, void *out, long ES, long PS, int sign);
int fft_r2c_rows_reg(gev_ctx *ctx, const void *real, void *spec);
int fft_c2r_rows_reg(gev_ctx *ctx, const void *spec, void *real);
// times the FP32 tile-width candidates of each pass once per context (a no-op after
// the first call and for FP64)
void fft_autotune(gev_ctx *ctx);
// FP32, power-of-two N: the backward z pass of a spectrum into out with
// solveModifiedPoissonFT's factor (coeff already divided by -N^3) applied on load
int fft_cols_z_poisson(gev_ctx *ctx, const void *spec, void *out, double coeff, double modif);
int fft_c2r_poisson_comp(gev_ctx *ctx, const void *srcFT, void *real, double coeff, double modif);
int kspace_poisson_raw(gev_ctx *ctx, const void *in, void *out, double coeff, double modif);
int pcls_relink(gev_ctx *ctx, gev_pcls *p);
int pcls_id_order(gev_ctx *ctx, gev_pcls *p);
int pcls_unpack_at(gev_ctx *ctx, gev_pcls *p, const gev_part *d, long count, long offset);
int pcls_pack_range(gev_ctx *ctx, gev_pcls *p, gev_part *d, long i0, long count);
int ctx_ensure_cube(gev_ctx *ctx, size_t bytes);
int ctx_ensure_red(gev_ctx *ctx, size_t elems);
// the deposit of kind 0 T00, 1 T0i, 2 Tij, 3 mass (coefficient 1) replacing the
// target's contents: projection_init + projection_*_project + _comm in one call
int projection_replace(gev_ctx *ctx, gev_pcls *p, gev_field *out, int kind, double a, const gev_field *phi);
int projection_replace_t00_tij(gev_ctx *ctx, gev_pcls *p, gev_field *T00, gev_field *Tij, double a,
                               const gev_field *phi);
