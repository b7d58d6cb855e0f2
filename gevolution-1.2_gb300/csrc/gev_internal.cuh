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

#define GEV_MAX_RADICES 12

struct FftPlan {
  int L;
  int nst;
  int R[GEV_MAX_RADICES];
};

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
  FftPlan planN{}, planH{};
  // scratch: one spectrum component for the input-preserving c2r, deposit cubes,
  // reductions
  void *d_fft_scratch = nullptr;
  size_t fft_scratch_bytes = 0;
  void *d_cube = nullptr;
  size_t cube_bytes = 0;
  double *d_red = nullptr;  // partial sums / max
  size_t red_elems = 0;
  long long launches = 0;
  size_t bytes_in_use = 0;
  std::string err;
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
  uint32_t *big = nullptr;    // list of cells needing the block-wide ID sort (+1 counter)
  uint32_t *scan_tmp = nullptr;
  size_t scan_tmp_elems = 0;
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
int pcls_relink(gev_ctx *ctx, gev_pcls *p);
int ctx_ensure_cube(gev_ctx *ctx, size_t bytes);
int ctx_ensure_red(gev_ctx *ctx, size_t elems);
