// gev_batch.cuh -- batched launches: one launch per kernel of a cycle for a cohort of
// simulations of one grid size (include/gev_sim.h, gev_batch_step).
//
// A kernel that takes part keeps its __global__ form for the ordinary launch and has
// its code in a __device__ body function of the same parameters; gev_launch either
// launches the kernel on the context's stream or, while the context records a cycle
// (ctx->rec set), records the body's launch: its grid, block and shared memory and
// its arguments packed into a trivially copyable struct.  The executor (gev_batch.cu)
// lays the packed arguments of a cohort's simulations side by side in a device table
// and launches the body's batched form once, gridDim.y = the cohort's size, each block
// reading its simulation's arguments from the table row blockIdx.y.  A body never
// reads blockIdx.y or gridDim.y, so inside it the launch looks like the ordinary one.
#pragma once

#include <atomic>
#include <cstring>
#include <vector>

#include "gev_internal.cuh"

// ------------------------------------------------------------ argument pack --
template <typename... A>
struct GevPack {};
template <>
struct GevPack<> {
  GevPack() = default;
};
template <typename H, typename... T>
struct GevPack<H, T...> {
  H h;
  GevPack<T...> t;
  GevPack() = default;
  template <typename X, typename... Y>
  __host__ __device__ GevPack(X x, Y... y) : h(x), t(y...) {}
};

template <auto F, typename... Done>
__device__ __forceinline__ void gev_apply(const GevPack<> &, const Done &...d) {
  F(d...);
}
template <auto F, typename H, typename... T, typename... Done>
__device__ __forceinline__ void gev_apply(const GevPack<H, T...> &p, const Done &...d) {
  gev_apply<F>(p.t, d..., p.h);
}

template <typename Sig>
struct GevBodyArgs;
template <typename... A>
struct GevBodyArgs<void (*)(A...)> {
  typedef GevPack<A...> type;
};

// the batched form of body F: block (x, s) runs F with simulation s's arguments, read
// once into locals.  It is compiled apart from the kernel, with the arguments as loads
// rather than parameters, so where a body leaves the pairing of multiplies and adds
// to the compiler (the FP32 stencils, transforms, k-space operators and the kick and
// drift) its fused multiply-adds may pair differently: the results then differ from
// the kernel's in the last bits.  Bodies written with explicitly rounded intrinsics
// (the fixed-point deposits, the sums) give the same bits either way.
template <auto F, int MT, int MB>
__global__ void __launch_bounds__(MT, MB)
    k_batched(const typename GevBodyArgs<decltype(F)>::type *__restrict__ tab) {
  const typename GevBodyArgs<decltype(F)>::type a = tab[blockIdx.y];
  gev_apply<F>(a);
}

typedef void (*GevBatchLaunch)(const void *tab, unsigned nsims, dim3 grid, dim3 block, size_t smem, cudaStream_t st);

template <auto F, int MT, int MB>
void gev_launch_batched(const void *tab, unsigned nsims, dim3 grid, dim3 block, size_t smem, cudaStream_t st) {
  typedef typename GevBodyArgs<decltype(F)>::type P;
  if (smem > 48 * 1024) {  // once per process: the batched form's dynamic shared memory limit
    static std::atomic<bool> set{false};
    if (!set.load(std::memory_order_relaxed)) {
      cudaFuncSetAttribute(k_batched<F, MT, MB>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
      set.store(true, std::memory_order_relaxed);
    }
  }
  k_batched<F, MT, MB><<<dim3(grid.x, nsims), block, smem, st>>>((const P *)tab);
}

// ---------------------------------------------------------------- recorder --
// One recorded operation of a cycle: a kernel (its batched form's launcher and packed
// arguments) or a device -> host copy.
struct GevOp {
  GevBatchLaunch launch = nullptr;  // nullptr: a copy
  dim3 grid, block;
  size_t smem = 0;
  size_t off = 0, bytes = 0;        // packed arguments in GevRecorder::args
  void *dst = nullptr;              // copy: host destination, device source
  const void *src = nullptr;
};

struct GevRecorder {
  std::vector<GevOp> ops;
  std::vector<unsigned char> args;
  bool bad = false;  // an operation that cannot be batched was recorded

  void clear() {
    ops.clear();
    args.clear();
    bad = false;
  }
  template <auto F, int MT, int MB, typename... A>
  void add(dim3 grid, dim3 block, size_t smem, A... a) {
    typedef typename GevBodyArgs<decltype(F)>::type P;
    static_assert(alignof(P) <= 16, "argument pack alignment");
    if (grid.y != 1 || grid.z != 1) bad = true;
    const P pk(a...);
    GevOp op;
    op.launch = &gev_launch_batched<F, MT, MB>;
    op.grid = grid;
    op.block = block;
    op.smem = smem;
    op.off = (args.size() + 15) & ~(size_t)15;
    op.bytes = sizeof(P);
    args.resize(op.off + sizeof(P));
    memcpy(args.data() + op.off, &pk, sizeof(P));
    ops.push_back(op);
  }
  void add_copy(void *dst, const void *src, size_t bytes) {
    GevOp op;
    op.dst = dst;
    op.src = src;
    op.bytes = bytes;
    ops.push_back(op);
  }
};

// Launches kernel `kern`, whose code is the body F, on the context's stream -- or
// records F's launch while the context records a cycle.  MT and MB are the
// kernel's launch bounds (MB = 1 where it names none).
template <auto F, int MT, int MB, typename K, typename... A>
inline void gev_launch(gev_ctx *ctx, K kern, dim3 grid, dim3 block, size_t smem, A... a) {
  if (ctx->rec)
    ctx->rec->template add<F, MT, MB>(grid, block, smem, a...);
  else
    kern<<<grid, block, smem, ctx->stream>>>(a...);
}

// gev_launch where B, else the plain launch (no batched form is compiled: the FP64
// form's kernels are never batched)
template <bool B, auto F, int MT, int MB, typename K, typename... A>
inline void gev_launch_if(gev_ctx *ctx, K kern, dim3 grid, dim3 block, size_t smem, A... a) {
  if constexpr (B)
    gev_launch<F, MT, MB>(ctx, kern, grid, block, smem, a...);
  else
    kern<<<grid, block, smem, ctx->stream>>>(a...);
}

// cudaMemsetAsync to zero, or the same as a recorded kernel (bytes a multiple of 4,
// the pointer 4-byte aligned)
__device__ __forceinline__ void k_zero4_body(uint32_t *p, size_t n4) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4; i += (size_t)gridDim.x * blockDim.x) p[i] = 0u;
}
__global__ void __launch_bounds__(256) k_zero4(uint32_t *p, size_t n4);
inline cudaError_t gev_zero_async(gev_ctx *ctx, void *p, size_t bytes) {
  if (!ctx->rec) return cudaMemsetAsync(p, 0, bytes, ctx->stream);
  if (bytes % 4 != 0 || ((uintptr_t)p & 3u) != 0) {
    ctx->rec->bad = true;
    return cudaSuccess;
  }
  gev_launch<k_zero4_body, 256, 1>(ctx, k_zero4, dim3(grid_for(ctx, bytes / 4, 256, 8)), dim3(256), 0,
                                   (uint32_t *)p, bytes / 4);
  return cudaSuccess;
}

// cudaMemcpyAsync device -> host, or the same recorded
inline cudaError_t gev_d2h_async(gev_ctx *ctx, void *dst, const void *src, size_t bytes) {
  if (!ctx->rec) return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream);
  ctx->rec->add_copy(dst, src, bytes);
  return cudaSuccess;
}
