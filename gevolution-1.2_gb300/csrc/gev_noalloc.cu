// gev_noalloc.cu -- gev_sum_noalloc: the field reduction (T00hom-style sum of one
// component) for callers that must not allocate device memory.
//
// Who cannot allocate: a host code that embeds this library inside its own time
// step usually sizes its fields to fill the GPU and hands all device memory to
// its own pool (or to PyTorch's caching allocator).  A cudaMalloc behind that
// pool's back can fail for lack of memory even though the pool has room, and
// cudaMalloc / cudaFree may synchronise the whole device, which stalls a time
// step whose kernels are queued ahead.  Such a caller owns the input and output
// buffers already; this entry point needs nothing else from it.
//
// The scratch (one FP64 partial sum per chunk of SUM_CHUNK values) lives in a
// file-scope __device__ array of SUM_MAX_PARTIALS doubles (1 MiB).  Every GPU
// that loads the library holds that megabyte until the process exits.  In host
// code the array's name is only a host-side stand-in, not a device address, so
// the host side looks the device address up with cudaGetSymbolAddress, once per
// device, with that device current, and passes it to the kernels.  CUDA loads
// modules and kernels lazily (the default since CUDA 12.2), and loading places
// the array and the kernels on the GPU, which allocates; the same set-up
// therefore loads all three kernels (cudaFuncGetAttributes), so that no later
// call, whatever its n or precision, loads anything.
#include <mutex>

#include "gev_internal.cuh"

namespace {

constexpr int SUM_THREADS = 256;
constexpr size_t SUM_CHUNK = 8192;               // values per partial sum (32 per thread)
constexpr size_t SUM_MAX_PARTIALS = 131072;      // 2^17 doubles = 1 MiB of scratch
constexpr int SUM_MAX_DEVICES = 64;

static_assert(SUM_CHUNK * SUM_MAX_PARTIALS == (size_t)GEV_SUM_NOALLOC_MAX_N,
              "the header's limit must match the scratch size");

static __device__ __align__(256) double g_sum_partials[SUM_MAX_PARTIALS];

// Block b sums values [b*SUM_CHUNK, min((b+1)*SUM_CHUNK, n)) in FP64: thread t
// takes every SUM_THREADS-th value from t (coalesced), then a fixed tree.  The
// partition depends only on n, so the result is the same on every GPU model and
// launch configuration.
template <typename T>
__global__ void __launch_bounds__(SUM_THREADS) k_sum_chunks(const T *__restrict__ f, size_t n,
                                                            double *__restrict__ partial) {
  __shared__ double sh[SUM_THREADS];
  const size_t base = (size_t)blockIdx.x * SUM_CHUNK;
  const size_t end = base + SUM_CHUNK < n ? base + SUM_CHUNK : n;
  double s = 0.;
#pragma unroll 8
  for (size_t i = base + threadIdx.x; i < end; i += SUM_THREADS) s += (double)f[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = SUM_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

// One block adds the np partials in a fixed order and writes out[0] (0 for np = 0).
__global__ void __launch_bounds__(1024) k_sum_partials(const double *__restrict__ partial, int np,
                                                       double *__restrict__ out) {
  __shared__ double sh[1024];
  double s = 0.;
  for (int i = threadIdx.x; i < np; i += 1024) s += partial[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = 512; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = sh[0];
}

std::mutex g_addr_mu;
void *g_addr[SUM_MAX_DEVICES] = {};

int say(char *errbuf, size_t errlen, int code, const char *fmt, long long a = 0, long long b = 0) {
  if (errbuf && errlen) snprintf(errbuf, errlen, fmt, a, b);
  return code;
}

}  // namespace

extern "C" int gev_sum_noalloc(int device, const void *data, int precision, size_t n, double *out, void *cuda_stream,
                               char *errbuf, size_t errbuf_len) {
  if (errbuf && errbuf_len) errbuf[0] = 0;
  if (device < 0 || device >= SUM_MAX_DEVICES)
    return say(errbuf, errbuf_len, GEV_EINVAL, "sum_noalloc: device %lld outside 0..%lld", device,
               SUM_MAX_DEVICES - 1);
  if (precision != GEV_PREC_FP64 && precision != GEV_PREC_MIXED)
    return say(errbuf, errbuf_len, GEV_EINVAL, "sum_noalloc: precision %lld is neither FP64 (0) nor mixed (1)",
               precision);
  if (!out || (n && !data)) return say(errbuf, errbuf_len, GEV_EINVAL, "sum_noalloc: null data or out pointer");
  if (n > (size_t)GEV_SUM_NOALLOC_MAX_N)
    return say(errbuf, errbuf_len, GEV_EINVAL,
               "sum_noalloc: n = %lld values exceeds the limit of %lld (2^30) that its fixed 1 MiB scratch serves",
               (long long)n, (long long)GEV_SUM_NOALLOC_MAX_N);

  int prev = -1;
  if (cudaGetDevice(&prev) != cudaSuccess) return say(errbuf, errbuf_len, GEV_ENODEV, "sum_noalloc: no CUDA device");
  if (prev != device && cudaSetDevice(device) != cudaSuccess)
    return say(errbuf, errbuf_len, GEV_ENODEV, "sum_noalloc: cannot make device %lld current", device);

  int rc = GEV_OK;
  double *partials = nullptr;
  {
    // set-up on the first call on this device: the device address of the scratch
    std::lock_guard<std::mutex> lk(g_addr_mu);
    if (!g_addr[device]) {
      void *p = nullptr;
      cudaFuncAttributes fa;
      cudaError_t e = cudaFuncGetAttributes(&fa, k_sum_chunks<double>);
      if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_sum_chunks<float>);
      if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_sum_partials);
      if (e == cudaSuccess) e = cudaGetSymbolAddress(&p, g_sum_partials);
      if (e != cudaSuccess || !p) {
        if (errbuf && errbuf_len)
          snprintf(errbuf, errbuf_len, "sum_noalloc: set-up (kernel load / cudaGetSymbolAddress): %s",
                   cudaGetErrorString(e));
        rc = GEV_ECUDA;
      } else {
        g_addr[device] = p;
      }
    }
    partials = (double *)g_addr[device];
  }
  if (rc == GEV_OK) {
    cudaStream_t st = (cudaStream_t)cuda_stream;
    const size_t np = (n + SUM_CHUNK - 1) / SUM_CHUNK;  // <= SUM_MAX_PARTIALS by the check above
    // every partial the second kernel reads is written by the first one of the same
    // call, so nothing left in the scratch by an earlier call is ever read
    if (np) {
      if (precision == GEV_PREC_FP64)
        k_sum_chunks<double><<<(unsigned)np, SUM_THREADS, 0, st>>>((const double *)data, n, partials);
      else
        k_sum_chunks<float><<<(unsigned)np, SUM_THREADS, 0, st>>>((const float *)data, n, partials);
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) {
      k_sum_partials<<<1, 1024, 0, st>>>(partials, (int)np, out);
      e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
      if (errbuf && errbuf_len) snprintf(errbuf, errbuf_len, "sum_noalloc: kernel launch: %s", cudaGetErrorString(e));
      rc = GEV_ECUDA;
    }
  }
  if (prev != device) cudaSetDevice(prev);
  return rc;
}
