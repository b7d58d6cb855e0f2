// gev_capi.cu -- context, field and FFT entry points of the C-ABI
// (include/gev_gb300.h).  The context owns the stream, the k-space and twiddle
// tables, and the scratch buffers (c2r staging spectrum, deposit cubes,
// reduction words); fields are plain device arrays in the layouts of
// gev_internal.cuh.
#include <cmath>
#include <cstring>
#include <vector>

#include "gev_internal.cuh"

int fft_init_kernels(int prec);
void fft_perm(const FftPlan &pl, std::vector<unsigned short> &perm);

namespace {

// gridk2 / kshift exactly as gevolution.hpp:222-227 builds them
template <typename T>
void kspace_tables(int N, std::vector<T> &g, std::vector<T> &ks) {
  g.resize(N);
  ks.resize(2 * N);
  for (int i = 0; i < N; i++) {
    double gi = 2. * (double)N * sin(M_PI * (double)i / (double)N);
    ks[2 * i] = (T)(gi * cos(M_PI * (double)i / (double)N));
    ks[2 * i + 1] = (T)(gi * -sin(M_PI * (double)i / (double)N));
    g[i] = (T)(gi * gi);
  }
}

template <typename T>
void twiddles(int L, std::vector<T> &tw) {
  tw.resize(2 * (size_t)L);
  for (int j = 0; j < L; j++) {
    long double ang = 2.0L * 3.14159265358979323846264338327950288L * (long double)j / (long double)L;
    tw[2 * j] = (T)cosl(ang);
    tw[2 * j + 1] = (T)-sinl(ang);
  }
}

template <typename T>
int upload_tables(gev_ctx *ctx) {
  std::vector<T> g, ks, twN, twH;
  kspace_tables<T>(ctx->N, g, ks);
  twiddles<T>(ctx->N, twN);
  twiddles<T>(ctx->N / 2, twH);
  const size_t sz = sizeof(T);
  GEV_CHECK_CUDA(ctx, cudaMalloc(&ctx->d_gridk2, g.size() * sz));
  GEV_CHECK_CUDA(ctx, cudaMalloc(&ctx->d_kshift, ks.size() * sz));
  GEV_CHECK_CUDA(ctx, cudaMalloc(&ctx->d_twN, twN.size() * sz));
  GEV_CHECK_CUDA(ctx, cudaMalloc(&ctx->d_twH, twH.size() * sz));
  GEV_CHECK_CUDA(ctx, cudaMemcpy(ctx->d_gridk2, g.data(), g.size() * sz, cudaMemcpyHostToDevice));
  GEV_CHECK_CUDA(ctx, cudaMemcpy(ctx->d_kshift, ks.data(), ks.size() * sz, cudaMemcpyHostToDevice));
  GEV_CHECK_CUDA(ctx, cudaMemcpy(ctx->d_twN, twN.data(), twN.size() * sz, cudaMemcpyHostToDevice));
  GEV_CHECK_CUDA(ctx, cudaMemcpy(ctx->d_twH, twH.data(), twH.size() * sz, cudaMemcpyHostToDevice));
  std::vector<unsigned short> pN, pH;
  fft_perm(ctx->planN, pN);
  fft_perm(ctx->planH, pH);
  GEV_CHECK_CUDA(ctx, cudaMalloc(&ctx->d_permN, pN.size() * 2));
  GEV_CHECK_CUDA(ctx, cudaMalloc(&ctx->d_permH, pH.size() * 2));
  GEV_CHECK_CUDA(ctx, cudaMemcpy(ctx->d_permN, pN.data(), pN.size() * 2, cudaMemcpyHostToDevice));
  GEV_CHECK_CUDA(ctx, cudaMemcpy(ctx->d_permH, pH.data(), pH.size() * 2, cudaMemcpyHostToDevice));
  return GEV_OK;
}

size_t real_size(const gev_ctx *ctx) { return ctx->prec == GEV_PREC_FP64 ? 8 : 4; }

template <typename T>
__global__ void k_from_double(const double *__restrict__ in, T *out, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = (T)in[i];
}
template <typename T>
__global__ void k_to_double(const T *__restrict__ in, double *out, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = (double)in[i];
}

}  // namespace

int ctx_ensure_cube(gev_ctx *ctx, size_t bytes) {
  if (ctx->cube_bytes >= bytes) return GEV_OK;
  if (ctx->d_cube) {
    GEV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    cudaFree(ctx->d_cube);
    ctx->bytes_in_use -= ctx->cube_bytes;
    ctx->d_cube = nullptr;
    ctx->cube_bytes = 0;
  }
  if (cudaMalloc(&ctx->d_cube, bytes) != cudaSuccess) {
    cudaGetLastError();
    return gev_fail(ctx, GEV_ENOMEM, "deposit scratch allocation failed");
  }
  ctx->cube_bytes = bytes;
  ctx->bytes_in_use += bytes;
  return GEV_OK;
}

int ctx_ensure_red(gev_ctx *ctx, size_t elems) {
  if (ctx->red_elems >= elems) return GEV_OK;
  if (ctx->d_red) {
    GEV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    cudaFree(ctx->d_red);
  }
  ctx->d_red = nullptr;
  ctx->red_elems = 0;
  if (cudaMalloc(&ctx->d_red, elems * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    return gev_fail(ctx, GEV_ENOMEM, "reduction scratch allocation failed");
  }
  ctx->red_elems = elems;
  return GEV_OK;
}

void ctx_retain(gev_ctx *ctx) { ctx->refs++; }

static cudaEvent_t timer_event(gev_ctx *ctx) {
  if (!ctx->event_pool.empty()) {
    cudaEvent_t e = ctx->event_pool.back();
    ctx->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return e;
}

GevTimed::GevTimed(gev_ctx *c, const char *name) : ctx(c) {
  if (!ctx || !ctx->timing) return;
  gev_ctx::TimedRegion r{name, timer_event(ctx), timer_event(ctx)};
  if (!r.start || !r.stop) return;
  cudaEventRecord(r.start, ctx->stream);
  idx = (long)ctx->timed.size();
  ctx->timed.push_back(r);
}

void GevTimed::stop() {
  if (idx >= 0) cudaEventRecord(ctx->timed[(size_t)idx].stop, ctx->stream);
  idx = -1;
}

// waits for the stream and folds the recorded regions into the per-name sums
static int timer_collect(gev_ctx *ctx) {
  GEV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  for (const auto &r : ctx->timed) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, r.start, r.stop) != cudaSuccess) {
      cudaGetLastError();
      ms = 0.f;
    }
    size_t k = 0;
    while (k < ctx->timed_names.size() && ctx->timed_names[k] != r.name) ++k;
    if (k == ctx->timed_names.size()) {
      ctx->timed_names.push_back(r.name);
      ctx->timed_count.push_back(0);
      ctx->timed_ms.push_back(0.);
    }
    ctx->timed_count[k] += 1;
    ctx->timed_ms[k] += (double)ms;
    ctx->event_pool.push_back(r.start);
    ctx->event_pool.push_back(r.stop);
  }
  ctx->timed.clear();
  return GEV_OK;
}

void ctx_release(gev_ctx *ctx) {
  if (--ctx->refs > 0) return;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  cudaFree(ctx->d_gridk2);
  cudaFree(ctx->d_kshift);
  cudaFree(ctx->d_twN);
  cudaFree(ctx->d_twH);
  cudaFree(ctx->d_permN);
  cudaFree(ctx->d_permH);
  cudaFree(ctx->d_fft_scratch);
  cudaFree(ctx->d_cube);
  cudaFree(ctx->d_red);
  for (const auto &r : ctx->timed) {
    cudaEventDestroy(r.start);
    cudaEventDestroy(r.stop);
  }
  for (cudaEvent_t e : ctx->event_pool) cudaEventDestroy(e);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

extern "C" {

const char *gev_strerror(int s) {
  switch (s) {
    case GEV_OK:
      return "ok";
    case GEV_EINVAL:
      return "invalid argument";
    case GEV_ENOMEM:
      return "device out of memory";
    case GEV_ECUDA:
      return "CUDA error";
    case GEV_ETIMEOUT:
      return "device wait timed out";
    case GEV_ENODEV:
      return "no usable CUDA device";
    default:
      return "unknown status";
  }
}

int gev_ctx_create(int device, int N, int precision, gev_ctx **out) {
  if (!out) return GEV_EINVAL;
  *out = nullptr;
  // N^3 < 2^32: cell keys and field indices are 32-bit
  if (N < 8 || N > 1536 || N % 2 != 0 || (precision != GEV_PREC_FP64 && precision != GEV_PREC_MIXED))
    return GEV_EINVAL;
  FftPlan pN, pH;
  if (fft_build_plan(N, &pN) != GEV_OK || fft_build_plan(N / 2, &pH) != GEV_OK) return GEV_EINVAL;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= device || device < 0) {
    cudaGetLastError();
    return GEV_ENODEV;
  }
  if (cudaSetDevice(device) != cudaSuccess) return GEV_ENODEV;
  gev_ctx *ctx = new gev_ctx();
  ctx->device = device;
  ctx->N = N;
  ctx->prec = precision;
  ctx->planN = pN;
  ctx->planH = pH;
  cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, device);
  int rc = GEV_OK;
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) rc = GEV_ECUDA;
  if (!rc) rc = precision == GEV_PREC_FP64 ? upload_tables<double>(ctx) : upload_tables<float>(ctx);
  if (!rc) rc = fft_init_kernels(precision);
  if (!rc) {
    const size_t spec = (size_t)N * N * (N / 2 + 1) * 2 * real_size(ctx);
    if (cudaMalloc(&ctx->d_fft_scratch, spec) != cudaSuccess)
      rc = GEV_ENOMEM;
    else {
      ctx->fft_scratch_bytes = spec;
      ctx->bytes_in_use += spec;
    }
  }
  if (!rc) rc = ctx_ensure_red(ctx, 1024);
  if (rc) {
    cudaGetLastError();
    gev_ctx_destroy(ctx);
    return rc;
  }
  *out = ctx;
  return GEV_OK;
}

int gev_ctx_destroy(gev_ctx *ctx) {
  if (!ctx) return GEV_OK;
  if (!ctx->closed) {
    ctx->closed = true;
    ctx_release(ctx);
  }
  return GEV_OK;
}

int gev_ctx_sync(gev_ctx *ctx) {
  if (!ctx) return GEV_EINVAL;
  GEV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return GEV_OK;
}

int gev_ctx_stream(gev_ctx *ctx, void **s) {
  if (!ctx || !s) return GEV_EINVAL;
  *s = (void *)ctx->stream;
  return GEV_OK;
}

int gev_ctx_info(gev_ctx *ctx, int *N, int *precision, size_t *bytes) {
  if (!ctx) return GEV_EINVAL;
  if (N) *N = ctx->N;
  if (precision) *precision = ctx->prec;
  if (bytes) *bytes = ctx->bytes_in_use;
  return GEV_OK;
}

const char *gev_ctx_last_error(gev_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int gev_ctx_launch_count(gev_ctx *ctx, long long *count) {
  if (!ctx || !count) return GEV_EINVAL;
  *count = ctx->launches;
  return GEV_OK;
}

int gev_ctx_set_timing(gev_ctx *ctx, int on) {
  if (!ctx) return GEV_EINVAL;
  if (!on && ctx->timing) {
    const int rc = timer_collect(ctx);
    if (rc) return rc;
  }
  ctx->timing = on != 0;
  return GEV_OK;
}

int gev_ctx_timing_report(gev_ctx *ctx, char *buf, size_t len, int reset) {
  if (!ctx || (!buf && len)) return GEV_EINVAL;
  const int rc = timer_collect(ctx);
  if (rc) return rc;
  std::string out;
  char line[256];
  for (size_t k = 0; k < ctx->timed_names.size(); ++k) {
    snprintf(line, sizeof line, "%s\t%ld\t%.6f\n", ctx->timed_names[k].c_str(), ctx->timed_count[k],
             ctx->timed_ms[k]);
    out += line;
  }
  if (len) {
    const size_t n = out.size() < len - 1 ? out.size() : len - 1;
    memcpy(buf, out.data(), n);
    buf[n] = 0;
  }
  if (reset) {
    ctx->timed_names.clear();
    ctx->timed_count.clear();
    ctx->timed_ms.clear();
  }
  return out.size() < len ? GEV_OK : gev_fail(ctx, GEV_EINVAL, "timing_report: buffer too small");
}

int gev_field_create(gev_ctx *ctx, int kind, int ncomp, gev_field **out) {
  if (!ctx || !out || ncomp < 1 || ncomp > 16 || (kind != GEV_FIELD_REAL && kind != GEV_FIELD_SPECTRUM))
    return gev_fail(ctx, GEV_EINVAL, "field_create: bad kind or component count");
  const int N = ctx->N;
  gev_field *f = new gev_field();
  f->ctx = ctx;
  ctx_retain(ctx);
  f->kind = kind;
  f->ncomp = ncomp;
  f->comp_elems = kind == GEV_FIELD_REAL ? (size_t)N * N * N : (size_t)N * N * (N / 2 + 1);
  f->elem_bytes = real_size(ctx) * (kind == GEV_FIELD_REAL ? 1 : 2);
  const size_t bytes = f->comp_elems * f->elem_bytes * ncomp;
  if (cudaMalloc(&f->d, bytes) != cudaSuccess) {
    cudaGetLastError();
    delete f;
    ctx_release(ctx);
    return gev_fail(ctx, GEV_ENOMEM, "field_create: device allocation failed");
  }
  ctx->bytes_in_use += bytes;
  GEV_CHECK_CUDA(ctx, cudaMemsetAsync(f->d, 0, bytes, ctx->stream));
  *out = f;
  return GEV_OK;
}

int gev_field_destroy(gev_field *f) {
  if (!f) return GEV_OK;
  gev_ctx *ctx = f->ctx;
  if (ctx) {
    cudaStreamSynchronize(ctx->stream);
    ctx->bytes_in_use -= f->comp_elems * f->elem_bytes * f->ncomp;
  }
  cudaFree(f->d);
  delete f;
  if (ctx) ctx_release(ctx);
  return GEV_OK;
}

int gev_field_upload(gev_field *f, const double *host) {
  if (!f || !host) return GEV_EINVAL;
  gev_ctx *ctx = f->ctx;
  const size_t nd = f->comp_elems * f->ncomp * (f->kind == GEV_FIELD_SPECTRUM ? 2 : 1);
  if (ctx->prec == GEV_PREC_FP64) {
    GEV_CHECK_CUDA(ctx, cudaMemcpyAsync(f->d, host, nd * 8, cudaMemcpyHostToDevice, ctx->stream));
  } else {
    double *tmp = nullptr;
    GEV_CHECK_CUDA(ctx, cudaMallocAsync(&tmp, nd * 8, ctx->stream));
    GEV_CHECK_CUDA(ctx, cudaMemcpyAsync(tmp, host, nd * 8, cudaMemcpyHostToDevice, ctx->stream));
    k_from_double<float><<<grid_for(ctx, nd, 256, 16), 256, 0, ctx->stream>>>(tmp, (float *)f->d, nd);
    GEV_LAUNCH_CHECK(ctx);
    GEV_CHECK_CUDA(ctx, cudaFreeAsync(tmp, ctx->stream));
  }
  GEV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return GEV_OK;
}

int gev_field_download(gev_field *f, double *host) {
  if (!f || !host) return GEV_EINVAL;
  gev_ctx *ctx = f->ctx;
  const size_t nd = f->comp_elems * f->ncomp * (f->kind == GEV_FIELD_SPECTRUM ? 2 : 1);
  if (ctx->prec == GEV_PREC_FP64) {
    GEV_CHECK_CUDA(ctx, cudaMemcpyAsync(host, f->d, nd * 8, cudaMemcpyDeviceToHost, ctx->stream));
  } else {
    double *tmp = nullptr;
    GEV_CHECK_CUDA(ctx, cudaMallocAsync(&tmp, nd * 8, ctx->stream));
    k_to_double<float><<<grid_for(ctx, nd, 256, 16), 256, 0, ctx->stream>>>((const float *)f->d, tmp, nd);
    GEV_LAUNCH_CHECK(ctx);
    GEV_CHECK_CUDA(ctx, cudaMemcpyAsync(host, tmp, nd * 8, cudaMemcpyDeviceToHost, ctx->stream));
    GEV_CHECK_CUDA(ctx, cudaFreeAsync(tmp, ctx->stream));
  }
  GEV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return GEV_OK;
}

int gev_field_zero(gev_field *f) {
  if (!f) return GEV_EINVAL;
  GEV_CHECK_CUDA(f->ctx, cudaMemsetAsync(f->d, 0, f->comp_elems * f->elem_bytes * f->ncomp, f->ctx->stream));
  return GEV_OK;
}

int gev_field_device_ptr(gev_field *f, void **ptr, size_t *bytes) {
  if (!f) return GEV_EINVAL;
  if (ptr) *ptr = f->d;
  if (bytes) *bytes = f->comp_elems * f->elem_bytes * f->ncomp;
  return GEV_OK;
}

int gev_fft_r2c(gev_ctx *ctx, const gev_field *real, gev_field *spec) {
  if (!ctx || !real || !spec || real->ctx != ctx || spec->ctx != ctx || real->kind != GEV_FIELD_REAL ||
      spec->kind != GEV_FIELD_SPECTRUM || real->ncomp != spec->ncomp)
    return gev_fail(ctx, GEV_EINVAL, "fft_r2c: real field and spectrum with equal component counts");
  GevTimed tm_(ctx, "phase:fft");
  for (int c = 0; c < real->ncomp; ++c) {
    int rc = fft_r2c_comp(ctx, (const char *)real->d + c * real->comp_elems * real->elem_bytes,
                          (char *)spec->d + c * spec->comp_elems * spec->elem_bytes);
    if (rc) return rc;
  }
  return GEV_OK;
}

int gev_fft_c2r(gev_ctx *ctx, const gev_field *spec, gev_field *real) {
  if (!ctx || !real || !spec || real->ctx != ctx || spec->ctx != ctx || real->kind != GEV_FIELD_REAL ||
      spec->kind != GEV_FIELD_SPECTRUM || real->ncomp != spec->ncomp)
    return gev_fail(ctx, GEV_EINVAL, "fft_c2r: spectrum and real field with equal component counts");
  GevTimed tm_(ctx, "phase:fft");
  for (int c = 0; c < real->ncomp; ++c) {
    int rc = fft_c2r_comp(ctx, (const char *)spec->d + c * spec->comp_elems * spec->elem_bytes,
                          (char *)real->d + c * real->comp_elems * real->elem_bytes, ctx->d_fft_scratch);
    if (rc) return rc;
  }
  return GEV_OK;
}

int gev_fft_c2r_poisson(gev_ctx *ctx, const gev_field *srcFT, gev_field *real, double coeff, double modif) {
  if (!ctx || !real || !srcFT || real->ctx != ctx || srcFT->ctx != ctx || real->kind != GEV_FIELD_REAL ||
      srcFT->kind != GEV_FIELD_SPECTRUM || real->ncomp != 1 || srcFT->ncomp != 1)
    return gev_fail(ctx, GEV_EINVAL, "fft_c2r_poisson: one spectrum component and one real component");
  GevTimed tm_(ctx, "phase:fft");
  return fft_c2r_poisson_comp(ctx, srcFT->d, real->d, coeff, modif);
}

}  // extern "C"
