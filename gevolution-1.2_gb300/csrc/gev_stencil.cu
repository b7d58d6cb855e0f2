// gev_stencil.cu -- prepareFTsource (tensor and scalar forms) and field
// reductions.  One thread per cell, x fastest so that a warp reads contiguous
// rows; the +-1 neighbours in y and z come from rows already in L1/L2.
// Periodic wrap replaces LATfield2's halo (updateHalo, main.cpp:518, 568).
#include <array>
#include <map>
#include <mutex>
#include <utility>

#include "gev_batch.cuh"

namespace {

// prepareFTsource (tensor), gevolution.hpp:56-147, PHINONLINEAR without
// ORIGINALMETRIC.  T and S may be the same array (each cell reads its own
// components before writing them).
template <typename T>
__global__ void k_source_tensor(const T *__restrict__ phi, const T *Tij, T *Sij, T coeff, int N, int lg, Div32 dN) {
  const unsigned V = (unsigned)N * N * N;  // < 2^32
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < V; i += gridDim.x * blockDim.x) {
    int x, y, z;
    cell_xyz(i, N, lg, dN, x, y, z);
    const Nb3 b = nb3(i, x, y, z, N);
    const T p = phi[i];
    const T pxp = phi[i + b.xp], pxm = phi[i + b.xm];
    const T pyp = phi[i + b.yp], pym = phi[i + b.ym];
    const T pzp = phi[i + b.zp], pzm = phi[i + b.zm];
    const T pxy = phi[i + b.xp + b.yp], pxz = phi[i + b.xp + b.zp], pyz = phi[i + b.yp + b.zp];
    const T h = (T)0.5;
    const size_t Vs = V;  // component offsets past 2^32 elements at N = 1024
    const T t00 = Tij[i], t01 = Tij[Vs + i], t02 = Tij[2 * Vs + i], t11 = Tij[3 * Vs + i], t12 = Tij[4 * Vs + i],
            t22 = Tij[5 * Vs + i];
    Sij[i] = coeff * t00 + h * (pxp - pxm) * (pxp - pxm);
    Sij[3 * Vs + i] = coeff * t11 + h * (pyp - pym) * (pyp - pym);
    Sij[5 * Vs + i] = coeff * t22 + h * (pzp - pzm) * (pzp - pzm);
    if constexpr (sizeof(T) == 8) {  // the reference's expression, term by term
      Sij[Vs + i] = coeff * t01 + (pxp * pyp - p * pxy) + h * p * p - h * pxp * pxp - h * pyp * pyp + h * pxy * pxy;
      Sij[2 * Vs + i] = coeff * t02 + (pxp * pzp - p * pxz) + h * p * p - h * pxp * pxp - h * pzp * pzp + h * pxz * pxz;
      Sij[4 * Vs + i] = coeff * t12 + (pyp * pzp - p * pyz) + h * p * p - h * pyp * pyp - h * pzp * pzp + h * pyz * pyz;
    } else {
      // FP32: with a = phi(x), b = phi(x+i), c = phi(x+j), d = phi(x+i+j) the sum
      // bc - ad + a^2/2 - b^2/2 - c^2/2 + d^2/2 equals ((a-d) - (b-c)) ((a-d) + (b-c)) / 2,
      // which never forms the O(phi^2) terms that cancel down to O((grad phi)^2)
      const T dxy = p - pxy, exy = pxp - pyp, dxz = p - pxz, exz = pxp - pzp, dyz = p - pyz, eyz = pyp - pzp;
      Sij[Vs + i] = coeff * t01 + h * (dxy - exy) * (dxy + exy);
      Sij[2 * Vs + i] = coeff * t02 + h * (dxz - exz) * (dxz + exz);
      Sij[4 * Vs + i] = coeff * t12 + h * (dyz - eyz) * (dyz + eyz);
    }
  }
}

// FP32 with N % 4 == 0: four consecutive x cells a thread (cell i, i % 4 == 0).  The
// rows at (y, z), (y +- 1, z), (y, z +- 1) and the streamed arrays are read as 16-byte
// vectors (every row offset is a multiple of 4 elements); the x neighbours outside
// the vector, phi(x0 - 1) and phi(x0 + 4), are scalar loads with the periodic wrap.
// Each cell's expression is the scalar kernel's, term for term.
__device__ __forceinline__ float4 ld4(const float *p) { return *reinterpret_cast<const float4 *>(p); }
__device__ __forceinline__ void st4(float *p, const float4 &v) { *reinterpret_cast<float4 *>(p) = v; }
__device__ __forceinline__ void unpack4(const float4 &v, float (&a)[4]) {
  a[0] = v.x;
  a[1] = v.y;
  a[2] = v.z;
  a[3] = v.w;
}
// the element 4 past the first of a vector at row offset `off`, wrapped when x0 + 4 == N
__device__ __forceinline__ unsigned next4(unsigned i, int x, int N) {
  return x + 4 == N ? i + 4u - (unsigned)N : i + 4u;
}

__device__ __forceinline__ void k_source_tensor4_body(const float *__restrict__ phi, const float *Tij, float *Sij,
                                                      float coeff, int N, int lg, Div32 dN) {
  const unsigned V = (unsigned)N * N * N, V4 = V / 4;
  const float h = 0.5f;
  for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < V4; q += gridDim.x * blockDim.x) {
    const unsigned i = q * 4u;
    int x, y, z;
    cell_xyz(i, N, lg, dN, x, y, z);
    const Nb3 b = nb3(i, x, y, z, N);
    float P[4], YP[4], YM[4], ZP[4], ZM[4], XY[4], XZ[4], YZ[4];
    // neighbour indices summed in 32 bits, where the periodic offsets wrap, before
    // they touch a pointer
    const unsigned iyp = i + b.yp, iym = i + b.ym, izp = i + b.zp, izm = i + b.zm, iyz = i + b.yp + b.zp;
    unpack4(ld4(phi + i), P);
    unpack4(ld4(phi + iyp), YP);
    unpack4(ld4(phi + iym), YM);
    unpack4(ld4(phi + izp), ZP);
    unpack4(ld4(phi + izm), ZM);
    unpack4(ld4(phi + iyz), YZ);
    const float pl = phi[i + b.xm], pr = phi[next4(i, x, N)];
    const float pry = phi[next4(iyp, x, N)], prz = phi[next4(izp, x, N)];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      XY[j] = j < 3 ? YP[j + 1] : pry;
      XZ[j] = j < 3 ? ZP[j + 1] : prz;
    }
    const size_t Vs = V;  // component offsets past 2^32 elements at N = 1024
    float T0[4], T1[4], T2[4], T3[4], T4[4], T5[4];
    unpack4(ld4(Tij + i), T0);
    unpack4(ld4(Tij + Vs + i), T1);
    unpack4(ld4(Tij + 2 * Vs + i), T2);
    unpack4(ld4(Tij + 3 * Vs + i), T3);
    unpack4(ld4(Tij + 4 * Vs + i), T4);
    unpack4(ld4(Tij + 5 * Vs + i), T5);
    float S0[4], S1[4], S2[4], S3[4], S4[4], S5[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const float p = P[j];
      const float pxp = j < 3 ? P[j + 1] : pr, pxm = j > 0 ? P[j - 1] : pl;
      const float pyp = YP[j], pym = YM[j], pzp = ZP[j], pzm = ZM[j];
      const float pxy = XY[j], pxz = XZ[j], pyz = YZ[j];
      S0[j] = coeff * T0[j] + h * (pxp - pxm) * (pxp - pxm);
      S3[j] = coeff * T3[j] + h * (pyp - pym) * (pyp - pym);
      S5[j] = coeff * T5[j] + h * (pzp - pzm) * (pzp - pzm);
      const float dxy = p - pxy, exy = pxp - pyp, dxz = p - pxz, exz = pxp - pzp, dyz = p - pyz, eyz = pyp - pzp;
      S1[j] = coeff * T1[j] + h * (dxy - exy) * (dxy + exy);
      S2[j] = coeff * T2[j] + h * (dxz - exz) * (dxz + exz);
      S4[j] = coeff * T4[j] + h * (dyz - eyz) * (dyz + eyz);
    }
    st4(Sij + i, make_float4(S0[0], S0[1], S0[2], S0[3]));
    st4(Sij + Vs + i, make_float4(S1[0], S1[1], S1[2], S1[3]));
    st4(Sij + 2 * Vs + i, make_float4(S2[0], S2[1], S2[2], S2[3]));
    st4(Sij + 3 * Vs + i, make_float4(S3[0], S3[1], S3[2], S3[3]));
    st4(Sij + 4 * Vs + i, make_float4(S4[0], S4[1], S4[2], S4[3]));
    st4(Sij + 5 * Vs + i, make_float4(S5[0], S5[1], S5[2], S5[3]));
  }
}

__global__ void k_source_tensor4(const float *__restrict__ phi, const float *Tij, float *Sij, float coeff, int N,
                                 int lg, Div32 dN) {
  k_source_tensor4_body(phi, Tij, Sij, coeff, N, lg, dN);
}

__device__ __forceinline__ void k_source_scalar4_body(const float *__restrict__ phi, const float *__restrict__ chi,
                                                      const float *source, float bgmodel, float *result, float coeff,
                                                      float coeff2, float coeff3, int N, int lg, Div32 dN) {
  const unsigned V4 = (unsigned)N * N * N / 4;
  for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < V4; q += gridDim.x * blockDim.x) {
    const unsigned i = q * 4u;
    int x, y, z;
    cell_xyz(i, N, lg, dN, x, y, z);
    const Nb3 b = nb3(i, x, y, z, N);
    float P[4], YP[4], YM[4], ZP[4], ZM[4], SRC[4], CHI[4], R[4];
    const unsigned iyp = i + b.yp, iym = i + b.ym, izp = i + b.zp, izm = i + b.zm;  // wrapped in 32 bits
    unpack4(ld4(phi + i), P);
    unpack4(ld4(phi + iyp), YP);
    unpack4(ld4(phi + iym), YM);
    unpack4(ld4(phi + izp), ZP);
    unpack4(ld4(phi + izm), ZM);
    unpack4(ld4(source + i), SRC);
    unpack4(ld4(chi + i), CHI);
    const float pl = phi[i + b.xm], pr = phi[next4(i, x, N)];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const float p = P[j];
      const float dx = (j > 0 ? P[j - 1] : pl) - (j < 3 ? P[j + 1] : pr);
      const float dy = YM[j] - YP[j];
      const float dz = ZM[j] - ZP[j];
      float r = coeff2 * (SRC[j] - bgmodel);
      r *= 1.f - 2.f * p;
      r += 0.125f * (dx * dx + dy * dy + dz * dz);
      r += (coeff3 - coeff) * p - coeff3 * CHI[j];
      R[j] = r;
    }
    st4(result + i, make_float4(R[0], R[1], R[2], R[3]));
  }
}
__global__ void k_source_scalar4(const float *__restrict__ phi, const float *__restrict__ chi, const float *source,
                                 float bgmodel, float *result, float coeff, float coeff2, float coeff3, int N,
                                 int lg, Div32 dN) {
  k_source_scalar4_body(phi, chi, source, bgmodel, result, coeff, coeff2, coeff3, N, lg, dN);
}

// prepareFTsource (scalar), gevolution.hpp:169-192; result may equal source
template <typename T>
__global__ void k_source_scalar(const T *__restrict__ phi, const T *__restrict__ chi, const T *source, T bgmodel,
                                T *result, T coeff, T coeff2, T coeff3, int N, int lg, Div32 dN) {
  const unsigned V = (unsigned)N * N * N;  // < 2^32
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < V; i += gridDim.x * blockDim.x) {
    int x, y, z;
    cell_xyz(i, N, lg, dN, x, y, z);
    const Nb3 b = nb3(i, x, y, z, N);
    const T p = phi[i];
    const T dx = phi[i + b.xm] - phi[i + b.xp];
    const T dy = phi[i + b.ym] - phi[i + b.yp];
    const T dz = phi[i + b.zm] - phi[i + b.zp];
    T r = coeff2 * (source[i] - bgmodel);
    r *= (T)1 - (T)2 * p;
    r += (T)0.125 * (dx * dx + dy * dy + dz * dz);
    r += (coeff3 - coeff) * p - coeff3 * chi[i];
    result[i] = r;
  }
}

// deterministic sum: fixed per-thread striding, fixed block tree, fixed final pass
template <typename T>
__global__ void k_sum_partial(const T *__restrict__ f, size_t n, double *partial) {
  __shared__ double sh[256];
  double s = 0.;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    s += (double)f[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

__global__ void k_sum_final(const double *partial, int nb, double *out) {
  __shared__ double sh[256];
  double s = 0.;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) s += partial[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = sh[0];
}

bool same_ctx(gev_ctx *ctx, const gev_field *f, int kind) { return f && f->ctx == ctx && f->kind == kind; }

// ---------------------------------------------------------------- tuning --
// The FP32 stencils are grid-stride loops over 4-cell vectors, each vector
// computed alone, so every launch shape gives the same bits; which shape runs
// fastest depends on the grid (a 64^3 field is 65,536 vectors, fewer than the GPU
// holds threads).  On the first call of the first context of a size in the process
// the candidates -- 128, 256 or 512 threads a block, at most 4, 8, 16 or 32 blocks a
// SM -- are timed on scratch fields of that size filled with bounded values (three
// rounds, the best time of each), and a shape replaces the default (256 threads, 16
// blocks a SM) only when it is more than 3% faster; later contexts of that size take
// the same shapes.  Grids above 256^3 keep the default: there every candidate
// fills the GPU many times over, and the scratch (13 fields) would be large.
constexpr int ST_THREADS[3] = {128, 256, 512};
constexpr int ST_PER_SM[4] = {4, 8, 16, 32};
constexpr int ST_TUNE_MAX_N = 256;

__global__ void k_st_fill(float *s, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    s[i] = (float)((unsigned)(i * 2654435761u) >> 8) * (1.f / 16777216.f) - 0.5f;
}

void launch_scalar4(gev_ctx *ctx, int threads, int per_sm, const float *phi, const float *chi, const float *source,
                    float bgmodel, float *result, float coeff, float coeff2, float coeff3) {
  const size_t V = (size_t)ctx->N * ctx->N * ctx->N;
  gev_launch<k_source_scalar4_body, 512, 1>(ctx, k_source_scalar4, dim3(grid_for(ctx, V / 4, threads, per_sm)),
                                            dim3(threads), 0, phi, chi, source, bgmodel, result, coeff, coeff2,
                                            coeff3, ctx->N, lg_pow2(ctx->N), make_div32(ctx->N));
}

void launch_tensor4(gev_ctx *ctx, int threads, int per_sm, const float *phi, const float *Tij, float *Sij,
                    float coeff) {
  const size_t V = (size_t)ctx->N * ctx->N * ctx->N;
  gev_launch<k_source_tensor4_body, 512, 1>(ctx, k_source_tensor4, dim3(grid_for(ctx, V / 4, threads, per_sm)),
                                            dim3(threads), 0, phi, Tij, Sij, coeff, ctx->N, lg_pow2(ctx->N),
                                            make_div32(ctx->N));
}

// mean ms of 5 launches after one untimed launch; +inf when a launch fails
template <typename F>
float st_time_ms(gev_ctx *ctx, F &&fn) {
  cudaEvent_t a = nullptr, b = nullptr;
  float ms = 3.4e38f;
  if (cudaEventCreate(&a) == cudaSuccess && cudaEventCreate(&b) == cudaSuccess) {
    fn();
    cudaEventRecord(a, ctx->stream);
    for (int k = 0; k < 5; ++k) fn();
    cudaEventRecord(b, ctx->stream);
    if (cudaGetLastError() == cudaSuccess && cudaEventSynchronize(b) == cudaSuccess &&
        cudaEventElapsedTime(&ms, a, b) == cudaSuccess)
      ms /= 5.f;
    else
      ms = 3.4e38f;
  }
  cudaGetLastError();
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  return ms;
}

// shapes already timed in this process, per (device, N): a later context of a size
// seen before takes them instead of timing again
std::mutex g_shapes_mu;
std::map<std::pair<int, int>, std::array<int, 4>> g_shapes;

void stencil_tune(gev_ctx *ctx);

void stencil_autotune(gev_ctx *ctx) {
  if (ctx->st_tuned) return;
  if (ctx->rec) {  // a recorded cycle cannot time anything: batch only tuned contexts
    ctx->rec->bad = true;
    return;
  }
  ctx->st_tuned = true;
  const int N = ctx->N;
  if (ctx->prec == GEV_PREC_FP64 || N % 4 != 0 || N > ST_TUNE_MAX_N) return;
  const auto key = std::make_pair(ctx->device, N);
  {
    std::lock_guard<std::mutex> lk(g_shapes_mu);
    const auto it = g_shapes.find(key);
    if (it != g_shapes.end()) {
      for (int k = 0; k < 2; ++k) {
        ctx->st_threads[k] = it->second[k];
        ctx->st_per_sm[k] = it->second[2 + k];
      }
      return;
    }
  }
  stencil_tune(ctx);
  std::lock_guard<std::mutex> lk(g_shapes_mu);
  g_shapes[key] = {ctx->st_threads[0], ctx->st_threads[1], ctx->st_per_sm[0], ctx->st_per_sm[1]};
}

// times the candidates on scratch fields of the context's size
void stencil_tune(gev_ctx *ctx) {
  const int N = ctx->N;
  const size_t V = (size_t)N * N * N;
  float *tmp = nullptr;
  if (cudaMallocAsync((void **)&tmp, 13 * V * sizeof(float), ctx->stream) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  k_st_fill<<<grid_for(ctx, 13 * V, 256, 8), 256, 0, ctx->stream>>>(tmp, 13 * V);
  float *phi = tmp, *chi = tmp + V, *src = tmp + 2 * V, *res = tmp + 3 * V, *Tij = tmp + V, *Sij = tmp + 7 * V;
  for (int which = 0; which < 2; ++which) {
    float t[3][4];
    for (auto &row : t)
      for (float &x : row) x = 3.4e38f;
    for (int round = 0; round < 3; ++round)
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 4; ++b) {
          const int th = ST_THREADS[a], ps = ST_PER_SM[b];
          // shapes that give the same grid as a smaller cap are the same launch
          if (b > 0 && grid_for(ctx, V / 4, th, ps) == grid_for(ctx, V / 4, th, ST_PER_SM[b - 1])) continue;
          const float ms = which == 0 ? st_time_ms(ctx, [&] {
            launch_scalar4(ctx, th, ps, phi, chi, src, 0.3f, res, 1e-3f, 1e-3f, 1e-3f);
          })
                                      : st_time_ms(ctx, [&] { launch_tensor4(ctx, th, ps, phi, Tij, Sij, 1e-3f); });
          t[a][b] = fminf(t[a][b], ms);
        }
    int ba = 1, bb = 2;  // the default, 256 threads and 16 blocks a SM
    const float tdef = t[1][2];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 4; ++b)
        if (t[a][b] < 0.97f * tdef && t[a][b] < t[ba][bb]) {
          ba = a;
          bb = b;
        }
    ctx->st_threads[which] = ST_THREADS[ba];
    ctx->st_per_sm[which] = ST_PER_SM[bb];
  }
  cudaFreeAsync(tmp, ctx->stream);
  cudaGetLastError();
}

}  // namespace

extern "C" {

int gev_ctx_stencil_shapes(gev_ctx *ctx, int threads[2], int per_sm[2]) {
  if (!ctx || !threads || !per_sm) return gev_fail(ctx, GEV_EINVAL, "ctx_stencil_shapes: null argument");
  for (int k = 0; k < 2; ++k) {
    threads[k] = ctx->st_threads[k];
    per_sm[k] = ctx->st_per_sm[k];
  }
  return GEV_OK;
}

int gev_ctx_set_stencil_shapes(gev_ctx *ctx, const int threads[2], const int per_sm[2]) {
  if (!ctx || !threads || !per_sm) return gev_fail(ctx, GEV_EINVAL, "ctx_set_stencil_shapes: null argument");
  for (int k = 0; k < 2; ++k)
    if ((threads[k] != 64 && threads[k] != 128 && threads[k] != 256 && threads[k] != 512) || per_sm[k] < 1 ||
        per_sm[k] > 64)
      return gev_fail(ctx, GEV_EINVAL, "ctx_set_stencil_shapes: 64, 128, 256 or 512 threads, 1..64 blocks a SM");
  for (int k = 0; k < 2; ++k) {
    ctx->st_threads[k] = threads[k];
    ctx->st_per_sm[k] = per_sm[k];
  }
  ctx->st_tuned = true;
  return GEV_OK;
}

int gev_prepare_source_tensor(gev_ctx *ctx, const gev_field *phi, const gev_field *Tij, gev_field *Sij, double coeff) {
  if (!ctx || !same_ctx(ctx, phi, GEV_FIELD_REAL) || !same_ctx(ctx, Tij, GEV_FIELD_REAL) ||
      !same_ctx(ctx, Sij, GEV_FIELD_REAL) || phi->ncomp != 1 || Tij->ncomp != 6 || Sij->ncomp != 6)
    return gev_fail(ctx, GEV_EINVAL, "prepare_source_tensor: phi (1 comp), Tij and Sij (6 comps) real fields");
  const size_t V = (size_t)ctx->N * ctx->N * ctx->N;
  const int blocks = grid_for(ctx, V, 256, 16);
  stencil_autotune(ctx);
  GevTimed tm_(ctx, "k_source_tensor");
  if (ctx->prec == GEV_PREC_FP64)
    k_source_tensor<double><<<blocks, 256, 0, ctx->stream>>>((const double *)phi->d, (const double *)Tij->d,
                                                             (double *)Sij->d, coeff, ctx->N, lg_pow2(ctx->N),
                                                             make_div32(ctx->N));
  else if (ctx->N % 4 == 0)
    launch_tensor4(ctx, ctx->st_threads[1], ctx->st_per_sm[1], (const float *)phi->d, (const float *)Tij->d,
                   (float *)Sij->d, (float)coeff);
  else
    k_source_tensor<float><<<blocks, 256, 0, ctx->stream>>>((const float *)phi->d, (const float *)Tij->d,
                                                            (float *)Sij->d, (float)coeff, ctx->N, lg_pow2(ctx->N),
                                                            make_div32(ctx->N));
  GEV_LAUNCH_CHECK(ctx);
  return GEV_OK;
}

int gev_prepare_source_scalar(gev_ctx *ctx, const gev_field *phi, const gev_field *chi, const gev_field *source,
                              double bgmodel, gev_field *result, double coeff, double coeff2, double coeff3) {
  if (!ctx || !same_ctx(ctx, phi, GEV_FIELD_REAL) || !same_ctx(ctx, chi, GEV_FIELD_REAL) ||
      !same_ctx(ctx, source, GEV_FIELD_REAL) || !same_ctx(ctx, result, GEV_FIELD_REAL) || phi->ncomp != 1 ||
      chi->ncomp != 1 || source->ncomp != 1 || result->ncomp != 1)
    return gev_fail(ctx, GEV_EINVAL, "prepare_source_scalar: four 1-component real fields");
  const size_t V = (size_t)ctx->N * ctx->N * ctx->N;
  const int blocks = grid_for(ctx, V, 256, 16);
  stencil_autotune(ctx);
  GevTimed tm_(ctx, "k_source_scalar");
  if (ctx->prec == GEV_PREC_FP64)
    k_source_scalar<double><<<blocks, 256, 0, ctx->stream>>>((const double *)phi->d, (const double *)chi->d,
                                                             (const double *)source->d, bgmodel, (double *)result->d,
                                                             coeff, coeff2, coeff3, ctx->N, lg_pow2(ctx->N),
                                                             make_div32(ctx->N));
  else if (ctx->N % 4 == 0)
    launch_scalar4(ctx, ctx->st_threads[0], ctx->st_per_sm[0], (const float *)phi->d, (const float *)chi->d,
                   (const float *)source->d, (float)bgmodel, (float *)result->d, (float)coeff, (float)coeff2,
                   (float)coeff3);
  else
    k_source_scalar<float><<<blocks, 256, 0, ctx->stream>>>(
        (const float *)phi->d, (const float *)chi->d, (const float *)source->d, (float)bgmodel, (float *)result->d,
        (float)coeff, (float)coeff2, (float)coeff3, ctx->N, lg_pow2(ctx->N), make_div32(ctx->N));
  GEV_LAUNCH_CHECK(ctx);
  return GEV_OK;
}

int gev_field_sum(gev_ctx *ctx, const gev_field *f, int comp, double *out) {
  if (!ctx || !f || f->ctx != ctx || f->kind != GEV_FIELD_REAL || comp < 0 || comp >= f->ncomp || !out)
    return gev_fail(ctx, GEV_EINVAL, "field_sum: real field and valid component");
  const size_t V = f->comp_elems;
  const int nb = ctx->sms * 4;
  int rc = ctx_ensure_red(ctx, (size_t)nb + 1);
  if (rc) return rc;
  if (ctx->prec == GEV_PREC_FP64)
    k_sum_partial<double><<<nb, 256, 0, ctx->stream>>>((const double *)f->d + comp * V, V, ctx->d_red);
  else
    k_sum_partial<float><<<nb, 256, 0, ctx->stream>>>((const float *)f->d + comp * V, V, ctx->d_red);
  GEV_LAUNCH_CHECK(ctx);
  k_sum_final<<<1, 256, 0, ctx->stream>>>(ctx->d_red, nb, ctx->d_red + nb);
  GEV_LAUNCH_CHECK(ctx);
  GEV_CHECK_CUDA(ctx, cudaMemcpyAsync(out, ctx->d_red + nb, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  GEV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return GEV_OK;
}

}  // extern "C"
