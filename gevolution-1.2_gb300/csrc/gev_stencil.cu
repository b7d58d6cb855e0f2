// gev_stencil.cu -- prepareFTsource (tensor and scalar forms) and field
// reductions.  One thread per cell, x fastest so that a warp reads contiguous
// rows; the +-1 neighbours in y and z come from rows already in L1/L2.
// Periodic wrap replaces LATfield2's halo (updateHalo, main.cpp:518, 568).
#include "gev_internal.cuh"

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
    const T t00 = Tij[i], t01 = Tij[V + i], t02 = Tij[2 * V + i], t11 = Tij[3 * V + i], t12 = Tij[4 * V + i],
            t22 = Tij[5 * V + i];
    Sij[i] = coeff * t00 + h * (pxp - pxm) * (pxp - pxm);
    Sij[3 * V + i] = coeff * t11 + h * (pyp - pym) * (pyp - pym);
    Sij[5 * V + i] = coeff * t22 + h * (pzp - pzm) * (pzp - pzm);
    if constexpr (sizeof(T) == 8) {  // the reference's expression, term by term
      Sij[V + i] = coeff * t01 + (pxp * pyp - p * pxy) + h * p * p - h * pxp * pxp - h * pyp * pyp + h * pxy * pxy;
      Sij[2 * V + i] = coeff * t02 + (pxp * pzp - p * pxz) + h * p * p - h * pxp * pxp - h * pzp * pzp + h * pxz * pxz;
      Sij[4 * V + i] = coeff * t12 + (pyp * pzp - p * pyz) + h * p * p - h * pyp * pyp - h * pzp * pzp + h * pyz * pyz;
    } else {
      // FP32: with a = phi(x), b = phi(x+i), c = phi(x+j), d = phi(x+i+j) the sum
      // bc - ad + a^2/2 - b^2/2 - c^2/2 + d^2/2 equals ((a-d) - (b-c)) ((a-d) + (b-c)) / 2,
      // which never forms the O(phi^2) terms that cancel down to O((grad phi)^2)
      const T dxy = p - pxy, exy = pxp - pyp, dxz = p - pxz, exz = pxp - pzp, dyz = p - pyz, eyz = pyp - pzp;
      Sij[V + i] = coeff * t01 + h * (dxy - exy) * (dxy + exy);
      Sij[2 * V + i] = coeff * t02 + h * (dxz - exz) * (dxz + exz);
      Sij[4 * V + i] = coeff * t12 + h * (dyz - eyz) * (dyz + eyz);
    }
  }
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

}  // namespace

extern "C" {

int gev_prepare_source_tensor(gev_ctx *ctx, const gev_field *phi, const gev_field *Tij, gev_field *Sij, double coeff) {
  if (!ctx || !same_ctx(ctx, phi, GEV_FIELD_REAL) || !same_ctx(ctx, Tij, GEV_FIELD_REAL) ||
      !same_ctx(ctx, Sij, GEV_FIELD_REAL) || phi->ncomp != 1 || Tij->ncomp != 6 || Sij->ncomp != 6)
    return gev_fail(ctx, GEV_EINVAL, "prepare_source_tensor: phi (1 comp), Tij and Sij (6 comps) real fields");
  const size_t V = (size_t)ctx->N * ctx->N * ctx->N;
  const int blocks = grid_for(ctx, V, 256, 16);
  if (ctx->prec == GEV_PREC_FP64)
    k_source_tensor<double><<<blocks, 256, 0, ctx->stream>>>((const double *)phi->d, (const double *)Tij->d,
                                                             (double *)Sij->d, coeff, ctx->N, lg_pow2(ctx->N),
                                                             make_div32(ctx->N));
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
  if (ctx->prec == GEV_PREC_FP64)
    k_source_scalar<double><<<blocks, 256, 0, ctx->stream>>>((const double *)phi->d, (const double *)chi->d,
                                                             (const double *)source->d, bgmodel, (double *)result->d,
                                                             coeff, coeff2, coeff3, ctx->N, lg_pow2(ctx->N),
                                                             make_div32(ctx->N));
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
