// gev_deposit.cu -- the CIC / CIC-NGP stress-energy deposits.
//
// Replaces projection_T00/T0i/Tij_project and their *_comm halo folds
// (gevolution.hpp:926-1301) and LATfield2's scalarProjectionCIC_project.
// The reference accumulates each cell's particles into a small "local cube"
// and then adds the cube to the 8 (or fewer) surrounding field cells.  Here the
// same two levels run as two passes with no atomics:
//   pass 1 (one thread per cell): sum the cell's particles -- contiguous in the
//           (cell, ID)-ordered store -- into its cube values, already multiplied
//           by the mass and metric factors the reference applies per cube;
//   pass 2 (one thread per field cell): gather the cube entries of the source
//           cells that touch it, with periodic wrap (the halo fold), in a fixed
//           order, and add them to the field.
// Every sum therefore has a fixed order: results are bit-reproducible run to
// run.  This is the FP64 form; the mixed form uses the fixed-point column
// sweep of gev_deposit_fx.cu.
#include "gev_internal.cuh"

int deposit_fx(gev_ctx *ctx, gev_pcls *p, gev_field *out, int kind, double mass, double a, const gev_field *phi,
               bool overwrite, gev_field *out2 = nullptr);

namespace {

enum { DEP_T00 = 0, DEP_T0I = 1, DEP_TIJ = 2, DEP_MASS = 3 };
constexpr int NVAL[4] = {8, 12, 30, 8};

struct DepParams {
  int N;
  double mass, a;
  double fx_scale;  // fixed-point scale (mixed form)
};

template <typename T>
__device__ __forceinline__ T ldf(const T *__restrict__ f, int x, int y, int z, int N) {
  return __ldg(&f[sidx(wrapi(x, N), wrapi(y, N), wrapi(z, N), N)]);
}

// pass 1, FP64 form: cube[k * C + c] (SoA so that pass 2 reads coalesced rows)
template <int KIND>
__global__ void __launch_bounds__(256) k_cube_fp64(PclsArrays P, const uint32_t *__restrict__ start,
                                                   const double *__restrict__ phi, DepParams dp, double *cube) {
  const int N = dp.N;
  const size_t C = (size_t)N * N * N;
  const double Nd = (double)N, dx = 1.0 / Nd;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < C; c += (size_t)gridDim.x * blockDim.x) {
    const int cx = (int)(c % N), cy = (int)((c / N) % N), cz = (int)(c / ((size_t)N * N));
    const uint32_t s = start[c], e = start[c + 1];
    double l[8];
    if (phi != nullptr && KIND != DEP_MASS && e > s) {
      l[0] = ldf(phi, cx, cy, cz, N);
      l[1] = ldf(phi, cx, cy, cz + 1, N);
      l[2] = ldf(phi, cx, cy + 1, cz, N);
      l[3] = ldf(phi, cx, cy + 1, cz + 1, N);
      l[4] = ldf(phi, cx + 1, cy, cz, N);
      l[5] = ldf(phi, cx + 1, cy, cz + 1, N);
      l[6] = ldf(phi, cx + 1, cy + 1, cz, N);
      l[7] = ldf(phi, cx + 1, cy + 1, cz + 1, N);
    } else {
#pragma unroll
      for (int k = 0; k < 8; ++k) l[k] = 0.;
    }
    const double rx = cx * dx, ry = cy * dx, rz = cz * dx;
    constexpr int NV = NVAL[KIND];
    double acc[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] = 0.;
    const double a = dp.a;
    for (uint32_t j = s; j < e; ++j) {
      const double u0 = (P.px[j] - rx) * Nd, u1 = (P.py[j] - ry) * Nd, u2 = (P.pz[j] - rz) * Nd;
      const double d0 = 1.0 - u0, d1 = 1.0 - u1, d2 = 1.0 - u2;
      if (KIND == DEP_MASS || KIND == DEP_T00) {
        double ee = a, ff = 0.;
        if (KIND == DEP_T00 && phi != nullptr) {
          const double q0 = ((const double *)P.vx)[j], q1 = ((const double *)P.vy)[j], q2 = ((const double *)P.vz)[j];
          const double f = q0 * q0 + q1 * q1 + q2 * q2;
          ee = sqrt(f + a * a);
          ff = 3. * ee + f / ee;
        }
        const double w[8] = {d0 * d1 * d2, d0 * d1 * u2, d0 * u1 * d2, d0 * u1 * u2,
                             u0 * d1 * d2, u0 * d1 * u2, u0 * u1 * d2, u0 * u1 * u2};
#pragma unroll
        for (int k = 0; k < 8; ++k) acc[k] += KIND == DEP_MASS ? w[k] : w[k] * (ee + ff * l[k]);
      } else if (KIND == DEP_T0I) {
        const double q0 = ((const double *)P.vx)[j], q1 = ((const double *)P.vy)[j], q2 = ((const double *)P.vz)[j];
        double w = dp.mass * q0;
        acc[0] += w * d1 * d2;
        acc[1] += w * u1 * d2;
        acc[2] += w * d1 * u2;
        acc[3] += w * u1 * u2;
        w = dp.mass * q1;
        acc[4] += w * d0 * d2;
        acc[5] += w * u0 * d2;
        acc[6] += w * d0 * u2;
        acc[7] += w * u0 * u2;
        w = dp.mass * q2;
        acc[8] += w * d0 * d1;
        acc[9] += w * u0 * d1;
        acc[10] += w * d0 * u1;
        acc[11] += w * u0 * u1;
      } else {  // DEP_TIJ
        const double q[3] = {((const double *)P.vx)[j], ((const double *)P.vy)[j], ((const double *)P.vz)[j]};
        double f = q[0] * q[0] + q[1] * q[1] + q[2] * q[2];
        const double ee = sqrt(f + a * a);
        const double inv_e = 1.0 / ee;
        f = 4. + a * a / (f + a * a);
        const double w8[8] = {d0 * d1 * d2, d0 * d1 * u2, d0 * u1 * d2, d0 * u1 * u2,
                              u0 * d1 * d2, u0 * d1 * u2, u0 * u1 * d2, u0 * u1 * u2};
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const double w = dp.mass * q[i] * q[i] * inv_e;
#pragma unroll
          for (int k = 0; k < 8; ++k) acc[8 * i + k] += w * w8[k] * (1. + f * l[k]);
        }
        const double qf = 0.25 * f;
        double w = dp.mass * q[0] * q[1] * inv_e;
        acc[24] += w * d2 * (1. + qf * (l[0] + l[2] + l[4] + l[6]));
        acc[25] += w * u2 * (1. + qf * (l[1] + l[3] + l[5] + l[7]));
        w = dp.mass * q[0] * q[2] * inv_e;
        acc[26] += w * d1 * (1. + qf * (l[0] + l[1] + l[4] + l[5]));
        acc[27] += w * u1 * (1. + qf * (l[2] + l[3] + l[6] + l[7]));
        w = dp.mass * q[1] * q[2] * inv_e;
        acc[28] += w * d0 * (1. + qf * (l[0] + l[1] + l[2] + l[3]));
        acc[29] += w * u0 * (1. + qf * (l[4] + l[5] + l[6] + l[7]));
      }
    }
    if (KIND == DEP_T00 || KIND == DEP_MASS) {
#pragma unroll
      for (int k = 0; k < 8; ++k) cube[k * C + c] = acc[k] * dp.mass;
    } else if (KIND == DEP_T0I) {
      // the link factors (1 + phi_a + phi_b), gevolution.hpp:1129-1144
      const double f[12] = {1. + l[0] + l[4], 1. + l[2] + l[6], 1. + l[1] + l[5], 1. + l[3] + l[7],
                            1. + l[0] + l[2], 1. + l[4] + l[6], 1. + l[1] + l[3], 1. + l[5] + l[7],
                            1. + l[0] + l[1], 1. + l[4] + l[5], 1. + l[2] + l[3], 1. + l[6] + l[7]};
#pragma unroll
      for (int k = 0; k < 12; ++k) cube[k * C + c] = acc[k] * f[k];
    } else {
#pragma unroll
      for (int k = 0; k < 30; ++k) cube[k * C + c] = acc[k];
    }
  }
}

// pass 2: gather the cube entries touching each field cell, fixed order
template <typename A>
__device__ __forceinline__ A cv(const A *__restrict__ cube, int k, size_t C, int x, int y, int z, int N) {
  return cube[k * C + sidx(wrapi(x, N), wrapi(y, N), wrapi(z, N), N)];
}

template <int KIND, typename A, typename T>
__global__ void __launch_bounds__(256) k_gather(const A *__restrict__ cube, T *out, int N, double inv_scale) {
  const size_t C = (size_t)N * N * N;
  for (size_t f = blockIdx.x * (size_t)blockDim.x + threadIdx.x; f < C; f += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(f % N), y = (int)((f / N) % N), z = (int)(f / ((size_t)N * N));
    if (KIND == DEP_T00 || KIND == DEP_MASS || KIND == DEP_TIJ) {
      const int ncomp = KIND == DEP_TIJ ? 3 : 1;
      for (int i = 0; i < ncomp; ++i) {
        A s = 0;
        // source cell (x - dx, y - dy, z - dz) contributes its corner (dx, dy, dz) = index 4dx + 2dy + dz
#pragma unroll
        for (int dz = 1; dz >= 0; --dz)
#pragma unroll
          for (int dy = 1; dy >= 0; --dy)
#pragma unroll
            for (int dxx = 1; dxx >= 0; --dxx) s += cv(cube, 8 * i + 4 * dxx + 2 * dy + dz, C, x - dxx, y - dy, z - dz, N);
        const int comp = KIND == DEP_TIJ ? (i == 0 ? 0 : (i == 1 ? 3 : 5)) : 0;
        out[comp * C + f] += (T)((double)s * inv_scale);
      }
      if (KIND == DEP_TIJ) {
        const A s01 = cv(cube, 24, C, x, y, z, N) + cv(cube, 25, C, x, y, z - 1, N);
        const A s02 = cv(cube, 26, C, x, y, z, N) + cv(cube, 27, C, x, y - 1, z, N);
        const A s12 = cv(cube, 28, C, x, y, z, N) + cv(cube, 29, C, x - 1, y, z, N);
        out[1 * C + f] += (T)((double)s01 * inv_scale);
        out[2 * C + f] += (T)((double)s02 * inv_scale);
        out[4 * C + f] += (T)((double)s12 * inv_scale);
      }
    } else {  // T0i: component i on links along i; CIC in the two transverse directions
      const A s0 = cv(cube, 0, C, x, y, z, N) + cv(cube, 1, C, x, y - 1, z, N) + cv(cube, 2, C, x, y, z - 1, N) +
                   cv(cube, 3, C, x, y - 1, z - 1, N);
      const A s1 = cv(cube, 4, C, x, y, z, N) + cv(cube, 5, C, x - 1, y, z, N) + cv(cube, 6, C, x, y, z - 1, N) +
                   cv(cube, 7, C, x - 1, y, z - 1, N);
      const A s2 = cv(cube, 8, C, x, y, z, N) + cv(cube, 9, C, x - 1, y, z, N) + cv(cube, 10, C, x, y - 1, z, N) +
                   cv(cube, 11, C, x - 1, y - 1, z, N);
      out[f] += (T)((double)s0 * inv_scale);
      out[C + f] += (T)((double)s1 * inv_scale);
      out[2 * C + f] += (T)((double)s2 * inv_scale);
    }
  }
}

template <int KIND>
int run_deposit(gev_ctx *ctx, gev_pcls *p, gev_field *out, double a, const gev_field *phi, double coeff,
                bool overwrite = false) {
  const int N = ctx->N;
  const size_t C = (size_t)N * N * N;
  const double dx = 1.0 / N;
  double mass = coeff / (dx * dx * dx);
  mass *= p->mass;
  if (KIND == DEP_T00 || KIND == DEP_TIJ) mass /= a;
  if (KIND == DEP_MASS) mass = p->mass / (dx * dx * dx);
  DepParams dp{N, mass, a, 0.};
  const int blocks = grid_for(ctx, C, 256, 16);
  if (ctx->prec == GEV_PREC_FP64) {
    int rc = ctx_ensure_cube(ctx, (size_t)NVAL[KIND] * C * 8);
    if (rc) return rc;
    if (overwrite) {
      rc = gev_field_zero(out);
      if (rc) return rc;
    }
    GevTimed tm_(ctx, "k_cube_fp64+k_gather");
    k_cube_fp64<KIND><<<blocks, 256, 0, ctx->stream>>>(p->cur, p->start, phi ? (const double *)phi->d : nullptr, dp,
                                                       (double *)ctx->d_cube);
    GEV_LAUNCH_CHECK(ctx);
    k_gather<KIND, double, double><<<blocks, 256, 0, ctx->stream>>>((const double *)ctx->d_cube, (double *)out->d, N, 1.);
    GEV_LAUNCH_CHECK(ctx);
  } else {
    int rc = deposit_fx(ctx, p, out, KIND, mass, a, phi, overwrite);
    if (rc) return rc;
  }
  return GEV_OK;
}

bool ok_field(gev_ctx *ctx, const gev_field *f, int ncomp) {
  return f && f->ctx == ctx && f->kind == GEV_FIELD_REAL && f->ncomp == ncomp;
}

}  // namespace

// projection_init + projection_T00 and projection_init + projection_Tij (coefficient
// 1); the mixed form deposits both in one sweep over the particles
int projection_replace_t00_tij(gev_ctx *ctx, gev_pcls *p, gev_field *T00, gev_field *Tij, double a,
                               const gev_field *phi) {
  if (ctx->prec == GEV_PREC_FP64) {
    int rc = run_deposit<DEP_T00>(ctx, p, T00, a, phi, 1., true);
    return rc ? rc : run_deposit<DEP_TIJ>(ctx, p, Tij, a, phi, 1., true);
  }
  const double dx = 1.0 / ctx->N;
  const double mass = 1. / (dx * dx * dx) * p->mass / a;  // as run_deposit: coeff / dx^3 * m / a
  return deposit_fx(ctx, p, T00, 4, mass, a, phi, true, Tij);
}

// projection_init followed by the deposit, in one pass for the mixed form
int projection_replace(gev_ctx *ctx, gev_pcls *p, gev_field *out, int kind, double a, const gev_field *phi) {
  switch (kind) {
    case DEP_T00:
      return run_deposit<DEP_T00>(ctx, p, out, a, phi, 1., true);
    case DEP_T0I:
      return run_deposit<DEP_T0I>(ctx, p, out, 1., phi, 1., true);
    case DEP_TIJ:
      return run_deposit<DEP_TIJ>(ctx, p, out, a, phi, 1., true);
    default:
      return run_deposit<DEP_MASS>(ctx, p, out, 1., nullptr, 1., true);
  }
}

extern "C" {

int gev_projection_T00(gev_ctx *ctx, gev_pcls *p, gev_field *T00, double a, const gev_field *phi, double coeff) {
  if (!ctx || !p || p->ctx != ctx || !ok_field(ctx, T00, 1) || (phi && !ok_field(ctx, phi, 1)) || a <= 0.)
    return gev_fail(ctx, GEV_EINVAL, "projection_T00: 1-component target, optional 1-component phi, a > 0");
  return run_deposit<DEP_T00>(ctx, p, T00, a, phi, coeff);
}
int gev_projection_T0i(gev_ctx *ctx, gev_pcls *p, gev_field *T0i, const gev_field *phi, double coeff) {
  if (!ctx || !p || p->ctx != ctx || !ok_field(ctx, T0i, 3) || (phi && !ok_field(ctx, phi, 1)))
    return gev_fail(ctx, GEV_EINVAL, "projection_T0i: 3-component target, optional 1-component phi");
  return run_deposit<DEP_T0I>(ctx, p, T0i, 1., phi, coeff);
}
int gev_projection_Tij(gev_ctx *ctx, gev_pcls *p, gev_field *Tij, double a, const gev_field *phi, double coeff) {
  if (!ctx || !p || p->ctx != ctx || !ok_field(ctx, Tij, 6) || (phi && !ok_field(ctx, phi, 1)) || a <= 0.)
    return gev_fail(ctx, GEV_EINVAL, "projection_Tij: 6-component target, optional 1-component phi, a > 0");
  return run_deposit<DEP_TIJ>(ctx, p, Tij, a, phi, coeff);
}
int gev_projection_T00_Tij(gev_ctx *ctx, gev_pcls *p, gev_field *T00, gev_field *Tij, double a, const gev_field *phi) {
  if (!ctx || !p || p->ctx != ctx || !ok_field(ctx, T00, 1) || !ok_field(ctx, Tij, 6) ||
      (phi && !ok_field(ctx, phi, 1)) || a <= 0.)
    return gev_fail(ctx, GEV_EINVAL, "projection_T00_Tij: 1- and 6-component targets, optional phi, a > 0");
  return projection_replace_t00_tij(ctx, p, T00, Tij, a, phi);
}
int gev_projection_mass(gev_ctx *ctx, gev_pcls *p, gev_field *rho) {
  if (!ctx || !p || p->ctx != ctx || !ok_field(ctx, rho, 1))
    return gev_fail(ctx, GEV_EINVAL, "projection_mass: 1-component target");
  return run_deposit<DEP_MASS>(ctx, p, rho, 1., nullptr, 1.);
}

}  // extern "C"
