// gev_deposit.cu -- the CIC / CIC-NGP stress-energy deposits.
//
// Replaces projection_T00/T0i/Tij_project and their *_comm halo folds
// (gevolution.hpp:926-1301) and LATfield2's scalarProjectionCIC_project.
// The reference accumulates each cell's particles into a small "local cube"
// and then adds the cube to the 8 (or fewer) surrounding field cells.  Here the
// same two levels run as two passes with no atomics:
//   pass 1 (a warp per 32 cells, a lane per particle): sum each cell's particles
//           -- contiguous in the (cell, ID)-ordered store -- into its cube values in
//           the reference's order of operations, multiplied by the mass and metric
//           factors the reference applies per cube;
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
  double dx, Nd;    // 1 / N and N (FP64 form)
  bool pow2;        // N a power of two: (pos - ref) / dx is (pos - ref) * N exactly
};

template <typename T>
__device__ __forceinline__ T ldf(const T *__restrict__ f, int x, int y, int z, int N) {
  return __ldg(&f[sidx(wrapi(x, N), wrapi(y, N), wrapi(z, N), N)]);
}

// One particle's contributions to its cell's cube, FP64 form, in the reference's
// order of operations (gevolution.hpp:955-1001 T00, 1085-1127 T0i, 1215-1270 Tij;
// the mass deposit of ic_basic.hpp's scalarProjectionCIC_project): every product and
// sum is an explicitly rounded intrinsic, evaluated left to right as the C++ source
// reads, and nothing is contracted into a multiply-add.  up = (pos - ref) / dx, dn =
// 1 - up.  The cube slots: T00 / mass the 8 corners (XYZ bits, z fastest); T0i the 12
// link sums (the 4 along x, y, z each); Tij the 3 x 8 diagonal corner sums, then
// the 6 off-diagonal plaquette sums (01 at z, z + 1; 02 at y, y + 1; 12 at x, x + 1).
__device__ __forceinline__ double m3(double a, double b, double c) { return __dmul_rn(__dmul_rn(a, b), c); }
template <int KIND>
__device__ __forceinline__ void contrib64(const PclsArrays &P, uint32_t j, const double (&l)[8], double rx, double ry,
                                          double rz, bool has_phi, const DepParams &dp, double (&c)[NVAL[KIND]]) {
  double up0, up1, up2;
  if (dp.pow2) {
    up0 = __dmul_rn(__dsub_rn(P.px[j], rx), dp.Nd);
    up1 = __dmul_rn(__dsub_rn(P.py[j], ry), dp.Nd);
    up2 = __dmul_rn(__dsub_rn(P.pz[j], rz), dp.Nd);
  } else {
    up0 = __ddiv_rn(__dsub_rn(P.px[j], rx), dp.dx);
    up1 = __ddiv_rn(__dsub_rn(P.py[j], ry), dp.dx);
    up2 = __ddiv_rn(__dsub_rn(P.pz[j], rz), dp.dx);
  }
  const double dn0 = __dsub_rn(1.0, up0), dn1 = __dsub_rn(1.0, up1), dn2 = __dsub_rn(1.0, up2);
  const double a = dp.a, aa = __dmul_rn(a, a);
  if constexpr (KIND == DEP_MASS || KIND == DEP_T00) {
    const double w[8] = {m3(dn0, dn1, dn2), m3(dn0, dn1, up2), m3(dn0, up1, dn2), m3(dn0, up1, up2),
                         m3(up0, dn1, dn2), m3(up0, dn1, up2), m3(up0, up1, dn2), m3(up0, up1, up2)};
    if constexpr (KIND == DEP_MASS) {
#pragma unroll
      for (int k = 0; k < 8; ++k) c[k] = w[k];
    } else {
      double e = a, f = 0.;
      if (has_phi) {
        const double *vx = (const double *)P.vx, *vy = (const double *)P.vy, *vz = (const double *)P.vz;
        const double q0 = vx[j], q1 = vy[j], q2 = vz[j];
        f = __dadd_rn(__dadd_rn(__dmul_rn(q0, q0), __dmul_rn(q1, q1)), __dmul_rn(q2, q2));
        e = __dsqrt_rn(__dadd_rn(f, aa));
        f = __dadd_rn(__dmul_rn(3., e), __ddiv_rn(f, e));
      }
#pragma unroll
      for (int k = 0; k < 8; ++k) c[k] = __dmul_rn(w[k], __dadd_rn(e, __dmul_rn(f, l[k])));
    }
  } else if constexpr (KIND == DEP_T0I) {
    const double *vx = (const double *)P.vx, *vy = (const double *)P.vy, *vz = (const double *)P.vz;
    double w = __dmul_rn(dp.mass, vx[j]);
    c[0] = m3(w, dn1, dn2);
    c[1] = m3(w, up1, dn2);
    c[2] = m3(w, dn1, up2);
    c[3] = m3(w, up1, up2);
    w = __dmul_rn(dp.mass, vy[j]);
    c[4] = m3(w, dn0, dn2);
    c[5] = m3(w, up0, dn2);
    c[6] = m3(w, dn0, up2);
    c[7] = m3(w, up0, up2);
    w = __dmul_rn(dp.mass, vz[j]);
    c[8] = m3(w, dn0, dn1);
    c[9] = m3(w, up0, dn1);
    c[10] = m3(w, dn0, up1);
    c[11] = m3(w, up0, up1);
  } else {  // DEP_TIJ
    const double *vx = (const double *)P.vx, *vy = (const double *)P.vy, *vz = (const double *)P.vz;
    const double q[3] = {vx[j], vy[j], vz[j]};
    double f = __dadd_rn(__dadd_rn(__dmul_rn(q[0], q[0]), __dmul_rn(q[1], q[1])), __dmul_rn(q[2], q[2]));
    const double e = __dsqrt_rn(__dadd_rn(f, aa));
    f = __dadd_rn(4., __ddiv_rn(aa, __dadd_rn(f, aa)));
    const double g[8] = {__dadd_rn(1., __dmul_rn(f, l[0])), __dadd_rn(1., __dmul_rn(f, l[1])),
                         __dadd_rn(1., __dmul_rn(f, l[2])), __dadd_rn(1., __dmul_rn(f, l[3])),
                         __dadd_rn(1., __dmul_rn(f, l[4])), __dadd_rn(1., __dmul_rn(f, l[5])),
                         __dadd_rn(1., __dmul_rn(f, l[6])), __dadd_rn(1., __dmul_rn(f, l[7]))};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const double w = __ddiv_rn(__dmul_rn(__dmul_rn(dp.mass, q[i]), q[i]), e);
      const double w0 = __dmul_rn(w, dn0), w1 = __dmul_rn(w, up0);
      const double w00 = __dmul_rn(w0, dn1), w01 = __dmul_rn(w0, up1), w10 = __dmul_rn(w1, dn1),
                   w11 = __dmul_rn(w1, up1);
      c[8 * i + 0] = __dmul_rn(__dmul_rn(w00, dn2), g[0]);
      c[8 * i + 1] = __dmul_rn(__dmul_rn(w00, up2), g[1]);
      c[8 * i + 2] = __dmul_rn(__dmul_rn(w01, dn2), g[2]);
      c[8 * i + 3] = __dmul_rn(__dmul_rn(w01, up2), g[3]);
      c[8 * i + 4] = __dmul_rn(__dmul_rn(w10, dn2), g[4]);
      c[8 * i + 5] = __dmul_rn(__dmul_rn(w10, up2), g[5]);
      c[8 * i + 6] = __dmul_rn(__dmul_rn(w11, dn2), g[6]);
      c[8 * i + 7] = __dmul_rn(__dmul_rn(w11, up2), g[7]);
    }
    const double qf = __dmul_rn(f, 0.25);
    auto h = [&](double x0, double x1, double x2, double x3) {
      return __dadd_rn(1., __dmul_rn(qf, __dadd_rn(__dadd_rn(__dadd_rn(x0, x1), x2), x3)));
    };
    double w = __ddiv_rn(__dmul_rn(__dmul_rn(dp.mass, q[0]), q[1]), e);
    c[24] = __dmul_rn(__dmul_rn(w, dn2), h(l[0], l[2], l[4], l[6]));
    c[25] = __dmul_rn(__dmul_rn(w, up2), h(l[1], l[3], l[5], l[7]));
    w = __ddiv_rn(__dmul_rn(__dmul_rn(dp.mass, q[0]), q[2]), e);
    c[26] = __dmul_rn(__dmul_rn(w, dn1), h(l[0], l[1], l[4], l[5]));
    c[27] = __dmul_rn(__dmul_rn(w, up1), h(l[2], l[3], l[6], l[7]));
    w = __ddiv_rn(__dmul_rn(__dmul_rn(dp.mass, q[1]), q[2]), e);
    c[28] = __dmul_rn(__dmul_rn(w, dn0), h(l[0], l[1], l[2], l[3]));
    c[29] = __dmul_rn(__dmul_rn(w, up0), h(l[4], l[5], l[6], l[7]));
  }
}

// phi at the cell's 8 corners (XYZ bits, z fastest), or zeros
__device__ __forceinline__ void corner_phi(const double *__restrict__ phi, int cx, int cy, int cz, int N,
                                           double (&l)[8]) {
#pragma unroll
  for (int k = 0; k < 8; ++k) l[k] = phi ? ldf(phi, cx + (k >> 2), cy + ((k >> 1) & 1), cz + (k & 1), N) : 0.;
}

// slot k of a cell's finished sums, as the reference's fold adds it: T00 and the
// mass deposit times the mass factor, T0i times the link's (1 + phi_a + phi_b)
// (gevolution.hpp:1129-1144, phi at the link's two corners), Tij as summed
template <int KIND>
__device__ __forceinline__ double cube_out(double acc, int k, const double *__restrict__ phi, int cx, int cy, int cz,
                                           const DepParams &dp) {
  if constexpr (KIND == DEP_T00 || KIND == DEP_MASS) return __dmul_rn(acc, dp.mass);
  if constexpr (KIND == DEP_T0I) {
    // links along x: corners (0,dy,dz)-(1,dy,dz); along y: (dx,0,dz)-(dx,1,dz); along z: (dx,dy,0)-(dx,dy,1)
    const int i = k >> 2, t = k & 3;
    int c0;
    if (i == 0) c0 = ((t & 1) << 1) | (t >> 1);  // dy = t & 1, dz = t >> 1
    else if (i == 1) c0 = ((t & 1) << 2) | (t >> 1);
    else c0 = ((t & 1) << 2) | ((t >> 1) << 1);
    const int c1 = c0 | (i == 0 ? 4 : (i == 1 ? 2 : 1));
    const int N = dp.N;
    const double l0 = phi ? ldf(phi, cx + (c0 >> 2), cy + ((c0 >> 1) & 1), cz + (c0 & 1), N) : 0.;
    const double l1 = phi ? ldf(phi, cx + (c1 >> 2), cy + ((c1 >> 1) & 1), cz + (c1 & 1), N) : 0.;
    return __dmul_rn(acc, __dadd_rn(__dadd_rn(1., l0), l1));
  }
  return acc;
}

// pass 1, FP64 form: cube[k * C + c] (SoA so that pass 2 reads coalesced rows).  A warp
// takes 32 consecutive cells and walks their particles -- contiguous in the (cell,
// ID)-ordered store -- 32 at a time: each lane forms one particle's contributions,
// and lane k then adds slot k's contributions in the particles' order, starting
// from 0 at each new cell, as the reference's loop over a cell's particles adds them.
// Every lane forms contributions whatever the cells hold (a thread a cell left most
// lanes idle beside the fullest cell of their warp, and FP64 issue is scarce); the
// ordered sums cost one addition a particle for each slot.  A cell's sums are staged
// in shared memory and the tile's cube rows written once, empty cells as 0.
constexpr int CUBE_WARPS = 2;
template <int KIND>
__global__ void __launch_bounds__(32 * CUBE_WARPS) k_cube_fp64(PclsArrays P, const uint32_t *__restrict__ start,
                                                              const double *__restrict__ phi, DepParams dp,
                                                              double *cube) {
  constexpr int NV = NVAL[KIND];
  __shared__ double sb[CUBE_WARPS][NV][33];  // the chunk's contributions, slot-major
  __shared__ double so[CUBE_WARPS][NV][32];  // the tile's cell sums
  __shared__ int sc[CUBE_WARPS][32];         // the chunk's particles' cells, tile-relative
  const int N = dp.N;
  const size_t C = (size_t)N * N * N;
  const int lane = threadIdx.x & 31, wb = threadIdx.x >> 5;
  const size_t ntiles = (C + 31) / 32;
  for (size_t t = blockIdx.x * (size_t)CUBE_WARPS + wb; t < ntiles; t += (size_t)gridDim.x * CUBE_WARPS) {
    const size_t c0 = t * 32, cend = c0 + 32 < C ? c0 + 32 : C;
    const uint32_t s0 = start[c0], s1 = start[cend];
#pragma unroll
    for (int k = 0; k < NV; ++k) so[wb][k][lane] = 0.;
    int cur = -1;
    double acc = 0.;
    for (uint32_t base = s0; base < s1; base += 32) {
      const uint32_t j = base + lane;
      if (j < s1) {
        const uint32_t c = P.cell[j];
        const int cx = (int)(c % (uint32_t)N), cy = (int)((c / (uint32_t)N) % (uint32_t)N),
                  cz = (int)(c / ((uint32_t)N * (uint32_t)N));
        double l[8];
        corner_phi(KIND != DEP_MASS ? phi : nullptr, cx, cy, cz, N, l);
        const double rx = __dmul_rn((double)cx, dp.dx), ry = __dmul_rn((double)cy, dp.dx),
                     rz = __dmul_rn((double)cz, dp.dx);
        double cj[NV];
        contrib64<KIND>(P, j, l, rx, ry, rz, phi != nullptr, dp, cj);
#pragma unroll
        for (int k = 0; k < NV; ++k) sb[wb][k][lane] = cj[k];
        sc[wb][lane] = (int)(c - (uint32_t)c0);
      }
      __syncwarp();
      const int m = (int)min(32u, s1 - base);
      if (lane < NV) {
        for (int i = 0; i < m; ++i) {
          const int ci = sc[wb][i];
          if (ci != cur) {
            if (cur >= 0 && cur < 32) {  // (a particle's cell is always one of the tile's)
              const uint32_t cc = (uint32_t)c0 + (uint32_t)cur;
              so[wb][lane][cur] = cube_out<KIND>(acc, lane, phi, (int)(cc % (uint32_t)N),
                                                 (int)((cc / (uint32_t)N) % (uint32_t)N),
                                                 (int)(cc / ((uint32_t)N * (uint32_t)N)), dp);
            }
            cur = ci;
            acc = 0.;
          }
          acc = __dadd_rn(acc, sb[wb][lane][i]);
        }
      }
      __syncwarp();
    }
    if (lane < NV && cur >= 0 && cur < 32) {
      const uint32_t cc = (uint32_t)c0 + (uint32_t)cur;
      so[wb][lane][cur] = cube_out<KIND>(acc, lane, phi, (int)(cc % (uint32_t)N), (int)((cc / (uint32_t)N) % (uint32_t)N),
                                         (int)(cc / ((uint32_t)N * (uint32_t)N)), dp);
    }
    __syncwarp();
    if (c0 + lane < cend) {
#pragma unroll
      for (int k = 0; k < NV; ++k) cube[k * C + c0 + lane] = so[wb][k][lane];
    }
    __syncwarp();
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
      // the source cells in the reference's order: the plane below first, each plane in
      // site order
      const A s0 = cv(cube, 3, C, x, y - 1, z - 1, N) + cv(cube, 2, C, x, y, z - 1, N) + cv(cube, 1, C, x, y - 1, z, N) +
                   cv(cube, 0, C, x, y, z, N);
      const A s1 = cv(cube, 7, C, x - 1, y, z - 1, N) + cv(cube, 6, C, x, y, z - 1, N) + cv(cube, 5, C, x - 1, y, z, N) +
                   cv(cube, 4, C, x, y, z, N);
      const A s2 = cv(cube, 11, C, x - 1, y - 1, z, N) + cv(cube, 10, C, x, y - 1, z, N) +
                   cv(cube, 9, C, x - 1, y, z, N) + cv(cube, 8, C, x, y, z, N);
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
  DepParams dp{N, mass, a, 0., dx, (double)N, (N & (N - 1)) == 0};
  const int blocks = grid_for(ctx, C, 256, 16);
  if (ctx->prec == GEV_PREC_FP64) {
    int rc = ctx_ensure_cube(ctx, (size_t)NVAL[KIND] * C * 8);
    if (rc) return rc;
    if (overwrite) {
      rc = gev_field_zero(out);
      if (rc) return rc;
    }
    GevTimed tm_(ctx, "k_cube_fp64+k_gather");
    const long ntiles = (long)((C + 31) / 32);
    k_cube_fp64<KIND><<<grid_for(ctx, (size_t)ntiles, CUBE_WARPS, 8),
                        32 * CUBE_WARPS, 0, ctx->stream>>>(p->cur, p->start, phi ? (const double *)phi->d : nullptr, dp,
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
