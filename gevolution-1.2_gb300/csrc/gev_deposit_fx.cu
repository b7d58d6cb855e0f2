// gev_deposit_fx.cu -- the mixed-precision deposit: per-particle FP32
// contributions accumulated as 64-bit fixed-point integers.
//
// Same physics as projection_T00/T0i/Tij_project (gevolution.hpp:926-1297) and
// scalarProjectionCIC_project.  Layout of the work:
//   * a block owns a column tile of TX x TY cells and a chunk of TZ cell
//     layers, and sweeps the chunk in z;
//   * for each source layer z it walks the particles of the layer's TY rows
//     (contiguous runs of the (cell, ID)-ordered store, one thread per
//     particle) and adds each corner contribution, converted exactly to an
//     int64 with a power-of-two scale, into two shared-memory layers (field
//     z and z + 1) with 64-bit shared atomics -- integer adds, so the result
//     does not depend on their order;
//   * when layer z is complete it is flushed: cells that only this block can
//     touch are added straight into the FP32 field; cells on a tile face
//     (shared with a neighbouring block, including the periodic wrap) go into
//     a compact int64 face buffer with global atomics, which a fix-up pass
//     then adds to the field and clears.
// HBM traffic is one read of the particles, one read-modify-write of the
// target components, and the small face buffer -- no per-cell scratch.
#include <cmath>

#include "gev_internal.cuh"

namespace {

enum { FX_T00 = 0, FX_T0I = 1, FX_TIJ = 2, FX_MASS = 3 };
constexpr int FX_NC[4] = {1, 3, 6, 1};
constexpr int TX = 32, TY = 16, TZ = 32, FX_THREADS = 256;

struct FxParams {
  int N, lg;  // lg = log2 N for a power of two, else -1
  float mass, a;
  long nPX, nPY, nPZ;  // face planes per direction
  int overwrite;       // 1: the target's previous contents are replaced instead of added to
};

__device__ __forceinline__ long face_index(int x, int y, int z, const FxParams &p) {
  const long NN = (long)p.N * p.N;
  if (x % TX == 0) return (long)(x / TX) * NN + (long)z * p.N + y;
  if (y % TY == 0) return p.nPX * NN + (long)(y / TY) * NN + (long)z * p.N + x;
  return (p.nPX + p.nPY) * NN + (long)(z / TZ) * NN + (long)y * p.N + x;
}

// v * 2^k rounded to the nearest integer (ties away from zero), with integer
// instructions only: on GB300 the float -> int64 conversion instruction issues
// on the FP64 pipe, which is 1/64 of the FP32 rate.  The scale is a power of
// two, so v * s is exact and its value is mantissa * 2^(exponent - 150).
__device__ __forceinline__ long long fixed_of(float y) {
  const unsigned b = __float_as_uint(y);
  const int sh = min((int)((b >> 23) & 0xffu) - 150, 39);  // the clamp only matters for inf / NaN
  const long long m = (long long)((b & 0x7fffffu) | 0x800000u);
  long long q;
  if (sh >= 0)
    q = m << sh;  // |y| < 2^62 keeps sh <= 38
  else if (sh >= -24)
    q = (m + (1ll << (-sh - 1))) >> (-sh);
  else
    q = 0;  // |y| < 0.5 (this also covers y = 0 and denormals)
  return (b >> 31) ? -q : q;
}

__device__ __forceinline__ void sadd(unsigned long long *a, float v, float s) {
  const long long q = fixed_of(v * s);
  if (q != 0) atomicAdd(a, (unsigned long long)q);
}

// The fixed-point scale comes from the data, on the device: max |q|^2 over the
// particles and the most particles in one cell.  A cell's sum has at most 8 x that
// many contributions (its 8 neighbouring cells), each below c_max of the kind, and
// must stay below 2^62; max reductions do not depend on order, so neither does the
// scale.
__global__ void __launch_bounds__(256) k_fx_bounds(const float *__restrict__ vx, const float *__restrict__ vy,
                                                   const float *__restrict__ vz, long n,
                                                   const uint32_t *__restrict__ count, long C, uint32_t *bounds) {
  float q2 = 0.f;
  uint32_t mc = 0u;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    q2 = fmaxf(q2, vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i]);
  for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < C; c += (long)gridDim.x * blockDim.x)
    mc = max(mc, count[c]);
  for (int o = 16; o > 0; o >>= 1) {
    q2 = fmaxf(q2, __shfl_xor_sync(0xffffffffu, q2, o));
    mc = max(mc, __shfl_xor_sync(0xffffffffu, mc, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&bounds[0], __float_as_uint(q2));  // q2 >= 0: the bit patterns order as the values
    atomicMax(&bounds[1], mc);
  }
}

// per-particle contribution bounds, |phi| <= 1 taken for the (1 + f phi) factors:
// T00 m (e + (3e + q^2/e)|phi|) <= m (4e + q^2/a); T0i m |q_i| (1 + 2|phi|) <= 3 m |q|;
// Tij m q_i q_j / e (1 + 5|phi|) <= 6 m q^2 / a; mass m.  Writes the power k of the
// scale 2^k into bounds[2], kept in [-60, 100] (FP32 scale and float_of_fixed stay exact).
__global__ void k_fx_scale(uint32_t *bounds, int kind, double mass, double a) {
  const double q2 = (double)__uint_as_float(bounds[0]);
  const double mc = (double)(bounds[1] > 0u ? bounds[1] : 1u);
  const double e = sqrt(q2 + a * a);
  double c;
  if (kind == FX_MASS)
    c = mass;
  else if (kind == FX_T00)
    c = mass * (4. * e + q2 / a);
  else if (kind == FX_T0I)
    c = 3. * mass * sqrt(q2);
  else
    c = 6. * mass * q2 / a;
  const double bound = fabs(c) * 8. * mc;
  int k = 100;
  if (bound > 0.) {
    int e2 = 0;
    frexp(bound, &e2);  // bound < 2^e2
    k = 62 - e2;
  }
  k = k < -60 ? -60 : (k > 100 ? 100 : k);
  bounds[2] = (uint32_t)k;
}

template <int KIND>
__global__ void __launch_bounds__(FX_THREADS) k_dep_fx(PclsArrays P, const uint32_t *__restrict__ start,
                                                       const float *__restrict__ phi, float *out,
                                                       unsigned long long *face, FxParams p,
                                                       const uint32_t *__restrict__ fxb) {
  constexpr int NC = FX_NC[KIND];
  const int ks = (int)fxb[2];
  const float scale = __int_as_float((127 + ks) << 23);  // 2^ks
  constexpr int SX = TX + 1, SY = TY + 1, SL = SX * SY;  // one shared layer per component
  extern __shared__ __align__(16) unsigned long long lay[];  // [2][NC][SY][SX]
  __shared__ uint32_t rowoff[TY + 1], rowbase[TY];
  const int N = p.N;
  const long C = (long)N * N * N;
  const long NN = (long)N * N;
  const int ntx = (N + TX - 1) / TX, nty = (N + TY - 1) / TY;
  const long fstride = (p.nPX + p.nPY + p.nPZ) * NN;  // face entries per component
  const int bx = blockIdx.x % ntx, by = (blockIdx.x / ntx) % nty, bz = blockIdx.x / (ntx * nty);
  const int x0 = bx * TX, y0 = by * TY, z0 = bz * TZ;
  const int nx = min(TX, N - x0), ny = min(TY, N - y0), nz = min(TZ, N - z0);
  for (int i = threadIdx.x; i < 2 * NC * SL; i += blockDim.x) lay[i] = 0ull;
  int cur = 0;  // layer holding field z = zs; 1 - cur holds z = zs + 1
  for (int zs = z0; zs < z0 + nz; ++zs) {
    if (threadIdx.x < 32) {  // the layer's TY row runs: one lane per row, then a warp scan of the counts
      const int yy = threadIdx.x;
      uint32_t s = 0, cnt = 0;
      if (yy < ny) {
        const long c0 = x0 + (long)N * (y0 + yy) + NN * zs;
        s = start[c0];
        cnt = start[c0 + nx] - s;
      }
      uint32_t inc = cnt;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, inc, o);
        if (yy >= o) inc += v;
      }
      if (yy < ny) {
        rowbase[yy] = s;
        rowoff[yy] = inc - cnt;
      }
      if (yy == ny - 1) rowoff[ny] = inc;
    }
    __syncthreads();
    const uint32_t total = rowoff[ny];
    unsigned long long *A = lay + cur * NC * SL, *B = lay + (1 - cur) * NC * SL;
    for (uint32_t t = threadIdx.x; t < total; t += blockDim.x) {
      int yy = 0;
      while (rowoff[yy + 1] <= t) ++yy;
      const uint32_t j = rowbase[yy] + (t - rowoff[yy]);
      const uint32_t cell = P.cell[j];
      const int cx = p.lg >= 0 ? (int)(cell & (uint32_t)(N - 1)) : (int)(cell % N);
      const int cy = p.lg >= 0 ? (int)((cell >> p.lg) & (uint32_t)(N - 1)) : (int)((cell / N) % N);
      const int lx = cx - x0, ly = cy - y0;
      const float u0 = P.rx[j], u1 = P.ry[j], u2 = P.rz[j];
      const float d0 = 1.f - u0, d1 = 1.f - u1, d2 = 1.f - u2;
      const float w[8] = {d0 * d1 * d2, d0 * d1 * u2, d0 * u1 * d2, d0 * u1 * u2,
                          u0 * d1 * d2, u0 * d1 * u2, u0 * u1 * d2, u0 * u1 * u2};
      float l[8];
      if (KIND != FX_MASS && phi != nullptr) {
        const int xp = cx + 1 == N ? 0 : cx + 1, yp = cy + 1 == N ? 0 : cy + 1, zp = zs + 1 == N ? 0 : zs + 1;
        l[0] = __ldg(&phi[sidx(cx, cy, zs, N)]);
        l[1] = __ldg(&phi[sidx(cx, cy, zp, N)]);
        l[2] = __ldg(&phi[sidx(cx, yp, zs, N)]);
        l[3] = __ldg(&phi[sidx(cx, yp, zp, N)]);
        l[4] = __ldg(&phi[sidx(xp, cy, zs, N)]);
        l[5] = __ldg(&phi[sidx(xp, cy, zp, N)]);
        l[6] = __ldg(&phi[sidx(xp, yp, zs, N)]);
        l[7] = __ldg(&phi[sidx(xp, yp, zp, N)]);
      } else {
#pragma unroll
        for (int k = 0; k < 8; ++k) l[k] = 0.f;
      }
      // corner k = 4 dx + 2 dy + dz goes to layer dz at (ly + dy, lx + dx)
      const int o00 = ly * SX + lx, o01 = (ly + 1) * SX + lx, o10 = ly * SX + lx + 1, o11 = (ly + 1) * SX + lx + 1;
      const int off[8] = {o00, o00, o01, o01, o10, o10, o11, o11};
      const float s = scale, m = p.mass, a = p.a;
      if (KIND == FX_MASS || KIND == FX_T00) {
        float ee = a, ff = 0.f;
        if (KIND == FX_T00 && phi != nullptr) {
          const float q0 = ((const float *)P.vx)[j], q1 = ((const float *)P.vy)[j], q2 = ((const float *)P.vz)[j];
          const float f = q0 * q0 + q1 * q1 + q2 * q2;
          ee = sqrtf(f + a * a);
          ff = 3.f * ee + f / ee;
        }
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          const float v = KIND == FX_MASS ? m * w[k] : m * w[k] * (ee + ff * l[k]);
          sadd(((k & 1) ? B : A) + off[k], v, s);
        }
      } else if (KIND == FX_T0I) {
        const float q0 = ((const float *)P.vx)[j], q1 = ((const float *)P.vy)[j], q2 = ((const float *)P.vz)[j];
        // x component: CIC in y, z; NGP in x (gevolution.hpp:1107-1144)
        float wq = m * q0;
        sadd(A + o00, wq * d1 * d2 * (1.f + l[0] + l[4]), s);
        sadd(A + o01, wq * u1 * d2 * (1.f + l[2] + l[6]), s);
        sadd(B + o00, wq * d1 * u2 * (1.f + l[1] + l[5]), s);
        sadd(B + o01, wq * u1 * u2 * (1.f + l[3] + l[7]), s);
        wq = m * q1;
        sadd(A + SL + o00, wq * d0 * d2 * (1.f + l[0] + l[2]), s);
        sadd(A + SL + o10, wq * u0 * d2 * (1.f + l[4] + l[6]), s);
        sadd(B + SL + o00, wq * d0 * u2 * (1.f + l[1] + l[3]), s);
        sadd(B + SL + o10, wq * u0 * u2 * (1.f + l[5] + l[7]), s);
        wq = m * q2;
        sadd(A + 2 * SL + o00, wq * d0 * d1 * (1.f + l[0] + l[1]), s);
        sadd(A + 2 * SL + o10, wq * u0 * d1 * (1.f + l[4] + l[5]), s);
        sadd(A + 2 * SL + o01, wq * d0 * u1 * (1.f + l[2] + l[3]), s);
        sadd(A + 2 * SL + o11, wq * u0 * u1 * (1.f + l[6] + l[7]), s);
      } else {  // FX_TIJ, components 00 01 02 11 12 22
        const float q[3] = {((const float *)P.vx)[j], ((const float *)P.vy)[j], ((const float *)P.vz)[j]};
        float f = q[0] * q[0] + q[1] * q[1] + q[2] * q[2];
        const float ee = sqrtf(f + a * a), inv_e = 1.f / ee;
        f = 4.f + a * a / (f + a * a);
        const int dslot[3] = {0, 3, 5};
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const float wi = m * q[i] * q[i] * inv_e;
#pragma unroll
          for (int k = 0; k < 8; ++k) sadd(((k & 1) ? B : A) + dslot[i] * SL + off[k], wi * w[k] * (1.f + f * l[k]), s);
        }
        const float qf = 0.25f * f;
        float wq = m * q[0] * q[1] * inv_e;  // 01 on plaquettes: CIC in z only
        sadd(A + 1 * SL + o00, wq * d2 * (1.f + qf * (l[0] + l[2] + l[4] + l[6])), s);
        sadd(B + 1 * SL + o00, wq * u2 * (1.f + qf * (l[1] + l[3] + l[5] + l[7])), s);
        wq = m * q[0] * q[2] * inv_e;  // 02: CIC in y only
        sadd(A + 2 * SL + o00, wq * d1 * (1.f + qf * (l[0] + l[1] + l[4] + l[5])), s);
        sadd(A + 2 * SL + o01, wq * u1 * (1.f + qf * (l[2] + l[3] + l[6] + l[7])), s);
        wq = m * q[1] * q[2] * inv_e;  // 12: CIC in x only
        sadd(A + 4 * SL + o00, wq * d0 * (1.f + qf * (l[0] + l[1] + l[2] + l[3])), s);
        sadd(A + 4 * SL + o10, wq * u0 * (1.f + qf * (l[4] + l[5] + l[6] + l[7])), s);
      }
    }
    __syncthreads();
    // flush field layer zs (complete now) and clear it: one cell of the layer per
    // thread, its components in turn (the output component index equals the slot)
    for (int ci = threadIdx.x; ci < SL; ci += blockDim.x) {
      const int ly = ci / SX, lx = ci - ly * SX;
      if (lx > nx || ly > ny) continue;
      int x = x0 + lx, y = y0 + ly;
      if (x == N) x = 0;
      if (y == N) y = 0;
      const bool onface = lx == 0 || lx == nx || ly == 0 || ly == ny || zs == z0;
      const long fi = onface ? face_index(x, y, zs, p) : 0;
      const size_t gi = sidx(x, y, zs, N);
#pragma unroll
      for (int comp = 0; comp < NC; ++comp) {
        const unsigned long long v = A[comp * SL + ci];
        if (v != 0ull) A[comp * SL + ci] = 0ull;
        if (onface) {
          if (v != 0ull) atomicAdd(&face[(long)comp * fstride + fi], v);
        } else if (p.overwrite) {
          out[(long)comp * C + gi] = float_of_fixed((long long)v, ks);
        } else if (v != 0ull) {
          out[(long)comp * C + gi] += float_of_fixed((long long)v, ks);
        }
      }
    }
    __syncthreads();
    cur = 1 - cur;
  }
  // the layer above the chunk belongs to the next chunk's lower face
  {
    unsigned long long *A = lay + cur * NC * SL;
    int zf = z0 + nz;
    if (zf == N) zf = 0;
    for (int ci = threadIdx.x; ci < SL; ci += blockDim.x) {
      const int ly = ci / SX, lx = ci - ly * SX;
      if (lx > nx || ly > ny) continue;
      int x = x0 + lx, y = y0 + ly;
      if (x == N) x = 0;
      if (y == N) y = 0;
      const long fi = face_index(x, y, zf, p);
#pragma unroll
      for (int comp = 0; comp < NC; ++comp) {
        const unsigned long long v = A[comp * SL + ci];
        if (v != 0ull) atomicAdd(&face[(long)comp * fstride + fi], v);
      }
    }
  }
}

// add the face accumulators into the field (or, with p.overwrite, store them) and
// clear them.  A cell on several face planes has one entry, on the first of its
// x, y, z planes (face_index); in overwrite mode the other planes' entries for it
// (always zero) are skipped so that they do not overwrite the cell.
__global__ void __launch_bounds__(256) k_face_fix(unsigned long long *face, float *out, int ncomp, FxParams p,
                                                  const uint32_t *__restrict__ fxb) {
  const int N = p.N;
  const int ks = (int)fxb[2];
  const long NN = (long)N * N, C = NN * N;
  const int planes = (int)(p.nPX + p.nPY + p.nPZ);
  const long rows = (long)ncomp * planes * N;  // face entries come in rows of N (face_index)
  for (long row = blockIdx.x; row < rows; row += gridDim.x) {
    const int comp = (int)(row / ((long)planes * N));
    const int rr = (int)(row - (long)comp * planes * N);
    const int pl = rr / N, q = rr - pl * N;
    unsigned long long *f = face + row * N;
    float *o = out + comp * C;
    for (int t = threadIdx.x; t < N; t += blockDim.x) {
      const unsigned long long v = f[t];
      if (v == 0ull && !p.overwrite) continue;
      if (v != 0ull) f[t] = 0ull;
      int x, y, z;
      bool canonical = true;
      if (pl < p.nPX) {  // x plane: rows z, columns y
        x = pl * TX;
        z = q;
        y = t;
      } else if (pl < p.nPX + p.nPY) {  // y plane: rows z, columns x
        y = (int)(pl - p.nPX) * TY;
        z = q;
        x = t;
        canonical = x % TX != 0;
      } else {  // z plane: rows y, columns x
        z = (int)(pl - p.nPX - p.nPY) * TZ;
        y = q;
        x = t;
        canonical = x % TX != 0 && y % TY != 0;
      }
      if (p.overwrite) {
        if (canonical) o[sidx(x, y, z, N)] = float_of_fixed((long long)v, ks);
      } else {
        o[sidx(x, y, z, N)] += float_of_fixed((long long)v, ks);
      }
    }
  }
}

}  // namespace

// the fixed-point deposit of the mixed form; kind: 0 T00, 1 T0i, 2 Tij, 3 mass.
// overwrite: every cell of the target is written (the sum of this deposit alone),
// which spares the caller zeroing it first and the kernel reading it back.
int deposit_fx(gev_ctx *ctx, gev_pcls *p, gev_field *out, int kind, double mass, double a, const gev_field *phi,
               bool overwrite) {
  const int N = ctx->N;
  const int NC = FX_NC[kind];
  FxParams fp;
  fp.N = N;
  fp.lg = lg_pow2(N);
  fp.mass = (float)mass;
  fp.a = (float)a;
  fp.nPX = (N + TX - 1) / TX;
  fp.nPY = (N + TY - 1) / TY;
  fp.nPZ = (N + TZ - 1) / TZ;
  fp.overwrite = overwrite ? 1 : 0;
  const size_t face_elems = (size_t)(fp.nPX + fp.nPY + fp.nPZ) * N * N * NC;
  // the face buffer lives behind the deposit scratch pointer, kept zeroed between uses
  if (ctx->cube_bytes < face_elems * 8) {
    int rc = ctx_ensure_cube(ctx, face_elems * 8);
    if (rc) return rc;
    GEV_CHECK_CUDA(ctx, cudaMemsetAsync(ctx->d_cube, 0, ctx->cube_bytes, ctx->stream));
  }
  const int ntx = (N + TX - 1) / TX, nty = (N + TY - 1) / TY, ntz = (N + TZ - 1) / TZ;
  const size_t smem = 2 * (size_t)NC * (TX + 1) * (TY + 1) * 8;
  unsigned long long *face = (unsigned long long *)ctx->d_cube;
  const float *fphi = phi ? (const float *)phi->d : nullptr;
  float *fo = (float *)out->d;
  const unsigned blocks = (unsigned)(ntx * nty * ntz);
  const long C = (long)N * N * N;
  GEV_CHECK_CUDA(ctx, cudaMemsetAsync(p->bounds, 0, 2 * sizeof(uint32_t), ctx->stream));
  k_fx_bounds<<<grid_for(ctx, (size_t)(p->n > C ? p->n : C), 256, 8), 256, 0, ctx->stream>>>(
      (const float *)p->cur.vx, (const float *)p->cur.vy, (const float *)p->cur.vz, p->n, p->count, C, p->bounds);
  GEV_LAUNCH_CHECK(ctx);
  k_fx_scale<<<1, 1, 0, ctx->stream>>>(p->bounds, kind, mass, a);
  GEV_LAUNCH_CHECK(ctx);
  switch (kind) {
    case FX_T00:
      cudaFuncSetAttribute(k_dep_fx<FX_T00>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      k_dep_fx<FX_T00><<<blocks, FX_THREADS, smem, ctx->stream>>>(p->cur, p->start, fphi, fo, face, fp, p->bounds);
      break;
    case FX_T0I:
      cudaFuncSetAttribute(k_dep_fx<FX_T0I>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      k_dep_fx<FX_T0I><<<blocks, FX_THREADS, smem, ctx->stream>>>(p->cur, p->start, fphi, fo, face, fp, p->bounds);
      break;
    case FX_TIJ:
      cudaFuncSetAttribute(k_dep_fx<FX_TIJ>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      k_dep_fx<FX_TIJ><<<blocks, FX_THREADS, smem, ctx->stream>>>(p->cur, p->start, fphi, fo, face, fp, p->bounds);
      break;
    default:
      cudaFuncSetAttribute(k_dep_fx<FX_MASS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      k_dep_fx<FX_MASS><<<blocks, FX_THREADS, smem, ctx->stream>>>(p->cur, p->start, nullptr, fo, face, fp, p->bounds);
  }
  GEV_LAUNCH_CHECK(ctx);
  const long face_rows = (long)NC * (fp.nPX + fp.nPY + fp.nPZ) * N;
  const long ff_blocks = face_rows < (long)ctx->sms * 16 ? face_rows : (long)ctx->sms * 16;
  k_face_fix<<<(unsigned)ff_blocks, 256, 0, ctx->stream>>>(face, fo, NC, fp, p->bounds);
  GEV_LAUNCH_CHECK(ctx);
  return GEV_OK;
}
