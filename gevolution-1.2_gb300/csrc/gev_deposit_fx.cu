// gev_deposit_fx.cu -- the mixed-precision deposit: per-particle FP32
// contributions accumulated as 64-bit fixed-point integers.
//
// Same physics as projection_T00/T0i/Tij_project (gevolution.hpp:926-1297) and
// scalarProjectionCIC_project.  Layout of the work:
//   * a block owns a column tile of TX x TY cells and a chunk of TZ cell
//     layers, and sweeps the chunk in z;
//   * for each source layer z it walks the particles of the layer's TY rows
//     (contiguous runs of the cell-ordered store, one thread per particle) and
//     adds each corner contribution into two shared-memory layers (field z and z + 1) with
//     64-bit shared atomics.  A contribution is the product of two integers:
//     the particle's prefactor rounded once to an int32 (scale 2^kq) and the
//     corner's weight factor rounded to 22 bits (scale 2^kg, one FFMA) -- the
//     scales come from the data (largest |q|, |phi|, fullest cell) so no sum
//     can overflow, and integer adds make the result independent of order;
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

// kinds; FX_T00TIJ deposits T00 (slot 0) and Tij (slots 1-6) in one sweep
enum { FX_T00 = 0, FX_T0I = 1, FX_TIJ = 2, FX_MASS = 3, FX_T00TIJ = 4 };
constexpr int FX_NC[5] = {1, 3, 6, 1, 7};
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

// The fixed-point scale comes from the data, on the device: max |q|^2 over the
// particles and the most particles in one cell.  A cell's sum has at most 8 x that
// many contributions (its 8 neighbouring cells), each below c_max of the kind, and
// must stay below 2^62; max reductions do not depend on order, so neither does the
// scale.
__global__ void __launch_bounds__(256) k_fx_bounds(const float *__restrict__ vx, const float *__restrict__ vy,
                                                   const float *__restrict__ vz, long n,
                                                   const uint32_t *__restrict__ count, const float *__restrict__ phi,
                                                   long C, uint32_t *bounds) {
  float q2 = 0.f, ph = 0.f;
  uint32_t mc = 0u;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    q2 = fmaxf(q2, vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i]);
  for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < C; c += (long)gridDim.x * blockDim.x) {
    mc = max(mc, count[c]);
    if (phi) ph = fmaxf(ph, fabsf(phi[c]));
  }
  for (int o = 16; o > 0; o >>= 1) {
    q2 = fmaxf(q2, __shfl_xor_sync(0xffffffffu, q2, o));
    ph = fmaxf(ph, __shfl_xor_sync(0xffffffffu, ph, o));
    mc = max(mc, __shfl_xor_sync(0xffffffffu, mc, o));
  }
  if ((threadIdx.x & 31) == 0) {  // non-negative floats: the bit patterns order as the values
    atomicMax(&bounds[0], __float_as_uint(q2));
    atomicMax(&bounds[1], mc);
    atomicMax(&bounds[4], __float_as_uint(ph));
  }
}

// per-particle contribution bounds, |phi| <= 1 taken for the (1 + f phi) factors:
// T00 m (e + (3e + q^2/e)|phi|) <= m (4e + q^2/a); T0i m |q_i| (1 + 2|phi|) <= 3 m |q|;
// Tij m q_i q_j / e (1 + 5|phi|) <= 6 m q^2 / a; mass m.  Writes the power k of the
// scale 2^k into bounds[2], kept in [-60, 100] (FP32 scale and float_of_fixed stay exact).
// Each contribution is Q * G: Q = round(p 2^kq) an int32 per particle and quantity
// (p its prefactor, e.g. m q_i^2 / e), G = round(g 2^kg) an integer below 2^22 per
// corner (g its weight factor, e.g. w_k (1 + f phi_k)), their product one 32x32->64
// multiply.  gmax bounds |g| (|phi| from the data), pmax bounds |p|; the 8 x (max
// particles per cell) contributions a cell receives stay below 2^62.  The sum's
// scale is 2^(kq + kg).  Powers are written to bounds[5 + 2 group] (kq) and
// bounds[6 + 2 group] (kg); bounds[2 + group] = kq + kg.
__device__ void fx_group(uint32_t *bounds, int group, double pmax, double gmax, double mc) {
  int eg = 0;
  frexp(gmax, &eg);  // gmax < 2^eg
  const int kg = 22 - eg;
  // |Q| <= Qlim with 8 mc Qlim 2^22 <= 2^62
  double qlim = ldexp(1.0, 37) / mc;
  if (qlim > 2147483647.0) qlim = 2147483647.0;
  int kq = 100;
  if (pmax > 0.) {
    int ep = 0, el = 0;
    frexp(pmax, &ep);                    // pmax < 2^ep
    frexp(qlim, &el);                    // qlim < 2^el, so 2^(el - 1) <= qlim
    kq = (el - 1) - ep;
  }
  kq = kq < -60 ? -60 : (kq > 100 ? 100 : kq);
  bounds[5 + 2 * group] = (uint32_t)kq;
  bounds[6 + 2 * group] = (uint32_t)kg;
  bounds[2 + group] = (uint32_t)(kq + kg);
}
// prefactor and weight-factor bounds per kind (|phi| <= phimax):
// mass p = m, g = w; T00 p = m e, g = w (1 + (3 + q^2/e^2) phi) <= 1 + 4 phimax;
// T0i p = m q_i, g = w (1 + 2 phi); Tij p = m q_i q_j / e <= m q^2 / a, g <= 1 + 5 phimax.
__global__ void k_fx_scale(uint32_t *bounds, int kind, double mass, double a) {
  const double q2 = (double)__uint_as_float(bounds[0]);
  const double mc = (double)(bounds[1] > 0u ? bounds[1] : 1u);
  const double ph = (double)__uint_as_float(bounds[4]);
  const double m = fabs(mass);
  const double e = sqrt(q2 + a * a);
  if (kind == FX_MASS) {
    fx_group(bounds, 0, m, 1., mc);
  } else if (kind == FX_T00 || kind == FX_T00TIJ) {
    fx_group(bounds, 0, m * e, 1. + 4. * ph, mc);
    if (kind == FX_T00TIJ) fx_group(bounds, 1, m * q2 / a, 1. + 5. * ph, mc);
  } else if (kind == FX_T0I) {
    fx_group(bounds, 0, m * sqrt(q2), 1. + 2. * ph, mc);
  } else {
    fx_group(bounds, 0, m * q2 / a, 1. + 5. * ph, mc);
  }
}

// round(y) for |y| < 2^31, integer instructions only
__device__ __forceinline__ int fixed32_of(float y) {
  const unsigned b = __float_as_uint(y);
  const int sh = (int)((b >> 23) & 0xffu) - 150;
  const int m = (int)((b & 0x7fffffu) | 0x800000u);
  int q;
  if (sh >= 0)
    q = sh < 8 ? m << sh : 0x7fffffff;  // the bound keeps |y| < 2^31
  else if (sh >= -24)
    q = (m + (1 << (-sh - 1))) >> (-sh);
  else
    q = 0;
  return (b >> 31) ? -q : q;
}
// round(g 2^kg) for |g| 2^kg <= 2^22: one FFMA with 1.5 * 2^23 (a single rounding
// to nearest even), then the integer in the low mantissa bits
__device__ __forceinline__ int gq(float g, float sg) {
  return __float_as_int(__fmaf_rn(g, sg, 12582912.0f)) - 0x4B400000;
}
__device__ __forceinline__ void iadd(unsigned long long *a, int Q, int G) {
  atomicAdd(a, (unsigned long long)((long long)Q * (long long)G));
}
__device__ __forceinline__ float pow2f(int k) { return __int_as_float((127 + k) << 23); }

// scale power of output component comp
template <int KIND>
__device__ __forceinline__ int comp_shift(int comp, int ks0, int ks1) {
  return (KIND == FX_T00TIJ && comp > 0) ? ks1 : ks0;
}

// where component comp of the deposit goes: the first output holds nc0 components
struct FxOut {
  float *o0, *o1;
  int nc0;
};
__device__ __forceinline__ float *comp_ptr(const FxOut &o, int comp, long C) {
  return comp < o.nc0 ? o.o0 + comp * C : o.o1 + (comp - o.nc0) * C;
}

// per-particle contributions.  A: the accumulator layer of field z = zs, B: of
// zs + 1, each [slot][SY][SX]; off[k] the cell of corner k = 4 dx + 2 dy + dz.
// sq = 2^kq, sg = 2^kg of the quantity's group.
template <int SL>
__device__ __forceinline__ void add_t00(unsigned long long *A, unsigned long long *B, const int *off,
                                        const float *w, const float *l, float m, float ee, float r, float sq,
                                        float sg) {
  const int Q = fixed32_of(m * ee * sq);  // m w (ee + ff phi) = (m ee) w (1 + r phi), r = ff / ee
#pragma unroll
  for (int k = 0; k < 8; ++k) iadd(((k & 1) ? B : A) + off[k], Q, gq(w[k] * (1.f + r * l[k]), sg));
}
template <int SL>
__device__ __forceinline__ void add_tij(unsigned long long *A, unsigned long long *B, const int *off, const float *w,
                                        const float *l, const float *q, float m, float inv_e, float f, float u0,
                                        float u1, float u2, float sq, float sg) {
  const float d0 = 1.f - u0, d1 = 1.f - u1, d2 = 1.f - u2;
  const int o00 = off[0], o01 = off[2], o10 = off[4];
  int G[8];  // the diagonal components share the corner factors w_k (1 + f phi_k)
#pragma unroll
  for (int k = 0; k < 8; ++k) G[k] = gq(w[k] * (1.f + f * l[k]), sg);
  const int dslot[3] = {0, 3, 5};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const int Q = fixed32_of(m * q[i] * q[i] * inv_e * sq);
#pragma unroll
    for (int k = 0; k < 8; ++k) iadd(((k & 1) ? B : A) + dslot[i] * SL + off[k], Q, G[k]);
  }
  const float qf = 0.25f * f;
  int Q = fixed32_of(m * q[0] * q[1] * inv_e * sq);  // 01 on plaquettes: CIC in z only
  iadd(A + 1 * SL + o00, Q, gq(d2 * (1.f + qf * (l[0] + l[2] + l[4] + l[6])), sg));
  iadd(B + 1 * SL + o00, Q, gq(u2 * (1.f + qf * (l[1] + l[3] + l[5] + l[7])), sg));
  Q = fixed32_of(m * q[0] * q[2] * inv_e * sq);  // 02: CIC in y only
  iadd(A + 2 * SL + o00, Q, gq(d1 * (1.f + qf * (l[0] + l[1] + l[4] + l[5])), sg));
  iadd(A + 2 * SL + o01, Q, gq(u1 * (1.f + qf * (l[2] + l[3] + l[6] + l[7])), sg));
  Q = fixed32_of(m * q[1] * q[2] * inv_e * sq);  // 12: CIC in x only
  iadd(A + 4 * SL + o00, Q, gq(d0 * (1.f + qf * (l[0] + l[1] + l[2] + l[3])), sg));
  iadd(A + 4 * SL + o10, Q, gq(u0 * (1.f + qf * (l[4] + l[5] + l[6] + l[7])), sg));
}

template <int KIND>
__global__ void __launch_bounds__(FX_THREADS, 3) k_dep_fx(PclsArrays P, const uint32_t *__restrict__ start,
                                                       const float *__restrict__ phi, FxOut out,
                                                       unsigned long long *face, FxParams p,
                                                       const uint32_t *__restrict__ fxb) {
  constexpr int NC = FX_NC[KIND];
  constexpr int SX = TX + 1, SY = TY + 1, SL = SX * SY;  // one shared layer per component
  constexpr bool USE_PHI = KIND != FX_MASS;
  extern __shared__ __align__(16) unsigned long long lay[];  // [2][NC][SY][SX]
  __shared__ uint32_t rowoff[TY + 1], rowbase[TY];
  const int ks0 = (int)fxb[2], ks1 = (int)fxb[3];  // accumulator scales 2^(kq + kg) of groups 0, 1
  const float sq0 = pow2f((int)fxb[5]), sg0 = pow2f((int)fxb[6]);
  const float sq1 = pow2f((int)fxb[7]), sg1 = pow2f((int)fxb[8]);
  const int N = p.N;
  const long C = (long)N * N * N;
  const long NN = (long)N * N;
  const int ntx = (N + TX - 1) / TX, nty = (N + TY - 1) / TY;
  const long fstride = (p.nPX + p.nPY + p.nPZ) * NN;  // face entries per component
  const int bx = blockIdx.x % ntx, by = (blockIdx.x / ntx) % nty, bz = blockIdx.x / (ntx * nty);
  const int x0 = bx * TX, y0 = by * TY, z0 = bz * TZ;
  const int nx = min(TX, N - x0), ny = min(TY, N - y0), nz = min(TZ, N - z0);
  const bool have_phi = USE_PHI && phi != nullptr;
  for (int i = threadIdx.x; i < 2 * NC * SL; i += blockDim.x) lay[i] = 0ull;
  int cur = 0;  // accumulator layer holding field z = zs; 1 - cur holds z = zs + 1
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
      int lo = 0, hi = ny;  // the row: the last yy with rowoff[yy] <= t (rowoff[ny] > t)
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (rowoff[mid] <= t)
          lo = mid;
        else
          hi = mid;
      }
      const int ly = lo;
      const uint32_t j = rowbase[ly] + (t - rowoff[ly]);
      const uint32_t cell = P.cell[j];
      const int cx = p.lg >= 0 ? (int)(cell & (uint32_t)(N - 1)) : (int)(cell % N);
      const int lx = cx - x0;
      const float u0 = P.rx[j], u1 = P.ry[j], u2 = P.rz[j];
      const float d0 = 1.f - u0, d1 = 1.f - u1, d2 = 1.f - u2;
      const float w[8] = {d0 * d1 * d2, d0 * d1 * u2, d0 * u1 * d2, d0 * u1 * u2,
                          u0 * d1 * d2, u0 * d1 * u2, u0 * u1 * d2, u0 * u1 * u2};
      // corner k = 4 dx + 2 dy + dz goes to layer dz at (ly + dy, lx + dx)
      const int o00 = ly * SX + lx, o01 = (ly + 1) * SX + lx, o10 = ly * SX + lx + 1, o11 = (ly + 1) * SX + lx + 1;
      const int off[8] = {o00, o00, o01, o01, o10, o10, o11, o11};
      float l[8];
      if (have_phi) {  // phi at the 8 corners (periodic)
        const int cy = ly + y0, xp = cx + 1 == N ? 0 : cx + 1, yp = cy + 1 == N ? 0 : cy + 1;
        const int zp = zs + 1 == N ? 0 : zs + 1;
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
      const float m = p.mass, a = p.a;
      if (KIND == FX_MASS) {
        const int Q = fixed32_of(m * sq0);
#pragma unroll
        for (int k = 0; k < 8; ++k) iadd(((k & 1) ? B : A) + off[k], Q, gq(w[k], sg0));
      } else if (KIND == FX_T0I) {
        const float q0 = ((const float *)P.vx)[j], q1 = ((const float *)P.vy)[j], q2 = ((const float *)P.vz)[j];
        // x component: CIC in y, z; NGP in x (gevolution.hpp:1107-1144)
        int Q = fixed32_of(m * q0 * sq0);
        iadd(A + o00, Q, gq(d1 * d2 * (1.f + l[0] + l[4]), sg0));
        iadd(A + o01, Q, gq(u1 * d2 * (1.f + l[2] + l[6]), sg0));
        iadd(B + o00, Q, gq(d1 * u2 * (1.f + l[1] + l[5]), sg0));
        iadd(B + o01, Q, gq(u1 * u2 * (1.f + l[3] + l[7]), sg0));
        Q = fixed32_of(m * q1 * sq0);
        iadd(A + SL + o00, Q, gq(d0 * d2 * (1.f + l[0] + l[2]), sg0));
        iadd(A + SL + o10, Q, gq(u0 * d2 * (1.f + l[4] + l[6]), sg0));
        iadd(B + SL + o00, Q, gq(d0 * u2 * (1.f + l[1] + l[3]), sg0));
        iadd(B + SL + o10, Q, gq(u0 * u2 * (1.f + l[5] + l[7]), sg0));
        Q = fixed32_of(m * q2 * sq0);
        iadd(A + 2 * SL + o00, Q, gq(d0 * d1 * (1.f + l[0] + l[1]), sg0));
        iadd(A + 2 * SL + o10, Q, gq(u0 * d1 * (1.f + l[4] + l[5]), sg0));
        iadd(A + 2 * SL + o01, Q, gq(d0 * u1 * (1.f + l[2] + l[3]), sg0));
        iadd(A + 2 * SL + o11, Q, gq(u0 * u1 * (1.f + l[6] + l[7]), sg0));
      } else {
        const float q[3] = {((const float *)P.vx)[j], ((const float *)P.vy)[j], ((const float *)P.vz)[j]};
        const float f2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2];
        if (KIND == FX_T00 || KIND == FX_T00TIJ) {
          float ee = a, r = 0.f;
          if (have_phi) {
            ee = sqrtf(f2 + a * a);
            r = (3.f * ee + f2 / ee) / ee;
          }
          add_t00<SL>(A, B, off, w, l, m, ee, r, sq0, sg0);
        }
        if (KIND == FX_TIJ || KIND == FX_T00TIJ) {
          constexpr int S0 = KIND == FX_T00TIJ ? 1 : 0;  // first Tij slot
          const float ee = sqrtf(f2 + a * a), inv_e = 1.f / ee;
          const float f = 4.f + a * a / (f2 + a * a);
          add_tij<SL>(A + S0 * SL, B + S0 * SL, off, w, l, q, m, inv_e, f, u0, u1, u2,
                      KIND == FX_T00TIJ ? sq1 : sq0, KIND == FX_T00TIJ ? sg1 : sg0);
        }
      }
    }
    __syncthreads();
    // flush field layer zs (complete now) and clear it: one cell of the layer per
    // thread, its components in turn
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
        } else {
          const float fv = float_of_fixed((long long)v, comp_shift<KIND>(comp, ks0, ks1));
          float *o = comp_ptr(out, comp, C) + gi;
          if (p.overwrite)
            *o = fv;
          else if (v != 0ull)
            *o += fv;
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
__global__ void __launch_bounds__(256) k_face_fix(unsigned long long *face, FxOut out, int ncomp, int fused,
                                                  FxParams p, const uint32_t *__restrict__ fxb) {
  const int N = p.N;
  const int ks0 = (int)fxb[2], ks1 = (int)fxb[3];
  const long NN = (long)N * N, C = NN * N;
  const int planes = (int)(p.nPX + p.nPY + p.nPZ);
  const long rows = (long)ncomp * planes * N;  // face entries come in rows of N (face_index)
  for (long row = blockIdx.x; row < rows; row += gridDim.x) {
    const int comp = (int)(row / ((long)planes * N));
    const int rr = (int)(row - (long)comp * planes * N);
    const int pl = rr / N, q = rr - pl * N;
    unsigned long long *f = face + row * N;
    float *o = comp_ptr(out, comp, C);
    const int ks = (fused && comp > 0) ? ks1 : ks0;
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

// the fixed-point deposit of the mixed form; kind: 0 T00, 1 T0i, 2 Tij, 3 mass,
// 4 T00 and Tij in one sweep (out: T00, out2: Tij).  overwrite: every cell of the
// target is written (the sum of this deposit alone), which spares the caller
// zeroing it first and the kernel reading it back.
int deposit_fx(gev_ctx *ctx, gev_pcls *p, gev_field *out, int kind, double mass, double a, const gev_field *phi,
               bool overwrite, gev_field *out2) {
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
  FxOut fo;
  fo.o0 = (float *)out->d;
  fo.o1 = out2 ? (float *)out2->d : nullptr;
  fo.nc0 = kind == FX_T00TIJ ? 1 : NC;
  const unsigned blocks = (unsigned)(ntx * nty * ntz);
  const long C = (long)N * N * N;
  GEV_CHECK_CUDA(ctx, cudaMemsetAsync(p->bounds, 0, 16 * sizeof(uint32_t), ctx->stream));
  k_fx_bounds<<<grid_for(ctx, (size_t)(p->n > C ? p->n : C), 256, 8), 256, 0, ctx->stream>>>(
      (const float *)p->cur.vx, (const float *)p->cur.vy, (const float *)p->cur.vz, p->n, p->count,
      kind == FX_MASS ? nullptr : fphi, C, p->bounds);
  GEV_LAUNCH_CHECK(ctx);
  k_fx_scale<<<1, 1, 0, ctx->stream>>>(p->bounds, kind, mass, a);
  GEV_LAUNCH_CHECK(ctx);
#define GEV_DEP_LAUNCH(K, PHI)                                                                       \
  cudaFuncSetAttribute(k_dep_fx<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);        \
  k_dep_fx<K><<<blocks, FX_THREADS, smem, ctx->stream>>>(p->cur, p->start, PHI, fo, face, fp, p->bounds)
  switch (kind) {
    case FX_T00:
      GEV_DEP_LAUNCH(FX_T00, fphi);
      break;
    case FX_T0I:
      GEV_DEP_LAUNCH(FX_T0I, fphi);
      break;
    case FX_TIJ:
      GEV_DEP_LAUNCH(FX_TIJ, fphi);
      break;
    case FX_T00TIJ:
      GEV_DEP_LAUNCH(FX_T00TIJ, fphi);
      break;
    default:
      GEV_DEP_LAUNCH(FX_MASS, nullptr);
  }
#undef GEV_DEP_LAUNCH
  GEV_LAUNCH_CHECK(ctx);
  const long face_rows = (long)NC * (fp.nPX + fp.nPY + fp.nPZ) * N;
  const long ff_blocks = face_rows < (long)ctx->sms * 16 ? face_rows : (long)ctx->sms * 16;
  k_face_fix<<<(unsigned)ff_blocks, 256, 0, ctx->stream>>>(face, fo, NC, kind == FX_T00TIJ ? 1 : 0, fp, p->bounds);
  GEV_LAUNCH_CHECK(ctx);
  return GEV_OK;
}
