// gev_deposit_fx.cu -- the mixed-precision deposits: per-particle FP32
// contributions accumulated as 64-bit fixed-point integers.
//
// Same physics as projection_T00/T0i/Tij_project (gevolution.hpp:926-1297) and
// scalarProjectionCIC_project.  Every contribution is the product of two integers:
// the particle's prefactor rounded once to an int32 (scale 2^kq) and the corner's
// weight factor rounded to 22 bits (scale 2^kg, one FFMA).  The scales come from the
// data (largest |q|, |phi|, fullest cell) so that no sum can overflow, and integer
// sums make every result independent of the order of the additions.
//
// T00 and Tij (the deposits of every step) are gathers: a prepass writes each
// particle's integer prefactors, then one thread per grid node sums, in int64
// registers, the contributions of the particles of its 8 neighbouring cells and
// writes the node once.  No atomics, barriers or halo buffers; HBM traffic is the
// particle positions and prefactors (read by 8 nodes each, mostly from L2), phi and
// one write of the target.
//
// T0i and the mass deposit are scatters:
//   * a block owns a column tile of TX x TY cells and a chunk of TZ cell
//     layers, and sweeps the chunk in z;
//   * for each source layer z it walks the particles of the layer's TY rows
//     (contiguous runs of the cell-ordered store, one thread per particle) and
//     adds each corner contribution into two shared-memory layers (field z and z + 1) with
//     64-bit shared atomics;
//   * when layer z is complete it is flushed: cells that only this block can
//     touch are added straight into the FP32 field; cells on a tile face
//     (shared with a neighbouring block, including the periodic wrap) go into
//     a compact int64 face buffer with global atomics, which a fix-up pass
//     then adds to the field and clears.
#include <cmath>

#include "gev_batch.cuh"

namespace {

// kinds; FX_T00TIJ deposits T00 and Tij in one gather
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

// the dense-cell tables of the gather deposit (k_dense_sums below)
// dense above 8 particles: measured over the last 20 cycles before z = 0 at 512^3 (the
// gather's remaining walks against the dense cells' own pass), the cycle took 37.32 ms
// with 8, 37.39 with 10, 37.58 with 12 and 37.83 with 16; before the small cells had
// eight lanes each (a warp a cell), 38.73 with 8 and 37.97 with 12
constexpr uint32_t DENSE_T = 8;
// dense cells of more particles than this take a whole warp (the smaller, eight lanes)
constexpr uint32_t DENSE_BIG = 64;
constexpr int DENSE_NS = 38;
constexpr uint32_t DENSE_NONE = 0xffffffffu;
constexpr int DENSE_MASK_WORDS = 16;
// Slots [0, cap) are for dense cells of up to `big` particles, summed by 8 lanes a cell;
// slots [cap, cap + cap_big) for larger ones, summed by a whole warp.
struct DenseTab {
  uint32_t *slot_of;  // per cell, valid for the cells above thr of this call
  uint32_t *list;     // slot -> cell
  uint32_t *count;    // [0] small and [1] big dense cells found (may exceed the caps)
  uint32_t cap, cap_big;
  uint32_t thr;       // cells with more particles are dense
  uint32_t big;       // dense cells with more particles take a whole warp
  long long *sums;    // slot * DENSE_NS + index
};


// The fixed-point scale comes from the data, on the device: max |q|^2 over the
// particles and the most particles in one cell.  A cell's sum has at most 8 x that
// many contributions (its 8 neighbouring cells), each below c_max of the kind, and
// must stay below 2^62; max reductions do not depend on order, so neither does the
// scale.
// For the gather kinds (D.slot_of set) the same pass over the cell counts gives every
// cell with more than D.thr particles the next dense slot (a warp-aggregated counter),
// or DENSE_NONE once the D.cap slots are taken: every such cell's entry is written,
// and the gather reads only such cells' entries (the counts and the cell starts it
// walks come from the same relink).
__device__ __forceinline__ void k_fx_bounds_body(const float *__restrict__ vx, const float *__restrict__ vy,
                                                   const float *__restrict__ vz, long n,
                                                   const uint32_t *__restrict__ count, const float *__restrict__ phi,
                                                   long C, uint32_t *bounds, DenseTab D) {
  float q2 = 0.f, ph = 0.f;
  uint32_t mc = 0u;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    q2 = fmaxf(q2, vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i]);
  // Dense slots: a thread counts its dense cells as it reduces, the warp takes the
  // slots of all its threads with one counter update (an exclusive scan of the
  // threads' counts gives each thread its first slot), and each thread then hands out
  // its own slots in a second pass over its cells (no warp-wide operation in either
  // loop, so both keep their loads in flight)
  const unsigned lane = threadIdx.x & 31u;
  const long c_first = (long)blockIdx.x * blockDim.x + threadIdx.x, c_step = (long)gridDim.x * blockDim.x;
  // the iterations that met a dense cell, one bit each (up to DENSE_MASK_WORDS * 32
  // iterations a thread; a grid with more makes the second pass read every count again)
  uint32_t ndense = 0u, nbig = 0u, dmask[DENSE_MASK_WORDS];
#pragma unroll
  for (int w = 0; w < DENSE_MASK_WORDS; ++w) dmask[w] = 0u;
  int it = 0;
  for (long c = c_first; c < C; c += c_step, ++it) {
    const uint32_t k = count[c];
    mc = max(mc, k);
    if (phi) ph = fmaxf(ph, fabsf(phi[c]));
    const bool dense = k > D.thr;
    ndense += dense ? 1u : 0u;
    nbig += k > D.big ? 1u : 0u;
    if (dense && it < DENSE_MASK_WORDS * 32) dmask[it >> 5] |= 1u << (it & 31);
  }
  const bool masked = it <= DENSE_MASK_WORDS * 32;
  if (D.slot_of != nullptr) {  // a gather kind (uniform: a kernel argument)
    // small and big dense cells apart (ndense counts both, nbig the big ones)
    const uint32_t nsmall = ndense - nbig;
    uint32_t is = nsmall, ib = nbig;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t ts = __shfl_up_sync(0xffffffffu, is, o), tb = __shfl_up_sync(0xffffffffu, ib, o);
      if ((int)lane >= o) {
        is += ts;
        ib += tb;
      }
    }
    const uint32_t tots = __shfl_sync(0xffffffffu, is, 31), totb = __shfl_sync(0xffffffffu, ib, 31);
    uint32_t bs = 0u, bb = 0u;
    if (lane == 0u) {
      if (tots > 0u) bs = atomicAdd(&D.count[0], tots);
      if (totb > 0u) bb = atomicAdd(&D.count[1], totb);
    }
    uint32_t ss = __shfl_sync(0xffffffffu, bs, 0) + is - nsmall, sb = __shfl_sync(0xffffffffu, bb, 0) + ib - nbig;
    if (ndense > 0u) {
      auto give = [&](long c) {
        const uint32_t k = count[c];
        if (k > D.big) {
          const bool ok = sb < D.cap_big;
          D.slot_of[c] = ok ? D.cap + sb : DENSE_NONE;
          if (ok) D.list[D.cap + sb] = (uint32_t)c;
          ++sb;
        } else if (k > D.thr) {
          const bool ok = ss < D.cap;
          D.slot_of[c] = ok ? ss : DENSE_NONE;
          if (ok) D.list[ss] = (uint32_t)c;
          ++ss;
        }
      };
      if (masked) {
        for (int w = 0; w < DENSE_MASK_WORDS; ++w)
          for (uint32_t m = dmask[w]; m != 0u; m &= m - 1u) give(c_first + (long)(32 * w + __ffs(m) - 1) * c_step);
      } else {
        for (long c = c_first; c < C; c += c_step) give(c);
      }
    }
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
__global__ void __launch_bounds__(256) k_fx_bounds(const float *__restrict__ vx, const float *__restrict__ vy,
                                                   const float *__restrict__ vz, long n,
                                                   const uint32_t *__restrict__ count, const float *__restrict__ phi,
                                                   long C, uint32_t *bounds, DenseTab D) {
  k_fx_bounds_body(vx, vy, vz, n, count, phi, C, bounds, D);
}

// per-particle contribution bounds, |phi| <= 1 taken for the (1 + f phi) factors:
// T00 m (e + (3e + q^2/e)|phi|) <= m (4e + q^2/a); T0i m |q_i| (1 + 2|phi|) <= 3 m |q|;
// Tij m q_i q_j / e (1 + 5|phi|) <= 6 m q^2 / a; mass m.  Writes the power k = kq + kg
// of the sum's scale 2^k into bounds[2 + group]: kq is kept in [-60, 100] and kg in
// [-4, 21], so k stays in [-64, 121], where float_of_fixed is exact (its scale 2^-k and
// its product stay normal for k in [-64, 126]).
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
  // gmax >= 1 (eg >= 1); kg >= -4 holds for gmax < 2^26, i.e. |phi| below about 1e7,
  // which any metric perturbation (|phi| << 1) satisfies by many orders of magnitude
  int kg = 22 - eg;
  kg = kg < -4 ? -4 : kg;
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
__device__ __forceinline__ void k_fx_scale_body(uint32_t *bounds, int kind, double mass, double a) {
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
__global__ void k_fx_scale(uint32_t *bounds, int kind, double mass, double a) {
  k_fx_scale_body(bounds, kind, mass, a);
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

template <int KIND>
__global__ void __launch_bounds__(FX_THREADS, 3) k_dep_fx(PclsArrays P, const uint32_t *__restrict__ start,
                                                       const float *__restrict__ phi, float *out,
                                                       unsigned long long *face, FxParams p,
                                                       const uint32_t *__restrict__ fxb) {
  constexpr int NC = FX_NC[KIND];
  constexpr int SX = TX + 1, SY = TY + 1, SL = SX * SY;  // one shared layer per component
  constexpr bool USE_PHI = KIND != FX_MASS;
  extern __shared__ __align__(16) unsigned long long lay[];  // [2][NC][SY][SX]
  __shared__ uint32_t rowoff[TY + 1], rowbase[TY];
  const int ks0 = (int)fxb[2];  // accumulator scale 2^(kq + kg)
  const float sq0 = pow2f((int)fxb[5]), sg0 = pow2f((int)fxb[6]);
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
      const float m = p.mass;
      if (KIND == FX_MASS) {
        const int Q = fixed32_of(m * sq0);
#pragma unroll
        for (int k = 0; k < 8; ++k) iadd(((k & 1) ? B : A) + off[k], Q, gq(w[k], sg0));
      } else {  // FX_T0I
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
          const float fv = float_of_fixed((long long)v, ks0);
          float *o = out + comp * C + gi;
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

// ---------------------------------------------------------------- gather --
// T00 and Tij as a gather: each grid node sums, in int64 registers, the
// contributions of the particles in its 8 neighbouring cells.
//
// Prefactor records, one per particle in store order, 12 words (three 16-byte
// vectors) written by k_fx_prep, so that a particle visit of the gather is three
// vector loads from one address:
//   [0..2] the in-cell offset (rx, ry, rz)      [3] Q00 = round(m e 2^kq0)
//   [4] rT = (3e + q^2/e) / e                    [5] fT = 4 + a^2 / (q^2 + a^2)
//   [6], [7], [8] Qd_i = round(m q_i^2 / e 2^kq1)
//   [9], [10], [11] Qo = round(m q_i q_j / e 2^kq1) for 01, 02, 12
// Words a kind does not deposit are zero.  T00 alone keeps a record of two
// words, (Q00, rT), and reads the offsets from the particle store.
constexpr int PREP_WORDS = 12;
struct PrepArrays {
  uint4 *rec;  // 3 vectors per particle
};
inline PrepArrays prep_arrays(void *base, long) {
  PrepArrays a;
  a.rec = (uint4 *)base;
  return a;
}

template <int KIND>
__device__ __forceinline__ void k_fx_prep_body(PclsArrays P, long n, PrepArrays A, FxParams p, int have_phi,
                                                 const uint32_t *__restrict__ fxb) {
  const float sq0 = pow2f((int)fxb[5]), sq1 = pow2f((int)fxb[7]);
  const float sqT = KIND == FX_T00TIJ ? sq1 : pow2f((int)fxb[5]);  // Tij's prefactor scale
  // every operation is an explicitly rounded intrinsic: no multiply-add is contracted
  // differently in one instantiation than in another, so each kind and the fused
  // kind produce the same bits
  const float m = p.mass, a = p.a, a2 = __fmul_rn(a, a);
  for (long j = blockIdx.x * (long)blockDim.x + threadIdx.x; j < n; j += (long)gridDim.x * blockDim.x) {
    const float q0 = ((const float *)P.vx)[j], q1 = ((const float *)P.vy)[j], q2 = ((const float *)P.vz)[j];
    const float f2 = __fadd_rn(__fadd_rn(__fmul_rn(q0, q0), __fmul_rn(q1, q1)), __fmul_rn(q2, q2));
    const float ee = __fsqrt_rn(__fadd_rn(f2, a2));
    uint4 v0 = make_uint4(0u, 0u, 0u, 0u);
    if (KIND != FX_T00) v0 = make_uint4(__float_as_uint(P.rx[j]), __float_as_uint(P.ry[j]), __float_as_uint(P.rz[j]), 0u);
    uint4 v1 = make_uint4(0u, 0u, 0u, 0u), v2 = make_uint4(0u, 0u, 0u, 0u);
    if (KIND == FX_T00 || KIND == FX_T00TIJ) {
      const float e00 = have_phi ? ee : a;
      const float r = have_phi ? __fdiv_rn(__fadd_rn(__fmul_rn(3.f, ee), __fdiv_rn(f2, ee)), ee) : 0.f;
      v0.w = (unsigned)fixed32_of(__fmul_rn(__fmul_rn(m, e00), sq0));
      v1.x = __float_as_uint(r);
    }
    if (KIND == FX_TIJ || KIND == FX_T00TIJ) {
      const float inv_e = __fdiv_rn(1.f, ee), mi = __fmul_rn(m, inv_e);
      v1.y = __float_as_uint(__fadd_rn(4.f, __fdiv_rn(a2, __fadd_rn(f2, a2))));
      v1.z = (unsigned)fixed32_of(__fmul_rn(__fmul_rn(__fmul_rn(q0, q0), mi), sqT));
      v1.w = (unsigned)fixed32_of(__fmul_rn(__fmul_rn(__fmul_rn(q1, q1), mi), sqT));
      v2.x = (unsigned)fixed32_of(__fmul_rn(__fmul_rn(__fmul_rn(q2, q2), mi), sqT));
      v2.y = (unsigned)fixed32_of(__fmul_rn(__fmul_rn(__fmul_rn(q0, q1), mi), sqT));
      v2.z = (unsigned)fixed32_of(__fmul_rn(__fmul_rn(__fmul_rn(q0, q2), mi), sqT));
      v2.w = (unsigned)fixed32_of(__fmul_rn(__fmul_rn(__fmul_rn(q1, q2), mi), sqT));
    }
    if (KIND == FX_T00) {
      reinterpret_cast<uint2 *>(A.rec)[j] = make_uint2(v0.w, v1.x);
    } else {
      uint4 *o = A.rec + 3 * j;
      o[0] = v0;
      o[1] = v1;
      o[2] = v2;
    }
  }
}
template <int KIND>
__global__ void __launch_bounds__(256) k_fx_prep(PclsArrays P, long n, PrepArrays A, FxParams p, int have_phi,
                                                 const uint32_t *__restrict__ fxb) {
  k_fx_prep_body<KIND>(P, n, A, p, have_phi, fxb);
}

// ------------------------------------------------------------ dense cells --
// In a clustered state single cells hold tens to hundreds of particles, and each of
// the cell's 8 corner nodes walks all of them: the thread with such a cell in its
// walk keeps its warp busy long after the other lanes are done.  Cells with more
// than D.thr particles are therefore summed once: a warp per cell forms the
// contributions the gather would form at each of the cell's 8 corners (the same FP32
// weight factors with the corner node's phi, rounded the same way) and adds them in
// int64; the gather adds a dense cell's sums at its corner instead of walking it.
// Integer sums do not depend on the grouping of the additions, so the result is the
// same bits whichever cells take this path.  A cell finds its sums through a direct
// cell -> slot map, which k_fx_bounds writes for the dense cells of this call as it
// reduces the cell counts, and which the gather reads only for cells holding more
// than D.thr particles.  Slots run out at `cap`; dense cells beyond it are walked as
// before.  (A warp per dense cell through a hash map, with the gather walking dense
// cells in a separate loop, ran slower than the plain walk: the lanes of a warp took
// both loop shapes one after the other.)
//
// The 38 sums of a slot, corner k = dx + 2 dy + 4 dz of the cell:
//   [k]          T00 at corner k
//   [8 + 3k + c] the diagonal Tij_cc at corner k
//   [32 + dz]    Tij_01 at corner (0, 0, dz)   (the plaquettes the gather's nodes own)
//   [34 + dy]    Tij_02 at corner (0, dy, 0)
//   [36 + dx]    Tij_12 at corner (dx, 0, 0)
// A group of G lanes per dense cell (G = 8 for the small ones, four cells a warp; 32 for
// the big ones): lane l of the group takes the cell's particles l, l + G, ... and forms
// their contributions at the cell's 8 corners as gather_node's add() forms them for a
// node; the lanes' int64 sums are added through shared memory (each lane writes its 38,
// then lane g of the group adds the G values of sums g, g + G, ...).
constexpr int DENSE_WARPS = 4;
template <int KIND, int G>
__device__ __forceinline__ void dense_cell(bool has, uint32_t s, const PclsArrays &P, const uint32_t *__restrict__ start,
                                           const PrepArrays &A, const float *__restrict__ phi, const FxParams &p,
                                           const Div32 &dN, const DenseTab &D, float sg00, float sgij,
                                           long long (*red)[33]) {
  constexpr bool DO00 = KIND == FX_T00 || KIND == FX_T00TIJ, DOIJ = KIND == FX_TIJ || KIND == FX_T00TIJ;
  const int N = p.N;
  const int lane = threadIdx.x & 31, gl = lane & (G - 1), g0 = lane - gl;
  long long acc[DENSE_NS];
#pragma unroll
  for (int k = 0; k < DENSE_NS; ++k) acc[k] = 0;
  if (has) {
    const uint32_t c = D.list[s];
    int x, y, z;
    cell_xyz(c, N, p.lg, dN, x, y, z);
    const Nb3 b = nb3(c, x, y, z, N);
    // phi at the cell's 8 corners f[dx + 2 dy + 4 dz] (indices summed in 32 bits)
    float f[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const unsigned ik = c + ((k & 1) ? b.xp : 0u) + ((k & 2) ? b.yp : 0u) + ((k & 4) ? b.zp : 0u);
      f[k] = phi != nullptr ? __ldg(&phi[ik]) : 0.f;
    }
    // the plaquette sums of the corner nodes that own them, in gather_node's order
    float s01[2], s02[2], s12[2];
#pragma unroll
    for (int d = 0; d < 2; ++d) {
      s01[d] = __fadd_rn(__fadd_rn(__fadd_rn(f[4 * d], f[2 + 4 * d]), f[1 + 4 * d]), f[3 + 4 * d]);
      s02[d] = __fadd_rn(__fadd_rn(__fadd_rn(f[2 * d], f[2 * d + 4]), f[1 + 2 * d]), f[1 + 2 * d + 4]);
      s12[d] = __fadd_rn(__fadd_rn(__fadd_rn(f[d], f[d + 4]), f[d + 2]), f[d + 6]);
    }
    const uint32_t j1 = start[c + 1];
    for (uint32_t j = start[c] + gl; j < j1; j += G) {
      uint4 v0, v1, v2 = make_uint4(0u, 0u, 0u, 0u);
      if constexpr (KIND == FX_T00) {
        const uint2 q = __ldg(reinterpret_cast<const uint2 *>(A.rec) + j);
        v0 = make_uint4(__float_as_uint(P.rx[j]), __float_as_uint(P.ry[j]), __float_as_uint(P.rz[j]), q.x);
        v1 = make_uint4(q.y, 0u, 0u, 0u);
      } else {
        const uint4 *rec = A.rec + 3 * (size_t)j;
        v0 = __ldg(rec);
        v1 = __ldg(rec + 1);
        v2 = __ldg(rec + 2);
      }
      const float u0 = __uint_as_float(v0.x), u1 = __uint_as_float(v0.y), u2 = __uint_as_float(v0.z);
      const float wl0[2] = {__fsub_rn(1.f, u0), u0}, wl1[2] = {__fsub_rn(1.f, u1), u1},
                  wl2[2] = {__fsub_rn(1.f, u2), u2};
      const float fT = __uint_as_float(v1.y), qf = __fmul_rn(0.25f, fT);
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const int dx = k & 1, dy = (k >> 1) & 1, dz = k >> 2;
        const float w = __fmul_rn(__fmul_rn(wl0[dx], wl1[dy]), wl2[dz]);
        if (DO00)
          acc[k] += (long long)(int)v0.w *
                    (long long)gq(__fmul_rn(w, __fadd_rn(1.f, __fmul_rn(__uint_as_float(v1.x), f[k]))), sg00);
        if (DOIJ) {
          const long long Gw = gq(__fmul_rn(w, __fadd_rn(1.f, __fmul_rn(fT, f[k]))), sgij);
          acc[8 + 3 * k] += (long long)(int)v1.z * Gw;
          acc[9 + 3 * k] += (long long)(int)v1.w * Gw;
          acc[10 + 3 * k] += (long long)(int)v2.x * Gw;
        }
      }
      if (DOIJ) {
#pragma unroll
        for (int d = 0; d < 2; ++d) {
          acc[32 + d] += (long long)(int)v2.y * (long long)gq(__fmul_rn(wl2[d], __fadd_rn(1.f, __fmul_rn(qf, s01[d]))), sgij);
          acc[34 + d] += (long long)(int)v2.z * (long long)gq(__fmul_rn(wl1[d], __fadd_rn(1.f, __fmul_rn(qf, s02[d]))), sgij);
          acc[36 + d] += (long long)(int)v2.w * (long long)gq(__fmul_rn(wl0[d], __fadd_rn(1.f, __fmul_rn(qf, s12[d]))), sgij);
        }
      }
    }
  }
#pragma unroll
  for (int k = 0; k < DENSE_NS; ++k) red[k][lane] = acc[k];
  __syncwarp();
  if (has) {
    long long *out = D.sums + (size_t)s * DENSE_NS;
    for (int k = gl; k < DENSE_NS; k += G) {
      long long v = 0;
#pragma unroll
      for (int l = 0; l < G; ++l) v += red[k][g0 + l];
      out[k] = v;
    }
  }
  __syncwarp();  // red is rewritten for the warp's next cells
}

// the small dense cells four to a warp, then the big ones a warp each
template <int KIND>
__device__ __forceinline__ void k_dense_sums_body(PclsArrays P, const uint32_t *__restrict__ start,
                                                                PrepArrays A, const float *__restrict__ phi, FxParams p,
                                                                Div32 dN, const uint32_t *__restrict__ fxb, DenseTab D) {
  __shared__ long long red[DENSE_WARPS][DENSE_NS][33];
  const float sg00 = pow2f((int)fxb[6]), sgij = pow2f(KIND == FX_T00TIJ ? (int)fxb[8] : (int)fxb[6]);
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const uint32_t warps = (gridDim.x * blockDim.x) >> 5, w0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t ns = min(D.count[0], D.cap), nb = min(D.count[1], D.cap_big);
  for (uint32_t base = w0 * 4u; base < ns; base += warps * 4u) {
    const uint32_t s = base + (uint32_t)(lane >> 3);
    dense_cell<KIND, 8>(s < ns, s, P, start, A, phi, p, dN, D, sg00, sgij, red[wib]);
  }
  for (uint32_t b = w0; b < nb; b += warps) dense_cell<KIND, 32>(true, D.cap + b, P, start, A, phi, p, dN, D, sg00, sgij, red[wib]);
}
template <int KIND>
__global__ void __launch_bounds__(32 * DENSE_WARPS) k_dense_sums(PclsArrays P, const uint32_t *__restrict__ start,
                                                                PrepArrays A, const float *__restrict__ phi, FxParams p,
                                                                Div32 dN, const uint32_t *__restrict__ fxb, DenseTab D) {
  k_dense_sums_body<KIND>(P, start, A, phi, p, dN, fxb, D);
}

// node i = (x, y, z): its 8 neighbouring cells' contributions, summed in int64 and
// converted once; out: T00 (1 comp) and / or Tij (6 comps, 00 01 02 11 12 22)
template <int KIND>
__device__ __forceinline__ void gather_node(unsigned i, int x, int y, int z, const PclsArrays &P,
                                            const uint32_t *__restrict__ start, const PrepArrays &A,
                                            const float *__restrict__ phi, float *t00, float *tij, const FxParams &p,
                                            int ks00, int ksij, float sg00, float sgij, const DenseTab &D) {
  constexpr bool DO00 = KIND == FX_T00 || KIND == FX_T00TIJ, DOIJ = KIND == FX_TIJ || KIND == FX_T00TIJ;
  const int N = p.N;
  const unsigned C = (unsigned)N * N * N;
  const Nb3 b = nb3(i, x, y, z, N);
  // phi at the node and its +x, +y, +z neighbours: the factors of the node's corner
  // (T00, diagonal Tij) and the three plaquette sums of the off-diagonal components
  float pn = 0.f, s01 = 0.f, s02 = 0.f, s12 = 0.f;
  if (phi != nullptr) {  // indices summed in 32 bits: the offsets wrap modulo 2^32
    const unsigned i100 = i + b.xp, i010 = i + b.yp, i001 = i + b.zp;
    const unsigned i110 = i100 + b.yp, i101 = i100 + b.zp, i011 = i010 + b.zp;
    const float f000 = __ldg(&phi[i]), f100 = __ldg(&phi[i100]), f010 = __ldg(&phi[i010]);
    const float f110 = __ldg(&phi[i110]), f001 = __ldg(&phi[i001]);
    const float f101 = __ldg(&phi[i101]), f011 = __ldg(&phi[i011]);
    pn = f000;
    s01 = __fadd_rn(__fadd_rn(__fadd_rn(f000, f010), f100), f110);  // l0 + l2 + l4 + l6 of the particles' cells
    s02 = __fadd_rn(__fadd_rn(__fadd_rn(f000, f001), f100), f101);  // l0 + l1 + l4 + l5
    s12 = __fadd_rn(__fadd_rn(__fadd_rn(f000, f001), f010), f011);  // l0 + l1 + l2 + l3
  }
  long long a00 = 0, ad0 = 0, ad1 = 0, ad2 = 0, ao01 = 0, ao02 = 0, ao12 = 0;
  // the contributions of particle j to this node, the node being corner (dx, dy, dz)
  // of the particle's cell
  auto add = [&](uint32_t j, int dx, int dy, int dz) {
    uint4 v0, v1, v2 = make_uint4(0u, 0u, 0u, 0u);
    if constexpr (KIND == FX_T00) {
      const uint2 q = __ldg(reinterpret_cast<const uint2 *>(A.rec) + j);
      v0 = make_uint4(__float_as_uint(P.rx[j]), __float_as_uint(P.ry[j]), __float_as_uint(P.rz[j]), q.x);
      v1 = make_uint4(q.y, 0u, 0u, 0u);
    } else {
      const uint4 *rec = A.rec + 3 * (size_t)j;
      v0 = __ldg(rec);
      v1 = __ldg(rec + 1);
      v2 = __ldg(rec + 2);
    }
    const float u0 = __uint_as_float(v0.x), u1 = __uint_as_float(v0.y), u2 = __uint_as_float(v0.z);
    const float w0 = dx ? u0 : __fsub_rn(1.f, u0), w1 = dy ? u1 : __fsub_rn(1.f, u1),
                w2 = dz ? u2 : __fsub_rn(1.f, u2);
    const float w = __fmul_rn(__fmul_rn(w0, w1), w2);
    if (DO00)
      a00 += (long long)(int)v0.w *
             (long long)gq(__fmul_rn(w, __fadd_rn(1.f, __fmul_rn(__uint_as_float(v1.x), pn))), sg00);
    if (DOIJ) {
      const float f = __uint_as_float(v1.y);
      const long long G = gq(__fmul_rn(w, __fadd_rn(1.f, __fmul_rn(f, pn))), sgij);
      ad0 += (long long)(int)v1.z * G;
      ad1 += (long long)(int)v1.w * G;
      ad2 += (long long)(int)v2.x * G;
      const float qf = __fmul_rn(0.25f, f);
      if (dx == 0 && dy == 0)
        ao01 += (long long)(int)v2.y * (long long)gq(__fmul_rn(w2, __fadd_rn(1.f, __fmul_rn(qf, s01))), sgij);
      if (dx == 0 && dz == 0)
        ao02 += (long long)(int)v2.z * (long long)gq(__fmul_rn(w1, __fadd_rn(1.f, __fmul_rn(qf, s02))), sgij);
      if (dy == 0 && dz == 0)
        ao12 += (long long)(int)v2.w * (long long)gq(__fmul_rn(w0, __fadd_rn(1.f, __fmul_rn(qf, s12))), sgij);
    }
  };
  // the 4 cell pairs (x - 1, x) of rows (y - dy, z - dz): all their bounds first;
  // for x > 0 the two cells' particles are one contiguous run of the store
  const unsigned cb[4] = {i, i + b.zm, i + b.ym, i + b.ym + b.zm};
  uint32_t s0[4], s1[4], s2[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    s0[q] = start[cb[q] + b.xm];
    s1[q] = start[cb[q]];
    s2[q] = start[cb[q] + 1];
  }
  // a dense cell's sums at this node's corner (dx, dy, dz) of it, if it has a slot
  auto dense = [&](uint32_t cell, int dx, int dy, int dz) -> bool {
    const uint32_t slot = D.slot_of[cell];
    if (slot >= D.cap + D.cap_big) return false;  // DENSE_NONE: no slot was left for it
    const long long *hs = D.sums + (size_t)slot * DENSE_NS;
    const int k = dx + 2 * dy + 4 * dz;
    if (DO00) a00 += hs[k];
    if (DOIJ) {
      ad0 += hs[8 + 3 * k];
      ad1 += hs[9 + 3 * k];
      ad2 += hs[10 + 3 * k];
      if (dx == 0 && dy == 0) ao01 += hs[32 + dz];
      if (dx == 0 && dz == 0) ao02 += hs[34 + dy];
      if (dy == 0 && dz == 0) ao12 += hs[36 + dx];
    }
    return true;
  };
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int dy = q >> 1, dz = q & 1;
    // cell A = (x - 1, ...), whose corner (1, dy, dz) this node is, particles [s0, eA);
    // cell B = (x, ...), corner (0, dy, dz), particles [s1, s2)
    const uint32_t eA = x > 0 ? s1[q] : start[cb[q] + b.xm + 1];
    const bool skipA = eA - s0[q] > D.thr && dense(cb[q] + b.xm, 1, dy, dz);
    const bool skipB = s2[q] - s1[q] > D.thr && dense(cb[q], 0, dy, dz);
    if (x > 0) {
      // one loop over the contiguous pair, a summed cell cut off its end: every lane of
      // a warp runs the same loop, whichever of its cells are dense
      const uint32_t jb = skipA ? s1[q] : s0[q], je = skipB ? s1[q] : s2[q];
      for (uint32_t j = jb; j < je; ++j) add(j, j < s1[q] ? 1 : 0, dy, dz);
    } else {
      if (!skipB)
        for (uint32_t j = s1[q]; j < s2[q]; ++j) add(j, 0, dy, dz);
      if (!skipA)
        for (uint32_t j = s0[q]; j < eA; ++j) add(j, 1, dy, dz);
    }
  }
  if (DO00) {
    const float v = float_of_fixed(a00, ks00);
    t00[i] = p.overwrite ? v : t00[i] + v;
  }
  if (DOIJ) {
    const long long acc[6] = {ad0, ao01, ao02, ad1, ao12, ad2};
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      const float v = float_of_fixed(acc[c], ksij);
      float *o = tij + (size_t)c * C + i;
      *o = p.overwrite ? v : *o + v;
    }
  }
}

// One thread per node.  While no cell holds more than PATCH_MC particles (the
// nearly uniform early state) a warp takes 32 consecutive nodes of the flat index;
// in a clustered state it takes the 32 nodes of a PX x PY x PZ patch (PX = 0: always
// the flat index, for grids that the patch does not divide).  There the particles a
// node walks (its 8 neighbouring cells) differ by orders of magnitude between
// nodes, and a warp waits for its longest walk: a compact patch holds nodes of more
// similar density than a line of 32 cells (lanes busy, counted from a 128^3 run at
// z = 0: 17.8% in lines, 26.1% in 8 x 2 x 2 patches).  Measured over the last 20
// cycles before z = 0 at 512^3: 13.41 ms against 14.58 ms in lines (4 x 4 x 2: 15.03,
// 8 x 4 x 1: 14.20, 16 x 2 x 1: 14.16); in the first cycles the lines are faster
// (the patch's nodes are four 32-byte row pieces rather than one 128-byte line).
// Each node is one thread's either way, so the bits do not depend on the choice.
// Five resident blocks per SM (48 registers, 124 B of spill stores): the loop is
// latency-bound, and warps hide more than the few spilled words cost, up to a point
// (the late 512^3 cycle took 8.82 ms in the gather at five blocks, 9.16 at six with 40
// registers and 424 B of spills, 9.16 at four with 64 and 10.73 at three with 80).
constexpr uint32_t PATCH_MC = 8;
template <int KIND, int PX, int PY, int PZ>
__device__ __forceinline__ void k_dep_gather_body(PclsArrays P, const uint32_t *__restrict__ start, PrepArrays A,
                                                    const float *__restrict__ phi, float *t00, float *tij, FxParams p,
                                                    Div32 dN, const uint32_t *__restrict__ fxb, DenseTab D) {
  const int ks00 = (int)fxb[2], ksij = KIND == FX_T00TIJ ? (int)fxb[3] : (int)fxb[2];
  const float sg00 = pow2f((int)fxb[6]), sgij = pow2f(KIND == FX_T00TIJ ? (int)fxb[8] : (int)fxb[6]);
  const int N = p.N;
  const unsigned C = (unsigned)N * N * N;
  if (PX == 0 || fxb[1] <= PATCH_MC) {
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < C; i += gridDim.x * blockDim.x) {
      int x, y, z;
      cell_xyz(i, N, p.lg, dN, x, y, z);
      gather_node<KIND>(i, x, y, z, P, start, A, phi, t00, tij, p, ks00, ksij, sg00, sgij, D);
    }
  } else if constexpr (PX > 0) {
    static_assert(PX * PY * PZ == 32, "a patch is one warp");
    const int lane = threadIdx.x & 31;
    const int lx = lane % PX, ly = (lane / PX) % PY, lz = lane / (PX * PY);
    const unsigned ppx = (unsigned)N / PX, ppy = (unsigned)N / PY, npatch = ppx * ppy * ((unsigned)N / PZ);
    const unsigned nw = (gridDim.x * blockDim.x) >> 5;
    for (unsigned q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < npatch; q += nw) {
      const unsigned r = q / ppx, qz = r / ppy;
      const int x = (int)(q - r * ppx) * PX + lx, y = (int)(r - qz * ppy) * PY + ly, z = (int)qz * PZ + lz;
      const unsigned i = (unsigned)x + (unsigned)N * ((unsigned)y + (unsigned)N * (unsigned)z);
      gather_node<KIND>(i, x, y, z, P, start, A, phi, t00, tij, p, ks00, ksij, sg00, sgij, D);
    }
  }
}
template <int KIND, int PX, int PY, int PZ>
__global__ void __launch_bounds__(256, 5) k_dep_gather(PclsArrays P, const uint32_t *__restrict__ start, PrepArrays A,
                                                    const float *__restrict__ phi, float *t00, float *tij, FxParams p,
                                                    Div32 dN, const uint32_t *__restrict__ fxb, DenseTab D) {
  k_dep_gather_body<KIND, PX, PY, PZ>(P, start, A, phi, t00, tij, p, dN, fxb, D);
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

// the fixed-point deposit of the mixed form; kind: 0 T00, 1 T0i, 2 Tij, 3 mass,
// 4 T00 and Tij in one gather (out: T00, out2: Tij).  overwrite: every cell of the
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
  const bool gather = kind == FX_T00 || kind == FX_TIJ || kind == FX_T00TIJ;
  // the face buffer (scatter kinds) lives behind the deposit scratch pointer, kept zeroed between uses
  if (!gather && ctx->cube_bytes < face_elems * 8) {
    int rc = ctx_ensure_cube(ctx, face_elems * 8);
    if (rc) return rc;
    GEV_CHECK_CUDA(ctx, cudaMemsetAsync(ctx->d_cube, 0, ctx->cube_bytes, ctx->stream));
  }
  const int ntx = (N + TX - 1) / TX, nty = (N + TY - 1) / TY, ntz = (N + TZ - 1) / TZ;
  const size_t smem = 2 * (size_t)NC * (TX + 1) * (TY + 1) * 8;
  unsigned long long *face = (unsigned long long *)ctx->d_cube;
  const float *fphi = phi ? (const float *)phi->d : nullptr;
  const unsigned blocks = (unsigned)(ntx * nty * ntz);
  const long C = (long)N * N * N;
  // gather kinds: the prefactor records live in the alt array set, which only a relink
  // writes (an allocation of their own only if that block were too small), and the
  // dense-cell tables after them when the block has room, else in an allocation of
  // their own (slots for one dense cell in 64 particles)
  void *rec = nullptr;
  const size_t rec_bytes = (size_t)(p->cap > 0 ? p->cap : 1) * PREP_WORDS * 4;
  DenseTab dt{nullptr, nullptr, nullptr, 0u, 0u, 0u, 0u, nullptr};
  if (gather) {
    rec = p->alt.block_bytes >= rec_bytes ? p->alt.block : p->prep;
    if (!rec) {
      const size_t bytes = rec_bytes;
      if (cudaMalloc(&p->prep, bytes) != cudaSuccess) {
        cudaGetLastError();
        return gev_fail(ctx, GEV_ENOMEM, "deposit: prefactor scratch allocation failed");
      }
      ctx->bytes_in_use += bytes;
      p->bytes += bytes;
      rec = p->prep;
    }
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const long np = p->cap > 0 ? p->cap : 1;
    const uint32_t dcap = (uint32_t)(np / 64 > 1024 ? np / 64 : 1024);
    const uint32_t dcap_big = (uint32_t)(np / 256 > 1024 ? np / 256 : 1024);
    const size_t nslots = (size_t)dcap + dcap_big;
    const size_t o_list = al((size_t)C * 4), o_count = o_list + al(nslots * 4), o_sums = o_count + 256;
    const size_t dense_bytes = o_sums + nslots * DENSE_NS * 8;
    char *base = nullptr;
    if (rec == p->alt.block && p->alt.block_bytes >= al(rec_bytes) + dense_bytes) {
      base = (char *)p->alt.block + al(rec_bytes);
    } else {
      if (!p->dense) {
        if (cudaMalloc(&p->dense, dense_bytes) != cudaSuccess) {
          cudaGetLastError();
          p->dense = nullptr;
          return gev_fail(ctx, GEV_ENOMEM, "deposit: dense-cell table allocation failed");
        }
        ctx->bytes_in_use += dense_bytes;
        p->bytes += dense_bytes;
      }
      base = (char *)p->dense;
    }
    dt.slot_of = (uint32_t *)base;
    dt.list = (uint32_t *)(base + o_list);
    dt.count = (uint32_t *)(base + o_count);
    dt.sums = (long long *)(base + o_sums);
    dt.cap = dcap;
    dt.cap_big = dcap_big;
    dt.thr = DENSE_T;
    dt.big = DENSE_BIG;
    GEV_CHECK_CUDA(ctx, gev_zero_async(ctx, dt.count, 8));
  }
  GevTimed tm_b(ctx, "k_fx_bounds+k_fx_scale");
  GEV_CHECK_CUDA(ctx, gev_zero_async(ctx, p->bounds, 16 * sizeof(uint32_t)));
  gev_launch<k_fx_bounds_body, 256, 1>(ctx, k_fx_bounds, dim3(grid_for(ctx, (size_t)(p->n > C ? p->n : C), 256, 8)),
                                       dim3(256), 0, (const float *)p->cur.vx, (const float *)p->cur.vy,
                                       (const float *)p->cur.vz, p->n, (const uint32_t *)p->count,
                                       kind == FX_MASS ? nullptr : fphi, C, p->bounds, dt);
  GEV_LAUNCH_CHECK(ctx);
  gev_launch<k_fx_scale_body, 32, 1>(ctx, k_fx_scale, dim3(1), dim3(1), 0, p->bounds, kind, mass, a);
  GEV_LAUNCH_CHECK(ctx);
  tm_b.stop();
  if (gather) {
    const PrepArrays pa = prep_arrays(rec, p->cap > 0 ? p->cap : 1);
    float *t00 = kind == FX_TIJ ? nullptr : (float *)out->d;
    float *tij = kind == FX_TIJ ? (float *)out->d : (out2 ? (float *)out2->d : nullptr);
    const int pb = grid_for(ctx, (size_t)p->n, 256, 16);
    // many small blocks (up to 384 a SM, about 77 waves of the five resident): the block scheduler
    // refills an SM as soon as a block's nodes are done, which the long latency-bound walks
    // of a few large blocks cannot (first 512^3 cycles: 29.7 ms a cycle at 96, 30.7 at 16,
    // 31.8 at 12; late cycles, patch walk: gather 12.87 ms at 384, 13.09 at 192, 13.40 at 96,
    // 13.84 at 48, 13.25 with one block per 256 nodes)
    const int gb = grid_for(ctx, (size_t)C, 256, 384);
    const Div32 dN = make_div32((unsigned)N);
    // the patch walk needs N divisible by its 8 x 2 x 2 shape
    const bool patch = N % 8 == 0;
#define GEV_DENSE(K)                                                                                         \
  do {                                                                                                       \
    GevTimed tm_d(ctx, "k_dense_sums");                                                                      \
    gev_launch<k_dense_sums_body<K>, 32 * DENSE_WARPS, 4>(ctx, k_dense_sums<K>, dim3(ctx->sms * 8),          \
                                                          dim3(32 * DENSE_WARPS), 0, p->cur,                 \
                                                          (const uint32_t *)p->start, pa, fphi, fp, dN,      \
                                                          (const uint32_t *)p->bounds, dt);                  \
    GEV_LAUNCH_CHECK(ctx);                                                                                   \
  } while (0)
#define GEV_GATHER(K)                                                                                               \
  do {                                                                                                              \
    if (patch)                                                                                                      \
      gev_launch<k_dep_gather_body<K, 8, 2, 2>, 256, 5>(ctx, k_dep_gather<K, 8, 2, 2>, dim3(gb), dim3(256), 0,      \
                                                        p->cur, (const uint32_t *)p->start, pa, fphi, t00, tij, fp, \
                                                        dN, (const uint32_t *)p->bounds, dt);                       \
    else                                                                                                            \
      gev_launch<k_dep_gather_body<K, 0, 0, 0>, 256, 5>(ctx, k_dep_gather<K, 0, 0, 0>, dim3(gb), dim3(256), 0,      \
                                                        p->cur, (const uint32_t *)p->start, pa, fphi, t00, tij, fp, \
                                                        dN, (const uint32_t *)p->bounds, dt);                       \
  } while (0)
    GevTimed tm_p(ctx, "k_fx_prep");
    if (kind == FX_T00) {
      gev_launch<k_fx_prep_body<FX_T00>, 256, 8>(ctx, k_fx_prep<FX_T00>, dim3(pb), dim3(256), 0, p->cur, p->n, pa, fp,
                                              (int)(fphi != nullptr), (const uint32_t *)p->bounds);
      GEV_LAUNCH_CHECK(ctx);
      tm_p.stop();
      GEV_DENSE(FX_T00);
      GevTimed tm_g(ctx, "k_dep_gather");
      GEV_GATHER(FX_T00);
    } else if (kind == FX_TIJ) {
      gev_launch<k_fx_prep_body<FX_TIJ>, 256, 8>(ctx, k_fx_prep<FX_TIJ>, dim3(pb), dim3(256), 0, p->cur, p->n, pa, fp,
                                              (int)(fphi != nullptr), (const uint32_t *)p->bounds);
      GEV_LAUNCH_CHECK(ctx);
      tm_p.stop();
      GEV_DENSE(FX_TIJ);
      GevTimed tm_g(ctx, "k_dep_gather");
      GEV_GATHER(FX_TIJ);
    } else {
      gev_launch<k_fx_prep_body<FX_T00TIJ>, 256, 8>(ctx, k_fx_prep<FX_T00TIJ>, dim3(pb), dim3(256), 0, p->cur, p->n, pa, fp,
                                              (int)(fphi != nullptr), (const uint32_t *)p->bounds);
      GEV_LAUNCH_CHECK(ctx);
      tm_p.stop();
      GEV_DENSE(FX_T00TIJ);
      GevTimed tm_g(ctx, "k_dep_gather");
      GEV_GATHER(FX_T00TIJ);
    }
    GEV_LAUNCH_CHECK(ctx);
    return GEV_OK;
  }
#define GEV_DEP_LAUNCH(K, PHI)                                                                       \
  cudaFuncSetAttribute(k_dep_fx<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);        \
  k_dep_fx<K><<<blocks, FX_THREADS, smem, ctx->stream>>>(p->cur, p->start, PHI, (float *)out->d, face, fp, \
                                                         p->bounds)
  GevTimed tm_s(ctx, "k_dep_fx+k_face_fix");
  if (kind == FX_T0I) {
    GEV_DEP_LAUNCH(FX_T0I, fphi);
  } else {
    GEV_DEP_LAUNCH(FX_MASS, nullptr);
  }
#undef GEV_DEP_LAUNCH
  GEV_LAUNCH_CHECK(ctx);
  const long face_rows = (long)NC * (fp.nPX + fp.nPY + fp.nPZ) * N;
  const long ff_blocks = face_rows < (long)ctx->sms * 16 ? face_rows : (long)ctx->sms * 16;
  k_face_fix<<<(unsigned)ff_blocks, 256, 0, ctx->stream>>>(face, (float *)out->d, NC, fp, p->bounds);
  GEV_LAUNCH_CHECK(ctx);
  return GEV_OK;
}
