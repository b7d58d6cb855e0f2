// gev_particles.cu -- the device particle store and the particle updates.
//
// Replaces LATfield2's Particles (per-cell std::lists, updateVel /
// moveParticles with callbacks; main.cpp:743-806) by a structure-of-arrays
// store kept in (cell, ID) order:
//   relink = periodic counting sort: atomic histogram of cell keys, exclusive
//   scan into cell starts, scatter, then each particle is ranked by ID within its
//   cell's run (so the order -- and every sum over it -- is independent of atomic
//   timing), then one gather of the payload.
// update_q / update_pos (gevolution.hpp:570-903) run one thread per particle
// in that order, so neighbouring threads gather neighbouring field cells.
#include <cmath>
#include <cstring>

#include "gev_batch.cuh"

namespace {

// ------------------------------------------------------------ keys ------
__device__ __forceinline__ int cell1(double p, double Nd, int N) {
  int c = (int)(p * Nd);
  return c >= N ? N - 1 : (c < 0 ? 0 : c);
}
__device__ __forceinline__ uint32_t cell_key(double x, double y, double z, int N) {
  const double Nd = (double)N;
  return (uint32_t)cell1(x, Nd, N) + (uint32_t)N * ((uint32_t)cell1(y, Nd, N) + (uint32_t)N * (uint32_t)cell1(z, Nd, N));
}
// periodic wrap into [0,1), as moveParticles does for the box {1,1,1}
__device__ __forceinline__ double wrap01(double p) {
  if (p >= 1.0)
    p -= 1.0;
  else if (p < 0.0) {
    p += 1.0;
    if (p >= 1.0) p -= 1.0;
  }
  return p;
}

// ------------------------------------------------------------ upload ----
template <typename V>
__device__ __forceinline__ void unpack_one(const gev_part &q, long i, PclsArrays &P, int N) {
    P.px[i] = q.pos[0];
    P.py[i] = q.pos[1];
    P.pz[i] = q.pos[2];
    ((V *)P.vx)[i] = (V)q.vel[0];
    ((V *)P.vy)[i] = (V)q.vel[1];
    ((V *)P.vz)[i] = (V)q.vel[2];
    P.id[i] = q.ID;
    P.cell[i] = cell_key(q.pos[0], q.pos[1], q.pos[2], N);
    if (sizeof(V) == 4) {
      const int lg = lg_pow2(N);
      int cx, cy, cz;
      pos_split(q.pos[0], N, lg, cx, P.rx[i]);
      pos_split(q.pos[1], N, lg, cy, P.ry[i]);
      pos_split(q.pos[2], N, lg, cz, P.rz[i]);
      P.cell[i] = (uint32_t)cx + (uint32_t)N * ((uint32_t)cy + (uint32_t)N * (uint32_t)cz);
    }
}
template <typename V>
__global__ void k_unpack(const gev_part *__restrict__ in, long n, PclsArrays P, int N) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    unpack_one<V>(in[i], i, P, N);
}
template <typename V>
__device__ __forceinline__ gev_part pack_one(const PclsArrays &P, long i) {
  gev_part q;
  q.pos[0] = P.px[i];
  q.pos[1] = P.py[i];
  q.pos[2] = P.pz[i];
  q.vel[0] = (double)((const V *)P.vx)[i];
  q.vel[1] = (double)((const V *)P.vy)[i];
  q.vel[2] = (double)((const V *)P.vz)[i];
  q.ID = P.id[i];
  return q;
}
template <typename V>
__global__ void k_pack(gev_part *__restrict__ out, long n, PclsArrays P) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    out[i] = pack_one<V>(P, i);
}

// Records read from / written to the caller's host buffer directly, when it is
// pinned or registered memory (the GPU reaches it over NVLink-C2C): no device
// staging copy.  A block moves 256 records (14336 bytes, 896 16-byte vectors)
// through shared memory, so that every host access of a warp is one contiguous
// run of 16-byte vectors; an odd record count leaves a last 8-byte half vector.
// Two blocks per SM keep several MB in flight, more than the host link needs, and
// leave the SMs to other streams' kernels.
constexpr int HREC = 256, HVEC = HREC * 56 / 16;
template <typename V>
__global__ void __launch_bounds__(256) k_unpack_host(const gev_part *in, long n, PclsArrays P, int N) {
  __shared__ uint4 s[HVEC];
  const long ntile = (n + HREC - 1) / HREC;
  for (long t = blockIdx.x; t < ntile; t += gridDim.x) {
    const long r0 = t * HREC;
    const int cnt = (int)(n - r0 < HREC ? n - r0 : HREC);
    const int nv = (cnt * 56) >> 4;
    const uint4 *src = reinterpret_cast<const uint4 *>(in + r0);  // r0 even: 16-byte aligned
    __syncthreads();
    for (int k = threadIdx.x; k < nv; k += blockDim.x) s[k] = src[k];
    if ((cnt & 1) && threadIdx.x == 0)
      reinterpret_cast<uint2 *>(s)[2 * nv] = reinterpret_cast<const uint2 *>(src)[2 * nv];
    __syncthreads();
    if ((int)threadIdx.x < cnt)
      unpack_one<V>(*reinterpret_cast<const gev_part *>(reinterpret_cast<const char *>(s) + threadIdx.x * 56),
                    r0 + threadIdx.x, P, N);
  }
}
// perm: when given, record i is particle perm[i] of the store (the store's own order
// is left as it is)
template <typename V>
__global__ void __launch_bounds__(256) k_pack_host(gev_part *out, long n, PclsArrays P,
                                                   const uint32_t *__restrict__ perm) {
  __shared__ uint4 s[HVEC];
  const long ntile = (n + HREC - 1) / HREC;
  for (long t = blockIdx.x; t < ntile; t += gridDim.x) {
    const long r0 = t * HREC;
    const int cnt = (int)(n - r0 < HREC ? n - r0 : HREC);
    const int nv = (cnt * 56) >> 4;
    __syncthreads();
    if ((int)threadIdx.x < cnt) {
      const long i = r0 + threadIdx.x;
      *reinterpret_cast<gev_part *>(reinterpret_cast<char *>(s) + threadIdx.x * 56) =
          pack_one<V>(P, perm ? (long)perm[i] : i);
    }
    __syncthreads();
    uint4 *dst = reinterpret_cast<uint4 *>(out + r0);
    for (int k = threadIdx.x; k < nv; k += blockDim.x) dst[k] = s[k];
    if ((cnt & 1) && threadIdx.x == 0)
      reinterpret_cast<uint2 *>(dst)[2 * nv] = reinterpret_cast<const uint2 *>(s)[2 * nv];
  }
}

// flag[0] = 1 if the particles are not in strictly increasing (cell, ID) order
__global__ void k_unordered(const uint32_t *__restrict__ cell, const int64_t *__restrict__ id, long n,
                            uint32_t *flag) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i + 1 < n; i += (long)gridDim.x * blockDim.x) {
    const uint32_t c0 = cell[i], c1 = cell[i + 1];
    if (c0 > c1 || (c0 == c1 && id[i] >= id[i + 1])) *flag = 1u;
  }
}

// ------------------------------------------------------------ sort ------
__global__ void k_count(const uint32_t *__restrict__ cell, long n, uint32_t *count, uint32_t *rank) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    rank[i] = atomicAdd(&count[cell[i]], 1u);
}

constexpr int SCAN_T = 256, SCAN_PER = 16, SCAN_TILE = SCAN_T * SCAN_PER;

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *sh, uint32_t &total) {
  // warp-shuffle scan then a scan of the warp totals
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[w] = x;
  __syncthreads();
  if (w == 0) {
    uint32_t t = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    sh[lane + 32] = t;
  }
  __syncthreads();
  total = sh[32 + (blockDim.x >> 5) - 1];
  const uint32_t before = w > 0 ? sh[32 + w - 1] : 0u;
  __syncthreads();
  return before + x - v;
}

__device__ __forceinline__ void k_scan_reduce_body(const uint32_t *__restrict__ in, long n, uint32_t *bsum) {
  __shared__ uint32_t sh[64];
  const long base = (long)blockIdx.x * SCAN_TILE;
  uint32_t s = 0;
  for (int k = 0; k < SCAN_PER; ++k) {
    const long i = base + (long)k * SCAN_T + threadIdx.x;
    if (i < n) s += in[i];
  }
  uint32_t total;
  block_exclusive_scan(s, sh, total);
  if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}
__global__ void __launch_bounds__(SCAN_T) k_scan_reduce(const uint32_t *__restrict__ in, long n, uint32_t *bsum) {
  k_scan_reduce_body(in, n, bsum);
}

// one block: exclusive scan of nb block sums in place
__device__ __forceinline__ void k_scan_blocks_body(uint32_t *bsum, long nb) {
  __shared__ uint32_t sh[64];
  const long per = (nb + blockDim.x - 1) / blockDim.x;
  const long b0 = threadIdx.x * per;
  uint32_t s = 0;
  for (long i = b0; i < b0 + per && i < nb; ++i) s += bsum[i];
  uint32_t total;
  uint32_t off = block_exclusive_scan(s, sh, total);
  for (long i = b0; i < b0 + per && i < nb; ++i) {
    const uint32_t v = bsum[i];
    bsum[i] = off;
    off += v;
  }
}
__global__ void __launch_bounds__(1024) k_scan_blocks(uint32_t *bsum, long nb) {
  k_scan_blocks_body(bsum, nb);
}

__device__ __forceinline__ void k_scan_down_body(const uint32_t *__restrict__ in, long n,
                                                      const uint32_t *__restrict__ bsum, uint32_t *out,
                                                      uint32_t total_n) {
  // one word of padding per 32: the thread-major accesses (tid * SCAN_PER + k) then
  // fall on 32 distinct banks instead of 2
  __shared__ uint32_t tile[SCAN_TILE + SCAN_TILE / 32];
  __shared__ uint32_t sh[64];
  auto pad = [](int i) { return i + (i >> 5); };
  const long base = (long)blockIdx.x * SCAN_TILE;
  for (int k = 0; k < SCAN_PER; ++k) {
    const long i = base + (long)k * SCAN_T + threadIdx.x;
    tile[pad(k * SCAN_T + threadIdx.x)] = i < n ? in[i] : 0u;
  }
  __syncthreads();
  uint32_t loc[SCAN_PER], s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_PER; ++k) {
    loc[k] = tile[pad(threadIdx.x * SCAN_PER + k)];
    s += loc[k];
  }
  uint32_t total;
  uint32_t off = block_exclusive_scan(s, sh, total) + bsum[blockIdx.x];
#pragma unroll
  for (int k = 0; k < SCAN_PER; ++k) {
    tile[pad(threadIdx.x * SCAN_PER + k)] = off;
    off += loc[k];
  }
  __syncthreads();
  for (int k = 0; k < SCAN_PER; ++k) {
    const long i = base + (long)k * SCAN_T + threadIdx.x;
    if (i < n) out[i] = tile[pad(k * SCAN_T + threadIdx.x)];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = total_n;
}
__global__ void __launch_bounds__(SCAN_T) k_scan_down(const uint32_t *__restrict__ in, long n,
                                                      const uint32_t *__restrict__ bsum, uint32_t *out,
                                                      uint32_t total_n) {
  k_scan_down_body(in, n, bsum, out, total_n);
}

__global__ void k_scatter(const uint32_t *__restrict__ cell, const uint32_t *__restrict__ rank, long n,
                          const uint32_t *__restrict__ start, uint32_t *perm) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    perm[start[cell[i]] + rank[i]] = (uint32_t)i;
}

// The (cell, ID) order: slot k of the run [s, e) of its cell holds particle via[k]
// (the store's own slot k where via is null); the particle's rank in the run is
// the number of the run's particles before it by (ID, slot) -- a permutation of the
// run even where IDs repeat, IDs in order of their slots -- and out[s + rank] gets
// the particle.  One thread a particle: the lanes of a warp mostly walk the same run,
// read from L1, and no thread sorts a cell alone (a thread a cell left most lanes
// idle beside the cells of a few particles).  The work is the sum over the cells of
// their squared counts.
__global__ void k_id_rank(const uint32_t *__restrict__ start, const uint32_t *__restrict__ cell,
                          const int64_t *__restrict__ id, const uint32_t *__restrict__ via, long n,
                          uint32_t *__restrict__ out) {
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
    const uint32_t i = via ? via[k] : (uint32_t)k;
    const uint32_t c = cell[i];
    const uint32_t s = start[c], e = start[c + 1];
    const int64_t my = id[i];
    uint32_t r = 0;
    for (uint32_t j = s; j < e; ++j) {
      const int64_t o = id[via ? via[j] : j];
      r += (o < my || (o == my && j < (uint32_t)k)) ? 1u : 0u;
    }
    if (s + r < e) out[s + r] = i;  // always, when slot k lies in its cell's run
  }
}

template <typename V>
__global__ void k_gather(PclsArrays src, PclsArrays dst, const uint32_t *__restrict__ perm, long n) {
  for (long j = blockIdx.x * (long)blockDim.x + threadIdx.x; j < n; j += (long)gridDim.x * blockDim.x) {
    const uint32_t i = perm[j];
    dst.px[j] = src.px[i];
    dst.py[j] = src.py[i];
    dst.pz[j] = src.pz[i];
    ((V *)dst.vx)[j] = ((const V *)src.vx)[i];
    ((V *)dst.vy)[j] = ((const V *)src.vy)[i];
    ((V *)dst.vz)[j] = ((const V *)src.vz)[i];
    dst.id[j] = src.id[i];
    dst.cell[j] = src.cell[i];
    if (sizeof(V) == 4) {
      dst.rx[j] = src.rx[i];
      dst.ry[j] = src.ry[i];
      dst.rz[j] = src.rz[i];
    }
  }
}

// relink without the ID order: particle i goes to start[cell] + rank, its rank
// among the particles of its cell taken by the atomic histogram.  The order
// inside a cell then follows atomic timing, which changes no result of the mixed
// form (its deposits add integers, the updates are per particle); downloads
// restore the (cell, ID) order first.
// Mixed form (FP32 momenta and offsets).  The source holds the drifted positions
// and their cell keys but not their in-cell offsets (k_kick_drift leaves them out):
// each particle's offsets are split from its position again, as the drift split
// them (pos_split, the same bits), and written with it.  A warp moves 32 PER
// consecutive particles per round, lane l the particles l, l + 32, l + 64,
// l + 96 (and so on), all payloads loaded before any store: every load and every store
// instruction of the warp covers 32 consecutive particles, and the destinations of
// consecutive particles (one cell's, or neighbouring cells') are consecutive too,
// so the scattered stores still fill whole lines.
// A lane holds PER particles' payloads (182 registers for 8, one block of 256
// threads per SM): in a clustered state the stores scatter within each dense
// cell's range and the loads wait longer, and more bytes in flight per warp beat
// more warps (the late-time 512^3 move took 5.19 ms with 8 or 6 a lane against 5.66
// with 4 at two blocks per SM on one GPU; 2 a lane at four blocks and 1 at six were
// slower than 4 on another).
constexpr int MOVE_PER = 8;
template <int PER>
__device__ __forceinline__ void k_move_body(PclsArrays src, PclsArrays dst, const uint32_t *__restrict__ start,
                                              const uint32_t *__restrict__ rank, long n, int N, int lg) {
  const float *svx = (const float *)src.vx, *svy = (const float *)src.vy, *svz = (const float *)src.vz;
  float *dvx = (float *)dst.vx, *dvy = (float *)dst.vy, *dvz = (float *)dst.vz;
  const int lane = threadIdx.x & 31;
  const long nw = (n + 32 * PER - 1) / (32 * PER), nwarps = ((long)gridDim.x * blockDim.x) >> 5;
  for (long w = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5; w < nw; w += nwarps) {
    const long i0 = w * (32 * PER) + lane;
    uint32_t c[PER], t[PER];
    double X[PER], Y[PER], Z[PER];
    long long D[PER];
    float VX[PER], VY[PER], VZ[PER];
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      const long i = i0 + 32 * k;
      if (i < n) {
        c[k] = src.cell[i];
        t[k] = rank[i];
        X[k] = src.px[i];
        Y[k] = src.py[i];
        Z[k] = src.pz[i];
        D[k] = src.id[i];
        VX[k] = svx[i];
        VY[k] = svy[i];
        VZ[k] = svz[i];
      }
    }
#pragma unroll
    for (int k = 0; k < PER; ++k)
      if (i0 + 32 * k < n) t[k] += start[c[k]];
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      if (i0 + 32 * k >= n) continue;
      int cx;
      float r0, r1, r2;
      pos_split(X[k], N, lg, cx, r0);
      pos_split(Y[k], N, lg, cx, r1);
      pos_split(Z[k], N, lg, cx, r2);
      const uint32_t j = t[k];
      dst.px[j] = X[k];
      dst.py[j] = Y[k];
      dst.pz[j] = Z[k];
      dvx[j] = VX[k];
      dvy[j] = VY[k];
      dvz[j] = VZ[k];
      dst.id[j] = D[k];
      dst.cell[j] = c[k];
      dst.rx[j] = r0;
      dst.ry[j] = r1;
      dst.rz[j] = r2;
    }
  }
}
template <int PER>
__global__ void __launch_bounds__(256, 1) k_move(PclsArrays src, PclsArrays dst, const uint32_t *__restrict__ start,
                                              const uint32_t *__restrict__ rank, long n, int N, int lg) {
  k_move_body<PER>(src, dst, start, rank, n, N, lg);
}

// ------------------------------------------------------- particle updates --
struct Params {
  double dtau, a, a2N, inv_a2, inv_a2N;
  int nfield, N, lg;
  // the same values rounded to FP32 on the host (round to nearest, as the device
  // conversion would), so the mixed form's loops convert nothing per particle
  float dtau_f, a_f, inv_a2_f, inv_a2N_f, inv_a_f, N_f;
};
inline Params make_params(double dtau, double a, double a2N, int nfield, int N) {
  Params p;
  p.dtau = dtau;
  p.a = a;
  p.a2N = a2N;
  p.inv_a2 = 1.0 / (a * a);
  p.inv_a2N = 1.0 / a2N;
  p.nfield = nfield;
  p.N = N;
  p.lg = lg_pow2(N);
  p.dtau_f = (float)p.dtau;
  p.a_f = (float)p.a;
  p.inv_a2_f = (float)p.inv_a2;
  p.inv_a2N_f = (float)p.inv_a2N;
  p.inv_a_f = (float)(1.0 / a);
  p.N_f = (float)N;
  return p;
}
// square root in the kernel's real type (sqrt of a float argument would otherwise
// resolve to the double overload and run on the FP64 pipe)
template <typename T>
__device__ __forceinline__ T tsqrt(T x) {
  if constexpr (sizeof(T) == 4)
    return sqrtf(x);
  else
    return sqrt(x);
}
// a parameter in the kernel's real type
template <typename T>
__device__ __forceinline__ T pv(double d, float f) {
  if constexpr (sizeof(T) == 4)
    return f;
  else
    return d;
}

// The linked cell of a particle and the index offsets (mod 2^32) of its six
// periodic neighbours, computed once per particle: every stencil value is then
// f[base + offsets], a few integer adds instead of a wrapped 3-D index.
struct CellNb {
  uint32_t base;  // x + N (y + N z)
  uint32_t xm, xp, ym, yp, zm, zp;
};
__device__ __forceinline__ CellNb cell_nb(uint32_t c, int N, int lg, int &cx, int &cy, int &cz) {
  if (lg >= 0) {
    cx = (int)(c & (uint32_t)(N - 1));
    cy = (int)((c >> lg) & (uint32_t)(N - 1));
    cz = (int)(c >> (2 * lg));
  } else {
    cx = (int)(c % (uint32_t)N);
    cy = (int)((c / (uint32_t)N) % (uint32_t)N);
    cz = (int)(c / ((uint32_t)N * (uint32_t)N));
  }
  const uint32_t n1 = (uint32_t)N, n2 = n1 * n1, n3 = n2 * n1;
  CellNb b;
  b.base = c;
  b.xm = cx == 0 ? n1 - 1u : 0u - 1u;
  b.xp = cx == N - 1 ? 1u - n1 : 1u;
  b.ym = cy == 0 ? n2 - n1 : 0u - n1;
  b.yp = cy == N - 1 ? n1 - n2 : n1;
  b.zm = cz == 0 ? n3 - n2 : 0u - n2;
  b.zp = cz == N - 1 ? n2 - n3 : n2;
  return b;
}
// f at the neighbour (DX, DY, DZ) in {-1, 0, 1}^3 of the cell
template <int DX, int DY, int DZ, typename T>
__device__ __forceinline__ T at(const T *__restrict__ f, const CellNb &b) {
  uint32_t i = b.base;
  if (DX < 0) i += b.xm;
  if (DX > 0) i += b.xp;
  if (DY < 0) i += b.ym;
  if (DY > 0) i += b.yp;
  if (DZ < 0) i += b.zm;
  if (DZ > 0) i += b.zp;
  return __ldg(f + i);
}

// The field values a particle update reads around its cell, as
// v<F, DX, DY, DZ>() with F = 0 phi, 1 chi, 2..4 the components of B.
// MemStencil loads each value where it is used.  RegStencil gathers every value
// the kick and the drift read (phi and chi on the cell's 8 corners, B^i on the 12
// nodes of the corners extended by one along axis i) into registers at once: one
// load per value for both updates, all of them in flight together.
template <typename T>
struct MemStencil {
  const T *phi, *chi, *B0, *B1, *B2;
  CellNb nb;
  bool has_chi, has_B;
  template <int F, int DX, int DY, int DZ>
  __device__ __forceinline__ T v() const {
    const T *f = F == 0 ? phi : F == 1 ? chi : F == 2 ? B0 : F == 3 ? B1 : B2;
    return at<DX, DY, DZ>(f, nb);
  }
};
template <typename T>
__device__ __forceinline__ MemStencil<T> mem_stencil(const T *phi, const T *chi, const T *Bi, size_t NV,
                                                     const CellNb &nb) {
  MemStencil<T> m;
  m.phi = phi;
  m.chi = chi;
  m.B0 = Bi;
  m.B1 = Bi ? Bi + NV : nullptr;
  m.B2 = Bi ? Bi + 2 * NV : nullptr;
  m.nb = nb;
  m.has_chi = chi != nullptr;
  m.has_B = Bi != nullptr;
  return m;
}
template <typename T>
struct RegStencil {
  T p[8], c[8], b0[12], b1[12], b2[12];
  bool has_chi, has_B;
  template <int F, int DX, int DY, int DZ>
  __device__ __forceinline__ T v() const {
    if constexpr (F == 0) return p[DX + 2 * DY + 4 * DZ];
    if constexpr (F == 1) return c[DX + 2 * DY + 4 * DZ];
    if constexpr (F == 2) return b0[(DX + 1) + 3 * (DY + 2 * DZ)];
    if constexpr (F == 3) return b1[DX + 2 * ((DY + 1) + 3 * DZ)];
    return b2[DX + 2 * DY + 4 * (DZ + 1)];
  }
};
template <int D>
__device__ __forceinline__ uint32_t nb_off(uint32_t m, uint32_t p) {
  return D < 0 ? m : (D > 0 ? p : 0u);
}
template <typename T>
__device__ __forceinline__ RegStencil<T> reg_stencil(const MemStencil<T> &m, bool chi_on, bool B_on) {
  RegStencil<T> r;
  const CellNb &b = m.nb;
  r.has_chi = m.has_chi;
  r.has_B = m.has_B;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const uint32_t i = b.base + ((k & 1) ? b.xp : 0u) + ((k & 2) ? b.yp : 0u) + ((k & 4) ? b.zp : 0u);
    r.p[k] = m.phi ? __ldg(m.phi + i) : (T)0;  // no phi: a drift with nfield = 0
    r.c[k] = chi_on ? __ldg(m.chi + i) : (T)0;
  }
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    // b0: x in {-1, 0, 1}, (y, z) in {0, 1}^2; b1: y in {-1, 0, 1}; b2: z in {-1, 0, 1}
    const int e0 = k % 3 - 1, u0 = (k / 3) & 1, w0 = k / 6;
    const int x1 = k & 1, e1 = (k >> 1) % 3 - 1, w1 = k / 6;
    const int x2 = k & 1, y2 = (k >> 1) & 1, e2 = (k >> 2) - 1;
    const uint32_t i0 = b.base + (e0 < 0 ? b.xm : e0 > 0 ? b.xp : 0u) + (u0 ? b.yp : 0u) + (w0 ? b.zp : 0u);
    const uint32_t i1 = b.base + (x1 ? b.xp : 0u) + (e1 < 0 ? b.ym : e1 > 0 ? b.yp : 0u) + (w1 ? b.zp : 0u);
    const uint32_t i2 = b.base + (x2 ? b.xp : 0u) + (y2 ? b.yp : 0u) + (e2 < 0 ? b.zm : e2 > 0 ? b.zp : 0u);
    r.b0[k] = B_on ? __ldg(m.B0 + i0) : (T)0;
    r.b1[k] = B_on ? __ldg(m.B1 + i1) : (T)0;
    r.b2[k] = B_on ? __ldg(m.B2 + i2) : (T)0;
  }
  return r;
}

// The per-particle physics of update_q (gevolution.hpp:570-678, GRADIENT_ORDER 1)
// and update_pos (810-871), on the particle's linked cell (its neighbours nb) and its
// in-cell offset r = pos*N - cell (ref_dist of the reference).  Field values are
// gathered with periodic wrap.

// q -> q - dtau e grad / dx (GR) or q - dtau a grad / dx (Newton)
template <typename T, int KIND, typename S>
__device__ __forceinline__ void kick_one(const S &st, const Params &pr, T r0, T r1, T r2, T &q0, T &q1, T &q2) {
  const int N = pr.N;
  const T s0 = (T)1 - r0, s1 = (T)1 - r1, s2 = (T)1 - r2;
  T g0, g1, g2;
  {
    const T f000 = st.template v<0, 0, 0, 0>(), f100 = st.template v<0, 1, 0, 0>(), f010 = st.template v<0, 0, 1, 0>(),
            f110 = st.template v<0, 1, 1, 0>(), f001 = st.template v<0, 0, 0, 1>(), f101 = st.template v<0, 1, 0, 1>(),
            f011 = st.template v<0, 0, 1, 1>(), f111 = st.template v<0, 1, 1, 1>();
    g0 = s1 * s2 * (f100 - f000) + r1 * s2 * (f110 - f010) + s1 * r2 * (f101 - f001) + r1 * r2 * (f111 - f011);
    g1 = s0 * s2 * (f010 - f000) + r0 * s2 * (f110 - f100) + s0 * r2 * (f011 - f001) + r0 * r2 * (f111 - f101);
    g2 = s0 * s1 * (f001 - f000) + r0 * s1 * (f101 - f100) + s0 * r1 * (f011 - f010) + r0 * r1 * (f111 - f110);
  }
  const T a = pv<T>(pr.a, pr.a_f);
  T e = (T)0, inv_e = (T)0;
  if (KIND == GEV_GR) {
    const T v2 = q0 * q0 + q1 * q1 + q2 * q2;
    const T e2 = v2 + a * a;
    T fac;
    if constexpr (sizeof(T) == 4) {
      // FP32: one reciprocal square root for e, 1/e and (v^2 + e^2) / e^2 = 1 + v^2 / e^2
      // (within 2 ulp, the rounding level of the form) instead of two IEEE divisions
      // and a square root
      const T r = rsqrtf(e2);
      inv_e = r;
      e = e2 * r;
      fac = (T)1 + v2 * (r * r);
    } else {
      fac = (v2 + e2) / e2;
      e = tsqrt<T>(e2);
      inv_e = (T)1 / e;
    }
    g0 *= fac;
    g1 *= fac;
    g2 *= fac;
  }
  if (pr.nfield >= 2 && st.has_chi) {
    const T f000 = st.template v<1, 0, 0, 0>(), f100 = st.template v<1, 1, 0, 0>(), f010 = st.template v<1, 0, 1, 0>(),
            f110 = st.template v<1, 1, 1, 0>(), f001 = st.template v<1, 0, 0, 1>(), f101 = st.template v<1, 1, 0, 1>(),
            f011 = st.template v<1, 0, 1, 1>(), f111 = st.template v<1, 1, 1, 1>();
    g0 -= s1 * s2 * (f100 - f000) + r1 * s2 * (f110 - f010) + s1 * r2 * (f101 - f001) + r1 * r2 * (f111 - f011);
    g1 -= s0 * s2 * (f010 - f000) + r0 * s2 * (f110 - f100) + s0 * r2 * (f011 - f001) + r0 * r2 * (f111 - f101);
    g2 -= s0 * s1 * (f001 - f000) + r0 * s1 * (f101 - f100) + s0 * r1 * (f011 - f010) + r0 * r1 * (f111 - f110);
  }
  if (KIND == GEV_GR && pr.nfield >= 3 && st.has_B) {
    const T t0 = (T)2 * r0, t1 = (T)2 * r1, t2 = (T)2 * r2;
    T p0, p1, p2;
    p0 = (s2 * (st.template v<3, 1, 0, 0>() - st.template v<3, 0, 0, 0>()) +
          r2 * (st.template v<3, 1, 0, 1>() - st.template v<3, 0, 0, 1>())) * q1;
    p0 += (s1 * (st.template v<4, 1, 0, 0>() - st.template v<4, 0, 0, 0>()) +
           r1 * (st.template v<4, 1, 1, 0>() - st.template v<4, 0, 1, 0>())) * q2;
    p0 += (s1 * s2 * ((r0 - (T)1) * st.template v<2, -1, 0, 0>() + ((T)1 - t0) * st.template v<2, 0, 0, 0>() + r0 * st.template v<2, 1, 0, 0>()) +
           r1 * s2 * ((r0 - (T)1) * st.template v<2, -1, 1, 0>() + ((T)1 - t0) * st.template v<2, 0, 1, 0>() + r0 * st.template v<2, 1, 1, 0>()) +
           s1 * r2 * ((r0 - (T)1) * st.template v<2, -1, 0, 1>() + ((T)1 - t0) * st.template v<2, 0, 0, 1>() + r0 * st.template v<2, 1, 0, 1>()) +
           r1 * r2 * ((r0 - (T)1) * st.template v<2, -1, 1, 1>() + ((T)1 - t0) * st.template v<2, 0, 1, 1>() + r0 * st.template v<2, 1, 1, 1>())) * q0;
    p1 = (s0 * (st.template v<4, 0, 1, 0>() - st.template v<4, 0, 0, 0>()) +
          r0 * (st.template v<4, 1, 1, 0>() - st.template v<4, 1, 0, 0>())) * q2;
    p1 += (s2 * (st.template v<2, 0, 1, 0>() - st.template v<2, 0, 0, 0>()) +
           r2 * (st.template v<2, 0, 1, 1>() - st.template v<2, 0, 0, 1>())) * q0;
    p1 += (s0 * s2 * ((r1 - (T)1) * st.template v<3, 0, -1, 0>() + ((T)1 - t1) * st.template v<3, 0, 0, 0>() + r1 * st.template v<3, 0, 1, 0>()) +
           r0 * s2 * ((r1 - (T)1) * st.template v<3, 1, -1, 0>() + ((T)1 - t1) * st.template v<3, 1, 0, 0>() + r1 * st.template v<3, 1, 1, 0>()) +
           s0 * r2 * ((r1 - (T)1) * st.template v<3, 0, -1, 1>() + ((T)1 - t1) * st.template v<3, 0, 0, 1>() + r1 * st.template v<3, 0, 1, 1>()) +
           r0 * r2 * ((r1 - (T)1) * st.template v<3, 1, -1, 1>() + ((T)1 - t1) * st.template v<3, 1, 0, 1>() + r1 * st.template v<3, 1, 1, 1>())) * q1;
    p2 = (s1 * (st.template v<2, 0, 0, 1>() - st.template v<2, 0, 0, 0>()) +
          r1 * (st.template v<2, 0, 1, 1>() - st.template v<2, 0, 1, 0>())) * q0;
    p2 += (s0 * (st.template v<3, 0, 0, 1>() - st.template v<3, 0, 0, 0>()) +
           r0 * (st.template v<3, 1, 0, 1>() - st.template v<3, 1, 0, 0>())) * q1;
    p2 += (s0 * s1 * ((r2 - (T)1) * st.template v<4, 0, 0, -1>() + ((T)1 - t2) * st.template v<4, 0, 0, 0>() + r2 * st.template v<4, 0, 0, 1>()) +
           r0 * s1 * ((r2 - (T)1) * st.template v<4, 1, 0, -1>() + ((T)1 - t2) * st.template v<4, 1, 0, 0>() + r2 * st.template v<4, 1, 0, 1>()) +
           s0 * r1 * ((r2 - (T)1) * st.template v<4, 0, 1, -1>() + ((T)1 - t2) * st.template v<4, 0, 1, 0>() + r2 * st.template v<4, 0, 1, 1>()) +
           r0 * r1 * ((r2 - (T)1) * st.template v<4, 1, 1, -1>() + ((T)1 - t2) * st.template v<4, 1, 1, 0>() + r2 * st.template v<4, 1, 1, 1>())) * q2;
    const T k = pv<T>(pr.inv_a2N, pr.inv_a2N_f) * inv_e;
    g0 += p0 * k;
    g1 += p1 * k;
    g2 += p2 * k;
  }
  const T m = pv<T>(pr.dtau, pr.dtau_f) * (KIND == GEV_GR ? e : a) * pv<T>((double)N, pr.N_f);
  q0 -= m * g0;
  q1 -= m * g1;
  q2 -= m * g2;
}

// the coordinate velocity of update_pos (GR): q (1 + (3 - q^2/e^2) phi - chi) / e + b / (a^2 N)
template <typename T, typename S>
__device__ __forceinline__ void drift_vel(const S &st, const Params &pr, T r0, T r1, T r2, T q0, T q1, T q2, T &v0,
                                          T &v1, T &v2) {
  const T s0 = (T)1 - r0, s1 = (T)1 - r1, s2 = (T)1 - r2;
  const T a = pv<T>(pr.a, pr.a_f);
  const T qq = q0 * q0 + q1 * q1 + q2 * q2;
  const T e2 = qq + a * a;
  T ph = (T)0, ch = (T)0;
  const T w000 = s0 * s1 * s2, w100 = r0 * s1 * s2, w010 = s0 * r1 * s2, w110 = r0 * r1 * s2;
  const T w001 = s0 * s1 * r2, w101 = r0 * s1 * r2, w011 = s0 * r1 * r2, w111 = r0 * r1 * r2;
  if (pr.nfield >= 1)
    ph = st.template v<0, 0, 0, 0>() * w000 + st.template v<0, 1, 0, 0>() * w100 + st.template v<0, 0, 1, 0>() * w010 +
         st.template v<0, 1, 1, 0>() * w110 + st.template v<0, 0, 0, 1>() * w001 + st.template v<0, 1, 0, 1>() * w101 +
         st.template v<0, 0, 1, 1>() * w011 + st.template v<0, 1, 1, 1>() * w111;
  if (pr.nfield >= 2)
    ch = st.template v<1, 0, 0, 0>() * w000 + st.template v<1, 1, 0, 0>() * w100 + st.template v<1, 0, 1, 0>() * w010 +
         st.template v<1, 1, 1, 0>() * w110 + st.template v<1, 0, 0, 1>() * w001 + st.template v<1, 1, 0, 1>() * w101 +
         st.template v<1, 0, 1, 1>() * w011 + st.template v<1, 1, 1, 1>() * w111;
  T fac;
  if constexpr (sizeof(T) == 4) {  // FP32: 1/e^2 and 1/e from one reciprocal square root
    const T r = rsqrtf(e2);
    fac = ((T)1 + ((T)3 - qq * (r * r)) * ph - ch) * r;
  } else {
    const T inv_e2 = (T)1 / e2;
    fac = ((T)1 + ((T)3 - qq * inv_e2) * ph - ch) * tsqrt<T>(inv_e2);
  }
  v0 = q0 * fac;
  v1 = q1 * fac;
  v2 = q2 * fac;
  if (pr.nfield >= 3) {
    const T b0 = st.template v<2, 0, 0, 0>() * s1 * s2 + st.template v<2, 0, 1, 0>() * r1 * s2 + st.template v<2, 0, 0, 1>() * s1 * r2 +
                 st.template v<2, 0, 1, 1>() * r1 * r2;
    const T b1 = st.template v<3, 0, 0, 0>() * s0 * s2 + st.template v<3, 1, 0, 0>() * r0 * s2 + st.template v<3, 0, 0, 1>() * s0 * r2 +
                 st.template v<3, 1, 0, 1>() * r0 * r2;
    const T b2 = st.template v<4, 0, 0, 0>() * s0 * s1 + st.template v<4, 1, 0, 0>() * r0 * s1 + st.template v<4, 0, 1, 0>() * s0 * r1 +
                 st.template v<4, 1, 1, 0>() * r0 * r1;
    const T ib = pv<T>(pr.inv_a2N, pr.inv_a2N_f);
    v0 += b0 * ib;
    v1 += b1 * ib;
    v2 += b2 * ib;
  }
}

// One particle's payload, read with independent loads before any field gather
// or store, so that all of it is in flight at once.
template <typename T, typename V>
struct Pcl {
  uint32_t cell;
  double x, y, z;
  T q0, q1, q2;
  float rx, ry, rz;  // the FP32 in-cell offset (mixed form)
};
template <typename T, typename V>
__device__ __forceinline__ Pcl<T, V> load_pcl(const PclsArrays &P, long i, bool pos) {
  Pcl<T, V> c;
  c.cell = P.cell[i];
  if (pos || sizeof(T) == 8) {
    c.x = P.px[i];
    c.y = P.py[i];
    c.z = P.pz[i];
  }
  c.q0 = (T)((const V *)P.vx)[i];
  c.q1 = (T)((const V *)P.vy)[i];
  c.q2 = (T)((const V *)P.vz)[i];
  if constexpr (sizeof(T) == 4) {
    c.rx = P.rx[i];
    c.ry = P.ry[i];
    c.rz = P.rz[i];
  }
  return c;
}
// the particle's linked cell and in-cell offset (the FP32 copy in the mixed form)
template <typename T, typename V>
__device__ __forceinline__ CellNb cell_of(const Pcl<T, V> &c, int N, int lg, T &r0, T &r1, T &r2) {
  int cx, cy, cz;
  const CellNb nb = cell_nb(c.cell, N, lg, cx, cy, cz);
  if constexpr (sizeof(T) == 4) {
    r0 = c.rx;
    r1 = c.ry;
    r2 = c.rz;
  } else {
    r0 = (T)(c.x * (double)N - cx);
    r1 = (T)(c.y * (double)N - cy);
    r2 = (T)(c.z * (double)N - cz);
  }
  return nb;
}
// the stencil a kernel reads: in registers for FP32, from memory for FP64 (whose
// 52 doubles would not fit beside the rest)
template <typename T>
__device__ __forceinline__ auto stencil(const T *phi, const T *chi, const T *Bi, int N, const CellNb &nb, bool chi_on,
                                        bool B_on) {
  const MemStencil<T> m = mem_stencil<T>(phi, chi_on ? chi : nullptr, B_on ? Bi : nullptr, (size_t)N * N * N, nb);
  if constexpr (sizeof(T) == 4)
    return reg_stencil<T>(m, m.has_chi, m.has_B);
  else
    return m;
}

// pos += dtau v, periodic wrap into [0, 1), new cell key (and offset) for the relink
// OFFSETS_LATER (mixed form, followed by k_move): the in-cell offsets are not
// stored here; k_move splits them from the stored position again (the same bits)
// as it moves the particle, which saves writing and re-reading them.
template <typename T, bool OFFSETS_LATER = false>
__device__ __forceinline__ uint32_t move_store(PclsArrays &P, long i, const Params &pr, T v0, T v1, T v2, double x,
                                               double y, double z) {
  const int N = pr.N, lg = pr.lg;
  const double dtau = pr.dtau;
  uint32_t key;
  if constexpr (sizeof(T) == 4) {
    const float dt = pr.dtau_f;
    x += f2d_bits(dt * v0);
    y += f2d_bits(dt * v1);
    z += f2d_bits(dt * v2);
    x = wrap01_bits(x);
    y = wrap01_bits(y);
    z = wrap01_bits(z);
    int cx, cy, cz;
    float r0, r1, r2;
    pos_split(x, N, lg, cx, r0);
    pos_split(y, N, lg, cy, r1);
    pos_split(z, N, lg, cz, r2);
    if (!OFFSETS_LATER) {
      P.rx[i] = r0;
      P.ry[i] = r1;
      P.rz[i] = r2;
    }
    key = (uint32_t)cx + (uint32_t)N * ((uint32_t)cy + (uint32_t)N * (uint32_t)cz);
  } else {
    x = wrap01(x + dtau * (double)v0);
    y = wrap01(y + dtau * (double)v1);
    z = wrap01(z + dtau * (double)v2);
    key = cell_key(x, y, z, N);
  }
  P.cell[i] = key;
  P.px[i] = x;
  P.py[i] = y;
  P.pz[i] = z;
  return key;
}

template <typename T>
__device__ __forceinline__ void block_max_to(T vmax, unsigned long long *maxbits) {
  for (int o = 16; o > 0; o >>= 1) {
    const T other = __shfl_xor_sync(0xffffffffu, vmax, o);
    vmax = other > vmax ? other : vmax;
  }
  __shared__ double sh[8];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = (double)vmax;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0.;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, sh[w]);
    atomicMax(maxbits, (unsigned long long)__double_as_longlong(m));
  }
}

// Particles::updateVel(update_q | update_q_Newton); the reduction is max q^2 / a^2
template <typename T, typename V, int KIND>
__global__ void __launch_bounds__(256) k_update_q(PclsArrays P, long n, const T *__restrict__ phi,
                                                  const T *__restrict__ chi, const T *__restrict__ Bi, Params pr,
                                                  unsigned long long *maxbits) {
  T vmax = (T)0;
  const bool chi_on = pr.nfield >= 2 && chi, B_on = KIND == GEV_GR && pr.nfield >= 3 && Bi;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const Pcl<T, V> c = load_pcl<T, V>(P, i, false);
    T r0, r1, r2;
    const CellNb nb = cell_of<T, V>(c, pr.N, pr.lg, r0, r1, r2);
    T q0 = c.q0, q1 = c.q1, q2 = c.q2;
    const auto st = stencil<T>(phi, chi, Bi, pr.N, nb, chi_on, B_on);
    kick_one<T, KIND>(st, pr, r0, r1, r2, q0, q1, q2);
    ((V *)P.vx)[i] = (V)q0;
    ((V *)P.vy)[i] = (V)q1;
    ((V *)P.vz)[i] = (V)q2;
    const T v2 = (q0 * q0 + q1 * q1 + q2 * q2) * pv<T>(pr.inv_a2, pr.inv_a2_f);
    vmax = v2 > vmax ? v2 : vmax;
  }
  block_max_to<T>(vmax, maxbits);
}

// Particles::moveParticles(update_pos | update_pos_Newton), then the wrap and the new key
template <typename T, typename V, int KIND>
__global__ void __launch_bounds__(256) k_update_pos(PclsArrays P, long n, const T *__restrict__ phi,
                                                    const T *__restrict__ chi, const T *__restrict__ Bi, Params pr) {
  const bool chi_on = pr.nfield >= 2 && chi, B_on = pr.nfield >= 3 && Bi;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const Pcl<T, V> c = load_pcl<T, V>(P, i, true);
    const T q0 = c.q0, q1 = c.q1, q2 = c.q2;
    T v0, v1, v2;
    if (KIND == GEV_NEWTON) {  // update_pos_Newton: dtau q / a
      const T ia = pv<T>(1.0 / pr.a, pr.inv_a_f);
      v0 = q0 * ia;
      v1 = q1 * ia;
      v2 = q2 * ia;
    } else {
      T r0, r1, r2;
      const CellNb nb = cell_of<T, V>(c, pr.N, pr.lg, r0, r1, r2);
      const auto st = stencil<T>(phi, chi, Bi, pr.N, nb, chi_on, B_on);
      drift_vel<T>(st, pr, r0, r1, r2, q0, q1, q2, v0, v1, v2);
    }
    move_store<T>(P, i, pr, v0, v1, v2, c.x, c.y, c.z);
  }
}

// updateVel(update_q) followed by moveParticles(update_pos) (main.cpp:775-798)
// in one pass: both read the same cell and the same phi / chi / B values.  The
// drift's scale factor (after the background half step) comes in pd.
template <typename T, typename V>
__device__ __forceinline__ void k_kick_drift_body(PclsArrays P, long n, const T *__restrict__ phi,
                                                    const T *__restrict__ chi, const T *__restrict__ Bi, Params pk,
                                                    Params pd, unsigned long long *maxbits, uint32_t *count,
                                                    uint32_t *rank) {
  T vmax = (T)0;
  const int nf = pk.nfield > pd.nfield ? pk.nfield : pd.nfield;
  const bool chi_on = nf >= 2 && chi, B_on = nf >= 3 && Bi;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const Pcl<T, V> c = load_pcl<T, V>(P, i, true);
    T r0, r1, r2;
    const CellNb nb = cell_of<T, V>(c, pk.N, pk.lg, r0, r1, r2);
    T q0 = c.q0, q1 = c.q1, q2 = c.q2;
    const auto st = stencil<T>(phi, chi, Bi, pk.N, nb, chi_on, B_on);
    kick_one<T, GEV_GR>(st, pk, r0, r1, r2, q0, q1, q2);
    ((V *)P.vx)[i] = (V)q0;
    ((V *)P.vy)[i] = (V)q1;
    ((V *)P.vz)[i] = (V)q2;
    const T vv = (q0 * q0 + q1 * q1 + q2 * q2) * pv<T>(pk.inv_a2, pk.inv_a2_f);
    vmax = vv > vmax ? vv : vmax;
    T v0, v1, v2;
    drift_vel<T>(st, pd, r0, r1, r2, q0, q1, q2, v0, v1, v2);
    // the mixed form (count given) leaves the in-cell offsets to k_move
    const uint32_t key = move_store<T, sizeof(T) == 4>(P, i, pd, v0, v1, v2, c.x, c.y, c.z);
    if (count) rank[i] = atomicAdd(&count[key], 1u);  // the histogram of the relink, fused
  }
  block_max_to<T>(vmax, maxbits);
}
template <typename T, typename V>
__global__ void __launch_bounds__(256, 2) k_kick_drift(PclsArrays P, long n, const T *__restrict__ phi,
                                                    const T *__restrict__ chi, const T *__restrict__ Bi, Params pk,
                                                    Params pd, unsigned long long *maxbits, uint32_t *count,
                                                    uint32_t *rank) {
  k_kick_drift_body<T, V>(P, n, phi, chi, Bi, pk, pd, maxbits, count, rank);
}

template <typename V>
size_t vbytes() {
  return sizeof(V);
}

// the arrays of one set carved from one allocation, each on a 256-byte boundary
int alloc_arrays(gev_ctx *ctx, PclsArrays &A, long cap, size_t vsz) {
  const size_t n = (size_t)cap;
  const bool mixed = vsz == 4;  // mixed form: FP32 in-cell offsets too
  const size_t sizes[11] = {n * 8, n * 8, n * 8, n * vsz, n * vsz, n * vsz, n * 8, n * 4,
                            mixed ? n * 4 : 0, mixed ? n * 4 : 0, mixed ? n * 4 : 0};
  size_t off[11], total = 0;
  for (int k = 0; k < 11; ++k) {
    off[k] = total;
    total += (sizes[k] + 255) & ~(size_t)255;
  }
  char *b = nullptr;
  GEV_CHECK_CUDA(ctx, cudaMalloc(&b, total));
  A.block = b;
  A.block_bytes = total;
  A.px = (double *)(b + off[0]);
  A.py = (double *)(b + off[1]);
  A.pz = (double *)(b + off[2]);
  A.vx = b + off[3];
  A.vy = b + off[4];
  A.vz = b + off[5];
  A.id = (int64_t *)(b + off[6]);
  A.cell = (uint32_t *)(b + off[7]);
  if (mixed) {
    A.rx = (float *)(b + off[8]);
    A.ry = (float *)(b + off[9]);
    A.rz = (float *)(b + off[10]);
  }
  ctx->bytes_in_use += total;
  return GEV_OK;
}
void free_arrays(PclsArrays &A) {
  cudaFree(A.block);
  A = PclsArrays();
}

int scan_cells(gev_ctx *ctx, gev_pcls *p) {
  const long C = (long)ctx->N * ctx->N * ctx->N;
  const long nb = (C + SCAN_TILE - 1) / SCAN_TILE;
  GevTimed tm_(ctx, "k_scan");
  gev_launch<k_scan_reduce_body, SCAN_T, 1>(ctx, k_scan_reduce, dim3((unsigned)nb), dim3(SCAN_T), 0,
                                            (const uint32_t *)p->count, C, p->scan_tmp);
  GEV_LAUNCH_CHECK(ctx);
  gev_launch<k_scan_blocks_body, 1024, 1>(ctx, k_scan_blocks, dim3(1), dim3(1024), 0, p->scan_tmp, nb);
  GEV_LAUNCH_CHECK(ctx);
  gev_launch<k_scan_down_body, SCAN_T, 1>(ctx, k_scan_down, dim3((unsigned)nb), dim3(SCAN_T), 0,
                                          (const uint32_t *)p->count, C, (const uint32_t *)p->scan_tmp, p->start,
                                          (uint32_t)p->n);
  GEV_LAUNCH_CHECK(ctx);
  return GEV_OK;
}

template <typename T, typename V>
int launch_update_q(gev_ctx *ctx, gev_pcls *p, int kind, double dtau, const gev_field *phi, const gev_field *chi,
                    const gev_field *Bi, int nfield, double a, double a2N, unsigned long long *mb) {
  const Params pr = make_params(dtau, a, a2N, nfield, ctx->N);
  GEV_CHECK_CUDA(ctx, cudaMemsetAsync(mb, 0, sizeof(unsigned long long), ctx->stream));
  const int blocks = grid_for(ctx, (size_t)p->n, 256, 16);
  const T *fphi = (const T *)phi->d, *fchi = chi ? (const T *)chi->d : nullptr, *fB = Bi ? (const T *)Bi->d : nullptr;
  if (kind == GEV_GR)
    k_update_q<T, V, GEV_GR><<<blocks, 256, 0, ctx->stream>>>(p->cur, p->n, fphi, fchi, fB, pr, mb);
  else
    k_update_q<T, V, GEV_NEWTON><<<blocks, 256, 0, ctx->stream>>>(p->cur, p->n, fphi, fchi, fB, pr, mb);
  GEV_LAUNCH_CHECK(ctx);
  return GEV_OK;
}

template <typename T, typename V>
int update_pos_t(gev_ctx *ctx, gev_pcls *p, int kind, double dtau, const gev_field *phi, const gev_field *chi,
                 const gev_field *Bi, int nfield, double a, double a2N) {
  const Params pr = make_params(dtau, a, a2N, nfield, ctx->N);
  const int blocks = grid_for(ctx, (size_t)p->n, 256, 16);
  const T *fphi = phi ? (const T *)phi->d : nullptr, *fchi = chi ? (const T *)chi->d : nullptr,
          *fB = Bi ? (const T *)Bi->d : nullptr;
  if (kind == GEV_GR)
    k_update_pos<T, V, GEV_GR><<<blocks, 256, 0, ctx->stream>>>(p->cur, p->n, fphi, fchi, fB, pr);
  else
    k_update_pos<T, V, GEV_NEWTON><<<blocks, 256, 0, ctx->stream>>>(p->cur, p->n, fphi, fchi, fB, pr);
  GEV_LAUNCH_CHECK(ctx);
  return pcls_relink(ctx, p);
}

bool field_ok(gev_ctx *ctx, const gev_field *f, int ncomp) {
  return f && f->ctx == ctx && f->kind == GEV_FIELD_REAL && f->ncomp == ncomp;
}

}  // namespace

int pcls_kick_async(gev_ctx *ctx, gev_pcls *p, int kind, double dtau, const gev_field *phi, const gev_field *chi,
                    const gev_field *Bi, int nfield, double a, double a2N, unsigned long long *maxbits_dev) {
  if (nfield < 2) chi = nullptr;
  if (nfield < 3) Bi = nullptr;
  return ctx->prec == GEV_PREC_FP64
             ? launch_update_q<double, double>(ctx, p, kind, dtau, phi, chi, Bi, nfield, a, a2N, maxbits_dev)
             : launch_update_q<float, float>(ctx, p, kind, dtau, phi, chi, Bi, nfield, a, a2N, maxbits_dev);
}

int pcls_kick_drift_async(gev_ctx *ctx, gev_pcls *p, double dtau_k, double a_k, int nfield_k, double dtau_d,
                          double a_d, int nfield_d, const gev_field *phi, const gev_field *chi, const gev_field *Bi,
                          unsigned long long *maxbits_dev) {
  const int N = ctx->N;
  const double a2N_k = a_k * a_k * N, a2N_d = a_d * a_d * N;
  const Params pk = make_params(dtau_k, a_k, a2N_k, nfield_k, N);
  const Params pd = make_params(dtau_d, a_d, a2N_d, nfield_d, N);
  GEV_CHECK_CUDA(ctx, gev_zero_async(ctx, maxbits_dev, sizeof(unsigned long long)));
  const int blocks = grid_for(ctx, (size_t)p->n, 256, 16);
  if (ctx->prec == GEV_PREC_FP64) {
    GevTimed tm_(ctx, "k_kick_drift");
    k_kick_drift<double, double><<<blocks, 256, 0, ctx->stream>>>(p->cur, p->n, (const double *)phi->d,
                                                                  (const double *)chi->d, (const double *)Bi->d, pk, pd,
                                                                  maxbits_dev, nullptr, nullptr);
    GEV_LAUNCH_CHECK(ctx);
    tm_.stop();
    GevTimed tr_(ctx, "relink");
    return pcls_relink(ctx, p);
  }
  // mixed form: histogram in the update, then scan and one move (no ID order)
  const long C = (long)N * N * N;
  GEV_CHECK_CUDA(ctx, gev_zero_async(ctx, p->count, C * sizeof(uint32_t)));
  GevTimed tm_(ctx, "k_kick_drift");
  gev_launch<k_kick_drift_body<float, float>, 256, 2>(ctx, k_kick_drift<float, float>, dim3(blocks), dim3(256), 0,
                                                      p->cur, p->n, (const float *)phi->d, (const float *)chi->d,
                                                      (const float *)Bi->d, pk, pd, maxbits_dev, p->count, p->rank);
  GEV_LAUNCH_CHECK(ctx);
  tm_.stop();
  if (p->n == 0) return GEV_OK;
  int rc = scan_cells(ctx, p);
  if (rc) return rc;
  GevTimed tv_(ctx, "k_move");
  gev_launch<k_move_body<MOVE_PER>, 256, 1>(ctx, k_move<MOVE_PER>,
                                            dim3(grid_for(ctx, (size_t)(p->n + MOVE_PER - 1) / MOVE_PER, 256, 16)),
                                            dim3(256), 0, p->cur, p->alt, (const uint32_t *)p->start,
                                            (const uint32_t *)p->rank, p->n, N, lg_pow2(N));
  GEV_LAUNCH_CHECK(ctx);
  std::swap(p->cur, p->alt);
  p->id_order = false;
  return GEV_OK;
}

// restore the (cell, ID) order after moves that skipped it
// The device address of a host buffer that kernels may access directly (pinned
// or registered memory, 16-byte aligned), or nullptr: pageable memory goes
// through a device staging copy instead.
static const void *host_alias(const void *h) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || a.devicePointer == nullptr || ((uintptr_t)a.devicePointer & 15u) != 0u)
    return nullptr;
  return a.devicePointer;
}

int pcls_relink(gev_ctx *ctx, gev_pcls *p);

// relink of uploaded particles: a store already in (cell, ID) order -- as
// gev_pcls_download writes it -- needs only its cell counts and starts (one read
// of the cell keys and IDs decides, and the host waits for that answer)
static int relink_uploaded(gev_ctx *ctx, gev_pcls *p) {
  if (p->n < 2) return pcls_relink(ctx, p);
  const long C = (long)ctx->N * ctx->N * ctx->N;
  const int pb = grid_for(ctx, (size_t)p->n, 256, 16);
  GEV_CHECK_CUDA(ctx, cudaMemsetAsync(p->bounds + 15, 0, sizeof(uint32_t), ctx->stream));
  {
    GevTimed tm_(ctx, "k_unordered");
    k_unordered<<<pb, 256, 0, ctx->stream>>>(p->cur.cell, p->cur.id, p->n, p->bounds + 15);
    GEV_LAUNCH_CHECK(ctx);
  }
  uint32_t unordered = 1u;
  GEV_CHECK_CUDA(ctx, cudaMemcpyAsync(&unordered, p->bounds + 15, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
  GEV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (unordered) return pcls_relink(ctx, p);
  GEV_CHECK_CUDA(ctx, cudaMemsetAsync(p->count, 0, C * sizeof(uint32_t), ctx->stream));
  k_count<<<pb, 256, 0, ctx->stream>>>(p->cur.cell, p->n, p->count, p->rank);
  GEV_LAUNCH_CHECK(ctx);
  int rc = scan_cells(ctx, p);
  if (rc) return rc;
  p->id_order = true;
  return GEV_OK;
}

// perm = the store's particles in (cell, ID) order (each cell's run ranked by ID)
static int id_permutation(gev_ctx *ctx, gev_pcls *p) {
  GevTimed tm_(ctx, "k_id_rank");
  k_id_rank<<<grid_for(ctx, (size_t)p->n, 256, 16), 256, 0, ctx->stream>>>(p->start, p->cur.cell, p->cur.id, nullptr,
                                                                          p->n, p->perm);
  GEV_LAUNCH_CHECK(ctx);
  return GEV_OK;
}

int pcls_id_order(gev_ctx *ctx, gev_pcls *p) {
  if (p->id_order || p->n == 0) return GEV_OK;
  const int pb = grid_for(ctx, (size_t)p->n, 256, 16);
  int rc = id_permutation(ctx, p);
  if (rc) return rc;
  if (ctx->prec == GEV_PREC_FP64)
    k_gather<double><<<pb, 256, 0, ctx->stream>>>(p->cur, p->alt, p->perm, p->n);
  else
    k_gather<float><<<pb, 256, 0, ctx->stream>>>(p->cur, p->alt, p->perm, p->n);
  GEV_LAUNCH_CHECK(ctx);
  std::swap(p->cur, p->alt);
  p->id_order = true;
  return GEV_OK;
}

int pcls_relink(gev_ctx *ctx, gev_pcls *p) {
  const long C = (long)ctx->N * ctx->N * ctx->N;
  if (p->n == 0) {
    GEV_CHECK_CUDA(ctx, cudaMemsetAsync(p->start, 0, (C + 1) * sizeof(uint32_t), ctx->stream));
    return GEV_OK;
  }
  GEV_CHECK_CUDA(ctx, cudaMemsetAsync(p->count, 0, C * sizeof(uint32_t), ctx->stream));
  const int pb = grid_for(ctx, (size_t)p->n, 256, 16);
  k_count<<<pb, 256, 0, ctx->stream>>>(p->cur.cell, p->n, p->count, p->rank);
  GEV_LAUNCH_CHECK(ctx);
  int rc = scan_cells(ctx, p);
  if (rc) return rc;
  k_scatter<<<pb, 256, 0, ctx->stream>>>(p->cur.cell, p->rank, p->n, p->start, p->perm);
  GEV_LAUNCH_CHECK(ctx);
  {
    GevTimed tm_(ctx, "k_id_rank");
    k_id_rank<<<pb, 256, 0, ctx->stream>>>(p->start, p->cur.cell, p->cur.id, p->perm, p->n, p->rank);
    GEV_LAUNCH_CHECK(ctx);
  }
  if (ctx->prec == GEV_PREC_FP64)
    k_gather<double><<<pb, 256, 0, ctx->stream>>>(p->cur, p->alt, p->rank, p->n);
  else
    k_gather<float><<<pb, 256, 0, ctx->stream>>>(p->cur, p->alt, p->rank, p->n);
  GEV_LAUNCH_CHECK(ctx);
  std::swap(p->cur, p->alt);
  p->id_order = true;
  return GEV_OK;
}

// device records d[0, count) into slots [offset, offset + count) of the store's
// arrays (cell keys and in-cell offsets derived as gev_pcls_upload does); the
// caller sets p->n and relinks
int pcls_unpack_at(gev_ctx *ctx, gev_pcls *p, const gev_part *d, long count, long offset) {
  if (count <= 0) return GEV_OK;
  if (offset < 0 || offset + count > p->cap) return gev_fail(ctx, GEV_EINVAL, "particles exceed the store's capacity");
  PclsArrays A = p->cur;
  const size_t vsz = ctx->prec == GEV_PREC_FP64 ? 8 : 4;
  A.px += offset;
  A.py += offset;
  A.pz += offset;
  A.vx = (char *)A.vx + offset * vsz;
  A.vy = (char *)A.vy + offset * vsz;
  A.vz = (char *)A.vz + offset * vsz;
  A.id += offset;
  A.cell += offset;
  if (A.rx) {
    A.rx += offset;
    A.ry += offset;
    A.rz += offset;
  }
  const int b = grid_for(ctx, (size_t)count, 256, 16);
  if (ctx->prec == GEV_PREC_FP64)
    k_unpack<double><<<b, 256, 0, ctx->stream>>>(d, count, A, ctx->N);
  else
    k_unpack<float><<<b, 256, 0, ctx->stream>>>(d, count, A, ctx->N);
  GEV_LAUNCH_CHECK(ctx);
  return GEV_OK;
}

// records [i0, i0 + count) of the store, in its current order, into d
int pcls_pack_range(gev_ctx *ctx, gev_pcls *p, gev_part *d, long i0, long count) {
  if (count <= 0) return GEV_OK;
  PclsArrays A = p->cur;
  const size_t vsz = ctx->prec == GEV_PREC_FP64 ? 8 : 4;
  A.px += i0;
  A.py += i0;
  A.pz += i0;
  A.vx = (char *)A.vx + i0 * vsz;
  A.vy = (char *)A.vy + i0 * vsz;
  A.vz = (char *)A.vz + i0 * vsz;
  A.id += i0;
  const int b = grid_for(ctx, (size_t)count, 256, 16);
  if (ctx->prec == GEV_PREC_FP64)
    k_pack<double><<<b, 256, 0, ctx->stream>>>(d, count, A);
  else
    k_pack<float><<<b, 256, 0, ctx->stream>>>(d, count, A);
  GEV_LAUNCH_CHECK(ctx);
  return GEV_OK;
}

extern "C" {

int gev_pcls_create(gev_ctx *ctx, long capacity, double mass, gev_pcls **out) {
  if (!ctx || !out || capacity < 0 || capacity > 0xFFFFFFFFL) return gev_fail(ctx, GEV_EINVAL, "pcls_create: bad capacity");
  gev_pcls *p = new gev_pcls();
  p->ctx = ctx;
  ctx_retain(ctx);
  p->cap = capacity;
  p->mass = mass;
  const size_t vsz = ctx->prec == GEV_PREC_FP64 ? 8 : 4;
  const long C = (long)ctx->N * ctx->N * ctx->N;
  const long cap = capacity > 0 ? capacity : 1;
  const size_t bytes0 = ctx->bytes_in_use;
  int rc = alloc_arrays(ctx, p->cur, cap, vsz);
  if (!rc) rc = alloc_arrays(ctx, p->alt, cap, vsz);
  if (!rc) {
    p->scan_tmp_elems = (size_t)((C + SCAN_TILE - 1) / SCAN_TILE) + 1;
    if (cudaMalloc(&p->count, C * 4) != cudaSuccess || cudaMalloc(&p->start, (C + 1) * 4) != cudaSuccess ||
        cudaMalloc(&p->rank, cap * 4) != cudaSuccess || cudaMalloc(&p->perm, cap * 4) != cudaSuccess ||
        cudaMalloc(&p->bounds, 16 * 4) != cudaSuccess ||
        cudaMalloc(&p->scan_tmp, p->scan_tmp_elems * 4) != cudaSuccess)
      rc = gev_fail(ctx, GEV_ENOMEM, "pcls_create: device allocation failed");
    else
      ctx->bytes_in_use += (size_t)C * 8 + (size_t)cap * 8 + p->scan_tmp_elems * 4;
  }
  p->bytes = ctx->bytes_in_use - bytes0;
  if (rc) {
    gev_pcls_destroy(p);
    cudaGetLastError();
    return rc == GEV_ECUDA ? GEV_ENOMEM : rc;
  }
  GEV_CHECK_CUDA(ctx, cudaMemsetAsync(p->start, 0, (C + 1) * 4, ctx->stream));
  *out = p;
  return GEV_OK;
}

int gev_pcls_destroy(gev_pcls *p) {
  if (!p) return GEV_OK;
  free_arrays(p->cur);
  free_arrays(p->alt);
  cudaFree(p->count);
  cudaFree(p->start);
  cudaFree(p->rank);
  cudaFree(p->perm);
  cudaFree(p->bounds);
  cudaFree(p->prep);
  cudaFree(p->dense);
  cudaFree(p->scan_tmp);
  gev_ctx *ctx = p->ctx;
  if (ctx) ctx->bytes_in_use -= p->bytes;
  delete p;
  if (ctx) ctx_release(ctx);
  return GEV_OK;
}

int gev_pcls_upload(gev_pcls *p, const gev_part *host, long n) {
  if (!p || (n > 0 && !host) || n < 0 || n > p->cap) return gev_fail(p ? p->ctx : nullptr, GEV_EINVAL, "pcls_upload: n exceeds capacity");
  gev_ctx *ctx = p->ctx;
  p->n = n;
  if (n > 0) {
    if (const gev_part *h = (const gev_part *)host_alias(host)) {
      const int hb = grid_for(ctx, (size_t)((n + HREC - 1) / HREC), 1, 2);
      GevTimed tm_(ctx, "k_unpack_host");
      if (ctx->prec == GEV_PREC_FP64)
        k_unpack_host<double><<<hb, 256, 0, ctx->stream>>>(h, n, p->cur, ctx->N);
      else
        k_unpack_host<float><<<hb, 256, 0, ctx->stream>>>(h, n, p->cur, ctx->N);
      GEV_LAUNCH_CHECK(ctx);
      tm_.stop();
      return relink_uploaded(ctx, p);
    }
    gev_part *d = nullptr;
    GEV_CHECK_CUDA(ctx, cudaMallocAsync(&d, n * sizeof(gev_part), ctx->stream));
    GEV_CHECK_CUDA(ctx, cudaMemcpyAsync(d, host, n * sizeof(gev_part), cudaMemcpyHostToDevice, ctx->stream));
    const int b = grid_for(ctx, (size_t)n, 256, 16);
    if (ctx->prec == GEV_PREC_FP64)
      k_unpack<double><<<b, 256, 0, ctx->stream>>>(d, n, p->cur, ctx->N);
    else
      k_unpack<float><<<b, 256, 0, ctx->stream>>>(d, n, p->cur, ctx->N);
    GEV_LAUNCH_CHECK(ctx);
    GEV_CHECK_CUDA(ctx, cudaFreeAsync(d, ctx->stream));
  }
  return relink_uploaded(ctx, p);
}

int gev_pcls_download(gev_pcls *p, gev_part *host, long *n) {
  if (!p || (!host && p->n > 0)) return gev_fail(p ? p->ctx : nullptr, GEV_EINVAL, "pcls_download: null buffer");
  gev_ctx *ctx = p->ctx;
  if (n) *n = p->n;
  gev_part *h = p->n > 0 ? (gev_part *)host_alias(host) : nullptr;
  if (h) {
    // the pack runs at the host link's rate, so it reads the particles through the
    // (cell, ID) permutation rather than moving the store into that order first
    const uint32_t *perm = nullptr;
    if (!p->id_order) {
      int rc = id_permutation(ctx, p);
      if (rc) return rc;
      perm = p->perm;
    }
    const int hb = grid_for(ctx, (size_t)((p->n + HREC - 1) / HREC), 1, 2);
    GevTimed tm_(ctx, "k_pack_host");
    if (ctx->prec == GEV_PREC_FP64)
      k_pack_host<double><<<hb, 256, 0, ctx->stream>>>(h, p->n, p->cur, perm);
    else
      k_pack_host<float><<<hb, 256, 0, ctx->stream>>>(h, p->n, p->cur, perm);
    GEV_LAUNCH_CHECK(ctx);
    tm_.stop();
    GEV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return GEV_OK;
  }
  int rc = pcls_id_order(ctx, p);
  if (rc) return rc;
  if (p->n > 0) {
    gev_part *d = nullptr;
    GEV_CHECK_CUDA(ctx, cudaMallocAsync(&d, p->n * sizeof(gev_part), ctx->stream));
    const int b = grid_for(ctx, (size_t)p->n, 256, 16);
    if (ctx->prec == GEV_PREC_FP64)
      k_pack<double><<<b, 256, 0, ctx->stream>>>(d, p->n, p->cur);
    else
      k_pack<float><<<b, 256, 0, ctx->stream>>>(d, p->n, p->cur);
    GEV_LAUNCH_CHECK(ctx);
    GEV_CHECK_CUDA(ctx, cudaMemcpyAsync(host, d, p->n * sizeof(gev_part), cudaMemcpyDeviceToHost, ctx->stream));
    GEV_CHECK_CUDA(ctx, cudaFreeAsync(d, ctx->stream));
  }
  GEV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return GEV_OK;
}

int gev_pcls_count(gev_pcls *p, long *n) {
  if (!p || !n) return GEV_EINVAL;
  *n = p->n;
  return GEV_OK;
}

int gev_update_q(gev_ctx *ctx, gev_pcls *p, int kind, double dtau, const gev_field *phi, const gev_field *chi,
                 const gev_field *Bi, int nfield, double a, double a2N, double *maxvel) {
  if (!ctx || !p || p->ctx != ctx || (kind != GEV_GR && kind != GEV_NEWTON) || nfield < 1 || !field_ok(ctx, phi, 1) ||
      (nfield >= 2 && !field_ok(ctx, chi, 1)) || (kind == GEV_GR && nfield >= 3 && !field_ok(ctx, Bi, 3)) || a <= 0.)
    return gev_fail(ctx, GEV_EINVAL, "update_q: needs phi (and chi for nfield>=2, Bi for nfield>=3) and a > 0");
  if (nfield < 2) chi = nullptr;
  if (nfield < 3) Bi = nullptr;
  int rc = ctx_ensure_red(ctx, 2);
  if (rc) return rc;
  unsigned long long *mb = (unsigned long long *)ctx->d_red;
  rc = pcls_kick_async(ctx, p, kind, dtau, phi, chi, Bi, nfield, a, a2N, mb);
  if (rc) return rc;
  if (maxvel) {
    unsigned long long bits = 0;
    GEV_CHECK_CUDA(ctx, cudaMemcpyAsync(&bits, mb, sizeof(bits), cudaMemcpyDeviceToHost, ctx->stream));
    GEV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    double m;
    memcpy(&m, &bits, sizeof(m));
    *maxvel = sqrt(m);
  }
  return GEV_OK;
}

int gev_update_q_pos(gev_ctx *ctx, gev_pcls *p, double dtau_kick, double a_kick, int nfield_kick, double dtau_drift,
                     double a_drift, int nfield_drift, const gev_field *phi, const gev_field *chi, const gev_field *Bi,
                     double *maxvel) {
  if (!ctx || !p || p->ctx != ctx || !field_ok(ctx, phi, 1) || !field_ok(ctx, chi, 1) || !field_ok(ctx, Bi, 3) ||
      a_kick <= 0. || a_drift <= 0. || nfield_kick < 1 || nfield_kick > 3 || nfield_drift < 0 || nfield_drift > 3)
    return gev_fail(ctx, GEV_EINVAL, "update_q_pos: phi, chi (1 comp) and Bi (3 comps), a > 0, nfield 1..3 / 0..3");
  int rc = ctx_ensure_red(ctx, 2);
  if (rc) return rc;
  unsigned long long *mb = (unsigned long long *)ctx->d_red;
  rc = pcls_kick_drift_async(ctx, p, dtau_kick, a_kick, nfield_kick, dtau_drift, a_drift, nfield_drift, phi, chi, Bi,
                             mb);
  if (rc) return rc;
  if (maxvel) {
    unsigned long long bits = 0;
    GEV_CHECK_CUDA(ctx, cudaMemcpyAsync(&bits, mb, sizeof(bits), cudaMemcpyDeviceToHost, ctx->stream));
    GEV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    double m;
    memcpy(&m, &bits, sizeof(m));
    *maxvel = sqrt(m);
  }
  return GEV_OK;
}

int gev_update_pos(gev_ctx *ctx, gev_pcls *p, int kind, double dtau, const gev_field *phi, const gev_field *chi,
                   const gev_field *Bi, int nfield, double a, double a2N) {
  if (!ctx || !p || p->ctx != ctx || (kind != GEV_GR && kind != GEV_NEWTON) || a <= 0. || nfield < 0 ||
      (kind == GEV_GR && ((nfield >= 1 && !field_ok(ctx, phi, 1)) || (nfield >= 2 && !field_ok(ctx, chi, 1)) ||
                          (nfield >= 3 && !field_ok(ctx, Bi, 3)))))
    return gev_fail(ctx, GEV_EINVAL, "update_pos: needs phi/chi/Bi for nfield >= 1/2/3 and a > 0");
  if (kind == GEV_NEWTON) nfield = 0;
  if (nfield < 1) phi = nullptr;
  if (nfield < 2) chi = nullptr;
  if (nfield < 3) Bi = nullptr;
  return ctx->prec == GEV_PREC_FP64
             ? update_pos_t<double, double>(ctx, p, kind, dtau, phi, chi, Bi, nfield, a, a2N)
             : update_pos_t<float, float>(ctx, p, kind, dtau, phi, chi, Bi, nfield, a, a2N);
}

}  // extern "C"
