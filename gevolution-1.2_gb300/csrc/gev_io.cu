// gev_io.cu -- Gadget-2 snapshots and hibernation points of the device state
// (include/gev_io.h).
//
// Gadget-2 (Particles_gevolution.hpp:30-251 saveGadget2, 574-665 loadGadget2):
// the per-particle conversion runs on the GPU -- one block per chunk of 1024
// particles in (cell, ID) order selects the tracers (ID % tracer_factor == 0),
// places them with a block scan at the chunk's offset (chunk offsets are an
// exclusive scan of per-chunk counts), and writes float positions, float
// velocities and IDs interleaved as the file holds them.  The host streams the
// batches into the file's three blocks.  The arithmetic is the reference's, in
// FP64 with every operation an explicitly rounded intrinsic (no contraction),
// then rounded to FP32.
//
// Hibernation points (hibernation.hpp:513-611, ic_read.hpp:290-320): sections
// are streamed through a pinned staging buffer with a 64-bit checksum each.
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/gev_io.h"
#include "gev_internal.cuh"

static_assert(sizeof(gev_gadget2_header) == 256, "the Gadget-2 header is 256 bytes");

namespace {

constexpr int G2_CHUNK = 1024;             // particles per selection chunk (one block)
constexpr long G2_BATCH = 1L << 22;        // tracers converted per file batch
constexpr size_t STAGE_BYTES = 64u << 20;  // checkpoint streaming buffer

struct G2Params {
  double box, rescale_vel, time, dtau_pos, dtau_vel, dx;
  long long tf;
  int N, lg, exact, idb;
  Div32 dN;
};

__global__ void __launch_bounds__(256) k_g2_count(const int64_t *__restrict__ id, long n, long long tf,
                                                  uint32_t *cnt) {
  __shared__ uint32_t ws[8];
  const long base = (long)blockIdx.x * G2_CHUNK;
  uint32_t c = 0;
  for (int k = 0; k < G2_CHUNK / 256; ++k) {
    const long i = base + k * 256 + threadIdx.x;
    if (i < n && id[i] % tf == 0) ++c;
  }
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int j = 0; j < 8; ++j) t += ws[j];
    cnt[blockIdx.x] = t;
  }
}

__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }
// modf's fractional part (x - trunc(x), exact)
__device__ __forceinline__ double dfrac(double x) { return dsub(x, trunc(x)); }

// one particle's record: Particles_gevolution.hpp:162-220
template <typename V, typename PH>
__device__ void g2_convert(const PclsArrays &P, long i, const PH *__restrict__ phi, const G2Params &g, float *pos,
                           float *vel) {
  const double x[3] = {P.px[i], P.py[i], P.pz[i]};
  const double v[3] = {(double)((const V *)P.vx)[i], (double)((const V *)P.vy)[i], (double)((const V *)P.vz)[i]};
  if (!g.exact) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      pos[k] = __double2float_rn(dmul(x[k], g.box));
      vel[k] = __double2float_rn(ddiv(dmul(v[k], g.rescale_vel), g.time));
    }
    return;
  }
  // EXACT_OUTPUT_REDSHIFTS: CIC phi and its gradient at the particle, from the
  // 8 corners of its cell
  double r[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) r[k] = dfrac(ddiv(x[k], g.dx));
  const double d0 = dsub(1., r[0]), d1 = dsub(1., r[1]), d2 = dsub(1., r[2]);
  int cx, cy, cz;
  cell_xyz(P.cell[i], g.N, g.lg, g.dN, cx, cy, cz);
  const Nb3 b = nb3(P.cell[i], cx, cy, cz, g.N);
  const unsigned i0 = P.cell[i], ix = i0 + b.xp, iy = i0 + b.yp, iz = i0 + b.zp;
  const unsigned ixy = ix + b.yp, ixz = ix + b.zp, iyz = iy + b.zp, ixyz = ixy + b.zp;
  const double f000 = (double)phi[i0], f100 = (double)phi[ix], f010 = (double)phi[iy], f110 = (double)phi[ixy];
  const double f001 = (double)phi[iz], f101 = (double)phi[ixz], f011 = (double)phi[iyz], f111 = (double)phi[ixyz];
  double ph = dmul(dmul(dmul(f000, d0), d1), d2);
  ph = dadd(ph, dmul(dmul(dmul(f100, r[0]), d1), d2));
  ph = dadd(ph, dmul(dmul(dmul(f010, d0), r[1]), d2));
  ph = dadd(ph, dmul(dmul(dmul(f110, r[0]), r[1]), d2));
  ph = dadd(ph, dmul(dmul(dmul(f001, d0), d1), r[2]));
  ph = dadd(ph, dmul(dmul(dmul(f101, r[0]), d1), r[2]));
  ph = dadd(ph, dmul(dmul(dmul(f011, d0), r[1]), r[2]));
  ph = dadd(ph, dmul(dmul(dmul(f111, r[0]), r[1]), r[2]));
  double gr[3];
  gr[0] = dmul(dmul(d1, d2), dsub(f100, f000));
  gr[1] = dmul(dmul(d0, d2), dsub(f010, f000));
  gr[2] = dmul(dmul(d0, d1), dsub(f001, f000));
  gr[0] = dadd(gr[0], dmul(dmul(r[1], d2), dsub(f110, f010)));
  gr[1] = dadd(gr[1], dmul(dmul(r[0], d2), dsub(f110, f100)));
  gr[2] = dadd(gr[2], dmul(dmul(r[0], d1), dsub(f101, f100)));
  gr[0] = dadd(gr[0], dmul(dmul(d1, r[2]), dsub(f101, f001)));
  gr[1] = dadd(gr[1], dmul(dmul(d0, r[2]), dsub(f011, f001)));
  gr[2] = dadd(gr[2], dmul(dmul(d0, r[1]), dsub(f011, f010)));
  gr[0] = dadd(gr[0], dmul(dmul(r[1], r[2]), dsub(f111, f011)));
  gr[1] = dadd(gr[1], dmul(dmul(r[0], r[2]), dsub(f111, f101)));
  gr[2] = dadd(gr[2], dmul(dmul(r[0], r[1]), dsub(f111, f110)));
  const double v2 = dadd(dadd(dmul(v[0], v[0]), dmul(v[1], v[1])), dmul(v[2], v[2]));
  const double e2 = dadd(v2, dmul(g.time, g.time));
  const double e = __dsqrt_rn(e2);
  const double v2e = dadd(v2, e2);
  const double fac = dadd(1., dmul(dsub(4., ddiv(v2e, e2)), ph));
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double p = dadd(dadd(1., x[k]), ddiv(dmul(dmul(g.dtau_pos, v[k]), fac), e));
    pos[k] = __double2float_rn(dmul(dfrac(p), g.box));
    const double kick = ddiv(ddiv(dmul(dmul(g.dtau_vel, v2e), gr[k]), g.dx), e);
    vel[k] = __double2float_rn(ddiv(dmul(dsub(v[k], kick), g.rescale_vel), g.time));
  }
}

// chunks [c0, c0 + gridDim.x): block b places chunk c0 + b's tracers at
// off[b] - obase of the batch buffers, in store order
template <typename V, typename PH>
__global__ void __launch_bounds__(256) k_g2_pack(PclsArrays P, long n, long c0, const long long *__restrict__ off,
                                                 long long obase, const PH *__restrict__ phi, G2Params g,
                                                 float *__restrict__ pos, float *__restrict__ vel,
                                                 unsigned char *__restrict__ ids) {
  __shared__ uint32_t ws[8];
  const long base = (c0 + blockIdx.x) * (long)G2_CHUNK;
  const long long o0 = off[blockIdx.x] - obase;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t run = 0;
  for (int k = 0; k < G2_CHUNK / 256; ++k) {
    const long i = base + k * 256 + threadIdx.x;
    const bool sel = i < n && P.id[i] % g.tf == 0;
    const unsigned bal = __ballot_sync(0xffffffffu, sel);
    if (lane == 0) ws[w] = __popc(bal);
    __syncthreads();
    uint32_t before = run + __popc(bal & ((1u << lane) - 1u)), tot = 0;
    for (int j = 0; j < 8; ++j) {
      if (j < w) before += ws[j];
      tot += ws[j];
    }
    __syncthreads();
    run += tot;
    if (sel) {
      const long long o = o0 + before;
      float pf[3], vf[3];
      g2_convert<V, PH>(P, i, phi, g, pf, vf);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        pos[3 * o + c] = pf[c];
        vel[3 * o + c] = vf[c];
      }
      const int64_t id = P.id[i];
      if (g.idb == 8)
        ((int64_t *)ids)[o] = id;
      else
        ((int32_t *)ids)[o] = (int32_t)(uint32_t)(uint64_t)id;
    }
  }
}

// loadGadget2's conversion (Particles_gevolution.hpp:638-657), in its float /
// double arithmetic, into particle records
__global__ void __launch_bounds__(256) k_g2_unpack(const float *__restrict__ pos, const float *__restrict__ vel,
                                                   const unsigned char *__restrict__ ids, long n, double box,
                                                   double vfac, int idb, gev_part *__restrict__ out) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    gev_part q;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      float pf = __double2float_rn(__ddiv_rn((double)pos[3 * i + c], box));
      if ((double)pf >= 1.) pf = __double2float_rn(__dsub_rn((double)pf, 1.));
      q.pos[c] = (double)pf;
      q.vel[c] = (double)__double2float_rn(__dmul_rn((double)vel[3 * i + c], vfac));
    }
    q.ID = idb == 8 ? (long)((const int64_t *)ids)[i] : (long)((const int32_t *)ids)[i];
    out[i] = q;
  }
}

// hibernate's B / (a^2 N) and readIC's B * a^2 / N^2, in FP64 then the field's type
template <typename R>
__global__ void k_scale(const R *__restrict__ in, R *__restrict__ out, size_t n, double s, int divide) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double v = divide ? __ddiv_rn((double)in[i], s) : __dmul_rn((double)in[i], s);
    out[i] = (R)v;
  }
}

// ---------------------------------------------------------------- host --
struct File {
  FILE *f = nullptr;
  ~File() {
    if (f) fclose(f);
  }
};

bool put(FILE *f, long long off, const void *p, size_t bytes) {
  return fseeko(f, (off_t)off, SEEK_SET) == 0 && fwrite(p, 1, bytes, f) == bytes;
}
bool get(FILE *f, long long off, void *p, size_t bytes) {
  return fseeko(f, (off_t)off, SEEK_SET) == 0 && fread(p, 1, bytes, f) == bytes;
}

G2Params g2_params(const gev_ctx *ctx, double box, double time, double dtau_pos, double dtau_vel, long long tf,
                   int exact, int idb) {
  G2Params g;
  g.box = box;
  g.time = time;
  g.rescale_vel = 1. / sqrt(time) / GEV_GADGET_VELOCITY_CONVERSION;  // Particles_gevolution.hpp:45
  g.dtau_pos = dtau_pos;
  g.dtau_vel = dtau_vel;
  g.dx = 1.0 / (double)ctx->N;
  g.tf = tf;
  g.N = ctx->N;
  g.lg = lg_pow2(ctx->N);
  g.exact = exact;
  g.idb = idb;
  g.dN = make_div32((unsigned)ctx->N);
  return g;
}

struct DevBuf {
  gev_ctx *ctx;
  void *p = nullptr;
  explicit DevBuf(gev_ctx *c) : ctx(c) {}
  ~DevBuf() {
    if (p) cudaFreeAsync(p, ctx->stream);
  }
};
struct HostBuf {
  void *p = nullptr;
  ~HostBuf() {
    if (p) cudaFreeHost(p);
  }
};

// the splitmix64 finaliser (Steele, Lea, Flood 2014; Vigna's constants) of each
// 8-byte word plus its index, summed: a checksum that a truncated, shifted or
// altered section fails
inline uint64_t mix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
struct Sum64 {
  uint64_t acc = 0, idx = 0;
  void add(const void *p, size_t bytes) {  // bytes a multiple of 8 except on the last call
    const unsigned char *c = (const unsigned char *)p;
    size_t i = 0;
    for (; i + 8 <= bytes; i += 8) {
      uint64_t w;
      memcpy(&w, c + i, 8);
      acc += mix64(w ^ (idx++ * 0x2545F4914F6CDD1Dull));
    }
    if (i < bytes) {
      uint64_t w = 0;
      memcpy(&w, c + i, bytes - i);
      acc += mix64(w ^ (idx++ * 0x2545F4914F6CDD1Dull));
    }
  }
};

struct CkptSection {
  uint64_t offset, bytes, checksum;
};
enum { SEC_PCLS = 0, SEC_PHI, SEC_CHI, SEC_B, SEC_BIFT, NSEC };
struct CkptHeader {
  char magic[8];
  uint32_t version, header_bytes;
  int32_t N, prec, elem_real, has_state;
  int64_t numpcl;
  double a, tau, dtau;
  int32_t cycle, pad0;
  double diag[4];  // a simulation's pending diagnostics: T00 sum, max bits, phi(k=0)
  uint32_t state_bytes, pad1;
  unsigned char state[512];
  CkptSection sec[NSEC];
  uint64_t header_checksum;
};
constexpr uint32_t CKPT_HEADER_BYTES = 4096;
static_assert(sizeof(CkptHeader) <= CKPT_HEADER_BYTES, "checkpoint header fits its slot");
static_assert(sizeof(gev_sim_state) <= 512, "state fits the header");
const char CKPT_MAGIC[8] = {'G', 'E', 'V', 'H', 'I', 'B', 'E', '1'};

uint64_t header_sum(const CkptHeader &h) {
  Sum64 s;
  s.add(&h, offsetof(CkptHeader, header_checksum));
  return s.acc;
}

bool field_shape(const gev_ctx *ctx, const gev_field *f, int kind, int ncomp) {
  return f && f->ctx == ctx && f->kind == kind && f->ncomp == ncomp;
}

// a device range to the file through the pinned stage (optionally scaled first)
int write_device(gev_ctx *ctx, FILE *f, long long off, const void *dsrc, size_t bytes, void *stage_h, void *stage_d,
                 Sum64 &sum, double scale, int real_bytes) {
  const char *src = (const char *)dsrc;
  for (size_t done = 0; done < bytes; done += STAGE_BYTES) {
    const size_t len = bytes - done < STAGE_BYTES ? bytes - done : STAGE_BYTES;
    const void *from = src + done;
    if (scale != 0.) {
      const size_t n = len / real_bytes;
      const int b = grid_for(ctx, n, 256, 8);
      if (real_bytes == 8)
        k_scale<double><<<b, 256, 0, ctx->stream>>>((const double *)from, (double *)stage_d, n, scale, 1);
      else
        k_scale<float><<<b, 256, 0, ctx->stream>>>((const float *)from, (float *)stage_d, n, scale, 1);
      GEV_LAUNCH_CHECK(ctx);
      from = stage_d;
    }
    GEV_CHECK_CUDA(ctx, cudaMemcpyAsync(stage_h, from, len, cudaMemcpyDeviceToHost, ctx->stream));
    GEV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    sum.add(stage_h, len);
    if (!put(f, off + (long long)done, stage_h, len)) return gev_fail(ctx, GEV_EINVAL, "checkpoint: write failed");
  }
  return GEV_OK;
}

// file bytes into a device range (optionally scaled on the way)
int read_device(gev_ctx *ctx, FILE *f, long long off, void *ddst, size_t bytes, void *stage_h, void *stage_d,
                Sum64 &sum, double scale, int real_bytes) {
  char *dst = (char *)ddst;
  for (size_t done = 0; done < bytes; done += STAGE_BYTES) {
    const size_t len = bytes - done < STAGE_BYTES ? bytes - done : STAGE_BYTES;
    if (!get(f, off + (long long)done, stage_h, len)) return gev_fail(ctx, GEV_EINVAL, "checkpoint: file truncated");
    sum.add(stage_h, len);
    if (scale != 0.) {
      GEV_CHECK_CUDA(ctx, cudaMemcpyAsync(stage_d, stage_h, len, cudaMemcpyHostToDevice, ctx->stream));
      const size_t n = len / real_bytes;
      const int b = grid_for(ctx, n, 256, 8);
      if (real_bytes == 8)
        k_scale<double><<<b, 256, 0, ctx->stream>>>((const double *)stage_d, (double *)(dst + done), n, scale, 0);
      else
        k_scale<float><<<b, 256, 0, ctx->stream>>>((const float *)stage_d, (float *)(dst + done), n, scale, 0);
      GEV_LAUNCH_CHECK(ctx);
    } else {
      GEV_CHECK_CUDA(ctx, cudaMemcpyAsync(dst + done, stage_h, len, cudaMemcpyHostToDevice, ctx->stream));
    }
    GEV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  }
  return GEV_OK;
}

size_t field_bytes(const gev_field *f) { return f->comp_elems * f->elem_bytes * f->ncomp; }

}  // namespace

extern "C" {

int gev_gadget2_save(gev_ctx *ctx, gev_pcls *p, const char *filename, const gev_gadget2_header *hdr,
                     int tracer_factor, double dtau_pos, double dtau_vel, const gev_field *phi, int exact_output,
                     int id_bytes) {
  if (!ctx || !p || p->ctx != ctx || !filename || !hdr || tracer_factor < 1 || (id_bytes != 4 && id_bytes != 8) ||
      hdr->time <= 0. || (phi && !field_shape(ctx, phi, GEV_FIELD_REAL, 1)))
    return gev_fail(ctx, GEV_EINVAL, "gadget2_save: bad arguments");
  if (hdr->num_files != 1)
    return gev_fail(ctx, GEV_EINVAL, "gadget2_save: one GPU writes one file (num_files must be 1)");
  if (exact_output && !phi)
    return gev_fail(ctx, GEV_EINVAL, "gadget2_save: the exact-output correction needs phi");
  int rc = pcls_id_order(ctx, p);
  if (rc) return rc;
  const long n = p->n;
  const long nch = (n + G2_CHUNK - 1) / G2_CHUNK;
  // tracer counts per chunk, and their exclusive scan on the host
  std::vector<long long> off((size_t)nch + 1, 0);
  if (nch > 0) {
    DevBuf cnt(ctx);
    GEV_CHECK_CUDA(ctx, cudaMallocAsync(&cnt.p, nch * sizeof(uint32_t), ctx->stream));
    k_g2_count<<<(unsigned)nch, 256, 0, ctx->stream>>>(p->cur.id, n, (long long)tracer_factor, (uint32_t *)cnt.p);
    GEV_LAUNCH_CHECK(ctx);
    std::vector<uint32_t> c((size_t)nch);
    GEV_CHECK_CUDA(ctx, cudaMemcpyAsync(c.data(), cnt.p, nch * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
    GEV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (long k = 0; k < nch; ++k) off[k + 1] = off[k] + c[k];
  }
  const long long S = off[nch];
  if (S != (long long)hdr->npart[1] || S > 0xFFFFFFFFll)
    return gev_fail(ctx, GEV_EINVAL, "gadget2_save: hdr.npart[1] does not match the particles to write");
  File F;
  F.f = fopen(filename, "wb");
  if (!F.f) return gev_fail(ctx, GEV_EINVAL, "gadget2_save: cannot open the file");
  // block layout and markers (Particles_gevolution.hpp:127-148); the markers are
  // uint32, as the reference writes them
  const long long hb = 256, idb = id_bytes;
  const long long o_pos = 3 * 4 + hb, o_vel = o_pos + 8 + 12 * S, o_id = o_vel + 8 + 12 * S;
  uint32_t m = (uint32_t)hb;
  bool ok = put(F.f, 0, &m, 4) && put(F.f, 4, hdr, 256) && put(F.f, 4 + hb, &m, 4);
  m = (uint32_t)(12ull * (unsigned long long)S);
  ok = ok && put(F.f, hb + 8, &m, 4) && put(F.f, o_vel - 8, &m, 4) && put(F.f, o_vel - 4, &m, 4) &&
       put(F.f, o_id - 8, &m, 4);
  m = (uint32_t)((unsigned long long)idb * (unsigned long long)S);
  ok = ok && put(F.f, o_id - 4, &m, 4) && put(F.f, o_id + idb * S, &m, 4);
  if (!ok) return gev_fail(ctx, GEV_EINVAL, "gadget2_save: write failed");
  if (S == 0) return GEV_OK;
  const G2Params g = g2_params(ctx, hdr->BoxSize, hdr->time, dtau_pos, dtau_vel, tracer_factor, exact_output, id_bytes);
  const long long cap = G2_BATCH;  // tracers per batch
  const size_t bpos = (size_t)cap * 12, bid = (size_t)cap * idb;
  DevBuf dpos(ctx), dvel(ctx), did(ctx), doff(ctx);
  HostBuf hbuf;
  GEV_CHECK_CUDA(ctx, cudaMallocAsync(&dpos.p, bpos, ctx->stream));
  GEV_CHECK_CUDA(ctx, cudaMallocAsync(&dvel.p, bpos, ctx->stream));
  GEV_CHECK_CUDA(ctx, cudaMallocAsync(&did.p, bid, ctx->stream));
  GEV_CHECK_CUDA(ctx, cudaMallocAsync(&doff.p, (size_t)(nch + 1) * sizeof(long long), ctx->stream));
  GEV_CHECK_CUDA(ctx, cudaMemcpyAsync(doff.p, off.data(), (size_t)(nch + 1) * sizeof(long long),
                                      cudaMemcpyHostToDevice, ctx->stream));
  GEV_CHECK_CUDA(ctx, cudaMallocHost(&hbuf.p, 2 * bpos + bid));
  char *hpos = (char *)hbuf.p, *hvel = hpos + bpos, *hid = hvel + bpos;
  long c0 = 0;
  while (c0 < nch) {
    // the longest run of chunks whose tracers fit the batch (a chunk holds at most
    // G2_CHUNK of them)
    long c1 = c0 + 1;
    while (c1 < nch && off[c1 + 1] - off[c0] <= cap) ++c1;
    const long long ob = off[c0], cnt = off[c1] - off[c0];
    if (cnt > 0) {
      const unsigned blocks = (unsigned)(c1 - c0);
      const long long *offp = (const long long *)doff.p + c0;
      if (ctx->prec == GEV_PREC_FP64)
        k_g2_pack<double, double><<<blocks, 256, 0, ctx->stream>>>(
            p->cur, n, c0, offp, ob, phi ? (const double *)phi->d : nullptr, g, (float *)dpos.p, (float *)dvel.p,
            (unsigned char *)did.p);
      else
        k_g2_pack<float, float><<<blocks, 256, 0, ctx->stream>>>(p->cur, n, c0, offp, ob,
                                                                 phi ? (const float *)phi->d : nullptr, g,
                                                                 (float *)dpos.p, (float *)dvel.p,
                                                                 (unsigned char *)did.p);
      GEV_LAUNCH_CHECK(ctx);
      GEV_CHECK_CUDA(ctx, cudaMemcpyAsync(hpos, dpos.p, cnt * 12, cudaMemcpyDeviceToHost, ctx->stream));
      GEV_CHECK_CUDA(ctx, cudaMemcpyAsync(hvel, dvel.p, cnt * 12, cudaMemcpyDeviceToHost, ctx->stream));
      GEV_CHECK_CUDA(ctx, cudaMemcpyAsync(hid, did.p, cnt * idb, cudaMemcpyDeviceToHost, ctx->stream));
      GEV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      if (!put(F.f, o_pos + 12 * ob, hpos, (size_t)cnt * 12) || !put(F.f, o_vel + 12 * ob, hvel, (size_t)cnt * 12) ||
          !put(F.f, o_id + idb * ob, hid, (size_t)(cnt * idb)))
        return gev_fail(ctx, GEV_EINVAL, "gadget2_save: write failed");
    }
    c0 = c1;
  }
  if (fflush(F.f) != 0) return gev_fail(ctx, GEV_EINVAL, "gadget2_save: write failed");
  return GEV_OK;
}

int gev_gadget2_load(gev_ctx *ctx, gev_pcls *p, const char *filename, gev_gadget2_header *hdr, int id_bytes) {
  if (!ctx || !p || p->ctx != ctx || !filename || !hdr || (id_bytes != 4 && id_bytes != 8))
    return gev_fail(ctx, GEV_EINVAL, "gadget2_load: bad arguments");
  File F;
  F.f = fopen(filename, "rb");
  if (!F.f) return gev_fail(ctx, GEV_EINVAL, "gadget2_load: cannot open the file");
  uint32_t m = 0;
  if (!get(F.f, 0, &m, 4) || m != 256u) return gev_fail(ctx, GEV_EINVAL, "gadget2_load: file type not recognized");
  if (!get(F.f, 4, hdr, 256)) return gev_fail(ctx, GEV_EINVAL, "gadget2_load: file truncated");
  const long long S = hdr->npart[1];
  if (p->n + S > p->cap) return gev_fail(ctx, GEV_EINVAL, "gadget2_load: the store has no room for the file");
  if (hdr->time <= 0. || hdr->BoxSize <= 0.) return gev_fail(ctx, GEV_EINVAL, "gadget2_load: bad header");
  // offsets as Particles_gevolution.hpp:610-612 computes them
  const long long o_pos = 256 + 3 * 4, o_vel = o_pos + 12 * S + 8, o_id = o_vel + o_vel - o_pos;
  const double rescale_vel = 1. / GEV_GADGET_VELOCITY_CONVERSION / sqrt(hdr->time);
  const double vfac = hdr->time / rescale_vel;
  const long long cap = G2_BATCH;
  DevBuf dpos(ctx), dvel(ctx), did(ctx), drec(ctx);
  HostBuf hbuf;
  const size_t bpos = (size_t)cap * 12, bid = (size_t)cap * id_bytes;
  if (S > 0) {
    GEV_CHECK_CUDA(ctx, cudaMallocAsync(&dpos.p, bpos, ctx->stream));
    GEV_CHECK_CUDA(ctx, cudaMallocAsync(&dvel.p, bpos, ctx->stream));
    GEV_CHECK_CUDA(ctx, cudaMallocAsync(&did.p, bid, ctx->stream));
    GEV_CHECK_CUDA(ctx, cudaMallocAsync(&drec.p, (size_t)cap * sizeof(gev_part), ctx->stream));
    GEV_CHECK_CUDA(ctx, cudaMallocHost(&hbuf.p, 2 * bpos + bid));
  }
  char *hpos = (char *)hbuf.p, *hvel = hpos + bpos, *hid = hvel + bpos;
  const long n0 = p->n;
  for (long long b0 = 0; b0 < S; b0 += cap) {
    const long long cnt = S - b0 < cap ? S - b0 : cap;
    if (!get(F.f, o_pos + 12 * b0, hpos, (size_t)cnt * 12) || !get(F.f, o_vel + 12 * b0, hvel, (size_t)cnt * 12) ||
        !get(F.f, o_id + id_bytes * b0, hid, (size_t)(cnt * id_bytes)))
      return gev_fail(ctx, GEV_EINVAL, "gadget2_load: file truncated");
    GEV_CHECK_CUDA(ctx, cudaMemcpyAsync(dpos.p, hpos, cnt * 12, cudaMemcpyHostToDevice, ctx->stream));
    GEV_CHECK_CUDA(ctx, cudaMemcpyAsync(dvel.p, hvel, cnt * 12, cudaMemcpyHostToDevice, ctx->stream));
    GEV_CHECK_CUDA(ctx, cudaMemcpyAsync(did.p, hid, cnt * id_bytes, cudaMemcpyHostToDevice, ctx->stream));
    k_g2_unpack<<<grid_for(ctx, (size_t)cnt, 256, 16), 256, 0, ctx->stream>>>(
        (const float *)dpos.p, (const float *)dvel.p, (const unsigned char *)did.p, cnt, hdr->BoxSize, vfac, id_bytes,
        (gev_part *)drec.p);
    GEV_LAUNCH_CHECK(ctx);
    int rc = pcls_unpack_at(ctx, p, (const gev_part *)drec.p, cnt, n0 + b0);
    if (rc) return rc;
    // the pinned batch buffers are refilled next: wait for their copies
    GEV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  }
  p->n = n0 + S;
  return pcls_relink(ctx, p);
}

int gev_checkpoint_info_read(const char *path, gev_checkpoint_info *info) {
  if (!path || !info) return GEV_EINVAL;
  File F;
  F.f = fopen(path, "rb");
  if (!F.f) return GEV_EINVAL;
  CkptHeader h;
  if (!get(F.f, 0, &h, sizeof(h)) || memcmp(h.magic, CKPT_MAGIC, 8) != 0 || h.version != 1u ||
      h.header_checksum != header_sum(h))
    return GEV_EINVAL;
  memset(info, 0, sizeof(*info));
  info->a = h.a;
  info->tau = h.tau;
  info->dtau = h.dtau;
  info->cycle = h.cycle;
  info->has_state = h.has_state;
  if (h.has_state) memcpy(&info->state, h.state, sizeof(gev_sim_state));
  info->numpcl = (long)h.numpcl;
  info->N = h.N;
  info->prec = h.prec;
  return GEV_OK;
}

// hibernate with an optional whole-simulation state and pending diagnostics
static int checkpoint_save(gev_ctx *ctx, const char *path, gev_pcls *p, const gev_field *phi, const gev_field *chi,
                           const gev_field *Bi, const gev_field *BiFT, double a, double tau, double dtau, int cycle,
                           const gev_sim_state *st, const double *diag) {
  if (!ctx || !path || !p || p->ctx != ctx || !field_shape(ctx, phi, GEV_FIELD_REAL, 1) ||
      !field_shape(ctx, chi, GEV_FIELD_REAL, 1) || (Bi && !field_shape(ctx, Bi, GEV_FIELD_REAL, 3)) ||
      (BiFT && !field_shape(ctx, BiFT, GEV_FIELD_SPECTRUM, 3)) || a <= 0.)
    return gev_fail(ctx, GEV_EINVAL, "checkpoint_save: bad arguments");
  int rc = pcls_id_order(ctx, p);
  if (rc) return rc;
  const int rb = ctx->prec == GEV_PREC_FP64 ? 8 : 4;
  CkptHeader h;
  memset(&h, 0, sizeof(h));
  memcpy(h.magic, CKPT_MAGIC, 8);
  h.version = 1;
  h.header_bytes = CKPT_HEADER_BYTES;
  h.N = ctx->N;
  h.prec = ctx->prec;
  h.elem_real = rb;
  h.numpcl = p->n;
  h.a = a;
  h.tau = tau;
  h.dtau = dtau;
  h.cycle = cycle;
  if (st) {
    h.has_state = 1;
    h.state_bytes = sizeof(gev_sim_state);
    memcpy(h.state, st, sizeof(gev_sim_state));
  }
  if (diag) memcpy(h.diag, diag, sizeof(h.diag));
  uint64_t o = CKPT_HEADER_BYTES;
  const uint64_t sizes[NSEC] = {(uint64_t)p->n * sizeof(gev_part), field_bytes(phi), field_bytes(chi),
                                Bi ? field_bytes(Bi) : 0, BiFT ? field_bytes(BiFT) : 0};
  for (int k = 0; k < NSEC; ++k) {
    h.sec[k].offset = sizes[k] ? o : 0;
    h.sec[k].bytes = sizes[k];
    o += sizes[k];
  }
  File F;
  F.f = fopen(path, "wb");
  if (!F.f) return gev_fail(ctx, GEV_EINVAL, "checkpoint_save: cannot open the file");
  DevBuf stage_d(ctx);
  HostBuf stage_h;
  GEV_CHECK_CUDA(ctx, cudaMallocAsync(&stage_d.p, STAGE_BYTES, ctx->stream));
  GEV_CHECK_CUDA(ctx, cudaMallocHost(&stage_h.p, STAGE_BYTES));
  // particles, as gev_part records in (cell, ID) order
  {
    Sum64 s;
    const long per = (long)(STAGE_BYTES / sizeof(gev_part));
    for (long i0 = 0; i0 < p->n; i0 += per) {
      const long cnt = p->n - i0 < per ? p->n - i0 : per;
      rc = pcls_pack_range(ctx, p, (gev_part *)stage_d.p, i0, cnt);
      if (rc) return rc;
      const size_t len = (size_t)cnt * sizeof(gev_part);
      GEV_CHECK_CUDA(ctx, cudaMemcpyAsync(stage_h.p, stage_d.p, len, cudaMemcpyDeviceToHost, ctx->stream));
      GEV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      s.add(stage_h.p, len);
      if (!put(F.f, (long long)(h.sec[SEC_PCLS].offset + (uint64_t)i0 * sizeof(gev_part)), stage_h.p, len))
        return gev_fail(ctx, GEV_EINVAL, "checkpoint_save: write failed");
    }
    h.sec[SEC_PCLS].checksum = s.acc;
  }
  const gev_field *fl[4] = {phi, chi, Bi, BiFT};
  for (int k = 0; k < 4; ++k) {
    const gev_field *f = fl[k];
    if (!f) continue;
    Sum64 s;
    // B is stored divided by a^2 N (hibernation.hpp:530-538)
    const double scale = (k == 2) ? a * a * (double)ctx->N : 0.;
    rc = write_device(ctx, F.f, (long long)h.sec[SEC_PHI + k].offset, f->d, field_bytes(f), stage_h.p, stage_d.p, s,
                      scale, rb);
    if (rc) return rc;
    h.sec[SEC_PHI + k].checksum = s.acc;
  }
  h.header_checksum = header_sum(h);
  std::vector<unsigned char> hb(CKPT_HEADER_BYTES, 0);
  memcpy(hb.data(), &h, sizeof(h));
  if (!put(F.f, 0, hb.data(), hb.size()) || fflush(F.f) != 0)
    return gev_fail(ctx, GEV_EINVAL, "checkpoint_save: write failed");
  return GEV_OK;
}

int gev_checkpoint_save(gev_ctx *ctx, const char *path, gev_pcls *p, const gev_field *phi, const gev_field *chi,
                        const gev_field *Bi, const gev_field *BiFT, double a, double tau, double dtau, int cycle,
                        const gev_sim_state *st) {
  return checkpoint_save(ctx, path, p, phi, chi, Bi, BiFT, a, tau, dtau, cycle, st, nullptr);
}

// reads one section through the host buffer without touching the device: true when
// all its bytes are there and match its checksum
static bool section_intact(FILE *f, const CkptSection &sec, void *buf, size_t bufbytes) {
  Sum64 s;
  for (uint64_t o = 0; o < sec.bytes; o += bufbytes) {
    const size_t len = (size_t)(sec.bytes - o < bufbytes ? sec.bytes - o : bufbytes);
    if (!get(f, (long long)(sec.offset + o), buf, len)) return false;
    s.add(buf, len);
  }
  return s.acc == sec.checksum;
}

static int checkpoint_load(gev_ctx *ctx, const char *path, gev_pcls *p, gev_field *phi, gev_field *chi, gev_field *Bi,
                           gev_field *BiFT, int flags, gev_checkpoint_info *info, double *diag) {
  if (!ctx || !path || (p && p->ctx != ctx) || (phi && !field_shape(ctx, phi, GEV_FIELD_REAL, 1)) ||
      (chi && !field_shape(ctx, chi, GEV_FIELD_REAL, 1)) || (Bi && !field_shape(ctx, Bi, GEV_FIELD_REAL, 3)) ||
      (BiFT && !field_shape(ctx, BiFT, GEV_FIELD_SPECTRUM, 3)))
    return gev_fail(ctx, GEV_EINVAL, "checkpoint_load: bad arguments");
  File F;
  F.f = fopen(path, "rb");
  if (!F.f) return gev_fail(ctx, GEV_EINVAL, "checkpoint_load: cannot open the file");
  CkptHeader h;
  if (!get(F.f, 0, &h, sizeof(h)) || memcmp(h.magic, CKPT_MAGIC, 8) != 0 || h.version != 1u)
    return gev_fail(ctx, GEV_EINVAL, "checkpoint_load: not a hibernation file");
  if (h.header_checksum != header_sum(h)) return gev_fail(ctx, GEV_EINVAL, "checkpoint_load: header damaged");
  if (h.N != ctx->N || h.prec != ctx->prec)
    return gev_fail(ctx, GEV_EINVAL, "checkpoint_load: grid size or precision form differs from the context's");
  if (p && h.numpcl > p->cap) return gev_fail(ctx, GEV_EINVAL, "checkpoint_load: the store has no room for the file");
  const int rb = h.elem_real;
  DevBuf stage_d(ctx);
  HostBuf stage_h;
  GEV_CHECK_CUDA(ctx, cudaMallocAsync(&stage_d.p, STAGE_BYTES, ctx->stream));
  GEV_CHECK_CUDA(ctx, cudaMallocHost(&stage_h.p, STAGE_BYTES));
  // every section this load reads is checked first, so that a damaged or truncated
  // file is refused before anything on the device is overwritten
  {
    bool ok = true;
    if (p) ok = h.sec[SEC_PCLS].bytes == h.numpcl * sizeof(gev_part) &&
                section_intact(F.f, h.sec[SEC_PCLS], stage_h.p, STAGE_BYTES);
    gev_field *fl0[3] = {phi, chi, Bi};
    for (int k = 0; ok && k < 3; ++k)
      if (fl0[k] && h.sec[SEC_PHI + k].bytes) ok = section_intact(F.f, h.sec[SEC_PHI + k], stage_h.p, STAGE_BYTES);
    if (ok && BiFT) {
      const bool from_b = h.sec[SEC_BIFT].bytes == 0 || (flags & GEV_CKPT_FROM_B);
      const CkptSection &sec = h.sec[from_b ? SEC_B : SEC_BIFT];
      if (sec.bytes) ok = section_intact(F.f, sec, stage_h.p, STAGE_BYTES);
    }
    if (!ok) return gev_fail(ctx, GEV_EINVAL, "checkpoint_load: file damaged or truncated (nothing was loaded)");
  }
  int rc;
  if (p) {
    Sum64 s;
    const long per = (long)(STAGE_BYTES / sizeof(gev_part));
    const long np = (long)h.numpcl;
    for (long i0 = 0; i0 < np; i0 += per) {
      const long cnt = np - i0 < per ? np - i0 : per;
      const size_t len = (size_t)cnt * sizeof(gev_part);
      if (!get(F.f, (long long)(h.sec[SEC_PCLS].offset + (uint64_t)i0 * sizeof(gev_part)), stage_h.p, len))
        return gev_fail(ctx, GEV_EINVAL, "checkpoint_load: file truncated");
      s.add(stage_h.p, len);
      GEV_CHECK_CUDA(ctx, cudaMemcpyAsync(stage_d.p, stage_h.p, len, cudaMemcpyHostToDevice, ctx->stream));
      rc = pcls_unpack_at(ctx, p, (const gev_part *)stage_d.p, cnt, i0);
      if (rc) return rc;
      GEV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    if (s.acc != h.sec[SEC_PCLS].checksum) return gev_fail(ctx, GEV_EINVAL, "checkpoint_load: particles damaged");
    p->n = np;
    rc = pcls_relink(ctx, p);
    if (rc) return rc;
  }
  gev_field *fl[3] = {phi, chi, Bi};
  for (int k = 0; k < 3; ++k) {
    gev_field *f = fl[k];
    if (!f) continue;
    const CkptSection &sec = h.sec[SEC_PHI + k];
    if (sec.bytes == 0 || sec.bytes != field_bytes(f))
      return gev_fail(ctx, GEV_EINVAL, "checkpoint_load: the file has no such field");
    Sum64 s;
    // readIC: B * a^2 / N^2 (ic_read.hpp:312-317; numpts * numpts is an int product)
    const double scale = (k == 2) ? h.a * h.a / (double)(ctx->N * ctx->N) : 0.;
    rc = read_device(ctx, F.f, (long long)sec.offset, f->d, field_bytes(f), stage_h.p, stage_d.p, s, scale, rb);
    if (rc) return rc;
    if (s.acc != sec.checksum) return gev_fail(ctx, GEV_EINVAL, "checkpoint_load: field damaged");
  }
  if (BiFT) {
    const CkptSection &sec = h.sec[SEC_BIFT];
    if (sec.bytes != 0 && !(flags & GEV_CKPT_FROM_B)) {
      if (sec.bytes != field_bytes(BiFT)) return gev_fail(ctx, GEV_EINVAL, "checkpoint_load: spectrum size differs");
      Sum64 s;
      rc = read_device(ctx, F.f, (long long)sec.offset, BiFT->d, field_bytes(BiFT), stage_h.p, stage_d.p, s, 0., rb);
      if (rc) return rc;
      if (s.acc != sec.checksum) return gev_fail(ctx, GEV_EINVAL, "checkpoint_load: spectrum damaged");
    } else {
      // plan_Bi->execute(FFT_FORWARD) of the rescaled B (ic_read.hpp:318)
      gev_field *tmp = Bi;
      if (!tmp) {
        rc = gev_field_create(ctx, GEV_FIELD_REAL, 3, &tmp);
        if (rc) return rc;
        const CkptSection &bs = h.sec[SEC_B];
        Sum64 s;
        rc = bs.bytes == field_bytes(tmp)
                 ? read_device(ctx, F.f, (long long)bs.offset, tmp->d, field_bytes(tmp), stage_h.p, stage_d.p, s,
                               h.a * h.a / (double)(ctx->N * ctx->N), rb)
                 : gev_fail(ctx, GEV_EINVAL, "checkpoint_load: the file holds neither BiFT nor B");
        if (!rc && s.acc != bs.checksum) rc = gev_fail(ctx, GEV_EINVAL, "checkpoint_load: field damaged");
        if (!rc) rc = gev_fft_r2c(ctx, tmp, BiFT);
        if (!rc && cudaStreamSynchronize(ctx->stream) != cudaSuccess)
          rc = gev_fail(ctx, GEV_ECUDA, "checkpoint_load: the transform of B failed");
        gev_field_destroy(tmp);
        if (rc) return rc;
      } else {
        if (h.sec[SEC_B].bytes == 0) return gev_fail(ctx, GEV_EINVAL, "checkpoint_load: the file holds neither BiFT nor B");
        rc = gev_fft_r2c(ctx, Bi, BiFT);
        if (rc) return rc;
      }
    }
  }
  if (info) {
    memset(info, 0, sizeof(*info));
    info->a = h.a;
    info->tau = h.tau;
    info->dtau = h.dtau;
    info->cycle = h.cycle;
    info->has_state = h.has_state;
    if (h.has_state) memcpy(&info->state, h.state, sizeof(gev_sim_state));
    info->numpcl = (long)h.numpcl;
    info->N = h.N;
    info->prec = h.prec;
  }
  if (diag) memcpy(diag, h.diag, sizeof(h.diag));
  GEV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return GEV_OK;
}

int gev_checkpoint_load(gev_ctx *ctx, const char *path, gev_pcls *p, gev_field *phi, gev_field *chi, gev_field *Bi,
                        gev_field *BiFT, int flags, gev_checkpoint_info *info) {
  return checkpoint_load(ctx, path, p, phi, chi, Bi, BiFT, flags, info, nullptr);
}

int gev_sim_hibernate(gev_sim *s, const char *path) {
  if (!s || !path) return GEV_EINVAL;
  GEV_CHECK_CUDA(s->ctx, cudaStreamSynchronize(s->ctx->stream));
  double diag[4] = {s->host_words[0], s->host_words[1], s->host_words[2], 0.};
  return checkpoint_save(s->ctx, path, s->pcls, s->phi, s->chi, s->Bi, s->BiFT, s->st.a, s->st.tau, s->st.dtau_old,
                         s->st.cycle, &s->st, diag);
}

int gev_sim_restart(gev_sim *s, const char *path, int flags) {
  if (!s || !path) return GEV_EINVAL;
  gev_checkpoint_info info;
  if (gev_checkpoint_info_read(path, &info) != GEV_OK)
    return gev_fail(s->ctx, GEV_EINVAL, "sim_restart: not a readable hibernation file");
  if (!info.has_state)
    return gev_fail(s->ctx, GEV_EINVAL, "sim_restart: the file holds no simulation state (use gev_checkpoint_load)");
  double diag[4];
  int rc = checkpoint_load(s->ctx, path, s->pcls, s->phi, s->chi, s->Bi, s->BiFT, flags, &info, diag);
  if (rc) return rc;
  s->st = info.state;
  s->pcls->mass = s->st.mass;
  memcpy(s->host_words, diag, 3 * sizeof(double));
  GEV_CHECK_CUDA(s->ctx, cudaMemcpyAsync(s->dev_words, diag, 3 * sizeof(double), cudaMemcpyHostToDevice,
                                         s->ctx->stream));
  GEV_CHECK_CUDA(s->ctx, cudaStreamSynchronize(s->ctx->stream));
  return GEV_OK;
}

}  // extern "C"
