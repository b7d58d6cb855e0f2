// gev_sim.cu -- one simulation's device state and the per-cycle driver that
// mirrors the body of gevolution's main loop (main.cpp:372-879) for CDM in GR
// mode: deposits, the phi / chi / B solves, the kick, the background half
// steps, the drift and the next time step.  The host keeps the FP64 scalar
// work (Hconf, the RK4 for a(tau), the dtau rule); everything per cell or per
// particle runs on the context's stream without a host synchronisation, so a
// cycle is a fixed launch sequence.  Diagnostics that the reference prints
// (T00hom, phi(k=0), max |v|) land in pinned host words and are read back only
// when the state is queried.
#include <cmath>
#include <cstring>

#include "gev_batch.cuh"

namespace {

double hconf(double a, double fourpiG, const gev_cosmology &c) {
  // background.hpp:137-140 without ncdm and fluid terms
  return sqrt((2. * fourpiG / 3.) * (((c.Omega_cdm + c.Omega_b) / a) + (c.Omega_Lambda * a * a) + (c.Omega_rad / a / a)));
}

void rk4bg(double &a, double fourpiG, const gev_cosmology &c, double dtau) {
  // background.hpp:167-177
  double k1a = a * hconf(a, fourpiG, c);
  double k2a = (a + k1a * dtau / 2.) * hconf(a + k1a * dtau / 2., fourpiG, c);
  double k3a = (a + k2a * dtau / 2.) * hconf(a + k2a * dtau / 2., fourpiG, c);
  double k4a = (a + k3a * dtau) * hconf(a + k3a * dtau, fourpiG, c);
  a += dtau * (k1a + 2. * k2a + 2. * k3a + k4a) / 6.;
}

// Fixed-order sum of a field component.  FP32 fields: 8 values (two 16-byte loads)
// added in a fixed FP32 tree, then one bit-built FP32 -> FP64 conversion and one
// FP64 add per 8 values (converting and adding every value in FP64 would issue two
// FP64-pipe instructions per cell on GB300).
template <typename T>
__device__ __forceinline__ void k_sum_to_body(const T *__restrict__ f, size_t n, double *partial) {
  __shared__ double sh[256];
  double s = 0.;
  if constexpr (sizeof(T) == 4) {
    const size_t n8 = n / 8;
    const float4 *f4 = reinterpret_cast<const float4 *>(f);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n8; i += (size_t)gridDim.x * blockDim.x) {
      const float4 a = f4[2 * i], b = f4[2 * i + 1];
      s += f2d_bits(((a.x + a.y) + (a.z + a.w)) + ((b.x + b.y) + (b.z + b.w)));
    }
    if (blockIdx.x == 0)
      for (size_t i = 8 * n8 + threadIdx.x; i < n; i += blockDim.x) s += f2d_bits((float)f[i]);
  } else {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
      s += (double)f[i];
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}
template <typename T>
__global__ void k_sum_to(const T *__restrict__ f, size_t n, double *partial) {
  k_sum_to_body<T>(f, n, partial);
}
__device__ __forceinline__ void k_sum_fin_body(const double *partial, int nb, double *out) {
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
__global__ void k_sum_fin(const double *partial, int nb, double *out) { k_sum_fin_body(partial, nb, out); }

#define RC(x)                 \
  do {                        \
    int rc_ = (x);            \
    if (rc_ != GEV_OK) return rc_; \
  } while (0)

int sum_async(gev_sim *s, const gev_field *f, double *dst_dev) {
  gev_ctx *ctx = s->ctx;
  const int nb = ctx->sms * 8;
  RC(ctx_ensure_red(ctx, (size_t)nb + 4));
  GevTimed tm_(ctx, "k_sum_to");
  if (ctx->prec == GEV_PREC_FP64)
    k_sum_to<double><<<nb, 256, 0, ctx->stream>>>((const double *)f->d, f->comp_elems, ctx->d_red);
  else
    gev_launch<k_sum_to_body<float>, 256, 1>(ctx, k_sum_to<float>, dim3(nb), dim3(256), 0, (const float *)f->d,
                                             f->comp_elems, ctx->d_red);
  GEV_LAUNCH_CHECK(ctx);
  gev_launch<k_sum_fin_body, 256, 1>(ctx, k_sum_fin, dim3(1), dim3(256), 0, (const double *)ctx->d_red, nb, dst_dev);
  GEV_LAUNCH_CHECK(ctx);
  return GEV_OK;
}

}  // namespace

__global__ void __launch_bounds__(256) k_zero4(uint32_t *p, size_t n4) { k_zero4_body(p, n4); }

int pcls_kick_drift_async(gev_ctx *ctx, gev_pcls *p, double dtau_k, double a_k, int nfield_k, double dtau_d,
                          double a_d, int nfield_d, const gev_field *phi, const gev_field *chi, const gev_field *Bi,
                          unsigned long long *maxbits_dev);

extern "C" {

int gev_sim_create(gev_ctx *ctx, long np, gev_sim **out) {
  if (!ctx || !out || np < 0) return gev_fail(ctx, GEV_EINVAL, "sim_create");
  gev_sim *s = new gev_sim();
  s->ctx = ctx;
  ctx_retain(ctx);
  int rc = gev_pcls_create(ctx, np, 0., &s->pcls);
  if (!rc) rc = gev_field_create(ctx, GEV_FIELD_REAL, 1, &s->phi);
  if (!rc) rc = gev_field_create(ctx, GEV_FIELD_REAL, 1, &s->chi);
  if (!rc) rc = gev_field_create(ctx, GEV_FIELD_REAL, 1, &s->source);
  if (!rc) rc = gev_field_create(ctx, GEV_FIELD_REAL, 6, &s->Sij);
  if (!rc) rc = gev_field_create(ctx, GEV_FIELD_REAL, 3, &s->Bi);
  if (!rc) rc = gev_field_create(ctx, GEV_FIELD_SPECTRUM, 1, &s->scalarFT);
  if (!rc) rc = gev_field_create(ctx, GEV_FIELD_SPECTRUM, 6, &s->SijFT);
  if (!rc) rc = gev_field_create(ctx, GEV_FIELD_SPECTRUM, 3, &s->BiFT);
  if (!rc && cudaMallocHost(&s->host_words, 4 * sizeof(double)) != cudaSuccess) rc = GEV_ENOMEM;
  if (!rc && cudaMalloc(&s->dev_words, 4 * sizeof(double)) != cudaSuccess) rc = GEV_ENOMEM;
  if (rc) {
    cudaGetLastError();
    gev_sim_destroy(s);
    return rc;
  }
  memset(s->host_words, 0, 4 * sizeof(double));
  cudaMemsetAsync(s->dev_words, 0, 4 * sizeof(double), ctx->stream);
  *out = s;
  return GEV_OK;
}

int gev_sim_destroy(gev_sim *s) {
  if (!s) return GEV_OK;
  if (s->ctx) cudaStreamSynchronize(s->ctx->stream);
  gev_pcls_destroy(s->pcls);
  gev_field_destroy(s->phi);
  gev_field_destroy(s->chi);
  gev_field_destroy(s->source);
  gev_field_destroy(s->Sij);
  gev_field_destroy(s->Bi);
  gev_field_destroy(s->scalarFT);
  gev_field_destroy(s->SijFT);
  gev_field_destroy(s->BiFT);
  if (s->host_words) cudaFreeHost(s->host_words);
  cudaFree(s->dev_words);
  if (s->gexec) cudaGraphExecDestroy(s->gexec);
  gev_ctx *ctx = s->ctx;
  delete s;
  if (ctx) ctx_release(ctx);
  return GEV_OK;
}

int gev_sim_field(gev_sim *s, int which, gev_field **out) {
  if (!s || !out) return GEV_EINVAL;
  gev_field *t[8] = {s->phi, s->chi, s->source, s->Sij, s->Bi, s->scalarFT, s->SijFT, s->BiFT};
  if (which < 0 || which > 7) return gev_fail(s->ctx, GEV_EINVAL, "sim_field: which in [0, 7]");
  *out = t[which];
  return GEV_OK;
}

int gev_sim_particles(gev_sim *s, gev_pcls **out) {
  if (!s || !out) return GEV_EINVAL;
  *out = s->pcls;
  return GEV_OK;
}

int gev_sim_set_state(gev_sim *s, const gev_sim_state *st) {
  if (!s || !st || st->a <= 0.) return GEV_EINVAL;
  s->st = *st;
  s->pcls->mass = st->mass;
  return GEV_OK;
}

int gev_sim_get_state(gev_sim *s, gev_sim_state *st) {
  if (!s || !st) return GEV_EINVAL;
  GEV_CHECK_CUDA(s->ctx, cudaStreamSynchronize(s->ctx->stream));
  const double V = (double)s->ctx->N * s->ctx->N * s->ctx->N;
  s->st.T00hom = s->host_words[0] / V;
  unsigned long long bits;
  memcpy(&bits, &s->host_words[1], sizeof(bits));
  double m2;
  memcpy(&m2, &bits, sizeof(m2));
  double mv = sqrt(m2);
  s->st.maxvel = mv / sqrt(mv * mv + 1.0);  // main.cpp:816-822
  s->st.phik0 = s->host_words[2];
  *st = s->st;
  return GEV_OK;
}

// the first part of a cycle, main.cpp:372-598: stress-energy, phi, chi and B
int gev_sim_step_fields(gev_sim *s) {
  if (!s) return GEV_EINVAL;
  gev_ctx *ctx = s->ctx;
  gev_sim_state &st = s->st;
  const int N = ctx->N;
  const double dx = 1.0 / (double)N;
  const double fourpiG = st.fourpiG;
  const double a = st.a;
  const gev_cosmology &cm = st.cosmo;

  // stress-energy (main.cpp:378-450)
  // (projection_init + projection_*: the target is replaced, not zeroed and re-read)
  // (T00 and Tij read the same particles and phi: one sweep deposits both)
  {
    GevTimed tm_(ctx, "phase:projections");
    RC(projection_replace_t00_tij(ctx, s->pcls, s->source, s->Sij, a, s->phi));
    if (st.vector_elliptic) RC(projection_replace(ctx, s->pcls, s->Bi, 1, 1., s->phi));
  }
  // the rest of this part is main.cpp's gravity solver time (main.cpp:454-602)
  GevTimed tm_solver(ctx, "phase:gravity solver");
  RC(sum_async(s, s->source, s->dev_words + 0));  // T00hom, main.cpp:459-463

  // phi (main.cpp:470-491)
  if (st.dtau_old > 0.) {
    const double H = hconf(a, fourpiG, cm);
    RC(gev_prepare_source_scalar(ctx, s->phi, s->chi, s->source, cm.Omega_cdm + cm.Omega_b, s->source,
                                 3. * H * dx * dx / st.dtau_old, fourpiG * dx * dx / a, 3. * H * H * dx * dx));
    RC(gev_fft_r2c(ctx, s->source, s->scalarFT));
    if (ctx->prec == GEV_PREC_FP64) {  // scalarFT keeps the potential: phi(k=0) is read from it below
      RC(gev_solve_poisson(ctx, s->scalarFT, s->scalarFT, 1. / (dx * dx), 3. * H / st.dtau_old));
      RC(gev_fft_c2r(ctx, s->scalarFT, s->phi));
    } else {  // the solve folded into the transform's first pass; scalarFT is scratch after it
      RC(gev_fft_c2r_poisson(ctx, s->scalarFT, s->phi, 1. / (dx * dx), 3. * H / st.dtau_old));
    }
  }
  // phi(k=0) for the background record (main.cpp:521-533)
  if (ctx->prec == GEV_PREC_FP64) {
    GEV_CHECK_CUDA(ctx, cudaMemcpyAsync(s->dev_words + 2, s->scalarFT->d, sizeof(double), cudaMemcpyDeviceToDevice,
                                        ctx->stream));
  }

  // chi (main.cpp:539-568)
  RC(gev_prepare_source_tensor(ctx, s->phi, s->Sij, s->Sij, 2. * fourpiG * dx * dx / a));
  RC(gev_fft_r2c(ctx, s->Sij, s->SijFT));
  if (st.vector_elliptic) {
    RC(gev_project_scalar(ctx, s->SijFT, s->scalarFT, 0));
    RC(gev_fft_c2r(ctx, s->scalarFT, s->chi));
    // B (main.cpp:570-598)
    RC(gev_fft_r2c(ctx, s->Bi, s->BiFT));
    RC(gev_project_vector(ctx, s->BiFT, s->BiFT, fourpiG * dx * dx, 0.));
  } else {
    // chi's projection and B's evolution (main.cpp:558, 586) share one read of SijFT;
    // neither c2r reads what the other's k-space step writes
    RC(gev_project_scalar_evolve_vector(ctx, s->SijFT, s->scalarFT, s->BiFT, a * a * st.dtau_old));
    RC(gev_fft_c2r(ctx, s->scalarFT, s->chi));
  }
  RC(gev_fft_c2r(ctx, s->BiFT, s->Bi));
  return GEV_OK;
}

// the rest of the cycle, main.cpp:743-872: kick, background half step, drift,
// background half step, next dtau.  Reads phi, chi and Bi only: the outputs the
// reference writes between the two parts (spectra, snapshots) may use every
// other field as scratch.
int gev_sim_step_particles(gev_sim *s) {
  if (!s) return GEV_EINVAL;
  gev_ctx *ctx = s->ctx;
  gev_sim_state &st = s->st;
  const int N = ctx->N;
  const double dx = 1.0 / (double)N;
  const double fourpiG = st.fourpiG;
  double a = st.a;
  const gev_cosmology &cm = st.cosmo;

  // particles (main.cpp:764-822): the kick at a, the background half step, the
  // drift at the new a -- the host runs the RK4 first so that one fused pass
  // does both particle updates, then the relink
  const double dtau = st.dtau;
  const double a_kick = a;
  const int nf_kick = 1. / a_kick < st.z_relax + 1. ? 3 : 2;
  rk4bg(a, fourpiG, cm, 0.5 * dtau);
  const int nf_drift = 1. / a < st.z_relax + 1. ? 3 : 0;
  {
    GevTimed tm_(ctx, "phase:update particles");
    RC(pcls_kick_drift_async(ctx, s->pcls, (dtau + st.dtau_old) / 2., a_kick, nf_kick, dtau, a, nf_drift, s->phi,
                             s->chi, s->Bi, (unsigned long long *)(s->dev_words + 1)));
  }
  rk4bg(a, fourpiG, cm, 0.5 * dtau);
  GEV_CHECK_CUDA(ctx, gev_d2h_async(ctx, s->host_words, s->dev_words, 4 * sizeof(double)));

  st.a = a;
  st.tau += dtau;
  st.dtau_old = dtau;
  const double H = hconf(a, fourpiG, cm);
  st.dtau = (st.Cf * dx < st.steplimit / H) ? st.Cf * dx : st.steplimit / H;  // main.cpp:869-872
  st.cycle++;
  return GEV_OK;
}

int gev_sim_step(gev_sim *s) {
  const int rc = gev_sim_step_fields(s);
  return rc ? rc : gev_sim_step_particles(s);
}

// The cycle of gev_sim_step as one CUDA graph.  The host runs the same code as
// gev_sim_step with the stream under capture (thread-local mode: other host threads
// keep driving their own streams), so the graph holds exactly the launches, copies
// and scalar arguments a direct cycle would enqueue.  From one cycle to the next
// the launch sequence keeps its shape and only scalar arguments and the particle
// arrays' halves change, so the simulation's executable graph is updated in place
// (cudaGraphExecUpdate) and instantiated again only when the shape changes.
// Direct cycles do what a cycle sets up on first use (the FFT tile tuner, the
// reduction and deposit scratch): the first two cycles of a run (the first has no
// phi solve) and every cycle with the per-kernel timers on.  A capture the runtime
// refuses leaves nothing enqueued; the host's side of the cycle (the background
// state, the particle arrays' halves) is put back and the cycle runs directly.
int gev_sim_step_graph(gev_sim *s) {
  if (!s) return GEV_EINVAL;
  gev_ctx *ctx = s->ctx;
  if (s->st.cycle < 2 || s->st.dtau_old <= 0. || ctx->timing) {
    s->graph_direct++;
    return gev_sim_step(s);
  }
  const gev_sim_state st0 = s->st;
  const PclsArrays cur0 = s->pcls->cur, alt0 = s->pcls->alt;
  auto direct = [&]() {
    cudaGetLastError();
    s->st = st0;
    s->pcls->cur = cur0;
    s->pcls->alt = alt0;
    s->graph_direct++;
    return gev_sim_step(s);
  };
  if (cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return direct();
  const int rc = gev_sim_step(s);
  cudaGraph_t g = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &g);
  if (rc != GEV_OK || ce != cudaSuccess || !g) {
    if (g) cudaGraphDestroy(g);
    return direct();
  }
  if (s->gexec) {
    cudaGraphExecUpdateResultInfo info;
    if (cudaGraphExecUpdate(s->gexec, g, &info) != cudaSuccess) {
      cudaGetLastError();
      cudaGraphExecDestroy(s->gexec);
      s->gexec = nullptr;
    }
  }
  if (!s->gexec) {
    if (cudaGraphInstantiate(&s->gexec, g, 0) != cudaSuccess) {
      s->gexec = nullptr;
      cudaGraphDestroy(g);
      return direct();
    }
    s->graph_builds++;
  }
  cudaGraphDestroy(g);
  if (cudaGraphLaunch(s->gexec, ctx->stream) != cudaSuccess) return direct();
  s->graph_launches++;
  return GEV_OK;
}

int gev_sim_graph_info(gev_sim *s, long *launches, long *builds, long *direct) {
  if (!s) return GEV_EINVAL;
  if (launches) *launches = s->graph_launches;
  if (builds) *builds = s->graph_builds;
  if (direct) *direct = s->graph_direct;
  return GEV_OK;
}

}  // extern "C"
