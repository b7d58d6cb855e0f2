// gev_ic.cu -- initial conditions generated on the device, following the
// power-spectrum ("mPk") branch of generateIC_basic (ic_basic.hpp:1626-2259)
// for CDM with the baryons folded in, GR, no massive neutrinos:
//   1. Gaussian displacement potential in k-space (generateDisplacementField,
//      ic_basic.hpp:1089-1379) with the standard lattice-Laplacian kernel
//      (ic_basic.hpp:748-771) and the GR gauge factor (1 + 7.5 H^2 / k^2);
//      the modes come from a counter-based hash of (seed, mode index) -- each
//      mode is independent of launch shape -- and P(k) is the sigma8-normalised
//      BBKS spectrum grown to z_in;
//   2. the sc1 template (64 particles on a 4^3 cell-centred lattice) tiled N/4
//      times per axis (initializeParticlePositions, ic_basic.hpp:1400-1434),
//      displaced by the CIC forward-difference gradient of the potential
//      (displace_pcls_ic_basic, ic_basic.hpp:60-91);
//   3. phi from the mass deposit and solveModifiedPoissonFT, velocities from
//      -grad phi with the linear rescale, B and chi from the T0i / Tij deposits
//      (ic_basic.hpp:2176-2252), all through the hot-path kernels.
#include <cmath>
#include <cstring>

#include "gev_internal.cuh"

namespace {

constexpr double C_SPEED_OF_LIGHT = 2997.92458;  // metadata.hpp:98, units of 100 km/s

// sc1_crystal.dat: template particle i sits at offsets 0.125 + 0.25 * digit
// with digits x + 4y + 16z listed in file order
__constant__ int c_sc1[64] = {0,  16, 20, 4,  5,  21, 17, 1,  32, 48, 52, 36, 37, 53, 49, 33,
                              40, 56, 60, 44, 45, 61, 57, 41, 8,  24, 28, 12, 13, 29, 25, 9,
                              10, 26, 30, 14, 15, 31, 27, 11, 42, 58, 62, 46, 47, 63, 59, 43,
                              34, 50, 54, 38, 39, 55, 51, 35, 2,  18, 22, 6,  7,  23, 19, 3};

__host__ __device__ inline uint64_t hash64(uint64_t seed, uint64_t c) {
  uint64_t z = seed * 0x9E3779B97F4A7C15ull + c * 0xD1B54A32D192ED03ull + 0x632BE59BD9B4E019ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__host__ __device__ inline double u01(uint64_t h) { return (double)((h >> 11) + 1) * (1.0 / 9007199254740992.0); }

// BBKS transfer function (Bardeen, Bond, Kaiser & Szalay 1986, eq. G3)
__host__ __device__ inline double bbks(double k, double Gamma) {
  const double q = k / Gamma;
  if (q < 1e-12) return 1.0;
  const double t = 1. + 3.89 * q + pow(16.1 * q, 2) + pow(5.46 * q, 3) + pow(6.71 * q, 4);
  return log(1. + 2.34 * q) / (2.34 * q) * pow(t, -0.25);
}

struct ICK {
  int N, ksphere;
  uint64_t seed;
  double amp, Gamma, n_s, L, coeff;
};

template <typename T>
__global__ void k_ic_potential(typename CT<T>::C *pot, ICK p, const T *__restrict__ gk2_unused) {
  typedef typename CT<T>::C C;
  const int N = p.N, NH = N / 2 + 1, kmax = N / 2 - 1;
  const size_t n = (size_t)N * N * NH;
  for (size_t id = blockIdx.x * (size_t)blockDim.x + threadIdx.x; id < n; id += (size_t)gridDim.x * blockDim.x) {
    const long kx = (long)(id % NH), ky = (long)((id / NH) % N), kz = (long)(id / ((size_t)NH * N));
    const long sy = ky <= N / 2 ? ky : N - ky, sz = kz <= N / 2 ? kz : N - kz;
    const double n2 = (double)(kx * kx + sy * sy + sz * sz);
    double re = 0., im = 0.;
    if (id != 0 && kx < kmax && sy < kmax && sz < kmax && !(p.ksphere && n2 >= (double)kmax * kmax)) {
      const double k2 = n2 * 4. * M_PI * M_PI;
      const double kphys = sqrt(k2) / p.L;
      const double Tk = bbks(kphys, p.Gamma);
      const double P = p.amp * pow(kphys, p.n_s) * Tk * Tk;
      const double spl = sqrt(0.5 * P * p.L) / p.L / p.L;
      const double sx_ = kx ? sin(M_PI * (double)kx / N) * N / (M_PI * kx) : 1.;
      const double sy_ = sy ? sin(M_PI * (double)sy / N) * N / (M_PI * sy) : 1.;
      const double sz_ = sz ? sin(M_PI * (double)sz / N) * N / (M_PI * sz) : 1.;
      double g0 = 2. * (double)N * sin(M_PI * (double)kx / (double)N);
      double g1 = 2. * (double)N * sin(M_PI * (double)ky / (double)N);
      double g2 = 2. * (double)N * sin(M_PI * (double)kz / (double)N);
      const double kern = g0 * g0 + g1 * g1 + g2 * g2;
      const double r1 = u01(hash64(p.seed, 2 * (uint64_t)id)), r2 = u01(hash64(p.seed, 2 * (uint64_t)id + 1));
      const double m = (1. + 7.5 * p.coeff / k2) / kern * sqrt(-2. * log(r1)) * spl * (sx_ * sy_ * sz_);
      re = cos(2. * M_PI * r2) * m;
      im = sin(2. * M_PI * r2) * m;
    }
    pot[id] = cmk<C>((T)re, (T)im);
  }
}

// particles on the tiled sc1 template, in ID order
template <typename V>
__global__ void k_ic_lattice(PclsArrays P, int N) {
  const int nt = N / 4;
  const long n = (long)N * N * N;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const int j = (int)(i % 64);
    const long t = i / 64;
    const long xt = t % nt, yt = (t / nt) % nt, zt = t / ((long)nt * nt);
    const int d = c_sc1[j];
    const float ox = 0.125f + 0.25f * (float)(d & 3), oy = 0.125f + 0.25f * (float)((d >> 2) & 3),
                oz = 0.125f + 0.25f * (float)(d >> 4);
    P.px[i] = ((double)xt + (double)ox) / (double)nt;
    P.py[i] = ((double)yt + (double)oy) / (double)nt;
    P.pz[i] = ((double)zt + (double)oz) / (double)nt;
    ((V *)P.vx)[i] = (V)0;
    ((V *)P.vy)[i] = (V)0;
    ((V *)P.vz)[i] = (V)0;
    P.id[i] = i;
  }
}

template <typename T>
__device__ __forceinline__ T fv(const T *__restrict__ f, int x, int y, int z, int N) {
  return __ldg(&f[sidx(wrapi(x, N), wrapi(y, N), wrapi(z, N), N)]);
}

// CIC-weighted forward-difference gradient / dx at the particle (ic_basic.hpp:71-86)
template <typename T>
__device__ __forceinline__ void cic_grad(const T *__restrict__ f, int cx, int cy, int cz, double r0_, double r1_,
                                         double r2_, int N, double *g) {
  const T r0 = (T)r0_, r1 = (T)r1_, r2 = (T)r2_, s0 = (T)1 - r0, s1 = (T)1 - r1, s2 = (T)1 - r2;
  const T f000 = fv(f, cx, cy, cz, N), f100 = fv(f, cx + 1, cy, cz, N), f010 = fv(f, cx, cy + 1, cz, N),
          f110 = fv(f, cx + 1, cy + 1, cz, N), f001 = fv(f, cx, cy, cz + 1, N), f101 = fv(f, cx + 1, cy, cz + 1, N),
          f011 = fv(f, cx, cy + 1, cz + 1, N), f111 = fv(f, cx + 1, cy + 1, cz + 1, N);
  g[0] = (double)(s1 * s2 * (f100 - f000) + r1 * s2 * (f110 - f010) + s1 * r2 * (f101 - f001) + r1 * r2 * (f111 - f011)) * N;
  g[1] = (double)(s0 * s2 * (f010 - f000) + r0 * s2 * (f110 - f100) + s0 * r2 * (f011 - f001) + r0 * r2 * (f111 - f101)) * N;
  g[2] = (double)(s0 * s1 * (f001 - f000) + r0 * s1 * (f101 - f100) + s0 * r1 * (f011 - f010) + r0 * r1 * (f111 - f110)) * N;
}

__device__ __forceinline__ int cell1(double p, int N) {
  int c = (int)(p * (double)N);
  return c >= N ? N - 1 : (c < 0 ? 0 : c);
}
__device__ __forceinline__ double wrap01(double p) {
  if (p >= 1.0)
    p -= 1.0;
  else if (p < 0.0) {
    p += 1.0;
    if (p >= 1.0) p -= 1.0;
  }
  return p;
}

// displace_pcls_ic_basic (coeff 1), then wrap and re-key
template <typename T>
__global__ void k_ic_displace(PclsArrays P, long n, const T *__restrict__ chi, int N) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    double x = P.px[i], y = P.py[i], z = P.pz[i];
    const int cx = cell1(x, N), cy = cell1(y, N), cz = cell1(z, N);
    double g[3];
    cic_grad(chi, cx, cy, cz, x * N - cx, y * N - cy, z * N - cz, N, g);
    x = wrap01(x + g[0]);
    y = wrap01(y + g[1]);
    z = wrap01(z + g[2]);
    P.px[i] = x;
    P.py[i] = y;
    P.pz[i] = z;
    P.cell[i] = (uint32_t)cell1(x, N) + (uint32_t)N * ((uint32_t)cell1(y, N) + (uint32_t)N * (uint32_t)cell1(z, N));
    if (P.rx != nullptr) {  // mixed form: FP32 in-cell offsets, split the same way the drift splits
      const int lg = lg_pow2(N);
      int ax, ay, az;
      pos_split(x, N, lg, ax, P.rx[i]);
      pos_split(y, N, lg, ay, P.ry[i]);
      pos_split(z, N, lg, az, P.rz[i]);
      P.cell[i] = (uint32_t)ax + (uint32_t)N * ((uint32_t)ay + (uint32_t)N * (uint32_t)az);
    }
  }
}

// initialize_q_ic_basic (ic_basic.hpp:118-153): q = -grad(phi) * rescale
template <typename T, typename V>
__global__ void k_ic_velocity(PclsArrays P, long n, const T *__restrict__ phi, int N, double rescale,
                              unsigned long long *maxbits) {
  double vmax = 0.;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const uint32_t c = P.cell[i];
    const int cx = (int)(c % N), cy = (int)((c / N) % N), cz = (int)(c / ((uint32_t)N * N));
    double g[3];
    cic_grad(phi, cx, cy, cz, P.px[i] * N - cx, P.py[i] * N - cy, P.pz[i] * N - cz, N, g);
    const double q0 = -g[0] * rescale, q1 = -g[1] * rescale, q2 = -g[2] * rescale;
    ((V *)P.vx)[i] = (V)q0;
    ((V *)P.vy)[i] = (V)q1;
    ((V *)P.vz)[i] = (V)q2;
    vmax = fmax(vmax, q0 * q0 + q1 * q1 + q2 * q2);
  }
  for (int o = 16; o > 0; o >>= 1) vmax = fmax(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
  if ((threadIdx.x & 31) == 0) atomicMax(maxbits, (unsigned long long)__double_as_longlong(vmax));
}

// ------------------------------------------------------------- host side --
double growth(double a, double Om, double OL) {
  // Heath (1977): D ~ H(a) int_0^a da' / (a' H(a'))^3, Simpson in a
  const int n = 4000;
  double s = 0.;
  for (int i = 0; i <= n; i++) {
    double x = a * (double)i / n, f = 0.;
    if (x > 0.) f = 1. / pow(x * sqrt(Om / (x * x * x) + OL), 3);
    s += f * ((i == 0 || i == n) ? 1. : (i % 2 ? 4. : 2.));
  }
  return sqrt(Om / (a * a * a) + OL) * s * a / n / 3.;
}

double tophat(double x) { return x < 1e-4 ? 1. - x * x / 10. : 3. * (sin(x) - x * cos(x)) / (x * x * x); }

// sigma8-normalised BBKS amplitude at z_in: P(k) = amp k^n_s T(k)^2
double pk_amplitude(const gev_ic_params &ic) {
  const double Om = ic.Omega_cdm + ic.Omega_b, Gamma = Om * ic.h;
  const int n = 20000;
  const double lk0 = log(1e-5), lk1 = log(1e3);
  double s = 0.;
  for (int i = 0; i <= n; i++) {
    const double k = exp(lk0 + (lk1 - lk0) * i / n);
    const double T = bbks(k, Gamma), W = tophat(8. * k);
    s += k * k * k * pow(k, ic.n_s) * T * T * W * W * ((i == 0 || i == n) ? 1. : (i % 2 ? 4. : 2.));
  }
  s *= (lk1 - lk0) / n / 3. / (2. * M_PI * M_PI);
  const double g = growth(1. / (1. + ic.z_in), Om, 1. - Om) / growth(1., Om, 1. - Om);
  return ic.sigma8 * ic.sigma8 / s * g * g;
}

double hconf(double a, double fourpiG, const gev_cosmology &c) {
  return sqrt((2. * fourpiG / 3.) * (((c.Omega_cdm + c.Omega_b) / a) + (c.Omega_Lambda * a * a) + (c.Omega_rad / a / a)));
}

// particleHorizon (background.hpp:200-212), Simpson in s = sqrt(a)
double particle_horizon(double a, double fourpiG, const gev_cosmology &c) {
  const int n = 20000;
  const double s0 = sqrt(a) * 1.0e-7, s1 = sqrt(a);
  double s = 0.;
  for (int i = 0; i <= n; i++) {
    const double x = s0 + (s1 - s0) * i / n;
    s += 2. / (x * hconf(x * x, 1., c)) * ((i == 0 || i == n) ? 1. : (i % 2 ? 4. : 2.));
  }
  return s * (s1 - s0) / n / 3. / sqrt(fourpiG);
}

#define RC(x)                      \
  do {                             \
    int rc_ = (x);                 \
    if (rc_ != GEV_OK) return rc_; \
  } while (0)

template <typename T, typename V>
int ic_t(gev_sim *s, const gev_ic_params &ic) {
  typedef typename CT<T>::C C;
  gev_ctx *ctx = s->ctx;
  const int N = ctx->N;
  const long n = (long)N * N * N;
  gev_sim_state &st = s->st;
  st = gev_sim_state();
  st.cosmo.Omega_cdm = ic.Omega_cdm;
  st.cosmo.Omega_b = ic.Omega_b;
  st.cosmo.Omega_m = ic.Omega_cdm + ic.Omega_b;
  st.cosmo.Omega_rad = 0.;
  st.cosmo.Omega_Lambda = 1. - st.cosmo.Omega_m - st.cosmo.Omega_rad;
  const double L = ic.boxsize;
  st.fourpiG = 1.5 * L * L / C_SPEED_OF_LIGHT / C_SPEED_OF_LIGHT;
  const double a = 1. / (1. + ic.z_in), fourpiG = st.fourpiG;
  st.a = a;
  st.Cf = ic.Cf;
  st.steplimit = ic.steplimit;
  st.z_relax = ic.z_in;
  st.tau = particle_horizon(a, fourpiG, st.cosmo);
  const double H = hconf(a, fourpiG, st.cosmo), dx = 1.0 / N;
  st.dtau = (st.Cf * dx < st.steplimit / H) ? st.Cf * dx : st.steplimit / H;
  st.dtau_old = 0.;
  st.cycle = 0;
  st.mass = (st.cosmo.Omega_cdm + st.cosmo.Omega_b) / (double)n;
  st.vector_elliptic = 0;
  s->pcls->mass = st.mass;
  s->pcls->n = n;

  // 1. displacement potential
  ICK p{N, ic.ksphere, ic.seed, pk_amplitude(ic), st.cosmo.Omega_m * ic.h, ic.n_s, L, H * H};
  const size_t nk = (size_t)N * N * (N / 2 + 1);
  k_ic_potential<T><<<grid_for(ctx, nk, 256, 16), 256, 0, ctx->stream>>>((C *)s->scalarFT->d, p, nullptr);
  GEV_LAUNCH_CHECK(ctx);
  RC(gev_fft_c2r(ctx, s->scalarFT, s->chi));
  // 2. template particles, displaced, relinked
  const int pb = grid_for(ctx, (size_t)n, 256, 16);
  k_ic_lattice<V><<<pb, 256, 0, ctx->stream>>>(s->pcls->cur, N);
  GEV_LAUNCH_CHECK(ctx);
  k_ic_displace<T><<<pb, 256, 0, ctx->stream>>>(s->pcls->cur, n, (const T *)s->chi->d, N);
  GEV_LAUNCH_CHECK(ctx);
  RC(pcls_relink(ctx, s->pcls));
  // 3. phi from the mass deposit
  RC(gev_field_zero(s->source));
  RC(gev_projection_mass(ctx, s->pcls, s->source));
  RC(gev_fft_r2c(ctx, s->source, s->scalarFT));
  GEV_CHECK_CUDA(ctx, cudaMemsetAsync(s->scalarFT->d, 0, sizeof(C), ctx->stream));
  RC(gev_solve_poisson(ctx, s->scalarFT, s->scalarFT, fourpiG / a, 3. * (H * H + fourpiG * st.cosmo.Omega_m / a)));
  RC(gev_fft_c2r(ctx, s->scalarFT, s->phi));
  // velocities with the linear rescale (Omega_rad(a) = 0 here)
  const double Om_a = st.cosmo.Omega_m / ((st.cosmo.Omega_cdm + st.cosmo.Omega_b) + st.cosmo.Omega_Lambda * a * a * a);
  const double rescale = a / H / (1.5 * Om_a);
  GEV_CHECK_CUDA(ctx, cudaMemsetAsync(s->dev_words + 1, 0, sizeof(double), ctx->stream));
  k_ic_velocity<T, V><<<pb, 256, 0, ctx->stream>>>(s->pcls->cur, n, (const T *)s->phi->d, N, rescale,
                                                   (unsigned long long *)(s->dev_words + 1));
  GEV_LAUNCH_CHECK(ctx);
  // B
  RC(gev_field_zero(s->Bi));
  RC(gev_projection_T0i(ctx, s->pcls, s->Bi, s->phi, 1.));
  RC(gev_fft_r2c(ctx, s->Bi, s->BiFT));
  RC(gev_project_vector(ctx, s->BiFT, s->BiFT, fourpiG / (double)N / (double)N, 0.));
  RC(gev_fft_c2r(ctx, s->BiFT, s->Bi));
  // chi
  RC(gev_field_zero(s->Sij));
  RC(gev_projection_Tij(ctx, s->pcls, s->Sij, a, s->phi, 1.));
  RC(gev_prepare_source_tensor(ctx, s->phi, s->Sij, s->Sij, 2. * fourpiG / a / (double)N / (double)N));
  RC(gev_fft_r2c(ctx, s->Sij, s->SijFT));
  RC(gev_project_scalar(ctx, s->SijFT, s->scalarFT, 0));
  RC(gev_fft_c2r(ctx, s->scalarFT, s->chi));
  GEV_CHECK_CUDA(ctx, cudaMemcpyAsync(s->host_words, s->dev_words, 4 * sizeof(double), cudaMemcpyDeviceToHost,
                                      ctx->stream));
  GEV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  unsigned long long bits;
  memcpy(&bits, &s->host_words[1], 8);
  double m2;
  memcpy(&m2, &bits, 8);
  double mv = sqrt(m2) / a;
  st.maxvel = mv / sqrt(mv * mv + 1.0);
  return GEV_OK;
}

}  // namespace

extern "C" int gev_sim_ic_generate(gev_sim *s, const gev_ic_params *ic) {
  if (!s || !ic || s->ctx->N % 4 != 0 || ic->boxsize <= 0. || ic->z_in <= 0. || ic->sigma8 <= 0.)
    return gev_fail(s ? s->ctx : nullptr, GEV_EINVAL, "sim_ic_generate: N multiple of 4, positive box, z_in, sigma8");
  if (s->pcls->cap < (long)s->ctx->N * s->ctx->N * s->ctx->N)
    return gev_fail(s->ctx, GEV_EINVAL, "sim_ic_generate: particle capacity below N^3");
  return s->ctx->prec == GEV_PREC_FP64 ? ic_t<double, double>(s, *ic) : ic_t<float, float>(s, *ic);
}
