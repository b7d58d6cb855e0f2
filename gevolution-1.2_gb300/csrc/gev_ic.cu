// gev_ic.cu -- initial conditions generated on the device, following the
// power-spectrum ("mPk") branch of generateIC_basic (ic_basic.hpp:1626-2259)
// for CDM with the baryons folded in, GR, no massive neutrinos:
//   1. Gaussian displacement potential in k-space: the CIC kernel
//      (generateCICKernel, ic_basic.hpp:737-1052; the sc1 template's with
//      `correct displacement`, else the lattice Laplacian) transformed forward,
//      then generateDisplacementField (ic_basic.hpp:1089-1379) with the GR gauge
//      factor (1 + 7.5 H^2 / k^2): the reference's sitmo stream (prng_engine.hpp)
//      laid over the k-space lines exactly as its discards lay it, one GPU thread
//      per (ky, kz) line, and the cubic spline of a tabulated sigma8-normalised
//      BBKS spectrum grown to z_in, read as the mPk branch reads a spectrum file;
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
#define GEV_SC1_DIGITS 0, 16, 20, 4, 5, 21, 17, 1, 32, 48, 52, 36, 37, 53, 49, 33, 40, 56, 60, 44, 45, 61, 57, 41, 8, 24, 28, 12, 13, 29, 25, 9, 10, 26, 30, 14, 15, 31, 27, 11, 42, 58, 62, 46, 47, 63, 59, 43, 34, 50, 54, 38, 39, 55, 51, 35, 2, 18, 22, 6, 7, 23, 19, 3
__constant__ int c_sc1[64] = {GEV_SC1_DIGITS};
const int sc1_digits[64] = {GEV_SC1_DIGITS};

// sitmo::prng_engine (prng_engine.hpp:88-230): draw d of the engine seeded with s
// is 32-bit half d & 1 (high) of word (d & 7) / 2 of block d / 8, a block being the
// Threefish-256 encryption (20 rounds, 5 key injections, the rotation constants of
// Skein 1.3) of the counter (d / 8, 0, 0, 0) under the key (s, 0, 0, 0)
__host__ __device__ inline uint64_t rotl64(uint64_t x, int r) { return (x << r) | (x >> (64 - r)); }
__host__ __device__ inline void sitmo_block(uint32_t seed, uint64_t block, uint64_t o[4]) {
  const int R[8][2] = {{14, 16}, {52, 57}, {23, 40}, {5, 37}, {25, 33}, {46, 12}, {58, 22}, {32, 32}};
  const uint64_t k[5] = {seed, 0, 0, 0, 0x1BD11BDAA9FC1A22ull ^ (uint64_t)seed};
  uint64_t b0 = block, b1 = 0, b2 = 0, b3 = 0;
#pragma unroll
  for (int r = 0; r < 20; ++r) {
    if (r % 4 == 0) {  // key injection r / 4
      const int s = r / 4;
      b0 += k[s % 5];
      b1 += k[(s + 1) % 5];
      b2 += k[(s + 2) % 5];
      b3 += k[(s + 3) % 5] + (uint64_t)s;
    }
    if (r % 2 == 0) {
      b0 += b1;
      b1 = rotl64(b1, R[r % 8][0]) ^ b0;
      b2 += b3;
      b3 = rotl64(b3, R[r % 8][1]) ^ b2;
    } else {
      b0 += b3;
      b3 = rotl64(b3, R[r % 8][0]) ^ b0;
      b2 += b1;
      b1 = rotl64(b1, R[r % 8][1]) ^ b2;
    }
  }
  o[0] = b0 + k[0];
  o[1] = b1 + k[1];
  o[2] = b2 + k[2];
  o[3] = b3 + k[3] + 5;
}

// BBKS transfer function (Bardeen, Bond, Kaiser & Szalay 1986, eq. G3)
__host__ __device__ inline double bbks(double k, double Gamma) {
  const double q = k / Gamma;
  if (q < 1e-12) return 1.0;
  const double t = 1. + 3.89 * q + pow(16.1 * q, 2) + pow(5.46 * q, 3) + pow(6.71 * q, 4);
  return log(1. + 2.34 * q) / (2.34 * q) * pow(t, -0.25);
}

// the 27 kernel values around the origin, K[(dx + 1) + 3 (dy + 1) + 9 (dz + 1)]
struct Stencil27 {
  double v[27];
};
template <typename T>
__global__ void k_ic_stencil(T *f, int N, Stencil27 K) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (int q = 0; q < 27; ++q) {  // += in index order: aliased cells (N = 2) add up
    const int dx = q % 3 - 1, dy = (q / 3) % 3 - 1, dz = q / 9 - 1;
    const size_t i = (size_t)((dx + N) % N) + (size_t)N * ((size_t)((dy + N) % N) + (size_t)N * (size_t)((dz + N) % N));
    f[i] = (T)((double)f[i] + K.v[q]);
  }
}

struct GdfParams {
  int N, kmax, ksphere, npk;
  uint32_t seed;
  double coeff, two_pi, four_pi2;
  const double *x, *y, *c;  // spline knots, values, half second derivatives
  const float *sinc;
  // the mixed form: the kernel spectrum as the DFT of its 27 values, in FP64 (an FP32
  // transform of the stencil, whose entries are O(N^2) while its spectrum near k = 0
  // is O(k^2), would lose the large scales); the FP64 form transforms the kernel field
  int dft;
  Stencil27 K;
};

__device__ inline double spline_eval(const GdfParams &p, double v) {
  int lo = 0, hi = p.npk - 1;
  while (hi > lo + 1) {
    const int mid = (lo + hi) / 2;
    if (p.x[mid] > v)
      hi = mid;
    else
      lo = mid;
  }
  const double h = __dsub_rn(p.x[lo + 1], p.x[lo]), t = __dsub_rn(v, p.x[lo]);
  const double ci = p.c[lo], cn = p.c[lo + 1];
  const double b = __dsub_rn(__ddiv_rn(__dsub_rn(p.y[lo + 1], p.y[lo]), h),
                             __ddiv_rn(__dmul_rn(h, __dadd_rn(cn, __dmul_rn(2.0, ci))), 3.0));
  const double d = __ddiv_rn(__dsub_rn(cn, ci), __dmul_rn(3.0, h));
  return __dadd_rn(p.y[lo], __dmul_rn(t, __dadd_rn(b, __dmul_rn(t, __dadd_rn(ci, __dmul_rn(t, d))))));
}

// the draws of one (ky, kz) line, read sequentially with the current block cached
struct SitmoCursor {
  uint32_t seed;
  uint64_t d, blk;
  uint64_t o[4];
  __device__ uint32_t next() {
    const uint64_t b = d >> 3;
    if (b != blk) {
      sitmo_block(seed, b, o);
      blk = b;
    }
    const uint64_t w = o[(d & 7) >> 1];
    const uint32_t r = (d & 1) ? (uint32_t)(w >> 32) : (uint32_t)w;
    ++d;
    return r;
  }
};

// generateDisplacementField<0> (ic_basic.hpp:1089-1379) on one rank: thread
// (ky, kz) walks its line in each quadrant pass that covers it -- A (ky, kz <=
// N/2), B (ky > N/2), C (kz > N/2, kx >= 1), D (both, kx >= 1), and the kx = 0
// modes of C and D from the lines of A and C, conjugated -- starting at the
// stream position the reference's discards give the line.  F holds the kernel
// spectrum on entry; modes are formed in FP64 with the reference's float
// and double types, every operation explicitly rounded.
template <typename T>
__global__ void __launch_bounds__(128) k_ic_modes(typename CT<T>::C *F, GdfParams p) {
  typedef typename CT<T>::C C;
  const int N = p.N, NH = N / 2 + 1;
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (t >= (long)N * N) return;
  const int ky = (int)(t % N), kz = (int)(t / N);
  const bool ylo = ky <= N / 2, zlo = kz <= N / 2;
  const int sy = ylo ? ky : N - ky, sz = zlo ? kz : N - kz;
  const uint64_t H = 65536;
  SitmoCursor cur;
  cur.seed = p.seed;
  cur.blk = ~0ull;
  // the line's factors e^{-2 pi i k d / N} for d = -1, 0, 1 along y and z (mixed form)
  double eyr[3] = {1., 1., 1.}, eyi[3] = {0., 0., 0.}, ezr[3] = {1., 1., 1.}, ezi[3] = {0., 0., 0.};
  if (p.dft) {
    double sy_, cy_, sz_, cz_;
    sincos(__ddiv_rn(__dmul_rn(p.two_pi, (double)ky), (double)N), &sy_, &cy_);
    sincos(__ddiv_rn(__dmul_rn(p.two_pi, (double)kz), (double)N), &sz_, &cz_);
    eyr[0] = cy_, eyi[0] = sy_, eyr[2] = cy_, eyi[2] = -sy_;
    ezr[0] = cz_, ezi[0] = sz_, ezr[2] = cz_, ezi[2] = -sz_;
  }
  auto walk = [&](uint64_t line, int kx0, int kx1, bool conj) {
    cur.d = line * H;
    for (int kx = kx0; kx <= kx1; ++kx) {
      C *f = F + (size_t)kx + (size_t)NH * ((size_t)ky + (size_t)N * (size_t)kz);
      const float k2 = __fadd_rn(__fadd_rn((float)(kx * kx), (float)(sy * sy)), (float)(sz * sz));
      if (kx >= p.kmax || sy >= p.kmax || sz >= p.kmax || (k2 >= (float)(p.kmax * p.kmax) && p.ksphere > 0)) {
        *f = cmk<C>((T)0, (T)0);
        continue;
      }
      const float s = __fmul_rn(__fmul_rn(p.sinc[kx], p.sinc[sy]), p.sinc[sz]);
      const float k2s = __double2float_rn(__dmul_rn((double)k2, p.four_pi2));
      uint32_t u1;
      float r1;
      do {
        u1 = cur.next();
        r1 = __fdiv_rn(__uint2float_rn(u1), 4294967296.0f);  // (float) u / (float) 0xFFFFFFFF
      } while (r1 == 0.f);
      const float r2 = __fdiv_rn(__uint2float_rn(cur.next()), 4294967296.0f);
      const double d1 = __dadd_rn(1., __ddiv_rn(__dmul_rn(7.5, p.coeff), (double)k2s));
      const double arg = __dmul_rn(p.two_pi, (double)r2);
      const double cr = cos(arg), sn = sin(arg);
      const double tr = __dmul_rn(cr, d1), ti = __dmul_rn(conj ? -sn : sn, d1);
      double Kr = (double)f->x, Ki = (double)f->y;
      if (p.dft) {  // sum over the stencil of K_d e^{-2 pi i k . d / N}
        double sx_, cx_;
        sincos(__ddiv_rn(__dmul_rn(p.two_pi, (double)kx), (double)N), &sx_, &cx_);
        const double exr[3] = {cx_, 1., cx_}, exi[3] = {sx_, 0., -sx_};
        Kr = 0.;
        Ki = 0.;
        for (int q = 0; q < 27; ++q) {
          const int a = q % 3, b = (q / 3) % 3, c = q / 9;
          const double yzr = __dsub_rn(__dmul_rn(eyr[b], ezr[c]), __dmul_rn(eyi[b], ezi[c]));
          const double yzi = __dadd_rn(__dmul_rn(eyr[b], ezi[c]), __dmul_rn(eyi[b], ezr[c]));
          const double er = __dsub_rn(__dmul_rn(exr[a], yzr), __dmul_rn(exi[a], yzi));
          const double ei = __dadd_rn(__dmul_rn(exr[a], yzi), __dmul_rn(exi[a], yzr));
          Kr = __dadd_rn(Kr, __dmul_rn(p.K.v[q], er));
          Ki = __dadd_rn(Ki, __dmul_rn(p.K.v[q], ei));
        }
      }
      const double nn = __dadd_rn(__dmul_rn(Kr, Kr), __dmul_rn(Ki, Ki));
      double qr = __ddiv_rn(__dadd_rn(__dmul_rn(tr, Kr), __dmul_rn(ti, Ki)), nn);
      double qi = __ddiv_rn(__dsub_rn(__dmul_rn(ti, Kr), __dmul_rn(tr, Ki)), nn);
      // log and sqrt of float arguments are <cmath>'s float overloads in the reference
      const float lg = __double2float_rn(log((double)r1));
      const double g = __dsqrt_rn(__dmul_rn(-2., (double)lg));
      const double sp = spline_eval(p, (double)__fsqrt_rn(k2s));
      qr = __dmul_rn(__dmul_rn(__dmul_rn(qr, g), sp), (double)s);
      qi = __dmul_rn(__dmul_rn(__dmul_rn(qi, g), sp), (double)s);
      *f = cmk<C>((T)qr, (T)qi);
    }
  };
  if (ylo && zlo) walk((uint64_t)kz * H + (uint64_t)ky, (ky == 0 && kz == 0) ? 1 : 0, N / 2, false);
  if (!ylo && zlo) walk((H + (uint64_t)kz) * H + (uint64_t)(N - ky), 0, N / 2, false);
  if (ylo && !zlo) {
    walk((2 * H + (uint64_t)(N - kz)) * H + (uint64_t)ky, 1, N / 2, false);
    walk((uint64_t)(N - kz) * H + (uint64_t)ky, 0, 0, true);
  }
  if (!ylo && !zlo) {
    walk((3 * H + (uint64_t)(N - kz)) * H + (uint64_t)(N - ky), 1, N / 2, false);
    walk((2 * H + (uint64_t)(N - kz)) * H + (uint64_t)(N - ky), 0, 0, true);
  }
  if (ky == 0 && kz == 0) F[0] = cmk<C>((T)0, (T)0);
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
  s *= a / n / 3.;
  return sqrt(Om / (a * a * a) + OL) * s;
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

// the tabulated spectrum the mPk branch reads (loadPowerSpectrum, ic_basic.hpp:343-471,
// and ic_basic.hpp:1679-1700): the BBKS P(k) [(Mpc/h)^3] at z_in on NPK log-spaced k
// [h/Mpc] covering every mode, as knots k L and values sqrt(P L / 2) / L^2
constexpr int NPK = 512;
void spline_knots(int N, const gev_ic_params &ic, double *x, double *y) {
  const double L = ic.boxsize, Om = ic.Omega_cdm + ic.Omega_b, amp = pk_amplitude(ic);
  const double lk0 = log(M_PI / L), lk1 = log(4. * M_PI * (double)N / L);
  for (int i = 0; i < NPK; i++) {
    const double k = exp(lk0 + (lk1 - lk0) * (double)i / (double)(NPK - 1));
    const double T = bbks(k, Om * ic.h);
    const double P = amp * pow(k, ic.n_s) * T * T;
    x[i] = k * L;
    y[i] = sqrt(0.5 * P * L);
    y[i] = y[i] / L / L;
  }
}

// gsl_interp_cspline: the natural cubic spline -- zero second derivative at both
// ends, the interior ones by elimination of the tridiagonal system; c holds half
// the second derivatives (the evaluation is spline_eval on the device)
void spline_init(int n, const double *x, const double *y, double *c) {
  for (int i = 0; i < n; i++) c[i] = 0.;
  if (n < 3) return;
  const int m = n - 2;
  std::vector<double> dg(m), of(m), rh(m);
  for (int i = 0; i < m; i++) {
    const double h0 = x[i + 1] - x[i], h1 = x[i + 2] - x[i + 1];
    dg[i] = 2.0 * (h0 + h1);
    of[i] = h1;
    rh[i] = 3.0 * ((y[i + 2] - y[i + 1]) / h1 - (y[i + 1] - y[i]) / h0);
  }
  for (int i = 1; i < m; i++) {
    const double w = of[i - 1] / dg[i - 1];
    dg[i] = dg[i] - w * of[i - 1];
    rh[i] = rh[i] - w * rh[i - 1];
  }
  c[m] = rh[m - 1] / dg[m - 1];
  for (int i = m - 1; i > 0; i--) c[i] = (rh[i - 1] - of[i - 1] * c[i + 1]) / dg[i - 1];
}

// generateCICKernel (ic_basic.hpp:737-1052) as the 27 values around the origin,
// K[(dx + 1) + 3 (dy + 1) + 9 (dz + 1)]: the lattice Laplacian, or (numpcl > 0) the
// kernel of the template particles pcl tiled numtile times, with the reference's
// float and double types term by term (this file builds with -ffp-contract=off)
void cic_kernel27(int N, long numpcl, const float *pcl, int numtile, double *K) {
  const long linesize = N;
  double renorm = (double)(linesize * linesize);
  for (int i = 0; i < 27; i++) K[i] = 0.;
  auto at = [&](int dx, int dy, int dz) -> double & { return K[(dx + 1) + 3 * (dy + 1) + 9 * (dz + 1)]; };
  if (numpcl == 0 || pcl == nullptr) {
    at(0, 0, 0) = 6. * renorm;
    at(1, 0, 0) = at(-1, 0, 0) = at(0, 1, 0) = at(0, 0, 1) = at(0, -1, 0) = at(0, 0, -1) = -renorm;
    return;
  }
  renorm /= (double)(numpcl * (long)numtile * (long)numtile * (long)numtile) / (double)(linesize * linesize * linesize);
  // octant o: per axis, measured from the far side (1 - p, step -1) or the near side (p, step +1)
  const int far[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
  for (long i = 0; i < numpcl; i++)
    for (int oct = 0; oct < 8; oct++) {
      float w[3];
      int sg[3];
      bool skip = false;
      for (int c = 0; c < 3; c++) {
        const float p = pcl[3 * i + c];
        if (far[oct][c]) {
          const double t = linesize * (1. - p) / numtile;  // double
          skip = skip || t >= 1.;
          w[c] = 1. - t;
          sg[c] = -1;
        } else {
          const float t = linesize * p / numtile;  // float
          skip = skip || t >= 1.;
          w[c] = 1. - t;
          sg[c] = 1;
        }
      }
      if (skip) continue;
      const float wx = w[0], wy = w[1], wz = w[2];
      const int sx = sg[0], sy = sg[1], sz = sg[2];
      float ww, q1;
      ww = wy * wz * renorm;  // 0-direction
      q1 = (wx > 0.9) ? 2. : 1.;
      at(0, 0, 0) += ww * wy * wz * q1;
      at(sx, 0, 0) -= ww * wy * wz;
      if (wx > 0.9) at(-sx, 0, 0) -= ww * wy * wz;
      at(0, 0, sz) += ww * wy * (1. - wz) * q1;
      at(sx, 0, sz) -= ww * wy * (1. - wz);
      if (wx > 0.9) at(-sx, 0, sz) -= ww * wy * (1. - wz);
      at(0, sy, 0) += ww * (1. - wy) * wz * q1;
      at(sx, sy, 0) -= ww * (1. - wy) * wz;
      if (wx > 0.9) at(-sx, sy, 0) -= ww * (1. - wy) * wz;
      at(0, sy, sz) += ww * (1. - wy) * (1. - wz) * q1;
      at(sx, sy, sz) -= ww * (1. - wy) * (1. - wz);
      if (wx > 0.9) at(-sx, sy, sz) -= ww * (1. - wy) * (1. - wz);
      ww = wx * wz * renorm;  // 1-direction
      q1 = (wy > 0.9) ? 2. : 1.;
      at(0, 0, 0) += ww * wx * wz * q1;
      at(sx, 0, 0) += ww * (1. - wx) * wz * q1;
      at(0, 0, sz) += ww * wx * (1. - wz) * q1;
      at(sx, 0, sz) += ww * (1. - wx) * (1. - wz) * q1;
      at(0, sy, 0) -= ww * wx * wz;
      at(sx, sy, 0) -= ww * (1. - wx) * wz;
      at(0, sy, sz) -= ww * wx * (1. - wz);
      at(sx, sy, sz) -= ww * (1. - wx) * (1. - wz);
      if (wy > 0.9) {
        at(0, -sy, 0) -= ww * wx * wz;
        at(sx, -sy, 0) -= ww * (1. - wx) * wz;
        at(0, -sy, sz) -= ww * wx * (1. - wz);
        at(sx, -sy, sz) -= ww * (1. - wx) * (1. - wz);
      }
      ww = wx * wy * renorm;  // 2-direction
      q1 = (wz > 0.9) ? 2. : 1.;
      at(0, 0, 0) += ww * wx * wy * q1;
      at(sx, 0, 0) += ww * (1. - wx) * wy * q1;
      at(0, sy, 0) += ww * wx * (1. - wy) * q1;
      at(sx, sy, 0) += ww * (1. - wx) * (1. - wy) * q1;
      at(0, 0, sz) -= ww * wx * wy;
      at(sx, 0, sz) -= ww * (1. - wx) * wy;
      at(0, sy, sz) -= ww * wx * (1. - wy);
      at(sx, sy, sz) -= ww * (1. - wx) * (1. - wy);
      if (wz > 0.9) {
        at(0, 0, -sz) -= ww * wx * wy;
        at(sx, 0, -sz) -= ww * (1. - wx) * wy;
        at(0, sy, -sz) -= ww * wx * (1. - wy);
        at(sx, sy, -sz) -= ww * (1. - wx) * (1. - wy);
      }
    }
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

  // 1. displacement potential: the kernel transformed forward (ic_basic.hpp:1670-1677)
  Stencil27 K;
  float pcl[192];
  for (int i = 0; i < 64; i++)
    for (int c = 0; c < 3; c++) pcl[3 * i + c] = 0.125f + 0.25f * (float)((sc1_digits[i] >> (2 * c)) & 3);
  if (ic.correct_displacement)
    cic_kernel27(N, 64, pcl, N / 4, K.v);
  else
    cic_kernel27(N, 0, nullptr, 1, K.v);
  RC(gev_field_zero(s->source));
  k_ic_stencil<T><<<1, 32, 0, ctx->stream>>>((T *)s->source->d, N, K);
  GEV_LAUNCH_CHECK(ctx);
  RC(gev_fft_r2c(ctx, s->source, s->scalarFT));
  // then generateDisplacementField over it, with the spline of the tabulated spectrum
  std::vector<double> tab(3 * NPK);
  spline_knots(N, ic, tab.data(), tab.data() + NPK);
  spline_init(NPK, tab.data(), tab.data() + NPK, tab.data() + 2 * NPK);
  std::vector<float> sinc(N);
  sinc[0] = 1.;
  for (int i = 1; i < N; i++) sinc[i] = sin(M_PI * (float)i / (float)N) * (float)N / (M_PI * (float)i);
  void *dtab = nullptr;
  GEV_CHECK_CUDA(ctx, cudaMallocAsync(&dtab, tab.size() * 8 + sinc.size() * 4, ctx->stream));
  GEV_CHECK_CUDA(ctx, cudaMemcpyAsync(dtab, tab.data(), tab.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
  GEV_CHECK_CUDA(ctx, cudaMemcpyAsync((char *)dtab + tab.size() * 8, sinc.data(), sinc.size() * 4,
                                      cudaMemcpyHostToDevice, ctx->stream));
  GdfParams gp;
  gp.N = N;
  gp.kmax = N / 2 - 1;
  gp.ksphere = ic.ksphere;
  gp.npk = NPK;
  gp.seed = (uint32_t)ic.seed;  // (unsigned int) ic.seed
  gp.coeff = H * H;             // gr_flag * Hconf^2
  gp.two_pi = 2. * M_PI;
  gp.four_pi2 = 4. * M_PI * M_PI;
  gp.x = (const double *)dtab;
  gp.y = gp.x + NPK;
  gp.c = gp.x + 2 * NPK;
  gp.sinc = (const float *)((const char *)dtab + tab.size() * 8);
  gp.dft = sizeof(T) == 4;
  gp.K = K;
  k_ic_modes<T><<<(unsigned)(((long)N * N + 127) / 128), 128, 0, ctx->stream>>>((C *)s->scalarFT->d, gp);
  GEV_LAUNCH_CHECK(ctx);
  GEV_CHECK_CUDA(ctx, cudaFreeAsync(dtab, ctx->stream));
  GEV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));  // the host tables above go out of scope
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
