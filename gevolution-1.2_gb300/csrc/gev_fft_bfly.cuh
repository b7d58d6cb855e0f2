// gev_fft_bfly.cuh -- in-register radix-2/3/4/8 DFT butterflies shared by the
// FFT kernels (gev_fft.cu: mixed-radix, shared-memory staged; gev_fft_reg.cu:
// power-of-two, register resident).  SIGN = -1 forward (e^{-2 pi i jk / R}),
// +1 backward; outputs in natural order, v[q] = sum_r v[r] e^{SIGN 2 pi i r q / R}.
#pragma once

#include "gev_internal.cuh"

template <typename T, int SIGN>
struct Bfly {
  typedef typename CT<T>::C C;
  // multiply by SIGN * i
  static __device__ __forceinline__ C mi(C a) { return SIGN < 0 ? cmk<C>(a.y, -a.x) : cmk<C>(-a.y, a.x); }
  static __device__ __forceinline__ void r2(C *v) {
    C a = v[0];
    v[0] = cadd(a, v[1]);
    v[1] = csub(a, v[1]);
  }
  static __device__ __forceinline__ void r4(C *v) {
    C a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]), a2 = cadd(v[1], v[3]), a3 = mi(csub(v[1], v[3]));
    v[0] = cadd(a0, a2);
    v[2] = csub(a0, a2);
    v[1] = cadd(a1, a3);
    v[3] = csub(a1, a3);
  }
  static __device__ __forceinline__ void r8(C *v) {
    const T c = (T)0.707106781186547524400844362104849039;
    C b[4], d[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      b[r] = cadd(v[r], v[r + 4]);
      d[r] = csub(v[r], v[r + 4]);
    }
    // d[r] *= e^{SIGN 2 pi i r / 8}
    d[1] = cmk<C>(c * (d[1].x - (T)SIGN * d[1].y), c * (d[1].y + (T)SIGN * d[1].x));
    d[2] = mi(d[2]);
    d[3] = cmk<C>(c * (-d[3].x - (T)SIGN * d[3].y), c * ((T)SIGN * d[3].x - d[3].y));
    r4(b);
    r4(d);
    v[0] = b[0];
    v[2] = b[1];
    v[4] = b[2];
    v[6] = b[3];
    v[1] = d[0];
    v[3] = d[1];
    v[5] = d[2];
    v[7] = d[3];
  }
  static __device__ __forceinline__ void r3(C *v) {
    const T s = (T)0.866025403784438646763723170752936183;
    C t1 = cadd(v[1], v[2]);
    C t2 = csub(v[0], cscale((T)0.5, t1));
    C t3 = cscale(s, mi(csub(v[1], v[2])));
    v[0] = cadd(v[0], t1);
    v[1] = cadd(t2, t3);
    v[2] = csub(t2, t3);
  }
  template <int R>
  static __device__ __forceinline__ void run(C *v) {
    if (R == 2) r2(v);
    if (R == 3) r3(v);
    if (R == 4) r4(v);
    if (R == 8) r8(v);
  }
};
