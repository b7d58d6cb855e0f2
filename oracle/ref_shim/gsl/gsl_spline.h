// gsl_spline.h -- stand-in for the GSL cubic-spline calls ic_basic.hpp makes
// (gsl_spline_alloc / init / eval / free with gsl_interp_cspline, and an unused
// gsl_interp_accel).  TEST INFRASTRUCTURE ONLY.
//
// GSL itself is not part of this project.  The spline is the natural cubic
// spline that gsl_interp_cspline documents: second derivatives zero at both
// ends, the interior ones from the tridiagonal system
//   h_{i-1} M_{i-1} + 2 (h_{i-1} + h_i) M_i + h_i M_{i+1} = 6 (dy_i / h_i - dy_{i-1} / h_{i-1}),
// solved by forward elimination and back substitution, and on [x_i, x_{i+1}]
//   y = y_i + t (b_i + t (c_i + t d_i)),  t = x - x_i,  c_i = M_i / 2,
//   b_i = dy_i / h_i - h_i (c_{i+1} + 2 c_i) / 3,  d_i = (c_{i+1} - c_i) / (3 h_i).
// The interval is found by bisection.  The same steps, in the same order, are the
// library's own spline (the initial conditions, gev_ic.cu) and the oracle's
// (gev_ic.c), so the three agree bit for bit; that they agree with a particular
// GSL release to the last bit is not claimed.
#ifndef GEV_GSL_SPLINE_SHIM
#define GEV_GSL_SPLINE_SHIM
#include <cstddef>
#include <cstdlib>
#include <cstring>

struct gsl_interp_type {
  int kind;
};
static const gsl_interp_type gev_gsl_cspline_type = {1};
static const gsl_interp_type *gsl_interp_cspline = &gev_gsl_cspline_type;

struct gsl_interp_accel {
  size_t cache;
};
inline gsl_interp_accel *gsl_interp_accel_alloc() { return (gsl_interp_accel *)std::calloc(1, sizeof(gsl_interp_accel)); }
inline void gsl_interp_accel_free(gsl_interp_accel *a) { std::free(a); }

struct gsl_spline {
  double *x, *y, *c;  // c: half the second derivative at each knot
  size_t size;
};

inline gsl_spline *gsl_spline_alloc(const gsl_interp_type *, size_t size) {
  gsl_spline *s = (gsl_spline *)std::calloc(1, sizeof(gsl_spline));
  s->size = size;
  s->x = (double *)std::calloc(size, sizeof(double));
  s->y = (double *)std::calloc(size, sizeof(double));
  s->c = (double *)std::calloc(size, sizeof(double));
  return s;
}
inline void gsl_spline_free(gsl_spline *s) {
  if (!s) return;
  std::free(s->x);
  std::free(s->y);
  std::free(s->c);
  std::free(s);
}

inline int gsl_spline_init(gsl_spline *s, const double *x, const double *y, size_t n) {
  std::memcpy(s->x, x, n * sizeof(double));
  std::memcpy(s->y, y, n * sizeof(double));
  for (size_t i = 0; i < n; i++) s->c[i] = 0.;
  if (n < 3) return 0;
  const size_t m = n - 2;  // unknowns c_1 .. c_{n-2}
  double *diag = (double *)std::malloc(m * sizeof(double)), *off = (double *)std::malloc(m * sizeof(double));
  double *rhs = (double *)std::malloc(m * sizeof(double));
  for (size_t i = 0; i < m; i++) {
    const double h0 = x[i + 1] - x[i], h1 = x[i + 2] - x[i + 1];
    diag[i] = 2.0 * (h0 + h1);
    off[i] = h1;
    rhs[i] = 3.0 * ((y[i + 2] - y[i + 1]) / h1 - (y[i + 1] - y[i]) / h0);
  }
  for (size_t i = 1; i < m; i++) {  // forward elimination
    const double w = off[i - 1] / diag[i - 1];
    diag[i] = diag[i] - w * off[i - 1];
    rhs[i] = rhs[i] - w * rhs[i - 1];
  }
  s->c[m] = rhs[m - 1] / diag[m - 1];
  for (size_t i = m - 1; i > 0; i--) s->c[i] = (rhs[i - 1] - off[i - 1] * s->c[i + 1]) / diag[i - 1];
  std::free(diag);
  std::free(off);
  std::free(rhs);
  return 0;
}

inline double gsl_spline_eval(const gsl_spline *s, double x, gsl_interp_accel *) {
  size_t lo = 0, hi = s->size - 1;
  while (hi > lo + 1) {
    const size_t mid = (lo + hi) / 2;
    if (s->x[mid] > x)
      hi = mid;
    else
      lo = mid;
  }
  const double h = s->x[lo + 1] - s->x[lo], t = x - s->x[lo];
  const double ci = s->c[lo], cn = s->c[lo + 1];
  const double b = (s->y[lo + 1] - s->y[lo]) / h - h * (cn + 2.0 * ci) / 3.0;
  const double d = (cn - ci) / (3.0 * h);
  return s->y[lo] + t * (b + t * (ci + t * d));
}
#endif
