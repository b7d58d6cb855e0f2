// gsl_integration.h -- stand-in for the one GSL routine background.hpp names.
// TEST INFRASTRUCTURE ONLY.  The harness never calls the quadratures that use it
// (bg_ncdm with num_ncdm = 0 returns before integrating; particleHorizon is not
// on the time-stepping path), so reaching it is an error.
#ifndef GEV_GSL_INTEGRATION_SHIM
#define GEV_GSL_INTEGRATION_SHIM
#include <cstdio>
#include <cstdlib>
struct gsl_function {
  double (*function)(double x, void *params);
  void *params;
};
inline int gsl_integration_qng(const gsl_function *, double, double, double, double, double *, double *, size_t *) {
  std::fprintf(stderr, "gsl_integration_qng is not available in the oracle shim\n");
  std::abort();
  return 0;
}
#endif
