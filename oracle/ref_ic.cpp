// ref_ic.cpp -- gevolution 1.2's own generateDisplacementField (ic_basic.hpp:
// 1089-1379) and sitmo engine (prng_engine.hpp) compiled against the
// single-rank LATfield2, MPI-IO and GSL-spline shims.
//
// TEST INFRASTRUCTURE ONLY (oracle/_ref): pins the restatement of the random
// stream and of its layout over the k-space lines in gev_ic.c.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <set>
#include <string>

#include "LATfield2.hpp"
#include "mpi_io_shim.hpp"

using namespace std;
using namespace LATfield2;

#include "metadata.hpp"
#include "background.hpp"
#include "Particles_gevolution.hpp"
#include "gevolution.hpp"
#include "ic_basic.hpp"

extern "C" {

// draws [d0, d0 + n) of the engine seeded with seed
void gevref_sitmo_draws(unsigned seed, unsigned long long d0, long n, unsigned *out) {
  sitmo::prng_engine e;
  e.seed(seed);
  e.discard(d0);
  for (long i = 0; i < n; i++) out[i] = e();
}

// generateDisplacementField<0>(potFT, coeff, spline(x, y), seed, ksphere): F holds
// the kernel spectrum (N^2 (N/2+1) complex, kx fastest) on entry, the modes on return
void gevref_displacement_field(int N, double *F, double coeff, int n, const double *x, const double *y,
                               unsigned seed, int ksphere) {
  int box[3] = {N, N, N};
  Lattice lat, latFT;
  lat.initialize(3, box, 1);
  latFT.initializeRealFFT(lat, 0);
  Field<Cplx> pot;
  pot.initialize(latFT, 1);
  memcpy(pot.data_.data(), F, sizeof(Cplx) * pot.data_.size());
  gsl_spline *sp = gsl_spline_alloc(gsl_interp_cspline, n);
  gsl_spline_init(sp, x, y, n);
  generateDisplacementField(pot, coeff, sp, seed, ksphere);
  gsl_spline_free(sp);
  memcpy(F, pot.data_.data(), sizeof(Cplx) * pot.data_.size());
}

// generateCICKernel(ker, numpcl, pcldata, numtile): the kernel's N^3 values, x fastest
void gevref_cic_kernel(int N, long numpcl, const float *pcldata, int numtile, double *out) {
  int box[3] = {N, N, N};
  Lattice lat;
  lat.initialize(3, box, 1);
  Field<Real> ker;
  ker.initialize(lat, 1);
  generateCICKernel(ker, numpcl, (float *)pcldata, numtile);
  Site x(lat);
  for (x.first(); x.test(); x.next()) out[x.coord(0) + (size_t)N * (x.coord(1) + (size_t)N * x.coord(2))] = ker(x);
}

}  // extern "C"
