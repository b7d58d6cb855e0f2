// ref_tools.cpp -- gevolution 1.2's own power-spectrum code (tools.hpp:53-345:
// extractCrossSpectrum, extractPowerSpectrum, writePowerSpectrum) compiled
// against the single-rank LATfield2 shim.  The Makefile compiles it twice:
// GEVREF_TAG names the exported writer, and EXACT_OUTPUT_REDSHIFTS selects
// the writer's interpolating variant as the reference's makefile flag would.
//
// TEST INFRASTRUCTURE ONLY (oracle/_ref): pins the restatements in
// gev_ic.c (gevo_power_spectrum) and gev_io.c (gevo_write_power_spectrum).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <iostream>

#include "LATfield2.hpp"
#include "mpi_io_shim.hpp"

using namespace std;
using namespace LATfield2;

#include "metadata.hpp"

#define GEVREF_CAT2(a, b) a##b
#define GEVREF_CAT(a, b) GEVREF_CAT2(a, b)
#define GEVREF_NS GEVREF_CAT(gevref_tools_ns_, GEVREF_TAG)

namespace GEVREF_NS {
#include "tools.hpp"
}

extern "C" {

#ifndef EXACT_OUTPUT_REDSHIFTS
// extractCrossSpectrum of two spectra of N^2 (N/2+1) complex per component
// (component-major, kx fastest); ncomp 1, 3 or 6 (6: symmetric tensor)
void gevref_cross_spectrum(int N, const double *f1, const double *f2, int ncomp, int numbins, int deconvolve,
                           int ktype, int comp1, int comp2, double *kbin, double *power, double *kscatter,
                           double *pscatter, int *occupation) {
  int box[3] = {N, N, N};
  Lattice lat, latFT;
  lat.initialize(3, box, 1);
  latFT.initializeRealFFT(lat, 0);
  Field<Cplx> a, b;
  if (ncomp == 6) {
    a.initialize(latFT, 3, 3, symmetric);
    b.initialize(latFT, 3, 3, symmetric);
  } else {
    a.initialize(latFT, ncomp);
    b.initialize(latFT, ncomp);
  }
  memcpy(a.data_.data(), f1, sizeof(Cplx) * a.data_.size());
  memcpy(b.data_.data(), f2, sizeof(Cplx) * b.data_.size());
  GEVREF_NS::extractCrossSpectrum(a, b, kbin, power, kscatter, pscatter, occupation, numbins, deconvolve != 0, ktype,
                                  comp1, comp2);
}
#endif

void GEVREF_CAT(gevref_write_power_spectrum_, GEVREF_TAG)(double *kbin, double *power, double *kscatter,
                                                          double *pscatter, int *occupation, int numbins,
                                                          double rescalek, double rescalep, const char *filename,
                                                          const char *description, double a, double z_target) {
  GEVREF_NS::writePowerSpectrum(kbin, power, kscatter, pscatter, occupation, numbins, rescalek, rescalep, filename,
                                description, a, z_target);
}

}  // extern "C"
