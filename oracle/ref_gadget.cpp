// ref_gadget.cpp -- gevolution 1.2's own Gadget-2 writer and reader
// (Particles_gevolution.hpp:30-251, 574-665) compiled against the single-rank
// LATfield2 and MPI-IO shims.  The Makefile compiles this file once per build
// variant of the reference: GEVREF_TAG names the exported functions, and
// EXACT_OUTPUT_REDSHIFTS / GADGET_ID_BYTES select the variant as the
// reference's own makefile flags would.
//
// TEST INFRASTRUCTURE ONLY (oracle/_ref): used to pin the restatement in
// gev_oracle.c and to make the golden Gadget-2 files under tests/golden/.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <list>
#include <set>
#include <string>

#include "LATfield2.hpp"
#include "mpi_io_shim.hpp"

using namespace std;
using namespace LATfield2;

#include "metadata.hpp"

#define GEVREF_CAT2(a, b) a##b
#define GEVREF_CAT(a, b) GEVREF_CAT2(a, b)
#define GEVREF_NS GEVREF_CAT(gevref_ns_, GEVREF_TAG)

namespace GEVREF_NS {
#include "Particles_gevolution.hpp"
}

extern "C" {

// particles in any order (the lists keep (cell, ID) order); phi: N^3 values, x
// fastest, or NULL; hdr: the 256-byte header
int GEVREF_CAT(gevref_gadget2_save_, GEVREF_TAG)(const char *fname, int N, long np, const gevo_part *src,
                                                  const double *phi, const void *hdr256, int tracer_factor,
                                                  double dtau_pos, double dtau_vel) {
  int box[3] = {N, N, N};
  Lattice lat;
  lat.initialize(3, box, 1);
  GEVREF_NS::Particles_gevolution<part_simple, part_simple_info, part_simple_dataType> pcls;
  part_simple_info info;
  memset(&info, 0, sizeof(info));
  part_simple_dataType dt;
  Real boxsize[3] = {1., 1., 1.};
  pcls.initialize(info, dt, &lat, boxsize);
  for (long i = 0; i < np; i++) {
    part_simple q;
    for (int l = 0; l < 3; l++) {
      q.pos[l] = src[i].pos[l];
      q.vel[l] = src[i].vel[l];
    }
    q.ID = (long)src[i].ID;
    pcls.addParticle_global(q);
  }
  Field<Real> f;
  f.initialize(lat, 1);
  if (phi) {
    Site x(lat);
    for (x.first(); x.test(); x.next())
      f(x) = phi[x.coord(0) + (size_t)N * (x.coord(1) + (size_t)N * x.coord(2))];
    f.updateHalo();
  }
  gadget2_header hdr;
  memcpy(&hdr, hdr256, sizeof(hdr));
  pcls.saveGadget2(string(fname), hdr, tracer_factor, dtau_pos, dtau_vel, phi ? &f : NULL);
  return 0;
}

// reads one file into a grid of N^3 cells; returns the particles in (cell, ID)
// order (at most cap of them) and the header
long GEVREF_CAT(gevref_gadget2_load_, GEVREF_TAG)(const char *fname, int N, gevo_part *dst, long cap, void *hdr256) {
  int box[3] = {N, N, N};
  Lattice lat;
  lat.initialize(3, box, 1);
  GEVREF_NS::Particles_gevolution<part_simple, part_simple_info, part_simple_dataType> pcls;
  part_simple_info info;
  memset(&info, 0, sizeof(info));
  part_simple_dataType dt;
  Real boxsize[3] = {1., 1., 1.};
  pcls.initialize(info, dt, &lat, boxsize);
  gadget2_header hdr;
  memset(&hdr, 0, sizeof(hdr));
  pcls.loadGadget2(string(fname), hdr);
  memcpy(hdr256, &hdr, sizeof(hdr));
  long n = 0;
  for (size_t c = 0; c < pcls.field_.cells_.size(); c++)
    for (std::list<part_simple>::iterator it = pcls.field_.cells_[c].parts.begin();
         it != pcls.field_.cells_[c].parts.end(); ++it) {
      if (n < cap) {
        for (int l = 0; l < 3; l++) {
          dst[n].pos[l] = it->pos[l];
          dst[n].vel[l] = it->vel[l];
        }
        dst[n].ID = it->ID;
      }
      n++;
    }
  return n;
}

}  // extern "C"
