// main_loop_gpu.cpp -- the GR body of gevolution's main loop (main.cpp:372-879,
// CDM only, parabolic B, no outputs) written against gevolution_gpu.hpp with
// the reference's own call sequence and names, so that the drop-in surface is
// exercised from C++ exactly as main.cpp would call it.
//
//   main_loop_gpu <state.bin> <steps> <out.bin> [<snapshot> <hibernation> <boxsize>]
//
// state.bin: int32 N, int32 pad, then doubles a, tau, dtau, dtau_old, fourpiG,
// Cf, steplimit, z_relax, mass, Omega_cdm, Omega_b, Omega_Lambda, Omega_rad,
// then N^3 gev_part records, phi (N^3), chi (N^3), Bi (3 N^3) and BiFT
// (3 N^2 (N/2+1) complex).  out.bin: a, then the N^3 particle records.  With
// the optional arguments the run ends as an output cycle would: a Gadget-2
// snapshot (header filled as output.hpp:362-403 fills it) and a hibernation point.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../gevolution-1.2_gb300/host/gevolution_gpu.hpp"

using namespace gevgpu;

struct Cosmo {
  double Omega_cdm, Omega_b, Omega_Lambda, Omega_rad;
};

// background.hpp:137-177 (no ncdm, no fluid)
static double Hconf(double a, double fourpiG, const Cosmo &c) {
  return sqrt((2. * fourpiG / 3.) * (((c.Omega_cdm + c.Omega_b) / a) + (c.Omega_Lambda * a * a) + (c.Omega_rad / a / a)));
}
static void rungekutta4bg(double &a, double fourpiG, const Cosmo &c, double dtau) {
  double k1a = a * Hconf(a, fourpiG, c);
  double k2a = (a + k1a * dtau / 2.) * Hconf(a + k1a * dtau / 2., fourpiG, c);
  double k3a = (a + k2a * dtau / 2.) * Hconf(a + k2a * dtau / 2., fourpiG, c);
  double k4a = (a + k3a * dtau) * Hconf(a + k3a * dtau, fourpiG, c);
  a += dtau * (k1a + 2. * k2a + 2. * k3a + k4a) / 6.;
}

int main(int argc, char **argv) {
  if (argc != 4 && argc != 7) {
    std::fprintf(stderr, "usage: %s state.bin steps out.bin [snapshot hibernation boxsize]\n", argv[0]);
    return 2;
  }
  FILE *in = std::fopen(argv[1], "rb");
  if (!in) return 2;
  int hdr[2];
  double sc[13];
  if (std::fread(hdr, 4, 2, in) != 2 || std::fread(sc, 8, 13, in) != 13) return 2;
  const int N = hdr[0];
  const long V = (long)N * N * N, K = (long)N * N * (N / 2 + 1);
  std::vector<gev_part> parts(V);
  std::vector<double> hphi(V), hchi(V), hB(3 * V), hBFT(6 * K);
  if (std::fread(parts.data(), sizeof(gev_part), V, in) != (size_t)V || std::fread(hphi.data(), 8, V, in) != (size_t)V ||
      std::fread(hchi.data(), 8, V, in) != (size_t)V || std::fread(hB.data(), 8, 3 * V, in) != (size_t)(3 * V) ||
      std::fread(hBFT.data(), 8, 6 * K, in) != (size_t)(6 * K))
    return 2;
  std::fclose(in);
  double a = sc[0], tau = sc[1], dtau = sc[2], dtau_old = sc[3], fourpiG = sc[4];
  const double Cf = sc[5], steplimit = sc[6], z_relax = sc[7], mass = sc[8];
  const Cosmo cosmo{sc[9], sc[10], sc[11], sc[12]};
  const int steps = std::atoi(argv[2]);

  // main.cpp:213-246
  int box[3] = {N, N, N};
  Lattice lat(3, box, 1);
  Lattice latFT;
  latFT.initializeRealFFT(lat, 0);
  Particles<> pcls_cdm;
  part_simple_info info{mass};
  Real boxSize[3] = {1., 1., 1.};
  pcls_cdm.initialize(info, part_simple_dataType(), &lat, boxSize, V);
  pcls_cdm.upload(parts.data(), V);
  Field<Real> phi, source, chi, Sij, Bi;
  Field<Cplx> scalarFT, SijFT, BiFT;
  source.initialize(lat, 1);
  phi.initialize(lat, 1);
  chi.initialize(lat, 1);
  scalarFT.initialize(latFT, 1);
  PlanFFT<Cplx> plan_source(&source, &scalarFT);
  PlanFFT<Cplx> plan_phi(&phi, &scalarFT);
  PlanFFT<Cplx> plan_chi(&chi, &scalarFT);
  Sij.initialize(lat, 3, 3, symmetric);
  SijFT.initialize(latFT, 3, 3, symmetric);
  PlanFFT<Cplx> plan_Sij(&Sij, &SijFT);
  Bi.initialize(lat, 3);
  BiFT.initialize(latFT, 3);
  PlanFFT<Cplx> plan_Bi(&Bi, &BiFT);
  phi.upload(hphi.data());
  chi.upload(hchi.data());
  Bi.upload(hB.data());
  BiFT.upload(hBFT.data());
  Field<Real> *update_cdm_fields[3] = {&phi, &chi, &Bi};
  double f_params[5];
  const double dx = 1.0 / (double)N;
  double maxvel = 0.;

  int cycle = 0;
  for (; cycle < steps; ++cycle) {
    projection_init(&source);
    projection_T00_project(&pcls_cdm, &source, a, &phi);
    projection_T00_comm(&source);
    projection_init(&Sij);
    projection_Tij_project(&pcls_cdm, &Sij, a, &phi);
    projection_Tij_comm(&Sij);
    if (dtau_old > 0.) {
      prepareFTsource<Real>(phi, chi, source, cosmo.Omega_cdm + cosmo.Omega_b, source,
                            3. * Hconf(a, fourpiG, cosmo) * dx * dx / dtau_old, fourpiG * dx * dx / a,
                            3. * Hconf(a, fourpiG, cosmo) * Hconf(a, fourpiG, cosmo) * dx * dx);
      plan_source.execute(FFT_FORWARD);
      solveModifiedPoissonFT(scalarFT, scalarFT, 1. / (dx * dx), 3. * Hconf(a, fourpiG, cosmo) / dtau_old);
      plan_phi.execute(FFT_BACKWARD);
    }
    phi.updateHalo();
    prepareFTsource<Real>(phi, Sij, Sij, 2. * fourpiG * dx * dx / a);
    plan_Sij.execute(FFT_FORWARD);
    projectFTscalar(SijFT, scalarFT);
    plan_chi.execute(FFT_BACKWARD);
    chi.updateHalo();
    evolveFTvector(SijFT, BiFT, a * a * dtau_old);
    plan_Bi.execute(FFT_BACKWARD);
    Bi.updateHalo();
    f_params[0] = a;
    f_params[1] = a * a * N;
    maxvel = pcls_cdm.updateVel(update_q, (dtau + dtau_old) / 2., update_cdm_fields, (1. / a < z_relax + 1. ? 3 : 2),
                                f_params);
    rungekutta4bg(a, fourpiG, cosmo, 0.5 * dtau);
    f_params[0] = a;
    f_params[1] = a * a * N;
    pcls_cdm.moveParticles(update_pos, dtau, update_cdm_fields, (1. / a < z_relax + 1. ? 3 : 0), f_params);
    rungekutta4bg(a, fourpiG, cosmo, 0.5 * dtau);
    maxvel /= sqrt(maxvel * maxvel + 1.0);
    tau += dtau;
    dtau_old = dtau;
    if (Cf * dx < steplimit / Hconf(a, fourpiG, cosmo))
      dtau = Cf * dx;
    else
      dtau = steplimit / Hconf(a, fourpiG, cosmo);
  }
  if (argc == 7) {
    const double boxsize = std::atof(argv[6]);
    gadget2_header hdr;
    std::memset(&hdr, 0, sizeof(hdr));
    hdr.num_files = 1;
    hdr.Omega0 = cosmo.Omega_cdm + cosmo.Omega_b;
    hdr.OmegaLambda = cosmo.Omega_Lambda;
    hdr.HubbleParam = 0.67;
    hdr.BoxSize = boxsize / GADGET_LENGTH_CONVERSION;
    hdr.time = a;
    hdr.redshift = (1. / a) - 1.;
    hdr.npart[1] = (uint32_t)V;
    hdr.npartTotal[1] = hdr.npart[1];
    hdr.mass[1] = 2.77459457e11 * (cosmo.Omega_cdm + cosmo.Omega_b) * boxsize * boxsize * boxsize / V /
                  GADGET_MASS_CONVERSION;
    pcls_cdm.saveGadget2(argv[4], hdr, 1);
    // main.cpp:845: hibernate(..., a, tau, dtau, cycle) with the step just taken
    hibernate(argv[5], &pcls_cdm, phi, chi, Bi, a, tau, dtau_old, cycle, &BiFT);
  }
  pcls_cdm.download(parts.data());
  // the power spectrum of B (output.hpp's Pk output path calls extractPowerSpectrum)
  const int numbins = 8;
  std::vector<Real> kbin(numbins), power(numbins), kscatter(numbins), pscatter(numbins);
  std::vector<int> occupation(numbins);
  extractPowerSpectrum(BiFT, kbin.data(), power.data(), kscatter.data(), pscatter.data(), occupation.data(), numbins,
                       true, KTYPE_LINEAR);
  FILE *out = std::fopen(argv[3], "wb");
  if (!out) return 2;
  std::fwrite(&a, 8, 1, out);
  std::fwrite(parts.data(), sizeof(gev_part), V, out);
  std::fwrite(power.data(), sizeof(Real), numbins, out);
  std::fwrite(occupation.data(), sizeof(int), numbins, out);
  std::fclose(out);
  std::printf("a = %.17g maxvel = %.6g\n", a, maxvel);
  return 0;
}
