// gev_pkout.cu -- power-spectrum outputs (include/gev_io.h): the ASCII writer
// of tools.hpp:268-345 and the writeSpectra sequence of output.hpp:1762-2204
// for CDM particles in GR.  Host code over the device primitives: every
// spectrum is binned on the GPU, and the host formats the table.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gev_io.h"
#include "gev_internal.cuh"

extern "C" {

int gev_write_power_spectrum(const double *kbin, const double *power, const double *kscatter, const double *pscatter,
                             const int *occupation, int numbins, double rescalek, double rescalep,
                             const char *filename, const char *description, double a, double z_target,
                             int exact_output) {
  if (!kbin || !power || !kscatter || !pscatter || !occupation || numbins < 0 || !filename || !description)
    return GEV_EINVAL;
  std::vector<double> p(power, power + numbins);
  for (double &v : p) v /= rescalep;
  if (exact_output && 1. / a < z_target + 1.) {
    // the table written one cycle earlier: its redshift, then its P(k) column
    // (tools.hpp:282-316)
    if (FILE *in = std::fopen(filename, "r")) {
      double w = 1.;
      int r = std::fscanf(in, "%*[^\n]\n");
      (void)r;
      if (std::fscanf(in, "# redshift z=%lf\n", &w) != 1) {
        std::fprintf(stderr, " error parsing power spectrum file header for interpolation (EXACT_OUTPUT_REDSHIFTS)\n");
        w = 1.;
      } else {
        w = (w - z_target) / (1. + w - 1. / a);
        r = std::fscanf(in, "%*[^\n]\n");
        for (int i = 0; i < numbins; i++) {
          if (occupation[i] <= 0) continue;
          if (std::fscanf(in, " %*e %le %*e %*e %*d \n", &p[i]) != 1) {
            std::fprintf(stderr, " error parsing power spectrum file data %d for interpolation (EXACT_OUTPUT_REDSHIFTS)\n",
                         i);
            break;
          }
        }
      }
      std::fclose(in);
      for (int i = 0; i < numbins; i++) p[i] = (1. - w) * p[i] + w * power[i] / rescalep;
      a = 1. / (z_target + 1.);
    }
  }
  FILE *out = std::fopen(filename, "w");
  if (!out) return GEV_EINVAL;
  std::fprintf(out, "# %s\n", description);
  std::fprintf(out, "# redshift z=%f\n", (1. / a) - 1.);
  std::fprintf(out, "# k              Pk             sigma(k)       sigma(Pk)      count\n");
  for (int i = 0; i < numbins; i++)
    if (occupation[i] > 0)
      std::fprintf(out, "  %e   %e   %e   %e   %d\n", kbin[i] / rescalek, p[i], kscatter[i] / rescalek,
                   pscatter[i] / rescalep / std::sqrt((double)occupation[i]), occupation[i]);
  return std::fclose(out) == 0 ? GEV_OK : GEV_EINVAL;
}

}  // extern "C"

namespace {

struct Writer {
  gev_sim *s;
  const gev_pk_settings *cfg;
  int pkcount;
  std::vector<double> kb, pw, ks, ps;
  std::vector<int> occ;
  Writer(gev_sim *sim, const gev_pk_settings *c, int k)
      : s(sim), cfg(c), pkcount(k), kb(c->numbins), pw(c->numbins), ks(c->numbins), ps(c->numbins), occ(c->numbins) {}
  // extractPowerSpectrum (KTYPE_LINEAR) of a spectrum on the GPU
  int spectrum(const gev_field *f, bool deconvolve, bool symmetric) {
    return gev_cross_spectrum(s->ctx, f, f, kb.data(), pw.data(), ks.data(), ps.data(), occ.data(), cfg->numbins,
                              deconvolve ? 1 : 0, 1, symmetric ? 1 : 0, -1, -1);
  }
  int write(const char *name, const char *description, double rescalep) {
    char file[4096];
    std::snprintf(file, sizeof(file), "%s%s%03d_%s.dat", cfg->output_path ? cfg->output_path : "",
                  cfg->basename_pk ? cfg->basename_pk : "", pkcount, name);
    return gev_write_power_spectrum(kb.data(), pw.data(), ks.data(), ps.data(), occ.data(), cfg->numbins,
                                    cfg->boxsize, rescalep, file, description, s->st.a, cfg->z_target,
                                    cfg->exact_output);
  }
};

#define RCW(x)                \
  do {                        \
    const int rc_ = (x);      \
    if (rc_) return rc_;      \
  } while (0)

}  // namespace

extern "C" {

int gev_sim_write_spectra(gev_sim *s, const gev_pk_settings *cfg, int pkcount) {
  if (!s || !cfg || cfg->numbins < 1 || cfg->boxsize <= 0.) return gev_fail(s ? s->ctx : nullptr, GEV_EINVAL, "write_spectra");
  gev_ctx *ctx = s->ctx;
  const gev_sim_state &st = s->st;
  const double a = st.a, fourpiG = st.fourpiG;
  const int N = ctx->N;
  const long numpts3d = (long)N * (long)N * (long)N;
  // (Real) numpts3d * (Real) numpts3d * 2. * M_PI * M_PI, the common normalisation
  const double base = (double)numpts3d * (double)numpts3d * 2. * M_PI * M_PI;
  const int m = cfg->out_pk;
  Writer w(s, cfg, pkcount);

  if (m & (GEV_MASK_RBARE | GEV_MASK_DBARE | GEV_MASK_POT)) {  // output.hpp:1785-1862, the mass density
    RCW(projection_replace(ctx, s->pcls, s->source, 3, 1., nullptr));
    RCW(gev_fft_r2c(ctx, s->source, s->scalarFT));
    if (m & (GEV_MASK_RBARE | GEV_MASK_DBARE)) RCW(w.spectrum(s->scalarFT, true, false));
    if (m & GEV_MASK_RBARE) RCW(w.write("rhoN", "power spectrum of rho_N", base * pow(a, 6.0)));
    if (m & GEV_MASK_DBARE)
      RCW(w.write("deltaN", "power spectrum of delta_N", base * st.cosmo.Omega_m * st.cosmo.Omega_m));
    if (m & GEV_MASK_POT) {
      RCW(gev_solve_poisson(ctx, s->scalarFT, s->scalarFT, fourpiG / a, 0.));
      RCW(w.spectrum(s->scalarFT, false, false));
      RCW(w.write("psiN", "power spectrum of psi_N", base));
    }
  }
  if (m & GEV_MASK_PHI) {  // 1922-1928
    RCW(gev_fft_r2c(ctx, s->phi, s->scalarFT));
    RCW(w.spectrum(s->scalarFT, false, false));
    RCW(w.write("phi", "power spectrum of phi", base));
  }
  if (m & GEV_MASK_CHI) {  // 1930-1936
    RCW(gev_fft_r2c(ctx, s->chi, s->scalarFT));
    RCW(w.spectrum(s->scalarFT, false, false));
    RCW(w.write("chi", "power spectrum of chi", base));
  }
  if (m & GEV_MASK_HIJ) {  // 1938-1959
    RCW(projection_replace(ctx, s->pcls, s->Sij, 2, a, s->phi));
    RCW(gev_prepare_source_tensor(ctx, s->phi, s->Sij, s->Sij, 2. * fourpiG / (double)N / (double)N / a));
    RCW(gev_fft_r2c(ctx, s->Sij, s->SijFT));
    RCW(gev_project_tensor(ctx, s->SijFT, s->SijFT));
    RCW(w.spectrum(s->SijFT, false, true));
    RCW(w.write("hij", "power spectrum of hij", 2. * M_PI * M_PI));
  }
  if (m & (GEV_MASK_T00 | GEV_MASK_DELTA)) {  // 1961-2025, GR
    RCW(projection_replace(ctx, s->pcls, s->source, 0, a, s->phi));
    RCW(gev_fft_r2c(ctx, s->source, s->scalarFT));
    RCW(w.spectrum(s->scalarFT, true, false));
    if (m & GEV_MASK_T00) RCW(w.write("T00", "power spectrum of T00", base * pow(a, 6.0)));
    if (m & GEV_MASK_DELTA) {
      const double om = st.cosmo.Omega_cdm + st.cosmo.Omega_b + 0.;  // + bg_ncdm(a) = 0: no ncdm species
      RCW(w.write("delta", "power spectrum of delta", base * om * om));
    }
  }
  if (m & GEV_MASK_B) {  // 2148-2152
    RCW(w.spectrum(s->BiFT, false, false));
    RCW(w.write("B", "power spectrum of B", a * a * a * a * N * N * 2. * M_PI * M_PI));
  }
  return GEV_OK;
}

}  // extern "C"
