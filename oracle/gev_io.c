/*
 * gev_io.c -- CPU restatement of gevolution 1.2's Gadget-2 snapshot writer and
 * reader (Particles_gevolution.hpp:30-251 saveGadget2, 574-665 loadGadget2) on
 * one rank.  TEST INFRASTRUCTURE ONLY (the checker for the GPU path); pinned
 * against the reference's own code compiled against the shims (ref_gadget.cpp).
 *
 * Built with -ffp-contract=off: every expression rounds as written, in the
 * reference's operation order.
 */
#define _POSIX_C_SOURCE 200809L
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gev_oracle.h"

#define G2_VEL_CONV 3.335640952e-6 /* GADGET_VELOCITY_CONVERSION, metadata.hpp:118 */

static int put(FILE *f, long long off, const void *p, size_t n) {
  return fseeko(f, (off_t)off, SEEK_SET) == 0 && fwrite(p, 1, n, f) == n;
}
static int get(FILE *f, long long off, void *p, size_t n) {
  return fseeko(f, (off_t)off, SEEK_SET) == 0 && fread(p, 1, n, f) == n;
}

/* phi at (x + dx, y + dy, z + dz), periodic (LATfield2's halo after updateHalo) */
static double phi_at(const double *phi, int N, int x, int y, int z) {
  return phi[(size_t)(x % N) + (size_t)N * ((size_t)(y % N) + (size_t)N * (size_t)(z % N))];
}

int gevo_gadget2_save(const char *fname, int N, long np, const gevo_part *src, const double *phi,
                      const void *hdr256, int tracer_factor, double dtau_pos, double dtau_vel, int exact,
                      int id_bytes) {
  gevo_gadget2_header hdr;
  memcpy(&hdr, hdr256, sizeof(hdr));
  if (hdr.num_files != 1 || tracer_factor < 1 || (exact && !phi) || (id_bytes != 4 && id_bytes != 8)) return -1;
  /* the per-cell lists in ascending ID order, walked site by site */
  gevo_part *p = (gevo_part *)malloc(sizeof(gevo_part) * (size_t)(np > 0 ? np : 1));
  memcpy(p, src, sizeof(gevo_part) * (size_t)np);
  gevo_sort(N, np, p, NULL);
  long long S = 0;
  for (long i = 0; i < np; i++)
    if (p[i].ID % tracer_factor == 0) S++;
  if (S != (long long)hdr.npart[1]) {
    free(p);
    return -1;
  }
  FILE *f = fopen(fname, "wb");
  if (!f) {
    free(p);
    return -1;
  }
  const double rescale_vel = 1. / sqrt(hdr.time) / G2_VEL_CONV; /* Particles_gevolution.hpp:45 */
  const double dx = 1.0 / (double)N;                            /* lat_resolution_ */
  const long long o_pos = 3 * 4 + 256, o_vel = o_pos + 8 + 12 * S, o_id = o_vel + 8 + 12 * S;
  uint32_t m = 256u;
  int ok = put(f, 0, &m, 4) && put(f, 4, &hdr, 256) && put(f, 260, &m, 4);
  m = (uint32_t)(3 * sizeof(float) * (size_t)hdr.npart[1]);
  ok = ok && put(f, 264, &m, 4) && put(f, o_vel - 8, &m, 4) && put(f, o_vel - 4, &m, 4) && put(f, o_id - 8, &m, 4);
  m = (uint32_t)((size_t)id_bytes * (size_t)hdr.npart[1]);
  ok = ok && put(f, o_id - 4, &m, 4) && put(f, o_id + (long long)id_bytes * S, &m, 4);
  long long k = 0;
  for (long i = 0; i < np && ok; i++) {
    const gevo_part *q = p + i;
    if (q->ID % tracer_factor != 0) continue;
    float pf[3], vf[3];
    if (!exact) { /* 213-219 */
      for (int l = 0; l < 3; l++) pf[l] = (float)(q->pos[l] * hdr.BoxSize);
      for (int l = 0; l < 3; l++) vf[l] = (float)(q->vel[l] * rescale_vel / hdr.time);
    } else { /* 166-211: phi and its gradient at the particle from its cell's 8 corners */
      double r[3], ip, ph, g[3];
      for (int l = 0; l < 3; l++) r[l] = modf(q->pos[l] / dx, &ip);
      const int cx = gevo_cell_of(N, q->pos[0]), cy = gevo_cell_of(N, q->pos[1]), cz = gevo_cell_of(N, q->pos[2]);
      const double f000 = phi_at(phi, N, cx, cy, cz), f100 = phi_at(phi, N, cx + 1, cy, cz);
      const double f010 = phi_at(phi, N, cx, cy + 1, cz), f110 = phi_at(phi, N, cx + 1, cy + 1, cz);
      const double f001 = phi_at(phi, N, cx, cy, cz + 1), f101 = phi_at(phi, N, cx + 1, cy, cz + 1);
      const double f011 = phi_at(phi, N, cx, cy + 1, cz + 1), f111 = phi_at(phi, N, cx + 1, cy + 1, cz + 1);
      ph = f000 * (1. - r[0]) * (1. - r[1]) * (1. - r[2]);
      ph += f100 * r[0] * (1. - r[1]) * (1. - r[2]);
      ph += f010 * (1. - r[0]) * r[1] * (1. - r[2]);
      ph += f110 * r[0] * r[1] * (1. - r[2]);
      ph += f001 * (1. - r[0]) * (1. - r[1]) * r[2];
      ph += f101 * r[0] * (1. - r[1]) * r[2];
      ph += f011 * (1. - r[0]) * r[1] * r[2];
      ph += f111 * r[0] * r[1] * r[2];
      g[0] = (1. - r[1]) * (1. - r[2]) * (f100 - f000);
      g[1] = (1. - r[0]) * (1. - r[2]) * (f010 - f000);
      g[2] = (1. - r[0]) * (1. - r[1]) * (f001 - f000);
      g[0] += r[1] * (1. - r[2]) * (f110 - f010);
      g[1] += r[0] * (1. - r[2]) * (f110 - f100);
      g[2] += r[0] * (1. - r[1]) * (f101 - f100);
      g[0] += (1. - r[1]) * r[2] * (f101 - f001);
      g[1] += (1. - r[0]) * r[2] * (f011 - f001);
      g[2] += (1. - r[0]) * r[1] * (f011 - f010);
      g[0] += r[1] * r[2] * (f111 - f011);
      g[1] += r[0] * r[2] * (f111 - f101);
      g[2] += r[0] * r[1] * (f111 - f110);
      double v2 = q->vel[0] * q->vel[0] + q->vel[1] * q->vel[1] + q->vel[2] * q->vel[2];
      const double e2 = v2 + hdr.time * hdr.time, e = sqrt(e2);
      v2 += e2;
      const double fac = 1. + (4. - (v2 / e2)) * ph;
      for (int l = 0; l < 3; l++)
        pf[l] = (float)(modf(1. + q->pos[l] + dtau_pos * q->vel[l] * fac / e, &ip) * hdr.BoxSize);
      for (int l = 0; l < 3; l++)
        vf[l] = (float)((q->vel[l] - dtau_vel * v2 * g[l] / dx / e) * rescale_vel / hdr.time);
    }
    ok = ok && put(f, o_pos + 12 * k, pf, 12) && put(f, o_vel + 12 * k, vf, 12);
    if (id_bytes == 8) {
      const int64_t id = (int64_t)q->ID;
      ok = ok && put(f, o_id + 8 * k, &id, 8);
    } else {
      const int32_t id = (int32_t)q->ID;
      ok = ok && put(f, o_id + 4 * k, &id, 4);
    }
    k++;
  }
  ok = fclose(f) == 0 && ok;
  free(p);
  return ok ? 0 : -1;
}

long gevo_gadget2_load(const char *fname, int N, gevo_part *dst, long cap, void *hdr256, int id_bytes) {
  FILE *f = fopen(fname, "rb");
  if (!f) return -1;
  uint32_t m = 0;
  gevo_gadget2_header hdr;
  if (!get(f, 0, &m, 4) || m != 256u || !get(f, 4, &hdr, 256)) {
    fclose(f);
    return -1;
  }
  memcpy(hdr256, &hdr, 256);
  const long long S = hdr.npart[1];
  if (S > cap) {
    fclose(f);
    return -1;
  }
  double rescale_vel = 1. / G2_VEL_CONV; /* 586, 608 */
  rescale_vel /= sqrt(hdr.time);
  const long long o_pos = 256 + 3 * 4, o_vel = o_pos + S * 12 + 8, o_id = o_vel + o_vel - o_pos;
  for (long long i = 0; i < S; i++) {
    float pf[3], vf[3];
    if (!get(f, o_pos + 12 * i, pf, 12) || !get(f, o_vel + 12 * i, vf, 12)) {
      fclose(f);
      return -1;
    }
    long id;
    if (id_bytes == 8) {
      int64_t v;
      if (!get(f, o_id + 8 * i, &v, 8)) {
        fclose(f);
        return -1;
      }
      id = (long)v;
    } else {
      int32_t v;
      if (!get(f, o_id + 4 * i, &v, 4)) {
        fclose(f);
        return -1;
      }
      id = (long)v;
    }
    for (int l = 0; l < 3; l++) { /* 638-643, float /= double and float *= double */
      pf[l] /= hdr.BoxSize;
      if (pf[l] >= 1.) pf[l] -= 1.;
      vf[l] *= hdr.time / rescale_vel;
    }
    for (int l = 0; l < 3; l++) {
      dst[i].pos[l] = pf[l];
      dst[i].vel[l] = vf[l];
    }
    dst[i].ID = id;
  }
  fclose(f);
  gevo_sort(N, (long)S, dst, NULL);
  return (long)S;
}

/* writePowerSpectrum (tools.hpp:268-345) on one rank; exact = the
 * EXACT_OUTPUT_REDSHIFTS build, which interpolates with the spectrum that an
 * earlier call left in the same file when 1/a < z_target + 1 */
int gevo_write_power_spectrum(const double *kbin, const double *power, const double *kscatter, const double *pscatter,
                              const int *occupation, int numbins, double rescalek, double rescalep,
                              const char *filename, const char *description, double a, double z_target, int exact) {
  double *power2 = (double *)malloc(sizeof(double) * (size_t)(numbins > 0 ? numbins : 1));
  for (int i = 0; i < numbins; i++) power2[i] = power[i] / rescalep;
  if (exact && 1. / a < z_target + 1.) {
    FILE *in = fopen(filename, "r");
    if (in) {
      double w = 1.;
      if (fscanf(in, "%*[^\n]\n") < 0) w = 1.;
      if (fscanf(in, "# redshift z=%lf\n", &w) != 1) {
        w = 1.;
      } else {
        w = (w - z_target) / (1. + w - 1. / a);
        if (fscanf(in, "%*[^\n]\n") < 0) w = w;
        for (int i = 0; i < numbins; i++)
          if (occupation[i] > 0 && fscanf(in, " %*e %le %*e %*e %*d \n", power2 + i) != 1) break;
      }
      fclose(in);
      for (int i = 0; i < numbins; i++) power2[i] = (1. - w) * power2[i] + w * power[i] / rescalep;
      a = 1. / (z_target + 1.);
    }
  }
  FILE *out = fopen(filename, "w");
  if (!out) {
    free(power2);
    return -1;
  }
  fprintf(out, "# %s\n", description);
  fprintf(out, "# redshift z=%f\n", (1. / a) - 1.);
  fprintf(out, "# k              Pk             sigma(k)       sigma(Pk)      count\n");
  for (int i = 0; i < numbins; i++)
    if (occupation[i] > 0)
      fprintf(out, "  %e   %e   %e   %e   %d\n", kbin[i] / rescalek, exact ? power2[i] : power[i] / rescalep,
              kscatter[i] / rescalek, pscatter[i] / rescalep / sqrt(occupation[i]), occupation[i]);
  fclose(out);
  free(power2);
  return 0;
}

/* hibernate's rescale of B before it is written (hibernation.hpp:529-538, the
 * parabolic vector method): every component divided by a^2 N */
void gevo_hibernate_b(int N, double *Bi, double a) {
  const size_t n = 3 * (size_t)N * N * N;
  for (size_t i = 0; i < n; i++) Bi[i] /= a * a * N;
}

/* readIC's restart of the vector potential from the stored B (ic_read.hpp:307-318):
 * every component multiplied by a^2 / (numpts * numpts), an int product, then the
 * forward transform (plan_Bi->execute(FFT_FORWARD)) into BiFT.  B is modified. */
void gevo_restart_bift_from_b(int N, double *Bi, double a, double *BiFT) {
  const size_t V = (size_t)N * N * N;
  const size_t K = (size_t)N * N * (N / 2 + 1) * 2;
  for (size_t i = 0; i < 3 * V; i++) Bi[i] *= a * a / (N * N);
  for (int c = 0; c < 3; c++) gevo_fft_r2c(N, Bi + c * V, BiFT + c * K);
}
