/*
 * gev_io.h -- particle snapshots and hibernation points of the device-resident
 * state, the file formats around the particle-mesh step.
 *
 * Gadget-2 snapshots (Particles_gevolution.hpp:30-251, 574-665; header
 * metadata.hpp:152-171).  The particles of a store are converted on the GPU
 * (positions to Gadget length units, q to Gadget velocities, the optional
 * EXACT_OUTPUT_REDSHIFTS drift and kick) and written in the reference's block
 * layout: [256][header][256] [12n][positions][12n] [12n][velocities][12n]
 * [8n or 4n][IDs][8n or 4n], little-endian, one file (num_files = 1).  The
 * particle order in the file is (cell, ID), the order of the reference's
 * per-cell lists on one rank.
 *
 * Hibernation points (hibernation.hpp:513-611 writes them, ic_read.hpp:58-716
 * reads them back).  HDF5 is not used: one binary file holds a header, the
 * particles as gev_part records in (cell, ID) order, phi, chi, B divided by
 * a^2 N as hibernate() stores it, and the spectrum BiFT, each section with a
 * 64-bit checksum.  A restart from the file continues bit for bit where the
 * hibernating run would have gone on.
 */
#ifndef GEV_IO_H
#define GEV_IO_H

#include "gev_sim.h"

#ifdef __cplusplus
extern "C" {
#endif

/* the 256-byte Gadget-2 file header, field for field as gadget2_header
 * (metadata.hpp:152-171) */
typedef struct {
  uint32_t npart[6];
  double mass[6];
  double time;
  double redshift;
  int32_t flag_sfr;
  int32_t flag_feedback;
  uint32_t npartTotal[6];
  int32_t flag_cooling;
  int32_t num_files;
  double BoxSize;
  double Omega0;
  double OmegaLambda;
  double HubbleParam;
  int32_t flag_age;
  int32_t flag_metals;
  uint32_t npartTotalHW[6];
  char fill[256 - 6 * 4 - 6 * 8 - 2 * 8 - 2 * 4 - 6 * 4 - 2 * 4 - 4 * 8 - 2 * 4 - 6 * 4];
} gev_gadget2_header;

/* Gadget units (metadata.hpp:111-121) */
#define GEV_GADGET_LENGTH_CONVERSION 0.001
#define GEV_GADGET_MASS_CONVERSION 1.0e10
#define GEV_GADGET_VELOCITY_CONVERSION 3.335640952e-6

/* saveGadget2 (Particles_gevolution.hpp:30-251).  Writes the particles whose
 * ID % tracer_factor == 0.  hdr->npart[1] must equal their number and
 * hdr->num_files must be 1 (GEV_EINVAL otherwise, and nothing is written).
 * exact_output = 0: positions * BoxSize, velocities * rescale / time (the
 * default build).  exact_output = 1: the EXACT_OUTPUT_REDSHIFTS build -- each
 * particle drifts by dtau_pos with its CIC-interpolated phi and kicks by
 * dtau_vel with the CIC gradient of phi; phi is required (main.cpp always
 * passes it; without it the reference's correction carries the previous
 * particle's integer part as phi).  id_bytes: GADGET_ID_BYTES, 8 or 4. */
int gev_gadget2_save(gev_ctx *ctx, gev_pcls *p, const char *filename, const gev_gadget2_header *hdr,
                     int tracer_factor, double dtau_pos, double dtau_vel, const gev_field *phi, int exact_output,
                     int id_bytes);

/* loadGadget2 (Particles_gevolution.hpp:574-665).  Reads one file, fills *hdr,
 * and adds its npart[1] particles to the store (addParticle_global), which must
 * have room for them.  Positions / BoxSize wrapped below 1 and velocities *
 * time / rescale, in the reference's float arithmetic. */
int gev_gadget2_load(gev_ctx *ctx, gev_pcls *p, const char *filename, gev_gadget2_header *hdr, int id_bytes);

/* hibernation points */
typedef struct {
  double a, tau, dtau; /* the arguments of hibernate(..., a, tau, dtau, cycle) */
  int cycle;
  int has_state;       /* 1: state holds the whole simulation state (gev_sim_hibernate) */
  gev_sim_state state;
  long numpcl;
  int N, prec;
} gev_checkpoint_info;

#define GEV_CKPT_FROM_B 1 /* restart: rebuild BiFT from B as readIC does, ignoring the stored spectrum */

/* hibernate (hibernation.hpp:513-611) for the fields and particles of a
 * caller's own loop.  Bi: the real-space B of the step (may be NULL when the
 * vector mode does not save it); it is stored divided by a^2 N.  BiFT may be
 * NULL; with it a restart is exact.  st may be NULL. */
int gev_checkpoint_save(gev_ctx *ctx, const char *path, gev_pcls *p, const gev_field *phi, const gev_field *chi,
                        const gev_field *Bi, const gev_field *BiFT, double a, double tau, double dtau, int cycle,
                        const gev_sim_state *st);
/* the restart branch of readIC (ic_read.hpp:58-716): replaces the store's
 * particles, phi, chi; Bi = B * a^2 / N^2 (ic_read.hpp:307-318) when Bi is given;
 * BiFT from the stored spectrum, or (no spectrum stored, or GEV_CKPT_FROM_B)
 * the forward transform of that Bi.  Any output may be NULL.  Checksums are
 * verified: a damaged file gives GEV_EINVAL.  info may be NULL. */
int gev_checkpoint_load(gev_ctx *ctx, const char *path, gev_pcls *p, gev_field *phi, gev_field *chi, gev_field *Bi,
                        gev_field *BiFT, int flags, gev_checkpoint_info *info);
/* reads only the header */
int gev_checkpoint_info_read(const char *path, gev_checkpoint_info *info);

/* the whole simulation of gev_sim.h */
int gev_sim_hibernate(gev_sim *s, const char *path);
int gev_sim_restart(gev_sim *s, const char *path, int flags);

/* power-spectrum outputs.
 * writePowerSpectrum (tools.hpp:268-345): the ASCII table of one spectrum (k,
 * P(k), sigma(k), sigma(P), count per occupied bin, k / rescalek and
 * P / rescalep).  exact_output = the EXACT_OUTPUT_REDSHIFTS build: when
 * 1/a < z_target + 1 and the file already holds the spectrum written one cycle
 * earlier, the table is interpolated linearly in redshift to z_target. */
int gev_write_power_spectrum(const double *kbin, const double *power, const double *kscatter, const double *pscatter,
                             const int *occupation, int numbins, double rescalek, double rescalep,
                             const char *filename, const char *description, double a, double z_target,
                             int exact_output);

/* the output masks of metadata.hpp:56-71 that a CDM-only GR run writes */
#define GEV_MASK_PHI 1
#define GEV_MASK_CHI 2
#define GEV_MASK_POT 4
#define GEV_MASK_B 8
#define GEV_MASK_T00 16
#define GEV_MASK_RBARE 64
#define GEV_MASK_HIJ 128
#define GEV_MASK_DELTA 4096
#define GEV_MASK_DBARE 8192

typedef struct {
  int out_pk;              /* sim.out_pk: an OR of GEV_MASK_* */
  int numbins;             /* sim.numbins */
  double boxsize;          /* sim.boxsize [Mpc/h] */
  double z_target;         /* sim.z_pk[pkcount] (read by exact_output) */
  int exact_output;        /* the EXACT_OUTPUT_REDSHIFTS build */
  const char *output_path; /* sim.output_path */
  const char *basename_pk; /* sim.basename_pk */
} gev_pk_settings;

/* writeSpectra (output.hpp:1762-2204) for the CDM particles of a GR simulation,
 * called between gev_sim_step_fields and gev_sim_step_particles as main.cpp
 * calls it: the spectra are binned on the GPU (gev_cross_spectrum) and written
 * as <output_path><basename_pk><pkcount %03d>_<name>.dat with the reference's
 * descriptions and normalisations.  Uses source, Sij, scalarFT and SijFT as
 * scratch, as the reference does. */
int gev_sim_write_spectra(gev_sim *s, const gev_pk_settings *cfg, int pkcount);

#ifdef __cplusplus
}
#endif
#endif
