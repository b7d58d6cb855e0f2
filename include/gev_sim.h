/*
 * gev_sim.h -- the device-resident simulation state and one cycle of
 * gevolution's main loop (main.cpp:372-879) for CDM in GR mode, on top of the
 * hot-path C-ABI in gev_gb300.h.
 *
 * The state mirrors the locals of main() that the loop body reads and writes:
 * the particles (pcls_cdm), the fields phi, chi, source, Sij, Bi and the
 * spectra scalarFT, SijFT, BiFT (main.cpp:217-246), and the scalars a, tau,
 * dtau, dtau_old, fourpiG and the cosmology.  gev_sim_step enqueues one cycle
 * without waiting for the GPU; gev_sim_get_state waits and also returns the
 * diagnostics the reference prints (T00hom, phi(k=0), max |v|).
 */
#ifndef GEV_SIM_H
#define GEV_SIM_H

#include "gev_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  double Omega_cdm, Omega_b, Omega_m, Omega_Lambda, Omega_rad;
} gev_cosmology;

typedef struct {
  double a, tau, dtau, dtau_old, fourpiG, Cf, steplimit, z_relax, maxvel, T00hom, phik0, mass;
  gev_cosmology cosmo;
  int vector_elliptic; /* 0: parabolic (default, parser.hpp:1136), 1: elliptic */
  int cycle;
} gev_sim_state;

/* gev_sim_field indices */
#define GEV_SIM_PHI 0
#define GEV_SIM_CHI 1
#define GEV_SIM_SOURCE 2
#define GEV_SIM_SIJ 3
#define GEV_SIM_BI 4
#define GEV_SIM_SCALARFT 5
#define GEV_SIM_SIJFT 6
#define GEV_SIM_BIFT 7

typedef struct gev_sim gev_sim;

int gev_sim_create(gev_ctx *ctx, long np, gev_sim **out);
int gev_sim_destroy(gev_sim *s);
int gev_sim_set_state(gev_sim *s, const gev_sim_state *st);
int gev_sim_get_state(gev_sim *s, gev_sim_state *st);
int gev_sim_field(gev_sim *s, int which, gev_field **out);
int gev_sim_particles(gev_sim *s, gev_pcls **out);
/* one cycle: deposits, phi / chi / B solves, kick, drift, background, next dtau */
int gev_sim_step(gev_sim *s);
/* the same cycle in its two parts, for a loop that writes outputs where
 * main.cpp writes them (between the field solves and the particle update):
 * gev_sim_step_fields = main.cpp:372-598 (stress-energy, phi, chi, B);
 * gev_sim_step_particles = main.cpp:743-872 (kick, drift, background, dtau).
 * Between the two, source, Sij, scalarFT and SijFT are free scratch. */
int gev_sim_step_fields(gev_sim *s);
int gev_sim_step_particles(gev_sim *s);
/* the cycle of gev_sim_step enqueued as one CUDA graph: the host code of the cycle
 * runs with the stream under capture (thread-local mode), and the simulation's
 * executable graph is updated in place with the new cycle's arguments
 * (instantiated again only if the launch sequence changed shape), then launched.
 * The results are the same bits as gev_sim_step's.  The first two cycles of a run,
 * and cycles with the per-kernel timers on, are enqueued directly (they set up
 * what the cycle tunes or allocates on first use); a capture the runtime refuses
 * also falls back to a direct cycle.  No call may be made on the simulation's
 * stream from another thread while this one runs. */
int gev_sim_step_graph(gev_sim *s);
/* cycles launched as a graph, graph instantiations, and cycles enqueued directly
 * by gev_sim_step_graph since the simulation was created (any pointer may be NULL) */
int gev_sim_graph_info(gev_sim *s, long *launches, long *builds, long *direct);

/* Batched cycles: one cycle of each of many simulations, with one launch per kernel
 * of the cycle for each cohort of simulations of one grid size.  Each simulation's
 * cycle is recorded (the host runs gev_sim_step's code, the launches are kept rather
 * than enqueued); simulations with the same launch sequence form a cohort, and each
 * kernel runs once for the whole cohort on the batch's stream, every block on its own
 * simulation's arguments -- the same bits as gev_sim_step.  The batch's stream waits
 * for the work already queued on each simulation's stream, and each simulation's
 * stream then waits for the batch, so the calls of gev_sim.h and gev_gb300.h on a
 * simulation keep their order.  Batched: mixed-form simulations from their third
 * cycle on (the first two tune and allocate on first use), with the per-kernel timers
 * off, on grids up to 256^3; every other simulation takes a direct cycle
 * (gev_sim_step) on its own stream, as does one whose cycle uses an operation that
 * has no batched form.  Nothing is waited for but the batch's staging buffers (a ring
 * of three). */
typedef struct gev_batch gev_batch;
int gev_batch_create(int device, gev_batch **out);
int gev_batch_destroy(gev_batch *b);
/* one cycle of each of sims[0 .. n-1] (distinct simulations on the batch's device).
 * A batch and its simulations are driven from one host thread at a time; separate
 * batches over separate simulations may run in separate threads.  GEV_EINVAL (null,
 * repeated or foreign simulations) leaves every simulation as it was; after any other
 * error the simulations of the call are in an undefined state. */
int gev_batch_step(gev_batch *b, gev_sim *const *sims, int n);
/* cycles run batched, cycles run directly, batched kernel launches (NULL to skip) */
int gev_batch_info(gev_batch *b, long *batched, long *direct, long *launches);
/* main.cpp's loop for each simulation, in batched steps: each of sims[0 .. n-1] runs
 * cycles until the first whose scale factor passes a_target[i]; cycles[i] = the cycles
 * it ran.  Returns once the device has finished them. */
int gev_batch_run(gev_batch *b, gev_sim *const *sims, int n, const double *a_target, int *cycles);

/* Zel'dovich initial conditions at z_in generated on the device, following the
 * power-spectrum branch of generateIC_basic (ic_basic.hpp:1626-2259): sc1
 * template tiled N/4 times, a tabulated BBKS spectrum normalised to sigma8 and
 * read through the mPk spline, the reference's sitmo stream laid over k-space as
 * generateDisplacementField lays it, baryons folded into CDM, no radiation.  Requires N % 4 == 0 and capacity >= N^3.  Sets the
 * whole state (a, tau, dtau, dtau_old = 0, fourpiG, cosmology, particle mass). */
typedef struct {
  double h, Omega_cdm, Omega_b, n_s, sigma8, z_in, boxsize, Cf, steplimit;
  uint64_t seed;              /* the sitmo stream is seeded with its low 32 bits, (unsigned int) ic.seed */
  int ksphere;                /* 1: k-domain = sphere */
  int correct_displacement;   /* 1: correct displacement = yes, the template's CIC kernel (ICFLAG_CORRECT_DISPLACEMENT) */
} gev_ic_params;
int gev_sim_ic_generate(gev_sim *s, const gev_ic_params *ic);

#ifdef __cplusplus
}
#endif
#endif
