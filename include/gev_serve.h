/*
 * gev_serve.h -- continuous batching of many independent simulations on one GPU:
 * a request loop that admits simulations (grid size, cosmology, seed, target
 * redshift) by HBM footprint, keeps their state on the device, advances all
 * admitted simulations concurrently, and hands back each one's result when it
 * reaches its target.
 *
 * Each admitted simulation owns a context (gev_gb300.h) and so a CUDA stream of
 * its own; scheduler threads inside the library enqueue one cycle
 * (gev_sim_step) per simulation in turn, each thread its own share of the
 * simulations, keeping a bounded number of cycles in flight on each stream, so
 * that the kernels of different simulations overlap on the device.  A simulation's work touches only its own buffers and every
 * kernel is deterministic, so its result is the same bits whether it runs alone
 * or among others.  Contexts of a grid size are pooled and reused; a new request
 * is admitted when the bytes its grid size needs fit under the budget.
 *
 * The result of a request is its state at the first cycle that passes the
 * target redshift (main.cpp's loop stops there): a, tau, the number of cycles,
 * and the power spectrum of phi (extractPowerSpectrum, tools.hpp:237-240) with
 * the reference's normalisation of its phi table.  Times are seconds since the
 * server started.
 */
#ifndef GEV_SERVE_H
#define GEV_SERVE_H

#include "gev_sim.h"

#ifdef __cplusplus
extern "C" {
#endif

#define GEV_SERVE_MAX_BINS 64
#define GEV_SERVE_MAX_WORKERS 16

typedef struct {
  int N;            /* grid points = particles per side (N % 4 == 0) */
  int prec;         /* GEV_PREC_FP64 or GEV_PREC_MIXED */
  double boxsize;   /* Mpc/h */
  double Omega_cdm, Omega_b, sigma8, n_s, h;
  double z_in, z_target;
  uint64_t seed;
  int numbins;      /* bins of the result's power spectrum, <= GEV_SERVE_MAX_BINS */
} gev_request;

typedef struct {
  long id;
  int N, prec, cycles, status; /* status: GEV_OK, or the error that ended it */
  double a, tau;
  double t_submit, t_admit, t_done;
  double kbin[GEV_SERVE_MAX_BINS], power[GEV_SERVE_MAX_BINS];
  int occupation[GEV_SERVE_MAX_BINS];
  int numbins;
} gev_result;

typedef struct {
  long submitted, admitted, completed, failed, active, pending;
  long max_active_seen;      /* the most simulations on the device at once */
  double particle_steps;     /* summed over completed cycles */
  double busy_seconds;       /* time with at least one simulation admitted */
  size_t bytes_budget, bytes_in_use, bytes_peak;
  long workers;              /* host threads that enqueue the simulations' cycles */
  long graph_cycles;         /* cycles launched as one CUDA graph each (gev_server_set_graphs) */
} gev_server_stats;

typedef struct gev_server gev_server;

/* bytes_budget: device bytes the server may hold (0: 90% of the free memory);
 * max_active: simulations on the device at once (0: no limit but the budget);
 * inflight: cycles enqueued ahead per simulation (0: 2) */
int gev_server_create(int device, size_t bytes_budget, int max_active, int inflight, gev_server **out);
/* the same with the number of host threads that enqueue the simulations' cycles
 * (1 .. GEV_SERVE_MAX_WORKERS; 0: 4 on hosts with 16 or more hardware threads, 2
 * with 8 or more, else 1, as gev_server_create chooses).  Worker 0 also admits
 * requests; each admitted simulation is enqueued by one worker only, so its
 * result does not depend on the count */
int gev_server_create_workers(int device, size_t bytes_budget, int max_active, int inflight, int workers,
                              gev_server **out);
/* on != 0: the schedulers enqueue each simulation's cycles with gev_sim_step_graph
 * (one CUDA graph a cycle, updated in place from cycle to cycle) instead of
 * gev_sim_step; results are the same bits either way.  Default off. */
int gev_server_set_graphs(gev_server *s, int on);
int gev_server_submit(gev_server *s, const gev_request *req, long *id);
/* up to max completed results not yet returned; *n their number */
int gev_server_poll(gev_server *s, gev_result *out, int max, int *n);
/* waits until no request is pending or active (timeout_s <= 0: no limit);
 * GEV_ETIMEOUT when the time runs out */
int gev_server_drain(gev_server *s, double timeout_s);
int gev_server_stats_get(gev_server *s, gev_server_stats *st);
/* the device bytes one simulation of grid N and precision form prec holds */
int gev_server_footprint(int device, int N, int prec, size_t *bytes);
int gev_server_destroy(gev_server *s);

#ifdef __cplusplus
}
#endif
#endif
