/*
 * gev_gb300.h -- C-ABI of the GB300 implementation of gevolution 1.2's
 * per-step particle-mesh hot path.
 *
 * One context owns one simulation grid (N^3 cells) on one GPU and one CUDA
 * stream.  Fields, spectra and particle stores are device-resident objects of
 * a context; every entry point enqueues work on the context's stream and
 * returns a status code (GEV_OK = 0).  Host buffers passed in or out are plain
 * arrays in the layouts below.  Nothing here falls back to the CPU: a missing
 * GPU or extension is an error.
 *
 * Host layouts (shared with the CPU oracle):
 *   real field   double[ncomp][N][N][N]            index c*N^3 + x + N*(y + N*z)
 *   spectrum     double[ncomp][N][N][N/2+1][2]     interleaved complex, kx fastest
 *   symmetric tensors store the components 00, 01, 02, 11, 12, 22
 *   particles    gev_part records {pos[3], vel[3], ID} (gevolution's part_simple)
 *
 * Each function names the gevolution-1.2 interface it replaces (file:line).
 */
#ifndef GEV_GB300_H
#define GEV_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define GEV_OK 0
#define GEV_EINVAL -1   /* bad argument (sizes, kinds, null handles) */
#define GEV_ENOMEM -2   /* device allocation failed */
#define GEV_ECUDA -3    /* CUDA runtime / launch error */
#define GEV_ETIMEOUT -4 /* a bounded device wait gave up */
#define GEV_ENODEV -5   /* no usable GPU */

/* ---- precision forms ---- */
#define GEV_PREC_FP64 0  /* fields, spectra, FFTs, deposits and particles in FP64 */
#define GEV_PREC_MIXED 1 /* FP32 fields/FFTs/momenta, FP64 positions, int64 fixed-point deposits */

/* ---- object kinds ---- */
#define GEV_FIELD_REAL 0
#define GEV_FIELD_SPECTRUM 1

/* ---- particle update kinds (the callbacks passed to updateVel / moveParticles) ---- */
#define GEV_GR 0     /* update_q / update_pos            gevolution.hpp:570, 810 */
#define GEV_NEWTON 1 /* update_q_Newton / update_pos_Newton gevolution.hpp:709, 900 */

typedef struct {
  double pos[3];
  double vel[3];
  int64_t ID;
} gev_part;

typedef struct gev_ctx gev_ctx;
typedef struct gev_field gev_field;
typedef struct gev_pcls gev_pcls;

/* ---- context (replaces Lattice/latFT set-up, main.cpp:213-215) ---- */
int gev_ctx_create(int device, int N, int precision, gev_ctx **out);
int gev_ctx_destroy(gev_ctx *ctx);
int gev_ctx_sync(gev_ctx *ctx);
int gev_ctx_stream(gev_ctx *ctx, void **cuda_stream); /* the cudaStream_t the context enqueues on */
int gev_ctx_info(gev_ctx *ctx, int *N, int *precision, size_t *device_bytes_in_use);
const char *gev_ctx_last_error(gev_ctx *ctx);
const char *gev_strerror(int status);
/* count of kernels this library launched on the context since creation */
int gev_ctx_launch_count(gev_ctx *ctx, long long *count);
/* device timing, no counterpart in the reference's API: the reference's
 * -DBENCHMARK build prints wall-time sums per phase of the main loop
 * (main.cpp:907-922).  While timing is on, the library brackets each of its
 * kernels, and each phase of gev_sim_step, with CUDA events on the context's
 * stream.  gev_ctx_timing_report waits for the stream and writes one line per
 * name, "name\tcount\ttotal_ms\n": kernel names (k_...) and the phases
 * "phase:projections", "phase:gravity solver", "phase:fft" (every 3-D
 * transform, inside the gravity solver) and "phase:update particles" (update_q
 * and update_pos with the relink).  reset != 0 clears the sums.  Returns
 * GEV_EINVAL if the report does not fit into len bytes (it is truncated). */
int gev_ctx_set_timing(gev_ctx *ctx, int on);
int gev_ctx_timing_report(gev_ctx *ctx, char *buf, size_t len, int reset);
/* the FFT tile widths in use, log2 of the lines a tile, for the r2c rows, y, z and
 * c2r rows passes: in the mixed form each is chosen by timing its candidates once,
 * on the context's first transform; every width gives the same bits */
int gev_ctx_fft_tiles(gev_ctx *ctx, int lg[4]);
/* pins the mixed form's FFT tile widths (rows 1..3, columns 2..4, at most 1024
 * threads a tile) instead of timing them; GEV_EINVAL for the FP64 form */
int gev_ctx_set_fft_tiles(gev_ctx *ctx, const int lg[4]);
/* the launch shapes of the mixed form's source stencils (prepareFTsource scalar
 * [0] and tensor [1]): threads a block and the cap on blocks a SM of their
 * grid-stride grids.  On a context's first stencil call each is chosen by timing
 * its candidates (128, 256, 512 threads; 4, 8, 16, 32 blocks a SM) on scratch
 * fields, for grids up to 256^3 (larger grids keep 256 threads and 16 blocks a
 * SM); every shape gives the same bits */
int gev_ctx_stencil_shapes(gev_ctx *ctx, int threads[2], int per_sm[2]);
/* pins those shapes instead of timing them: 64, 128, 256 or 512 threads, 1..64
 * blocks a SM */
int gev_ctx_set_stencil_shapes(gev_ctx *ctx, const int threads[2], const int per_sm[2]);

/* ---- fields (Field<Real> / Field<Cplx>::initialize, main.cpp:226-237) ---- */
int gev_field_create(gev_ctx *ctx, int kind, int ncomp, gev_field **out);
int gev_field_destroy(gev_field *f);
int gev_field_upload(gev_field *f, const double *host);
int gev_field_download(gev_field *f, double *host);
/* projection_init (LATfield2, main.cpp:378/416/426/438): zero all components */
int gev_field_zero(gev_field *f);
int gev_field_device_ptr(gev_field *f, void **ptr, size_t *bytes);

/* ---- particles (Particles<part_simple,...>::initialize / addParticle_global,
 *      ic_basic.hpp:1990, 1429) ---- */
int gev_pcls_create(gev_ctx *ctx, long capacity, double mass, gev_pcls **out);
int gev_pcls_destroy(gev_pcls *p);
/* copies n records in, wraps nothing, links them to their cells (counting sort) */
int gev_pcls_upload(gev_pcls *p, const gev_part *host, long n);
/* copies the records out in (cell, ID) order */
int gev_pcls_download(gev_pcls *p, gev_part *host, long *n);
int gev_pcls_count(gev_pcls *p, long *n);

/* ---- stress-energy deposits; each accumulates into its target like the reference
 *      and includes the periodic halo fold of the matching *_comm ---- */
/* projection_T00_project + projection_T00_comm, gevolution.hpp:926-1024 */
int gev_projection_T00(gev_ctx *ctx, gev_pcls *p, gev_field *T00, double a, const gev_field *phi, double coeff);
/* projection_T0i_project + projection_T0i_comm, gevolution.hpp:1045-1149 */
int gev_projection_T0i(gev_ctx *ctx, gev_pcls *p, gev_field *T0i, const gev_field *phi, double coeff);
/* projection_Tij_project + projection_Tij_comm, gevolution.hpp:1172-1301 */
int gev_projection_Tij(gev_ctx *ctx, gev_pcls *p, gev_field *Tij, double a, const gev_field *phi, double coeff);
/* scalarProjectionCIC_project + _comm (LATfield2; main.cpp:402, ic_basic.hpp:2180) */
int gev_projection_mass(gev_ctx *ctx, gev_pcls *p, gev_field *rho);
/* projection_init + projection_T00_project and projection_init + projection_Tij_project
 * (+ _comm), coefficient 1, as main.cpp:378-450 calls them: both targets are replaced,
 * in one sweep over the particles (the mixed form; the FP64 form runs the two deposits) */
int gev_projection_T00_Tij(gev_ctx *ctx, gev_pcls *p, gev_field *T00, gev_field *Tij, double a, const gev_field *phi);

/* ---- real-space sources ---- */
/* prepareFTsource (tensor), gevolution.hpp:56-147; Sij may equal Tij */
int gev_prepare_source_tensor(gev_ctx *ctx, const gev_field *phi, const gev_field *Tij, gev_field *Sij, double coeff);
/* prepareFTsource (scalar), gevolution.hpp:169-192; result may equal source */
int gev_prepare_source_scalar(gev_ctx *ctx, const gev_field *phi, const gev_field *chi, const gev_field *source,
                              double bgmodel, gev_field *result, double coeff, double coeff2, double coeff3);

/* ---- FFT (PlanFFT<Cplx>::execute, main.cpp:477-596); all components ---- */
int gev_fft_r2c(gev_ctx *ctx, const gev_field *real, gev_field *spectrum);
/* backward transform; never modifies its input spectrum */
int gev_fft_c2r(gev_ctx *ctx, const gev_field *spectrum, gev_field *real);
/* solveModifiedPoissonFT(srcFT, potFT, coeff, modif) then the c2r of potFT (main.cpp:483-488)
 * without writing potFT: srcFT is kept.  The mixed form on power-of-two grids applies the
 * Poisson factor inside the transform's first pass; the bits are those of the two calls. */
int gev_fft_c2r_poisson(gev_ctx *ctx, const gev_field *srcFT, gev_field *real, double coeff, double modif);
/* one unnormalised 1-D transform of a half spectrum along y (axis 1) or z (axis 2), in place,
 * sign -1 forward / +1 backward: one of the passes of the 3-D transforms above */
int gev_fft_axis(gev_ctx *ctx, gev_field *spectrum, int axis, int sign);

/* ---- k-space operators ---- */
int gev_solve_poisson(gev_ctx *ctx, const gev_field *srcFT, gev_field *potFT, double coeff,
                      double modif); /* solveModifiedPoissonFT, gevolution.hpp:501 */
int gev_project_scalar(gev_ctx *ctx, const gev_field *SijFT, gev_field *chiFT,
                       int add); /* projectFTscalar, gevolution.hpp:211 */
int gev_evolve_vector(gev_ctx *ctx, const gev_field *SijFT, gev_field *BiFT,
                      double a2dtau); /* evolveFTvector, gevolution.hpp:284 */
/* projectFTscalar(SijFT, chiFT) and evolveFTvector(SijFT, BiFT, a2dtau) as main.cpp:558 and 586
 * call them in the parabolic vector method, in one pass over SijFT; the same bits as the two */
int gev_project_scalar_evolve_vector(gev_ctx *ctx, const gev_field *SijFT, gev_field *chiFT, gev_field *BiFT,
                                     double a2dtau);
int gev_project_vector(gev_ctx *ctx, const gev_field *SiFT, gev_field *BiFT, double coeff,
                       double modif); /* projectFTvector, gevolution.hpp:350 */
int gev_project_tensor(gev_ctx *ctx, const gev_field *SijFT,
                       gev_field *hijFT); /* projectFTtensor, gevolution.hpp:411 */

/* ---- particle updates ---- */
/* Particles::updateVel(update_q | update_q_Newton, dtau, {phi, chi, Bi}, nfield, {a, a2N});
 * main.cpp:775; *maxvel receives the reduction (sqrt of the maximum q^2/a^2) */
int gev_update_q(gev_ctx *ctx, gev_pcls *p, int kind, double dtau, const gev_field *phi, const gev_field *chi,
                 const gev_field *Bi, int nfield, double a, double a2N, double *maxvel);
/* Particles::moveParticles(update_pos | update_pos_Newton, ...); main.cpp:798; the
 * relink to the new cells is the on-device counting sort */
int gev_update_pos(gev_ctx *ctx, gev_pcls *p, int kind, double dtau, const gev_field *phi, const gev_field *chi,
                   const gev_field *Bi, int nfield, double a, double a2N);
/* updateVel(update_q) then moveParticles(update_pos) with the relink, as main.cpp:775-798
 * runs them in GR (kick at a_kick, background half step on the host, drift at a_drift), in
 * one pass over the particles; phi, chi and Bi are all required.  In the mixed form the
 * relink leaves each cell's particles in atomic order, which changes no result (its
 * deposits add integers); downloads restore the (cell, ID) order.  *maxvel as gev_update_q,
 * or NULL to return without waiting. */
int gev_update_q_pos(gev_ctx *ctx, gev_pcls *p, double dtau_kick, double a_kick, int nfield_kick, double dtau_drift,
                     double a_drift, int nfield_drift, const gev_field *phi, const gev_field *chi, const gev_field *Bi,
                     double *maxvel);

/* ---- reductions ---- */
/* sum of one component over all cells (T00hom, main.cpp:459-463); deterministic order */
int gev_field_sum(gev_ctx *ctx, const gev_field *f, int comp, double *out);

/* ---- spectra ---- */
/* extractCrossSpectrum (tools.hpp:53-212) / extractPowerSpectrum (237-240) over device
 * spectra, without copying them to the host: numbins bins of |k| up to sqrt(3) k_Nyquist,
 * linear k (ktype 1, KTYPE_LINEAR) or grid k (ktype 0, KTYPE_GRID), the CIC window
 * deconvolved when deconvolve != 0.  comp1, comp2 >= 0 correlate one component of each
 * field; otherwise all components are summed (f1 and f2 with equal counts) and
 * symmetric != 0 reads 6 components as the symmetric tensor 00 01 02 11 12 22 with the
 * off-diagonal terms counted twice.  f2 may be f1.  Fills host arrays of numbins entries
 * as the reference does: mean k, mean power, k scatter, power scatter, modes per bin.
 * The per-bin sums are exact integer sums (bit-reproducible); waits for the stream. */
int gev_cross_spectrum(gev_ctx *ctx, const gev_field *f1, const gev_field *f2, double *kbin, double *power,
                       double *kscatter, double *pscatter, int *occupation, int numbins, int deconvolve, int ktype,
                       int symmetric, int comp1, int comp2);

/* ---- reduction that allocates nothing (no counterpart in gevolution-1.2) ----
 * For host codes that must not allocate device memory while they run: their
 * fields fill the GPU and all device memory belongs to their own pool (or to
 * PyTorch's caching allocator), where a cudaMalloc behind the pool's back can
 * fail, and cudaMalloc / cudaFree may synchronise the device in the middle of a
 * queued time step.  Needs no context and calls no allocating routine.
 *
 * Sums the n values at device pointer `data` (double for GEV_PREC_FP64, float for
 * GEV_PREC_MIXED) in FP64 and a fixed order that depends only on n, and writes
 * the sum to out[0] (device memory) on `cuda_stream` (NULL: the legacy default
 * stream) of GPU `device`.  Returns when the work is enqueued; the caller
 * synchronises.  n may be 0 (sum 0); n above GEV_SUM_NOALLOC_MAX_N is rejected
 * with GEV_EINVAL.  On error a message goes to errbuf (may be NULL).
 *
 * Scratch: 1 MiB of partial sums in a static device array, held on every GPU
 * that loads the library until the process exits.  The first call on a device,
 * with any n and either precision, does all of the set-up: it loads the
 * function's kernels and the array onto the GPU (CUDA loads modules lazily, and
 * loading allocates) and looks up the array's device address
 * (cudaGetSymbolAddress); later calls load and allocate nothing.  Make that first
 * call before any stream capture.  All calls on a GPU share the one array: calls whose work
 * overlaps on that GPU (other streams, other host threads) race and must be
 * serialised by the caller.  Nothing in it has to start at zero. */
#define GEV_SUM_NOALLOC_MAX_N 1073741824LL /* 2^30 values, e.g. one component of a 1024^3 field */
int gev_sum_noalloc(int device, const void *data, int precision, size_t n, double *out, void *cuda_stream,
                    char *errbuf, size_t errbuf_len);

#ifdef __cplusplus
}
#endif
#endif
