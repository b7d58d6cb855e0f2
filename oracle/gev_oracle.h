/*
 * gev_oracle.h -- CPU restatement (FP64, single core) of gevolution 1.2's
 * per-step particle-mesh path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
 * The product path never calls it and has no CPU fallback.
 *
 * Every function cites the reference file:line whose arithmetic it restates
 * (paths are relative to the gevolution-1.2 source tree).  Parts of the path
 * that live in the external library LATfield2 v1.1 (particle lists and their
 * relink, CIC halo folds, FFT conventions) are restated from the call sites in
 * gevolution.hpp / main.cpp / ic_basic.hpp; their conventions are fixed here:
 *
 *   - Real fields: flat periodic arrays, no halo, x fastest:
 *       f[c*N^3 + x + N*(y + N*z)]
 *   - Symmetric tensors: 6 components in the order 00, 01, 02, 11, 12, 22.
 *   - Half spectra (r2c): interleaved complex, kx fastest, kx in [0, N/2]:
 *       F[c*N*N*NH + kx + NH*(ky + N*kz)],  NH = N/2 + 1
 *     coordinates kx, ky, kz play the roles of rKSite coord(0), (1), (2).
 *   - FFT: unnormalised, FFTW sign convention (forward e^{-i...}); the c2r
 *     never modifies its complex input.
 *   - Particles: records {pos[3], vel[3], ID} (part_simple), pos in box units
 *     [0,1), vel = q/m.  A particle belongs to cell floor(pos/dx) (clamped to
 *     N-1).  Each cell's list is ordered by ascending ID; the store is the
 *     concatenation of the lists in site order (x fastest).
 *   - Deposits accumulate into a field with an upper halo and fold the halo
 *     back in the order x, y, z (the *_comm folds).
 *   - updateVel returns sqrt(max over particles of the callback's value).
 *   - moveParticles wraps pos into [0,1) per axis (p>=1 -> p-1, p<0 -> p+1,
 *     then once more p>=1 -> p-1) and relinks.
 */
#ifndef GEV_ORACLE_H
#define GEV_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  double pos[3];
  double vel[3];
  int64_t ID;
} gevo_part;

/* ---- FFT (project-written mixed-radix, double) ---- */
void gevo_fft1d(int L, double *data, int sign); /* in place, sign -1 forward */
void gevo_fft_r2c(int N, const double *in, double *out);
void gevo_fft_c2r(int N, const double *in, double *out);

/* ---- k-space operators (gevolution.hpp:211-535) ---- */
void gevo_kspace_tables(int N, double *gridk2, double *kshift /* 2N */);
void gevo_poisson(int N, const double *srcFT, double *potFT, double coeff, double modif);
void gevo_project_scalar(int N, const double *SijFT, double *chiFT, int add);
void gevo_evolve_vector(int N, const double *SijFT, double *BiFT, double a2dtau);
void gevo_project_vector(int N, const double *SiFT, double *BiFT, double coeff, double modif);
void gevo_project_tensor(int N, const double *SijFT, double *hijFT);

/* ---- real-space sources (gevolution.hpp:56-192) ---- */
void gevo_prepare_source_tensor(int N, const double *phi, const double *Tij, double *Sij, double coeff);
void gevo_prepare_source_scalar(int N, const double *phi, const double *chi, const double *source,
                                double bgmodel, double *result, double coeff, double coeff2,
                                double coeff3);

/* ---- particle store ---- */
int gevo_cell_of(int N, double p);
void gevo_wrap(double *p);
/* sort by (cell, ID); fills cell_start[N^3+1] if non-NULL */
void gevo_sort(int N, long np, gevo_part *p, long *cell_start);

/* ---- deposits (gevolution.hpp:926-1297; LATfield2 scalarProjectionCIC_*) ---- */
void gevo_deposit_T00(int N, long np, const gevo_part *p, const long *cell_start, double mass,
                      double a, const double *phi, double coeff, double *T00);
void gevo_deposit_T0i(int N, long np, const gevo_part *p, const long *cell_start, double mass,
                      const double *phi, double coeff, double *T0i);
void gevo_deposit_Tij(int N, long np, const gevo_part *p, const long *cell_start, double mass,
                      double a, const double *phi, double coeff, double *Tij);
void gevo_deposit_mass(int N, long np, const gevo_part *p, const long *cell_start, double mass,
                       double *rho);

/* ---- particle updates (gevolution.hpp:570-903) ----
 * kind 0 = GR (update_q / update_pos), 1 = Newton (update_q_Newton / update_pos_Newton).
 * fields: phi, chi, Bi (3 comps); nfield as in Particles::updateVel/moveParticles.
 * params: {a, a^2 N}.  kick returns sqrt(max v^2/a^2). drift relinks (sorts). */
double gevo_kick(int N, long np, gevo_part *p, int kind, double dtau, const double *phi,
                 const double *chi, const double *Bi, int nfield, double a, double a2N);
void gevo_drift(int N, long np, gevo_part *p, int kind, double dtau, const double *phi,
                const double *chi, const double *Bi, int nfield, double a, double a2N,
                long *cell_start);

/* ---- background (background.hpp:137-177), no ncdm / fluid ---- */
typedef struct {
  double Omega_cdm, Omega_b, Omega_m, Omega_Lambda, Omega_rad;
} gevo_cosmo;
double gevo_hconf(double a, double fourpiG, const gevo_cosmo *c);
void gevo_rk4bg(double *a, double fourpiG, const gevo_cosmo *c, double dtau);

/* ---- full simulation state and one GR time step (main.cpp:372-879) ---- */
typedef struct {
  int N;
  long np;
  gevo_part *p;
  long *cell_start; /* N^3 + 1 */
  double mass;      /* particle mass in units of the critical density */
  double *phi, *chi, *source, *Sij, *Bi; /* real fields */
  double *scalarFT, *SijFT, *BiFT;        /* half spectra */
  double a, tau, dtau, dtau_old, fourpiG, Cf, steplimit, z_relax, maxvel, T00hom, phik0;
  gevo_cosmo cosmo;
  int vector_elliptic;
  int cycle;
  /* wall time in seconds of the phases of main.cpp's BENCHMARK breakdown
   * (main.cpp:907-922), summed over cycles: [0] projections, [1] gravity solver,
   * [2] thereof FFTs, [3] update momenta, [4] move particles; fft_count counts the
   * 3-D transforms as main.cpp does */
  double t_phase[5];
  long fft_count;
} gevo_sim;

int gevo_sim_alloc(gevo_sim *s, int N, long np);
void gevo_sim_free(gevo_sim *s);
/* one cycle of the main loop body (GR): deposits, phi/chi/B solves, kick, drift,
 * background, next dtau.  Returns 0. */
int gevo_sim_step(gevo_sim *s);
/* the same cycle in two parts, for a loop that takes spectra where main.cpp
 * writes them: main.cpp:372-598 (deposits, phi, chi, B) and main.cpp:743-872
 * (kick, background, drift, next dtau) */
int gevo_sim_step_fields(gevo_sim *s);
int gevo_sim_step_particles(gevo_sim *s);
double gevo_next_dtau(const gevo_sim *s);

/* ---- initial conditions (restating the mPk path of ic_basic.hpp) ----
 * the displacement potential from the sitmo stream, the CIC kernel and the
 * spline of a tabulated BBKS spectrum; see gev_ic.c */
typedef struct {
  double h, Omega_cdm, Omega_b, n_s, sigma8, z_in, boxsize, Cf, steplimit;
  uint64_t seed;     /* the sitmo seed is its low 32 bits, (unsigned int) ic.seed */
  int ksphere;
  int correct_displacement; /* ICFLAG_CORRECT_DISPLACEMENT: the template's CIC kernel */
} gevo_icparams;
/* BBKS linear P(k) [(Mpc/h)^3] at z_in for k [h/Mpc], sigma8-normalised */
double gevo_ic_pk(const gevo_icparams *ic, double k);
/* amplitude factor A*D(z_in)^2/D(0)^2 so that P = amp * k^n_s T(k)^2 */
double gevo_ic_pk_amplitude(const gevo_icparams *ic);
double gevo_bbks_T(double k, double Gamma);
void gevo_ic_potential_k(int N, const gevo_icparams *ic, double *potFT);
int gevo_ic_generate(gevo_sim *s, const gevo_icparams *ic);

/* the sitmo stream (prng_engine.hpp) and generateDisplacementField's layout of it */
void gevo_sitmo_block(uint32_t seed, uint64_t block, uint64_t out[4]);
uint32_t gevo_sitmo_draw(uint32_t seed, uint64_t d);
void gevo_spline_init(int n, const double *x, const double *y, double *c);
double gevo_spline_eval(int n, const double *x, const double *y, const double *c, double v);
void gevo_displacement_field(int N, double *F, double coeff, int n, const double *x, const double *y, uint32_t seed,
                             int ksphere);
void gevo_cic_kernel(int N, long numpcl, const float *pcldata, int numtile, double K[27]);

/* ---- power spectrum (tools.hpp:53-212, extractPowerSpectrum) ---- */
void gevo_power_spectrum(int N, const double *FT, int ncomp, int symmetric, int numbins,
                         int deconvolve, double *kbin, double *power, double *kscatter,
                         double *pscatter, int *occupation);

/* ---- Gadget-2 snapshots (Particles_gevolution.hpp:30-251, 574-665) ----
 * the 256-byte header (metadata.hpp:152-171) */
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
  char fill[64];
} gevo_gadget2_header;
/* saveGadget2 of one rank: particles in any order (written in (cell, ID)
 * order); exact = the EXACT_OUTPUT_REDSHIFTS build (needs phi, N^3 values x
 * fastest); id_bytes = GADGET_ID_BYTES.  Returns 0, or -1 on a bad header, a
 * tracer count that differs from npart[1], or an I/O error. */
int gevo_gadget2_save(const char *fname, int N, long np, const gevo_part *p, const double *phi,
                      const void *hdr256, int tracer_factor, double dtau_pos, double dtau_vel, int exact,
                      int id_bytes);
/* loadGadget2: the particles in (cell, ID) order (at most cap), the header;
 * returns their number or -1 */
long gevo_gadget2_load(const char *fname, int N, gevo_part *dst, long cap, void *hdr256, int id_bytes);

/* hibernation of B and its restart (the parabolic vector method): hibernate
 * divides B by a^2 N before writing it (hibernation.hpp:529-538); readIC multiplies
 * the stored B by a^2 / (N N) and transforms it forward into BiFT
 * (ic_read.hpp:307-318).  Both modify Bi (3 components). */
void gevo_hibernate_b(int N, double *Bi, double a);
void gevo_restart_bift_from_b(int N, double *Bi, double a, double *BiFT);

/* writePowerSpectrum (tools.hpp:268-345); exact = the EXACT_OUTPUT_REDSHIFTS build */
int gevo_write_power_spectrum(const double *kbin, const double *power, const double *kscatter, const double *pscatter,
                              const int *occupation, int numbins, double rescalek, double rescalep,
                              const char *filename, const char *description, double a, double z_target, int exact);

#ifdef __cplusplus
}
#endif
#endif
