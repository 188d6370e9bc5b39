/*
 * mctomo.h - C ABI of the GB300 forward-modelling library for MCTomo's
 * rjMCMC hot path (libmctomo_gpu.so).
 *
 * Every entry point returns an int status: MCT_OK (0); MCT_MODEL_INVALID (1),
 * the analogue of the reference's like = huge(like) (the sampler rejects the
 * proposal); or a negative error. No entry point exits the process.
 *
 * Arrays use the reference's Fortran layouts (column-major; grids (nz,ny,nx)),
 * 1-based site indices, FP64 at the boundary unless stated. Calls taking host
 * pointers are synchronous and thread-safe. Calls suffixed _device take device
 * pointers and a cudaStream_t (passed as void*) and run asynchronously.
 */
#ifndef MCTOMO_H_
#define MCTOMO_H_

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MCT_OK 0
#define MCT_MODEL_INVALID 1
#define MCT_ERR_ARG (-1)
#define MCT_ERR_CUDA (-2)
#define MCT_ERR_NOMEM (-3)
#define MCT_ERR_OUTSIDE (-4)
#define MCT_ERR_UNSUPPORTED (-5)
#define MCT_ERR_TIMEOUT (-6)
#define MCT_ERR_INTERNAL (-7)

/* Library version string. */
const char *mct_version(void);

/* Text of the last error recorded by this thread (empty if none). */
const char *mct_last_error(void);

/* ------------------------------------------------------------------------
 * Voronoi -> grid map (nearest nucleus), replaces kdtree_to_grid
 * (src/mcmc_loc2.f90:2002-2082 for d=3, mcmc2d/mcmc.f90:1469-1525 for d=2)
 * and its kdtree2 search (src/kdtree2.f90:1028-1069,1369-1599), including
 * kdtree2's tie rule. points: (d, n) column-major = RTI%points(:,1:ncells);
 * params: (3, n) = RTI%parameters (vp, vs, rho). grid_lo = (xmin,ymin,zmin),
 * grid_step = (dx,dy,dz). box: 1-based inclusive (ix0,ix1,iy0,iy1,iz0,iz1),
 * or NULL for the whole grid. Outputs are (nz,ny,nx) (or (ny,nx) for d=2);
 * nodes outside the box are not written. vp/vs/rho may be NULL.
 * ---------------------------------------------------------------------- */
int mct_kdtree_to_grid(int d, int n, const double *points, const double *params,
                       int nx, int ny, int nz, const double *grid_lo,
                       const double *grid_step, const int *box, int *sites_id,
                       double *vp, double *vs, double *rho);

/* Batched form on device memory: nchains chains, nucleus arrays strided by
 * ncell_max (points [nchains][ncell_max][d], params [nchains][ncell_max][3]),
 * boxes [nchains][6] or NULL, outputs [nchains][grid]. The launch is
 * asynchronous on stream; the device-side inputs are checked on the device:
 * a box reaching outside the grid is clipped to it, and a chain whose
 * clipped box is empty or whose ncells lies outside [1, ncell_max] is
 * skipped (its outputs untouched) with MCT_ERR_ARG recorded. A node whose
 * tie resolution fails (a kd-tree deeper than the fixed search stacks, only
 * on degenerate nucleus sets) gets sites_id 0 and vp = vs = rho = 0, with
 * MCT_ERR_INTERNAL recorded. mct_grid_status reads what was recorded. */
int mct_grid_nearest_batch_device(int d, int nchains, int ncell_max,
                                  const int *ncells, const double *points,
                                  const double *params, int nx, int ny, int nz,
                                  const double *grid_lo, const double *grid_step,
                                  const int *box, int *sites_id, double *vp,
                                  double *vs, double *rho, void *stream);

/* Waits for stream, then returns in *status the first error recorded on the
 * device by any gridding call since the previous mct_grid_status (MCT_OK if
 * none) and clears it. No counterpart in the reference, whose kdtree2 runs
 * on the host and stops the program on errors. */
int mct_grid_status(void *stream, int *status);

/* Same as mct_grid_nearest_batch_device, same arguments and results, but it
 * allocates no device memory: its scratch is a fixed array of
 * MCT_GRID_NOALLOC_SCRATCH_BYTES per device inside the library. No counterpart
 * in the reference (which grids on the host); it serves callers that may not
 * allocate while they run (pre-reserved device memory, proposals enqueued
 * ahead on one stream). A call needing more scratch than the array holds
 * (about 4 B per node per chain plus the kd-tree storage) returns
 * MCT_ERR_ARG. The first call on a device does a one-time address lookup;
 * make it before any stream capture; the address is not looked up again, so
 * calls after a cudaDeviceReset in the same process are not supported. All
 * calls on a device share the array: calls that overlap in time race and
 * must be ordered by the caller. Device-side errors: as the allocating form,
 * read with mct_grid_status. */
#define MCT_GRID_NOALLOC_SCRATCH_BYTES (32u * 1024u * 1024u)
int mct_grid_nearest_batch_device_noalloc(int d, int nchains, int ncell_max,
                                          const int *ncells, const double *points,
                                          const double *params, int nx, int ny, int nz,
                                          const double *grid_lo, const double *grid_step,
                                          const int *box, int *sites_id, double *vp,
                                          double *vs, double *rho, void *stream);

/* ------------------------------------------------------------------------
 * Surface-wave dispersion of one layered column, replaces surfdisp96
 * (surfmodes/surfdisp96.f:52-382) with its argument list: REAL*4 model
 * (thkm, vpm, vsm, rhom of nlayer, last layer the half-space), iflsph must be
 * 0 (flat earth), iwave 1 Love / 2 Rayleigh, mode = 1, igr 0 phase / 1 group,
 * kmax periods t[kmax] (<= 60), dphase the search increment. cp/cg receive
 * the phase / group velocities; *ierr the reference's error flag.
 * ---------------------------------------------------------------------- */
int mct_surfdisp96(const float *thkm, const float *vpm, const float *vsm,
                   const float *rhom, int nlayer, int iflsph, int iwave,
                   int mode, int igr, int kmax, const double *t, double dphase,
                   double *cp, double *cg, int *ierr);

/* Multimode variant, replaces surfdisp_mmodes (surfdisp96.f:385-701):
 * cp/cg are (kmax, mode) column-major. */
int mct_surfdisp_mmodes(const float *thkm, const float *vpm, const float *vsm,
                        const float *rhom, int nlayer, int iflsph, int iwave,
                        int mode, int igr, int kmax, const double *t,
                        double dphase, double *cp, double *cg, int *ierr);

/* The surface-mode search parameters, T_MODES_PARA
 * (surfmodes/surfmodes.f90:23-30). The reference's surface likelihood sets
 * tolmin = tol, tolmax = 10 tol, smin_min = 1e-3f, smin_max = 5e-3f and
 * dc = dcm = dc1 = dc2 = dPhaseVel (src/likelihood_surf.F90:173-182). */
typedef struct {
  int modetype;      /* 1 Rayleigh, 0 Love */
  int nmodes;        /* modes (the generalized R/T path computes the fundamental) */
  int phase_group;   /* 0 phase only, 1 phase and group */
  double tolmin, tolmax, smin_min, smin_max;
  double dc, dcm, dc1, dc2;
} mct_modes_para;

/* surfmodes (surfmodes/surfmodes.f90:39-108) with the reference's routing:
 * a column without a low-velocity layer slower than the top layer
 * (setup_grt's nlvls1 = 0, :320-450) goes to surfdisp96 with the model cast
 * to REAL*4; a column with one goes to the generalized R/T fundamental-mode
 * search (RayleighModes / LoveModes, :185-303), FP64 throughout. freqs[np]
 * in Hz (np <= 60). Fluid layers (vs = 0) return MCT_ERR_UNSUPPORTED. */
int mct_surfmodes_para(const double *thick, const double *vp, const double *vs,
                       const double *rho, int nlayers, const double *freqs, int np,
                       const mct_modes_para *paras, double *phase, double *group,
                       int *ierr);

/* surfmodes with the example decks' tolerance (LIKE_SET%TOL = 1e-6,
 * examples/example1/MCTomo.inp:55): mct_surfmodes_para with tolmin 1e-6,
 * tolmax 1e-5, smin 1e-3f / 5e-3f and dc for every increment. */
int mct_surfmodes(const double *thick, const double *vp, const double *vs,
                  const double *rho, int nlayers, const double *freqs, int np,
                  int modetype, int phase_group, double dc, double *phase,
                  double *group, int *ierr);

/* surfmodes' routing for many columns (host only): route[c] = 1 where
 * setup_grt counts a low-velocity layer slower than the top layer (nlvls1 >
 * 0, surfmodes/surfmodes.f90:320-450; the generalized R/T search), 0 where
 * not (surfdisp96), -2 where such a column has a fluid layer (the
 * Stoneley-mode path, not built). Layer arrays [ncol][nl_max] FP64. */
int mct_surfmodes_route(int ncol, int nl_max, const int *nl, const double *vp,
                        const double *vs, int modetype, int *route);

/* The generalized R/T fundamental-mode search (RayleighModes / LoveModes,
 * surfmodes/surfmodes.f90:185-303, allmodes 0) for many columns, whatever
 * their layering: layer arrays [ncol][nl_max] FP64 (last layer of each
 * column the half-space), nl[ncol]; freqs[np] in Hz; phase / group
 * [ncol][np] (entries after a frequency without a root stay 0); ierr[ncol]:
 * 0, 1 (no root, the reference's ierr), 2 (the trial-velocity list would
 * exceed the reference's 20,000 entries), -1 (a layer count outside
 * 2..nl_max), -2 (a fluid layer, not built).
 * nevals (optional) receives the secular-function evaluations. */
int mct_grt_batch(int ncol, int nl_max, const int *nl, const double *thk,
                  const double *vp, const double *vs, const double *rho, int np,
                  const double *freqs, const mct_modes_para *paras, double *phase,
                  double *group, int *ierr, unsigned long long *nevals);

/* Device-pointer variant on the caller's stream (asynchronous; scratch is
 * allocated and freed in stream order). nevals, if given, is a device
 * counter that the kernel adds to. */
int mct_grt_batch_device(int ncol, int nl_max, const int *nl, const double *thk,
                         const double *vp, const double *vs, const double *rho,
                         int np, const double *freqs, const mct_modes_para *paras,
                         double *phase, double *group, int *ierr,
                         unsigned long long *nevals, void *stream);

/* Many columns at once (host buffers): layer arrays [ncol][nl_max] REAL*4,
 * nl[ncol]; cp/cg [ncol][mode][np]; ierr[ncol]. precision 0 = FP64 root
 * search as the reference; 1 = FP32 bracketing confirmed in FP64, then FP64
 * polish (same roots). ndltar (optional, 2 entries) counts the FP64 and
 * FP32 period-equation evaluations the root searches used; with precision 0
 * the FP64 count is the reference's own (values the kernel evaluates ahead
 * of a scan and the scan never reaches are not counted). */
int mct_surfdisp_batch(int ncol, int nl_max, const int *nl, const float *thk,
                       const float *vp, const float *vs, const float *rho,
                       int np, const double *periods, int iwave, int mode,
                       int igr, double dphase, int multimode, int precision,
                       double *cp, double *cg, int *ierr,
                       unsigned long long *ndltar);

/* Same on device memory, asynchronous on stream. */
int mct_surfdisp_batch_device(int ncol, int nl_max, const int *nl,
                              const float *thk, const float *vp,
                              const float *vs, const float *rho, int np,
                              const double *periods, int iwave, int mode,
                              int igr, double dphase, int multimode,
                              int precision, double *cp, double *cg, int *ierr,
                              unsigned long long *ndltar, void *stream);


/* ------------------------------------------------------------------------
 * 2D first-arrival travel times, replaces fm2d's modrays
 * (fm2d/fm2dray_cartesian.f90:67-480) with its Cartesian argument list:
 * sources (scx, scz)[nsrc], receivers (rcx, rcz)[nrc], srsin (nrc*nsrc, 2)
 * column-major (column 1: path exists, source-major), velvin the padded
 * vertex grid (nvz+2, nvx+2) column-major, grid dicing gdx/gdz, source-grid
 * refinement asgr with level sgdl and extent sgs, fom 0 first / 1 mixed
 * order. ttime (nrc, nsrc) is written where a path exists. tfield (optional)
 * receives the final (nnz, nnx) field per source. Only uar = 1 (no ray paths)
 * and wrgf = 0 are supported; earth and snb are accepted and unused, as in
 * the Cartesian reference. MCT_ERR_OUTSIDE when a source or receiver lies
 * outside the grid (the reference stops the program).
 * ---------------------------------------------------------------------- */
int mct_modrays(int nsrc, const double *scx, const double *scz, int nrc,
                const double *rcx, const double *rcz, const int *srsin,
                int wrgf, int nvx, int nvz, double goxd, double gozd,
                double dvxd, double dvzd, const double *velvin, int gdx,
                int gdz, int asgr, int sgdl, int sgs, double earth, int fom,
                double snb, double *ttime, int uar, int *crazyray,
                double *tfield);

/* Many velocity maps (e.g. every period of every chain) sharing the
 * stations: velv [nmaps][(nvx+2)*(nvz+2)], srs [srs_nmaps][nsrc][nrc] path
 * flags (map m uses set m % srs_nmaps), ttime [nmaps][nsrc][nrc], tfield
 * optional [nmaps][nsrc][nnx*nnz]. precision 0 evaluates the upwind updates
 * in FP64 as the reference; 1 solves each update's quadratic in FP32 on
 * times shifted to a neighbouring accepted time (times stay FP64); 2 does the
 * same with int32 fixed-point times (half the shared memory per solve). */
int mct_modrays_batch(int nmaps, int nsrc, const double *scx,
                      const double *scz, int nrc, const double *rcx,
                      const double *rcz, int srs_nmaps, const int *srs,
                      int nvx, int nvz, double goxd, double gozd, double dvxd,
                      double dvzd, const double *velv, int gdx, int gdz,
                      int asgr, int sgdl, int sgs, int fom, double *ttime,
                      double *tfield, int precision);

/* Group delays along ray paths: modrays with uar = 0 (ray paths traced from
 * each receiver down the phase travel-time field, fm2d/fm2dray_cartesian.f90
 * rpaths 801-1455) followed by CalGroupTime (src/likelihood_surf.F90:455-494)
 * on the group-velocity maps gvel[nmaps][nvx][nvz] (Fortran (nvz, nvx), the
 * model grid). Arguments as mct_modrays_batch; ttime receives the phase
 * times, gtime the group times and raylen the ray lengths
 * ([nmaps][nsrc][nrc]), crazy[nmaps] the rays that reached the point limit
 * (the reference's crazyray; their gtime and raylen are 0). */
int mct_modrays_group_batch(int nmaps, int nsrc, const double *scx, const double *scz, int nrc,
                            const double *rcx, const double *rcz, int srs_nmaps, const int *srs, int nvx,
                            int nvz, double goxd, double gozd, double dvxd, double dvzd,
                            const double *velv, const double *gvel, int gdx, int gdz, int asgr, int sgdl,
                            int sgs, int fom, double *ttime, double *gtime, double *raylen, int *crazy,
                            int precision);


/* ------------------------------------------------------------------------
 * Surface-wave likelihood with device-resident chains, replaces
 * likelihood() case 2 (src/likelihood.f90:57-93) -> surf_likelihood
 * (src/likelihood_surf.F90:110-410) and the kdtree_to_grid call before it.
 * ---------------------------------------------------------------------- */
typedef struct {
  int nx, ny, nz;                    /* T_GRID (src/settings.f90:20-28) */
  double xmin, ymin, zmin, dx, dy, dz;
  double scaling, water_depth;
} mct_grid;

#define MCT_LAW_EXPLICIT 0   /* vp, vs, rho taken from the nucleus parameters */
#define MCT_LAW_REFERENCE 1  /* vp = 1.73 vs, rho = 1.74 vp^0.25 (src/utils.f90:98-135) */
#define MCT_LAW_FIXED_RHO 2  /* vp = 1.73 vs, rho = rho_value */

typedef struct {
  int raylov;          /* 1 Rayleigh, 0 Love (T_LIKE_SET%raylov) */
  int phase_group;     /* 0 phase velocity; 1 group velocity: times along the
                          rays of the phase field (rpaths + CalGroupTime),
                          sigma uses the ray length */
  double dphase;       /* dPhaseVel */
  int gridx, gridy, sgref, sgdic, sgext, order;   /* fm2d settings */
  int sigdep;          /* 0 data sigma, else sigma = n0*srdist + n1 (srdist:
                          phase time, ray length for phase_group 1,
                          source-receiver distance for straight rays) */
  int material_law;    /* MCT_LAW_* */
  double rho_value;
  int precision;       /* dispersion root search: 0 FP64, 1 FP32 bracketing */
  int tt_precision;    /* fm2d updates: 0 FP64, 1 double-float, 2 FP32 + fixed-point times */
  int straight;        /* isStraight: 1 = straight rays, no fast marching */
} mct_surf_settings;

typedef struct {
  int nsrc, nrev, np;
  const double *src;      /* (2, nsrc) station x, y */
  const double *rev;      /* (2, nrev) */
  const double *freqs;    /* (np) frequencies, Hz */
  const int *raystat;     /* (nsrc*nrev, np): 1 where a path is observed */
  const double *ttime;    /* (nsrc*nrev, np) observed times */
  const double *sigma;    /* (nsrc*nrev, np) data sigma, or NULL */
  int nrays;
} mct_surf_data;

typedef struct mct_surf_ctx mct_surf_ctx;

/* Allocates nslots device-resident chain slots of at most ncell_max nuclei. */
int mct_surf_create(const mct_grid *grid, const mct_surf_settings *settings,
                    const mct_surf_data *data, int nslots, int ncell_max,
                    mct_surf_ctx **ctx);
int mct_surf_destroy(mct_surf_ctx *ctx);
/* Runs the context's work on a stream of the device's highest priority
 * (high != 0) or of normal priority (the default), after its pending work.
 * No counterpart in the reference: for the served loop, where contexts of
 * different kinds share the GPU. Refused while a submitted batch is pending. */
int mct_surf_set_priority(mct_surf_ctx *ctx, int high);
/* Limits the context's 2D travel-time launches to a share of the device's
 * SMs (share in (0, 1): that share of the SM count times the kernels'
 * resident blocks per SM; 0 or 1: the whole device, the default), so that
 * other contexts' kernels on other streams find free SMs while they run.
 * Results do not depend on it. No counterpart in the reference: for the
 * served loop. MCT_ERR_ARG outside [0, 1]. */
int mct_surf_set_sm_share(mct_surf_ctx *ctx, double share);

/* Evaluates one proposal per listed chain against its slot's committed
 * state. points / params: [nchains][ncell_max][3] (x, y, z) and
 * (vp, vs, rho); n0 / n1: [nchains][np] noise hyper-parameters. out:
 * [nchains][4] = like (-log L, DBL_MAX when the model is rejected), misfit,
 * unweighted misfit, status (0 valid; bit 1 check_model, bit 2 dispersion
 * failure, bit 4 crazy ray, bit 8 zero sigma). Host pointers, synchronous. */
int mct_surf_forward(mct_surf_ctx *ctx, int nchains, const int *slots,
                     const int *ncells, const double *points,
                     const double *params, const double *n0,
                     const double *n1, double *out);
/* Accept (1) or reject (0) each proposal of the last forward. */
int mct_surf_commit(mct_surf_ctx *ctx, const int *accept);
/* Device-pointer forms, asynchronous on stream (NULL = the context's stream)
 * and free of host synchronisation. */
int mct_surf_forward_device(mct_surf_ctx *ctx, int nchains, const int *slots,
                            const int *ncells, const double *points,
                            const double *params, const double *n0,
                            const double *n1, double *out, void *stream);
int mct_surf_commit_device(mct_surf_ctx *ctx, const int *accept,
                           void *stream);
/* Noise-only likelihood, replaces surf_noise_likelihood
 * (src/likelihood_surf.F90:56-99): each listed slot's committed travel times
 * re-reduced with new noise parameters n0, n1 (nchains x np), sigma = n0 *
 * travel time + n1 for every path; no forward solve. out as mct_surf_forward
 * (unweighted misfit included); status bit 8 for a zero sigma (the
 * reference's fatal error), bit 16 for a slot with nothing committed; the
 * call then returns MCT_MODEL_INVALID. */
int mct_surf_noise_likelihood(mct_surf_ctx *ctx, int nchains, const int *slots,
                              const double *n0, const double *n1, double *out);
/* Last forward's travel times (np, nsrc, nrev) = phaseTime(k,j,i) and phase
 * maps (np, nx, ny) for batch position index; either pointer may be NULL. */
int mct_surf_phase_time(mct_surf_ctx *ctx, int index, double *phase_time,
                        double *phase_vel);
/* Stage timing of the next max_steps forwards (CUDA events, no host
 * synchronisation in the forward), and its read-back: stage_ms[4] = summed
 * milliseconds of gridding, layering + dispersion, fm2d, misfit; launches =
 * kernels launched by forwards and commits since the start. */
int mct_surf_profile_start(mct_surf_ctx *ctx, int max_steps);
int mct_surf_profile_read(mct_surf_ctx *ctx, double *stage_ms, int *steps,
                          long long *launches);
/* The context's CUDA stream. */
int mct_surf_stream(mct_surf_ctx *ctx, void **stream);

/* Serving. No counterpart in the reference, whose sampler calls the
 * likelihood synchronously; these let a host loop keep many chains resident
 * and overlap its own work with the GPU's.
 * mct_surf_device_bytes: the device memory a context with these arguments
 * allocates (no allocation made), so a server can size nslots to the free
 * memory. mct_surf_admit: claims a free slot for a new chain (its first
 * forward computes every column); MCT_ERR_NOMEM when all are claimed.
 * mct_surf_evict: releases a claimed slot. Slots can also be addressed
 * directly without admit/evict. mct_surf_submit: starts the forward of
 * mct_surf_forward and returns at once (the arrays are copied before it
 * returns); one submitted batch per context at a time, and the blocking
 * calls on the context return MCT_ERR_ARG until it is polled.
 * mct_surf_poll: *done = 0 while the batch runs; when it has finished, *done
 * = 1, out (nchains x 4) is filled as by mct_surf_forward and the batch's
 * status is returned; mct_surf_commit then applies to it. A context is used
 * by one host thread at a time. */
int mct_surf_device_bytes(const mct_grid *grid, const mct_surf_settings *settings,
                          const mct_surf_data *data, int nslots, int ncell_max,
                          size_t *bytes);
int mct_surf_admit(mct_surf_ctx *ctx, int *slot);
int mct_surf_evict(mct_surf_ctx *ctx, int slot);
int mct_surf_submit(mct_surf_ctx *ctx, int nchains, const int *slots,
                    const int *ncells, const double *points,
                    const double *params, const double *n0,
                    const double *n1);
int mct_surf_poll(mct_surf_ctx *ctx, double *out, int *done);
/* Posterior statistics, replaces stat_rti (src/mcmc_loc2.f90:1966-2000) for
 * the models held on the device: mct_surf_stat_add adds each listed slot's
 * committed model (after mct_surf_commit) to the slot's sums of vp, vp^2,
 * vs and vs^2 per grid node, in the reference's order of operations, and
 * counts it (RTI%nthin); the caller decides when (after burn-in, every
 * thin-th sample, at temperature 1). The first call allocates the sums
 * (4 x nodes x nslots doubles). mct_surf_stat_read gives a slot's means and
 * mean squares, the sums over the count as write_mean / write_var
 * (src/read_write.f90:223-292) write them (zero when nothing was added),
 * each (nz, ny, nx) in Fortran order; any output may be NULL.
 * mct_surf_stat_reset clears a slot (mct_surf_admit does too). */
int mct_surf_stat_add(mct_surf_ctx *ctx, int nchains, const int *slots);
int mct_surf_stat_read(mct_surf_ctx *ctx, int slot, double *mean_vp, double *mean_vs, double *msq_vp,
                       double *msq_vs, int *nthin);
int mct_surf_stat_reset(mct_surf_ctx *ctx, int slot);


/* ------------------------------------------------------------------------
 * 3D first-arrival travel times, replaces the reference's C entry point
 * fastMarching3D (fastmarching/fastMarching.cpp:26-30) with the same
 * arguments: grid nx,ny,nz with spacing dx,dy,dz and origin xmin,ymin,zmin;
 * vel (nx,ny,nz) C order (= Fortran (nz,ny,nx)); src[3]; rev (nrev,3);
 * order 1 mixed second order, anything else first order (as the
 * reference); ttime[nrev]; tfield (optional) the final field in vel's
 * layout.
 *
 * Two GPU solvers, chosen by a flag OR-ed into order:
 *  MCT_EIK3_HEAP  - the reference's heap march (SFMM) itself, its pops,
 *                   pushes and FP64 updates in the same order: results
 *                   identical to the reference's, both orders. One group
 *                   of 8 lanes marches each solve, so it is fast only for
 *                   many solves at once.
 *  MCT_EIK3_TILES - a tile-based fast iterative method on the same update
 *                   operator (FP32 updates on fixed-point times): first
 *                   order within 1e-4 s of the reference; the mixed second
 *                   order only approximately (within 5e-2 s, typically
 *                   1e-3 s), since the reference's second-order result
 *                   depends on its acceptance order.
 * Without a flag: the heap march for order 1, tiles for first order.
 * An infinite accepted time (a region cut off by obstacles), where the
 * reference asserts, returns MCT_ERR_INTERNAL from the heap march.
 * ---------------------------------------------------------------------- */
#define MCT_EIK3_TILES 0x10
#define MCT_EIK3_HEAP 0x20
int mct_fast_marching3d(int nx, int ny, int nz, double dx, double dy,
                        double dz, double xmin, double ymin, double zmin,
                        const double *vel, const double *src,
                        const double *rev, int nrev, int order, double *ttime,
                        double *tfield);

/* Many solves at once: ngrids velocity grids vel[ngrids][nx][ny][nz], solve
 * i runs on grid solve_grid[i] from src[i][3]; the nrev receivers rev[nrev][3]
 * are shared; ttime[nsolve][nrev]; tfield optional [nsolve][nx][ny][nz];
 * order 0 or 1, optionally OR-ed with MCT_EIK3_TILES or MCT_EIK3_HEAP;
 * passes (optional) receives the number of tile passes run (0 for the heap
 * march). */
int mct_eikonal3d_batch(int nsolve, int nx, int ny, int nz, double dx,
                        double dy, double dz, double xmin, double ymin,
                        double zmin, int ngrids, const double *vel,
                        const int *solve_grid, const double *src, int nrev,
                        const double *rev, int order, double *ttime,
                        double *tfield, int *passes);

/* The tile solver's configuration (tile shape index * 4 + local sweeps
 * index, 0..47: shapes 8x8x8, 4x8x16, 8x4x16, 16x8x4, 8x16x4, 8x8x4, 8x4x8,
 * 4x8x8, 4x4x8, 4x8x4, 8x4x4, 4x4x4; 12, 24, 48 or 96 sweeps per visit). No counterpart in the
 * reference, whose solver has no tuning.
 * cfg = -1: tuned per (device, grid shape, order), the default; the tuner
 * times every configuration on the first call for a key. Configurations
 * differ in the last units of the fixed-point times (2^-shift s), so times
 * can differ by that much between processes whose tuners chose differently:
 * pin one (0..47) for reproducible times. Returns the previous setting. With
 * cfg < -1, returns the configuration tuned on the current device for
 * (nx, ny, nz, order), or -1 if none yet, and changes nothing. */
int mct_eik3_tile_config(int cfg, int nx, int ny, int nz, int order);


/* ------------------------------------------------------------------------
 * Body-wave (P and S) likelihood for many chains, replaces likelihood()
 * cases 0/1 (src/likelihood.f90:57-93) -> body_likelihood
 * (src/likelihood_body.F90:151-337) and the kdtree_to_grid call before it.
 * Events are the sources, stations the receivers; solves run from the
 * stations when events outnumber them (reciprocity), as the reference does.
 * ---------------------------------------------------------------------- */
typedef struct {
  int order;     /* 0 first order, 1 mixed second order */
  int np;        /* 1: P only (datatype 0), 2: P and S (datatype 1) */
  int sigdep;    /* 0 data sigma, else sigma = n0*time + n1 */
  int solver;    /* 3D solver: 0 default (heap march for order 1, tiles for
                    order 0), MCT_EIK3_TILES or MCT_EIK3_HEAP */
  int dynamic;   /* LIKE_SET%dynamic: 1 keeps the stations' travel-time fields
                    (like%field5d, 2 x nslots x np x nrev x nodes FP64) for
                    mct_body_location_likelihood; the solves then always run
                    from the stations */
} mct_body_settings;

typedef struct {
  int nsrc, nrev, np;
  const double *rev;      /* (3, nrev) station x, y, z */
  const int *raystat;     /* (nsrc*nrev, np): 1 where a pick exists */
  const double *ttime;    /* (nsrc*nrev, np) observed arrival times */
  const double *sigma;    /* (nsrc*nrev, np) data sigma, or NULL */
  int nrays;
} mct_body_data;

typedef struct mct_body_ctx mct_body_ctx;

int mct_body_create(const mct_grid *grid, const mct_body_settings *settings,
                    const mct_body_data *data, int nslots, int ncell_max,
                    mct_body_ctx **ctx);
int mct_body_destroy(mct_body_ctx *ctx);
/* Runs the context's work on a stream of the device's highest priority
 * (high != 0) or of normal priority (the default), after its pending work.
 * No counterpart in the reference: for the served loop, where contexts of
 * different kinds share the GPU. */
int mct_body_set_priority(mct_body_ctx *ctx, int high);
/* points/params [nchains][ncell_max][3] ((x,y,z) and (vp,vs,rho)),
 * locations [nchains][nsrc][4] event (x, y, z, origin time) (RTI%locations),
 * n0/n1 [nchains][np]; out [nchains][4] = like, misfit, unweighted misfit,
 * status. Host pointers, synchronous. */
int mct_body_forward(mct_body_ctx *ctx, int nchains, const int *ncells,
                     const double *points, const double *params,
                     const double *locations, const double *n0,
                     const double *n1, double *out);
/* mct_body_submit: starts the forward of mct_body_forward and returns at
 * once (the arrays are copied before it returns); the batch runs on a
 * worker thread of the context, since the 3D solver waits on the host
 * between its passes. One submitted batch per context at a time; the other
 * calls on the context return MCT_ERR_ARG until it is polled.
 * mct_body_poll: *done = 0 while the batch runs; when it has finished, *done
 * = 1, out (nchains x 4) is filled as by mct_body_forward and the batch's
 * status is returned; mct_body_commit then applies to it. No counterpart in
 * the reference: one host thread can keep several contexts busy. */
int mct_body_submit(mct_body_ctx *ctx, int nchains, const int *ncells,
                    const double *points, const double *params,
                    const double *locations, const double *n0,
                    const double *n1);
int mct_body_poll(mct_body_ctx *ctx, double *out, int *done);
/* After the Metropolis test: chains with accept[c] != 0 (and a valid
 * forward) keep the last forward's travel times as their state (the
 * reference keeps the accepted like and restores the backup on reject,
 * src/mcmc_loc2.f90:456-465). */
int mct_body_commit(mct_body_ctx *ctx, int nchains, const int *accept);
/* Noise-only likelihood, replaces body_noise_likelihood
 * (src/likelihood_body.F90:38-80): chains 0..nchains-1's committed travel
 * times re-reduced with new noise parameters n0, n1 (nchains x np) and
 * origin times (locations, nchains x nsrc x 4, the 4th entry used); sigma =
 * n0 * travel time + n1 for every pair. out as mct_body_forward (status 16:
 * nothing committed yet). */
/* Location step with stored fields, replaces body_location_likelihood
 * (src/likelihood_body.F90:82-149, settings.dynamic = 1): chains
 * 0..nchains-1's committed fields (one per station and phase, from their
 * last accepted forward) read at the proposed event locations
 * (Interpolate3d, :976-1005) and the misfit with origin times, sigma =
 * n0 * time + n1; out [nchains][4] as mct_body_forward (status 16: nothing
 * committed yet); phase_time (optional) [nchains][np][nsrc*nrev] the times.
 * mct_body_location_commit: the accepted location steps' times become the
 * chains' committed times. MCT_ERR_UNSUPPORTED without stored fields (the
 * reference's location step is then a full forward). */
int mct_body_location_likelihood(mct_body_ctx *ctx, int nchains, const double *locations, const double *n0,
                                 const double *n1, double *out, double *phase_time);
int mct_body_location_commit(mct_body_ctx *ctx, int nchains, const int *accept);
int mct_body_noise_likelihood(mct_body_ctx *ctx, int nchains,
                              const double *locations, const double *n0,
                              const double *n1, double *out);
/* Last forward's travel times (np, nsrc, nrev) = phaseTime(k,j,i) for batch
 * position index, and the number of tile passes the solves took. */
int mct_body_phase_time(mct_body_ctx *ctx, int index, double *phase_time,
                        int *passes);


/* ------------------------------------------------------------------------
 * 2D travel-time likelihood for many chains, replaces the 2D code's
 * likelihood call (mcmc2d/likelihood_joint.f90:56) -> body_likelihood
 * (mcmc2d/likelihood_dd.F90:349-529) and the kdtree_to_grid call before it
 * (mcmc2d/mcmc.f90:1469-1525): nearest-nucleus velocity grid (ny, nx),
 * padded vertex grid, modrays from every source (or straight rays), then
 * sigma and the misfit; datatype 1 adds the differential times of every
 * source pair. The grid's y axis is divided by its scaling for the
 * travel times, as the reference's call does; nz is ignored.
 * ---------------------------------------------------------------------- */
typedef struct {
  int gridx, gridy;   /* fm2d B-spline refinement of the vertex grid */
  int sgref;          /* 1: refined source grid */
  int sgdic, sgext;   /* source grid refinement factor and extent */
  int order;          /* fm2d: 0 first order, 1 mixed order (fom) */
  int sigdep;         /* 0 data sigma, else sigma = n0 * time + n1 */
  int datatype;       /* 0 travel times; 1 travel times + differential times */
  int straight;       /* 1: straight rays (isStraight) instead of fm2d */
  int precision;      /* fm2d: 0 FP64 in the reference's order, 1 double-float */
} mct_tt2d_settings;

typedef struct {
  int nsrc, nrev;
  const double *src;      /* (2, nsrc) source x, y (dat%src) */
  const double *rev;      /* (2, nrev) receiver x, y (dat%rev) */
  const int *raystat;     /* (nsrc*nrev): 1 where a time exists (dat%raystat(:,1,1)) */
  const double *ttime;    /* (nsrc*nrev) observed times (dat%ttime(:,1,1)) */
  const double *sigma;    /* (nsrc*nrev) data sigma (dat%ttime(:,2,1)), or NULL */
  int nrays;
  /* datatype 1: (nrev, nsrc*(nsrc-1)/2) column-major as dat%dtime(:,:,1)
   * and dat%dcc(:,:,1) (pairs i<j in order), and dat%ndtime */
  const double *dtime;
  const double *dcc;
  int ndtime;
} mct_tt2d_data;

typedef struct mct_tt2d_ctx mct_tt2d_ctx;

/* MCT_ERR_ARG also where the reference's differential-time test
 * (abs(dat%dtime(ddindex,k,1)), indices swapped) would read outside
 * dat%dtime. */
int mct_tt2d_create(const mct_grid *grid, const mct_tt2d_settings *settings,
                    const mct_tt2d_data *data, int nslots, int ncell_max,
                    mct_tt2d_ctx **ctx);
int mct_tt2d_destroy(mct_tt2d_ctx *ctx);
/* Runs the context's work on a stream of the device's highest priority
 * (high != 0) or of normal priority (the default), after its pending work.
 * No counterpart in the reference: for the served loop, where contexts of
 * different kinds share the GPU. */
int mct_tt2d_set_priority(mct_tt2d_ctx *ctx, int high);
/* As mct_surf_set_sm_share, for the context's fm2d launches. */
int mct_tt2d_set_sm_share(mct_tt2d_ctx *ctx, double share);
/* points [nchains][ncell_max][2] (x, y) = RTI%points, params
 * [nchains][ncell_max][3] (velocity first) = RTI%parameters, n0/n1
 * [nchains][2] = RTI%snoise0/1 (travel times, differential times);
 * out [nchains][4] = like, misfit, unweighted misfit, status (8: zero
 * sigma, the reference's fatal error; like = DBL_MAX when nonzero). Host
 * pointers, synchronous. */
int mct_tt2d_forward(mct_tt2d_ctx *ctx, int nchains, const int *ncells,
                     const double *points, const double *params,
                     const double *n0, const double *n1, double *out);
/* mct_tt2d_submit / mct_tt2d_poll: mct_tt2d_forward split as
 * mct_surf_submit / mct_surf_poll are (the arrays copied into pinned
 * staging before submit returns, the batch on the context's stream, poll
 * without blocking). One submitted batch at a time; the other calls on the
 * context return MCT_ERR_ARG until it is polled. */
int mct_tt2d_submit(mct_tt2d_ctx *ctx, int nchains, const int *ncells,
                    const double *points, const double *params,
                    const double *n0, const double *n1);
int mct_tt2d_poll(mct_tt2d_ctx *ctx, double *out, int *done);
/* After the Metropolis test: chains with accept[c] != 0 (and a valid
 * forward) keep the last forward's times as their state, as the
 * reference keeps the accepted like and restores the backed-up one on
 * reject (mcmc2d/mcmc.f90:456-465). */
int mct_tt2d_commit(mct_tt2d_ctx *ctx, int nchains, const int *accept);
/* Noise-only likelihood, replaces the 2D body_noise_likelihood
 * (mcmc2d/likelihood_dd.F90:32-106): chains 0..nchains-1's committed times
 * with new n0/n1; sigma = n0 * srdist + n1 (srdist: the times when sigdep
 * != 0, else the source-receiver distances), the differential sigma
 * log-sum kept in an integer as the reference does; out as
 * mct_tt2d_forward (unweighted misfit: the committed forward's; status 16:
 * nothing committed yet). */
int mct_tt2d_noise_likelihood(mct_tt2d_ctx *ctx, int nchains,
                              const double *n0, const double *n1, double *out);
/* Last forward's times (nsrc, nrev) = phaseTime(k,j,1) of batch position
 * index. */
int mct_tt2d_phase_time(mct_tt2d_ctx *ctx, int index, double *phase_time);

/* ------------------------------------------------------------------------
 * The sampler's random number stream, replaces the module mt19937
 * (src/mt19937.f90): MT19937 seeded as init_genrand(seed) (:96-115; the
 * reference seeds it from init_random_seed, src/initialise.f90:119), draws
 * as grnd (:117-172, u / (2^32 - 1) of the 32-bit output u), unirand
 * (:224-236) and gasdev (:200-222, polar Box-Muller on two grnd draws, host
 * libm log and sqrt). Each generator counts its draws like RTI%randcount.
 * Host only: no GPU is used. One generator per chain; a generator is not
 * safe to use from two threads at once.
 * ---------------------------------------------------------------------- */
typedef struct mct_rng mct_rng;
int mct_rng_create(unsigned seed, mct_rng **rng);
void mct_rng_destroy(mct_rng *rng);
int mct_rng_seed(mct_rng *rng, unsigned seed);
double mct_rng_unirand(mct_rng *rng);
double mct_rng_gasdev(mct_rng *rng);
/* the raw 32-bit output (genrand_int32), counted as one draw */
unsigned mct_rng_u32(mct_rng *rng);
long long mct_rng_count(const mct_rng *rng);

/* ------------------------------------------------------------------------
 * Proposal steps and acceptance test of the reference's Metropolis-Hastings
 * loop (src/mcmc_loc2.f90:72-687): proposeType2 (:1384-1432), cell_birth
 * (:1521-1613), cell_death (:1615-1683), cell_move (:1685-1765), vel_change
 * (:1767-1835), bsigma_change / ssigma_change (:1837-1903). Host only.
 * mct_mcmc_set holds the T_MCMC_SET fields the steps read; mct_mcmc_state
 * the chain's RTI%points / RTI%parameters (ncell_max x 3 each, one nucleus
 * per row: x, y, z and vp, vs, rho) and noise levels. The cell containing a
 * point (the reference's CGAL locate) is its nearest nucleus, the first in
 * index order on an exact tie. Source relocation (type 7) is not restated.
 * ---------------------------------------------------------------------- */
typedef struct {
  int ncell_min, ncell_max;
  int kernel;      /* 0: birth/death values from the local cell (Gaussian), 1: from the prior */
  int datatype;    /* 0 P, 1 P and S, 2 surface waves, 3 joint */
  int sigdep;      /* noise levels are sampled */
  int locate;      /* source locations are sampled (type 7, not supported) */
  double xmin, xmax, ymin, ymax, zmin, zmax;
  double vpmin, vpmax, vsmin, vsmax;
  double sigma_vp, sigma_vs, sigma_vp2, sigma_vs2;   /* value steps (upper, deeper half) */
  double pd, pd2;                                    /* move steps, percent of the extent */
  double sigma_bn0, sigma_bn1, bn0_min, bn0_max, bn1_min, bn1_max;
  double sigma_sn0, sigma_sn1, sn0_min, sn0_max, sn1_min, sn1_max;
} mct_mcmc_set;

typedef struct {
  int ncells;
  double *points;        /* [ncell_max][3] */
  double *parameters;    /* [ncell_max][3] vp, vs, rho */
  int nbnoise, nsnoise;  /* periods / phases of the body and surface noise levels */
  double *bnoise0, *bnoise1, *snoise0, *snoise1;
} mct_mcmc_state;

typedef struct {
  int ptype;       /* 1 birth, 2 death, 3 move, 4 value, 5 body noise, 6 surface noise */
  int index;       /* the cell (1-based) or period changed */
  int valid;       /* 0: the reference's lerr = .false. (the state is not a proposal) */
  double prob;     /* the proposal's log-density term of the acceptance ratio */
  double random;   /* the acceptance draw */
} mct_mcmc_step;

/* One proposal of iteration iter applied to state in place. Unless redo
 * (the last proposal's model was invalid and the reference repeats it with
 * the same type and acceptance draw), first draws step->random and the type
 * with proposeType2. The caller keeps a copy of the state to restore on
 * rejection, as the reference does. */
int mct_mcmc_propose(const mct_mcmc_set *set, mct_rng *rng, int iter, int redo, mct_mcmc_state *state,
                     mct_mcmc_step *step);
/* The acceptance test of the step given the proposal's -log L (like_new)
 * and the current one (like_old): 1 accept, 0 reject. */
int mct_mcmc_accept(const mct_mcmc_set *set, const mct_mcmc_step *step, double like_new, double like_old);
/* The same test in the parallel-tempering loop mcmc_pt
 * (src/mcmc_loc2.f90:881-886, 933-938, 979-981): the likelihood ratio is
 * divided by the chain's temperature (> 0). */
int mct_mcmc_accept_tempered(const mct_mcmc_set *set, const mct_mcmc_step *step, double like_new,
                             double like_old, double temperature);

/* ------------------------------------------------------------------------
 * Parallel tempering (mcmc_pt, src/mcmc_loc2.f90:1222-1275): chains
 * 1..nchains (RTI%number_of_chains) share a temperature ladder values0 of
 * nchains values (number_of_1s ones, then the temperature file's values,
 * src/initialise.f90:128-134). values / indices are each chain's current
 * temperature and its 1-based ladder position (RTI%temperature_values /
 * _indices); mct_pt_init sets them to the ladder in order. Every
 * tempering_step iterations from tempering_start, mct_pt_choose picks two
 * chains as choose_t1 / choose_t2 (:2148-2236; jump_type 0: a random chain
 * of another temperature, 1: a random ladder neighbour, 2: the nearest
 * ladder value) and mct_pt_swap offers them a swap given their current
 * -log L, as do_tempering (:2240-2280): 1 swapped, 0 not. Both draw from
 * the stream of the reference's first process (its chain 1). Host only. */
typedef struct {
  int nchains;
  int number_of_1s;
  int jump_type;
  const double *values0;   /* [nchains] */
  double *values;          /* [nchains] */
  int *indices;            /* [nchains] */
  long long accepted, total;
} mct_pt;
int mct_pt_init(mct_pt *pt);
int mct_pt_choose(mct_pt *pt, mct_rng *rng, int *t1_chain, int *t2_chain);
int mct_pt_swap(mct_pt *pt, mct_rng *rng, int t1_chain, int t2_chain, double like_t1, double like_t2);

/* ------------------------------------------------------------------------
 * The sample stream (samples_*.out, run_time_sample_*.dat): one T_SAMPLE
 * (src/run_time_info.f90:62-76) per iteration. mct_mcmc_record fills it as
 * the MCMC loop does after the acceptance test (src/mcmc_loc2.f90:253-263,
 * 305-315, 345-355, 425-436, 487-497, 578-582): zeros and the step's type;
 * for an accepted step the new cell's nucleus and values (birth), the
 * removed cell (death), the moved nucleus (move), the cell's new values
 * (value change) or the period's new noise levels (noise steps); then the
 * chain's current number of cells, -log L, misfit and unweighted misfit.
 * state is the chain's state after the decision (restored on rejection).
 * mct_samples_write appends records to a file (creating it) in
 * write_samples' stream layout (run_time_info.f90:306-340): int32 step,
 * 1-byte accepted, int32 vindex, int64 ncells, misfit, unweighted misfit,
 * like, dim coordinates (dim 2 for the 2D code, 3), 3 values, noise0,
 * noise1, unpadded little-endian. mct_samples_read reads up to n records
 * and returns how many it read (< 0: error). Host only.
 * ---------------------------------------------------------------------- */
typedef struct {
  int step, accepted, vindex;
  long long ncells;
  double misfit, unweighted_misfit, like;
  double coord[3], values[3];
  double noise0, noise1;
} mct_sample;
int mct_mcmc_record(const mct_mcmc_state *state, const mct_mcmc_step *step, int accepted, double like,
                    double misfit, double unweighted_misfit, mct_sample *sample);
int mct_samples_write(const char *filename, int dim, const mct_sample *samples, int n);
int mct_samples_read(const char *filename, int dim, mct_sample *samples, int n);

#ifdef __cplusplus
}
#endif
#endif /* MCTOMO_H_ */
