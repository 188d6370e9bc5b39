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
 * boxes [nchains][6] or NULL, outputs [nchains][grid]. */
int mct_grid_nearest_batch_device(int d, int nchains, int ncell_max,
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

/* surfmodes (surfmodes/surfmodes.f90:39-108): FP64 layer model cast to
 * REAL*4, freqs[np] in Hz, modetype 1 Rayleigh / 0 Love, phase_group 0/1.
 * A column with a low-velocity layer that the reference routes to its
 * generalized R/T solver returns MCT_ERR_UNSUPPORTED. */
int mct_surfmodes(const double *thick, const double *vp, const double *vs,
                  const double *rho, int nlayers, const double *freqs, int np,
                  int modetype, int phase_group, double dc, double *phase,
                  double *group, int *ierr);

/* Many columns at once (host buffers): layer arrays [ncol][nl_max] REAL*4,
 * nl[ncol]; cp/cg [ncol][mode][np]; ierr[ncol]. precision 0 = FP64 root
 * search as the reference; 1 = FP32 bracketing confirmed in FP64, then FP64
 * polish (same roots). ndltar (optional, 2 entries) counts FP64 and FP32
 * period-equation evaluations. */
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

#ifdef __cplusplus
}
#endif
#endif /* MCTOMO_H_ */
