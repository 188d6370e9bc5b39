// ORACLE (test infrastructure only): declarations of the CPU restatements of
// the MCTomo forward-modelling hot path. These functions are the checker for
// the GPU library and the timed CPU baseline; the product never links them.
#ifndef MCT_ORACLE_H_
#define MCT_ORACLE_H_
#ifdef __cplusplus
extern "C" {
#endif

int orc_kdtree_to_grid(int d, int n, const double *points, const double *params,
                       int nx, int ny, int nz, double xmin, double ymin,
                       double zmin, double dx, double dy, double dz, int ix0,
                       int ix1, int iy0, int iy1, int iz0, int iz1,
                       int *sites_id, double *vp, double *vs, double *rho);
int orc_kdtree_nearest(int d, int n, const double *points, const double *qv);

int orc_surfdisp96(const float *thkm, const float *vpm, const float *vsm,
                   const float *rhom, int nlayer, int iwave, int mode, int igr,
                   int kmax, const double *t, double dphase, double *cp,
                   double *cg, long long *ndltar);
int orc_surfdisp_mmodes(const float *thkm, const float *vpm, const float *vsm,
                        const float *rhom, int nlayer, int iwave, int mode,
                        int igr, int kmax, const double *t, double dphase,
                        double *cp, double *cg, long long *ndltar);
double orc_dltar(double wvno, double omega, int ifunc, const float *thkm,
                 const float *vpm, const float *vsm, const float *rhom,
                 int nlayer);
float orc_gtsolh(float a, float b);
int orc_count_lvl(const double *vp, const double *vs, int nl, int modetype);
int orc_surfmodes(const double *thick, const double *vp, const double *vs,
                  const double *rho, int nl, const double *freqs, int np,
                  int modetype, int phase_group, double dc, double *phase,
                  double *group, long long *ndltar);

int orc_modrays(int nsrc, const double *scx, const double *scz, int nrc,
                const double *rcx, const double *rcz, const int *srs, int nvx,
                int nvz, double goxd, double gozd, double dvxd, double dvzd,
                const double *velvin, int gdx, int gdz, int asgr, int sgdl,
                int sgs, int fom, double snb, double *ttime, double *tfield);
int orc_modrays_group(int nsrc, const double *scx, const double *scz, int nrc,
                      const double *rcx, const double *rcz, const int *srs, int nvx,
                      int nvz, double goxd, double gozd, double dvxd, double dvzd,
                      const double *velvin, int gdx, int gdz, int asgr, int sgdl,
                      int sgs, int fom, const double *gvel, double *ttime, double *gtime,
                      double *raylen, int *crazy);
int orc_straight_group(int nsrc, const double *src, int nrev, const double *rev, const int *raystat, int nx,
                       int ny, double xmin, double ymin, double dx, double dy, const double *vel, double *time,
                       double *dist);

int orc_fm2d_trace(int src, int *idx, double *t, int max);
int orc_fm2d_trace_count(void);
int orc_fast_marching3d(int nx, int ny, int nz, double dx, double dy, double dz,
                        double xmin, double ymin, double zmin, const double *vel,
                        const double *src, const double *rev, int nrev,
                        int order, double *ttime, double *tfield);

int orc_check_model(const double *vs, int nz, int ny, int nx);
int orc_convert_to_layer(const double *vp, const double *vs, const double *rho,
                         int nz, double dz, double scaling, double water_depth,
                         double *alpha, double *beta, double *rho_k,
                         double *thick);
int orc_surf_misfit(int nsrc, int nrev, int np, const double *phase_time,
                    const double *dat_ttime, const int *raystat,
                    const double *srdist, int sigdep, const double *n0,
                    const double *n1, int nrays, double *sigma_out,
                    double *out);
int orc_tt2d_misfit(int nsrc, int nrev, const double *phase_time, const double *dat_ttime,
                    const double *dat_sigma, const int *raystat, int sigdep, int datatype,
                    const double *dtime, const double *dcc, int ndtime, const double *n0,
                    const double *n1, int nrays, double *out);
int orc_tt2d_noise(int nsrc, int nrev, const double *phase_time, const double *dat_ttime,
                   const int *raystat, const double *srdist, int datatype, const double *dtime,
                   const double *dcc, int ndtime, const double *n0, const double *n1, int nrays,
                   double *out);
int orc_location_times(int nx, int ny, int nz, double xmin, double ymin, double zmin, double dx, double dy,
                       double dz, double scaling, int np, int nsrc, int nrev, const double *fields,
                       const double *events, double *times);
int orc_body_misfit(int nsrc, int nrev, int np, const double *phase_time,
                    const double *t0, const double *dat_ttime,
                    const int *raystat, const double *srdist, int sigdep,
                    const double *n0, const double *n1, int nrays,
                    double *sigma_out, double *out);
int orc_surf_likelihood(const int *gi, const double *gd, const int *iset, double dphase,
                        double rho_value, int n, const double *points, const double *params,
                        int np, const double *freqs, int nsrc, const double *src, int nrev,
                        const double *rev, const int *raystat, const double *ttime,
                        const double *sigma, int nrays, const double *n0, const double *n1,
                        const int *col_mask, double *pvel_io, double *phase_time, double *out);
double orc_vs2vp(double vs);
double orc_vp2rho(double vp);

#ifdef __cplusplus
}
#endif
#endif
