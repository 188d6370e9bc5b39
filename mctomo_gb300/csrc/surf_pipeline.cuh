// Device-side description of one batched surface-wave forward.
#pragma once
#include <cuda_runtime.h>
#include "fm2d.cuh"

#include "../../include/mctomo.h"

struct SurfBatch {
  // grid and settings
  int nx, ny, nz;
  double xmin, ymin, zmin, dx, dy, dz, scaling, water_depth;
  int law; double rho_value;
  int iwave, precision; double dphase;
  int sigdep;
  int igr;                   // 1: group velocities (phaseGroup = 1)
  int straight;              // 1: straight rays (isStraight = 1), no fast marching
  int np, nsrc, nrev, nrays;
  const double *periods;     // [np]
  const int *raystat;        // [np][nsrc*nrev]
  const double *dtime;       // [np][nsrc*nrev]
  const double *dsigma;      // [np][nsrc*nrev]
  // inputs (device)
  int nchains, ncell_max;
  const int *slots;          // [nchains]
  const int *ncells;         // [nchains]
  const double *points;      // [nchains][ncell_max][3]
  const double *params_in;   // [nchains][ncell_max][3]
  const double *n0, *n1;     // [nchains][np]
  double *out;               // [nchains][4]: like, misfit, unweighted misfit, status
  // working state for the batch
  double *params;            // [nchains][ncell_max][3] after material laws
  int *sites;                // [nchains][nodes]
  double *vp, *vs, *rho;     // [nchains][nodes]
  int *tie_count, *tie_nodes; void *kd_scratch; int *dev_status;
  int *status;               // [nchains]
  int *list_count; int2 *list;   // changed columns
  int nl_max;
  int *lnl; float *lthk, *lvp, *lvs, *lrho;   // [nchains*ncol][nl_max]
  double *lcp, *lcg; int *lierr;               // [nchains*ncol][np]
  int *lorder;                                 // [nchains*ncol] dispersion column order
  unsigned long long *ndltar;
  double *pvel;              // [nchains][np][nx][ny]
  double *velv;              // [nchains*np][(nx+2)*(ny+2)]
  double *ttime;             // [nchains*np][nsrc][nrev] phase times (fm2d)
  double *gvel;              // [nchains][np][nx][ny] group maps (igr)
  double *gtime, *raylen;    // [nchains*np][nsrc][nrev] times along rays and ray lengths (igr or straight)
  int *crazy;                // [nchains*np] rays that reached the point limit
  const double *sdist;       // [nsrc*nrev] source-receiver distances (straight)
  // committed per-slot state
  int *committed;            // [nslots]
  double *cvp, *cvs, *crho;  // [nslots][nodes]
  double *cpvel;             // [nslots][np][nx][ny]
  double *cttime;            // [nslots][np][nsrc][nrev] committed phase times
  double *csrd;              // [nslots][np][nsrc][nrev] their srdist (sigma = n0 srdist + n1)
  double *cgvel;             // [nslots][np][nx][ny] committed group maps (igr)
  // reuse of committed refined-box results in fm2d (reuse = 1: refined
  // source boxes, no rays, FP64 or double-float times)
  int reuse, spc, map_tmp_max;
  double *cvelv;             // [nslots][np][(nx+2)(ny+2)] committed padded phase maps
  double *cref_t;            // [nslots][spc][map_tmp_max] committed refined-box mappings
  short *cref_s;
  int *cmap, *csolve;        // per forward: [nchains*np], [nchains*spc] committed map / solve or -1
  int *ref_list, *ref_count; // [nslots*spc], [1]
  const double *map_tmp_t;   // the forward's mappings (fm2d scratch)
  const short *map_tmp_s;
};

// Optional per-stage timing: events recorded around the stages of each
// forward (no host synchronisation), read back after the timed region.
struct SurfProfile {
  int enabled = 0, max_steps = 0, step = 0;
  cudaEvent_t *ev = nullptr;        // [max_steps][5]
  long long launches = 0;           // kernels launched by forwards
};

struct SurfPlan {
  Fm2dJob fm2d;              // static parts (stations, settings, scratch, solve list)
  Fm2dPlan fm2d_plan;
  int nsolve_per_chain;
  const double *src_xy, *rev_xy;   // [nsrc][2], [nrev][2] station coordinates (straight rays)
};

int surf_forward(SurfBatch &b, const SurfPlan &plan, cudaStream_t s, SurfProfile *prof = nullptr);
int surf_commit(SurfBatch &b, const int *accept_dev, cudaStream_t s);
// Noise-only likelihood of committed slots (no forward solve).
int surf_noise(const SurfBatch &b, int nchains, const int *slots, const double *n0, const double *n1, double *out,
               cudaStream_t s);
