// GRT fundamental-mode dispersion (grt.cu): the job description and the
// launcher used by the C ABI.
#pragma once
#include "mct_common.cuh"

struct GrtJob {
  int ncol, nl_max, np, modetype, phase_group;
  const int *nl;                          // [ncol] layers per column (last = half-space)
  const double *thk, *vp, *vs, *rho;      // [nl_max][ncol], column-major
  const double *freqs;                    // [np] Hz
  double tolmin, tolmax, smin_min, smin_max, dc;
  double *mu, *v;                         // scratch [nl_max][ncol], [2 nl_max][ncol]
  double *scratch;                        // grt_scratch_doubles(n) trial velocities
  const int *cols;                        // optional list of the n columns to run (else 0..ncol-1)
  int n;                                  // columns to run
  unsigned *next;                         // pool counter (device, one word)
  double *phase, *group;                  // [ncol][np]
  int *ierr;                              // [ncol]: 0, 1 (no root), 2 (trial list over 20,000),
                                          // -1 (layer count), -2 (fluid layer)
  unsigned long long *nevals;             // [1] secular-function evaluations (added to)
};

// Trial-velocity entries per thread: a first pass with room for 8,192, then
// a narrow pass with the reference's 20,000 over the columns that needed more.
constexpr int kGrtCap0 = 8192, kGrtCap1 = 20000;
// Resident threads of the persistent GRT grid for n columns in pass 0 / 1
// (modetype 1 Rayleigh, 0 Love).
int grt_threads(int n, int pass, int modetype);
// Doubles of trial-velocity scratch the two passes need for n columns.
size_t grt_scratch_doubles(int n, int modetype);
// Enqueues on stream s the transposition of the row-major [ncol][nl_max]
// layer arrays rows[0..3] (thk, vp, vs, rho) into cols4 (4 x nl_max x ncol
// doubles) and the two passes of the GRT kernel; J's layer pointers are set
// from cols4.
int launch_grt(const GrtJob &J, const double *const rows[4], double *cols4, cudaStream_t s);
