// 3D eikonal job description (tile-based fast iterative method).
#pragma once
#include <cuda_runtime.h>
#include <cstddef>

struct Eik3Job {
  int nsolve;
  int nx, ny, nz;                 // grid, z fastest in memory (vel[nx][ny][nz])
  double dx, dy, dz;
  const double *vel;              // [ngrids][nx][ny][nz] velocities
  float *slow;                    // [ngrids][nx][ny][nz] scratch: FP32 slowness, < 0 marks an obstacle
  int ngrids;
  const int *solve_grid;          // [nsolve] velocity grid of each solve
  const double *src;              // [nsolve][3] source relative to the grid origin
  int order;                      // 0 first order, 1 mixed second order
  int shift;                      // times stored in units of 2^-shift s
  int *T;                         // [nsolve][nx][ny][nz] scratch: fixed-point times
  unsigned char *flags;           // [nsolve][tiles] scratch
  int *list, *count;              // scratch: active (solve, tile) list
  int nrev;                       // receivers per solve
  const double *rev;              // [sets][nrev][3] relative to the origin
  int rev_per_solve;              // 1: set = solve index (unless solve_rev given)
  const int *solve_rev;           // optional [nsolve]: receiver set of each solve
  double *ttime;                  // [nsolve][nrev]
};

size_t eik3_tiles(const Eik3Job &j);
int eik3_shift_for(double tmax_bound);
int launch_eik3(Eik3Job &job, cudaStream_t s, int max_passes, int *passes_out, double *tfield);
