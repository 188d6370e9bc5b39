// 3D eikonal job description: tile-based fast iterative method (method 1)
// or the exact heap march (method 2).
#pragma once
#include <cuda_runtime.h>
#include <cstddef>

// Method selection (the low bits of the public order argument carry the
// order; these bits select the solver).
enum Eik3Method { EIK3_DEFAULT = 0, EIK3_TILES = 1, EIK3_HEAP = 2 };

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
  int method;                     // EIK3_TILES or EIK3_HEAP (resolved, never EIK3_DEFAULT)
  // tile iteration scratch
  int shift;                      // times stored in units of 2^-shift s
  const int *grid_shift;          // optional [ngrids]: the shift of each grid's solves (overrides shift)
  int *T;                         // [nsolve][nx][ny][nz] scratch: fixed-point times
  unsigned char *flags;           // [nsolve][tiles] scratch
  int *list, *count;              // scratch: active (solve, tile) list
  // heap march scratch (solves run in chunks of hchunk)
  double *ht;                     // [hchunk][nn] arrival times
  unsigned char *hst;             // [hchunk][nn] OPEN / NARROW / FROZEN
  double *hkey;                   // [hchunk][hcap] heap entry keys
  unsigned *hid;                  // [hchunk][hcap] heap entry nodes (+ position slot)
  unsigned *hpos;                 // [hchunk][nn][2] heap positions of a node's entries
  double2 *hvn;                   // [ngrids][nn] (velocity, -1/velocity^2)
  int hchunk;
  unsigned hcap;
  int *herr;                      // [1] error bits
  // receivers
  int nrev;                       // receivers per solve
  const double *rev;              // [sets][nrev][3] relative to the origin
  int rev_per_solve;              // 1: set = solve index (unless solve_rev given)
  const int *solve_rev;           // optional [nsolve]: receiver set of each solve
  double *ttime;                  // [nsolve][nrev]
};

size_t eik3_tiles(const Eik3Job &j);
int eik3_shift_for(double tmax_bound);
// Resolves EIK3_DEFAULT: the heap march for the mixed second-order scheme
// (whose result depends on the acceptance order), tiles for first order.
int eik3_resolve_method(int order, int method);
// Heap-march scratch per solve (times, states, heap, entry positions), the
// bytes for a chunk of solves, and carving it (sets ht..hpos, hchunk, hcap).
struct Carve;
size_t eik3_heap_bytes_per_solve(int nx, int ny, int nz);
size_t eik3_heap_scratch_bytes(int nx, int ny, int nz, int chunk);
void eik3_heap_take(Eik3Job &job, Carve &cv, int chunk);
unsigned eik3_heap_cap(int nx, int ny, int nz);
int launch_eik3(Eik3Job &job, cudaStream_t s, int max_passes, int *passes_out, double *tfield);
int launch_eik3_heap(Eik3Job &job, cudaStream_t s, double *tfield);
