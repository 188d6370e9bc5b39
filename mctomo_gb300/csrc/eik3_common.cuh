// Device helpers shared by the two 3D travel-time solvers (tile iteration
// and heap march): grid dimensions, node indexing in the reference's
// vel[nx][ny][nz] layout (z fastest) and the reference's trilinear
// interpolation with its max-face clamp (ndgridmap/ndgridmap.hpp:158-191,
// 433-490: getVel / getTime).
#pragma once
#include <cuda_runtime.h>
#include <cstddef>

struct E3Dims {
  int nx, ny, nz;
};

__device__ __forceinline__ size_t e3_nidx(const E3Dims &d, int i, int j, int k) {
  return (size_t)k + (size_t)d.nz * ((size_t)j + (size_t)d.ny * i);
}

// Cell of a point: (int)(p/h) per axis, clamped to the grid
// (ndgridmap.hpp coordinate lookup).
__device__ __forceinline__ void e3_point_cell(const E3Dims &d, const double h[3], const double p[3], int pc[3]) {
  const int dimsz[3] = {d.nx, d.ny, d.nz};
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    int c = (int)(p[q] / h[q]);
    if (c < 0) c = 0; else if (c >= dimsz[q]) c = dimsz[q] - 1;
    pc[q] = c;
  }
}

// Corner v (0..7) of the cell of pc: bit 2 steps x, bit 1 y, bit 0 z, each
// clamped to the last node (so corners on a max face repeat).
__device__ __forceinline__ void e3_corner(const E3Dims &d, const int pc[3], int v, int vc[3]) {
  const int dimsz[3] = {d.nx, d.ny, d.nz};
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    vc[q] = pc[q] + ((v >> (3 - q - 1)) & 1);
    if (vc[q] >= dimsz[q]) vc[q] = dimsz[q] - 1;
  }
}

// Trilinear interpolation with the reference's weights: a corner clamped
// onto the cell's own node gets weight |s - h| / h instead of s / h, so
// points on a max face read 2x / 4x / 8x the value there, as the
// reference does.
template <class F>
__device__ double e3_trilinear(const E3Dims &d, const double h[3], const double p[3], F value) {
  int pc[3];
  e3_point_cell(d, h, p, pc);
  double acc = 0;
  for (int v = 0; v < 8; ++v) {
    int vc[3];
    e3_corner(d, pc, v, vc);
    double w = 1.0;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      double di = (double)(unsigned)(vc[q] - pc[q]);
      double s = p[q] - h[q] * (double)(unsigned)pc[q];
      double wj = fabs(di * h[q] - h[q] + s);
      w = w * wj / h[q];
    }
    acc = acc + w * value(vc[0], vc[1], vc[2]);
  }
  return acc;
}
