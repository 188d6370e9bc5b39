// Shared helpers for the MCTomo GB300 forward-modelling library.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <mutex>
#include "../../include/mctomo.h"

#define MCT_CUDA_TRY(expr)                                                  \
  do {                                                                      \
    cudaError_t _e = (expr);                                                \
    if (_e != cudaSuccess) {                                                \
      mct_set_error(#expr, cudaGetErrorString(_e), __FILE__, __LINE__);      \
      return MCT_ERR_CUDA;                                                  \
    }                                                                       \
  } while (0)

void mct_set_error(const char *what, const char *why, const char *file, int line);

// Raises a kernel's dynamic shared-memory limit to bytes on the current
// device, once per (device, kernel) and safely from several host threads; the
// CUDA return code is checked. The record does not survive cudaDeviceReset
// (calls after a reset in the same process are not supported).
int mct_smem_attr_raw(const void *func, int bytes);
template <class K> inline int mct_smem_attr(K *kernel, int bytes) {
  return mct_smem_attr_raw(reinterpret_cast<const void *>(kernel), bytes);
}

// Replaces a context's stream by a new non-blocking stream of the device's
// highest priority (high != 0) or of normal priority, after the old stream's
// work has finished.
inline int mct_restream(cudaStream_t *stream, int high) {
  int least = 0, greatest = 0;
  MCT_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
  MCT_CUDA_TRY(cudaStreamSynchronize(*stream));
  cudaStream_t s = nullptr;
  MCT_CUDA_TRY(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, high ? greatest : least));
  cudaStreamDestroy(*stream);
  *stream = s;
  return MCT_OK;
}

// Grow-only device buffer (reused across synchronous drop-in calls).
struct DevBuf {
  void *p = nullptr;
  size_t cap = 0;
  int reserve(size_t bytes) {
    if (bytes <= cap) return MCT_OK;
    if (p) cudaFree(p);
    p = nullptr; cap = 0;
    size_t want = bytes + bytes / 4 + 256;
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) { mct_set_error("cudaMalloc", cudaGetErrorString(e), __FILE__, __LINE__); return MCT_ERR_NOMEM; }
    cap = want;
    return MCT_OK;
  }
  template <class T> T *as() const { return static_cast<T *>(p); }
  void release() { if (p) cudaFree(p); p = nullptr; cap = 0; }
};

// Carves aligned sub-buffers out of one allocation.
struct Carve {
  char *base; size_t off;
  explicit Carve(void *b) : base(static_cast<char *>(b)), off(0) {}
  template <class T> T *take(size_t n) {
    off = (off + 255) & ~size_t(255);
    T *r = reinterpret_cast<T *>(base + off);
    off += n * sizeof(T);
    return r;
  }
};
inline size_t carve_size(std::initializer_list<size_t> bytes) {
  size_t off = 0;
  for (size_t b : bytes) { off = (off + 255) & ~size_t(255); off += b; }
  return off + 256;
}

// ---- launchers implemented in the kernel translation units ------------------

// Gridding: nearest nucleus for every node of a box, for many chains.
struct GridJob {
  int d;                 // 2 or 3
  int nx, ny, nz;
  double xmin, ymin, zmin, dx, dy, dz;
  int nchains;
  int ncell_max;         // stride of the per-chain nucleus arrays
  const int *ncells;     // [nchains]
  const double *points;  // [nchains][ncell_max][d]
  const double *params;  // [nchains][ncell_max][3]  (vp, vs, rho)
  const int *box;        // [nchains][6] 1-based inclusive ix0,ix1,iy0,iy1,iz0,iz1 (nullptr = full grid)
  int *sites_id;         // [nchains][nx][ny][nz]   (Fortran (nz,ny,nx) per chain)
  double *vp, *vs, *rho; // same layout; may be nullptr
  // scratch
  int *tie_count;        // [nchains]
  int *tie_nodes;        // [nchains][nx*ny*nz]
  void *kd_scratch;      // per-chain kd-tree storage, kd_scratch_bytes(ncell_max) each
  int *status;           // [1] error word
};
size_t kd_scratch_bytes(int ncell_max);
int launch_grid_nearest(const GridJob &job, cudaStream_t s);
// Waits for the stream, then returns and clears the device's sticky gridding
// error word (the first nonzero status of any gridding launch since the last
// read).
int grid_status_read(void *stream, int *status);

// Dispersion: surfdisp96 per column.
struct DispJob {
  int ncol;
  const int *ncol_dev;   // optional device-side column count (<= ncol)
  int nl_max;            // stride of the layer arrays
  const int *nl;         // [ncol]
  const float *thk, *vp, *vs, *rho;  // [ncol][nl_max] REAL*4 model
  int np;
  const double *periods; // [np]
  int iwave;             // 1 Love, 2 Rayleigh
  int mode;              // number of modes (1 = fundamental only)
  int igr;               // 0 phase, 1 group
  double dphase;
  int multimode;         // 0: surfdisp96, 1: surfdisp_mmodes
  int precision;         // 0: FP64 bracketing, 1: FP32 bracketing + FP64 polish
  double *cp, *cg;       // [ncol][mode][np]
  int *ierr;             // [ncol]
  unsigned long long *ndltar; // optional [2]: FP64 and FP32 period-equation evaluations used
  int *order;            // optional [ncol] scratch: columns are run in order of layer count
};
int launch_surfdisp(const DispJob &job, cudaStream_t s);
