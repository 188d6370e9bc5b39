// mct_grid_nearest_batch_device_noalloc: the batched nearest-nucleus
// gridding of mct_grid_nearest_batch_device, with its scratch (per-chain tie
// counters, tie-node lists, kd-tree storage and the error word) taken from a
// fixed device array of this file instead of an allocation per call.
//
// Who needs it: a caller that must not allocate device memory while it runs,
// e.g. a sampler that enqueues whole proposals ahead of time on its own
// stream and cannot let a call take the allocator's lock or grow a memory
// pool in the middle of a run, or a host whose device memory is fully
// reserved up front. The allocating entry point takes its scratch with a
// stream-ordered allocation on every call; this one never calls an
// allocator.
//
// Limits and rules for callers:
//  * scratch is MCT_GRID_NOALLOC_SCRATCH_BYTES (32 MiB) per device; a call
//    whose chains, grid and nucleus count need more is rejected with
//    MCT_ERR_ARG before anything is launched;
//  * the first call on a device looks up the array's device address with
//    that device current; make that first call before any stream capture.
//    The address is kept for the life of the process: after cudaDeviceReset
//    (which destroys the device's copy of the array) further calls are not
//    supported;
//  * errors found on the device (bad per-chain inputs, a failed tie
//    resolution) are recorded as for the allocating entry point and read
//    with mct_grid_status;
//  * the array is shared by every call on the device: two calls whose work
//    overlaps in time (different streams, or different host threads without
//    ordering between them) race on it and produce wrong grids. Order such
//    calls on one stream or with events.
#include "mct_common.cuh"
#include <string>

namespace {

constexpr size_t kScratchBytes = MCT_GRID_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_grid_scratch[kScratchBytes];

std::mutex g_setup_mu;
void *g_scratch_ptr[kMaxDevices] = {};

int scratch_for_current_device(void **out) {
  int dev = -1;
  MCT_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    mct_set_error("mct_grid_nearest_batch_device_noalloc", "device ordinal beyond 63", __FILE__, __LINE__);
    return MCT_ERR_ARG;
  }
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    MCT_CUDA_TRY(cudaGetSymbolAddress(&p, g_grid_scratch));
    if (!p) {
      mct_set_error("cudaGetSymbolAddress", "null address for the scratch array", __FILE__, __LINE__);
      return MCT_ERR_CUDA;
    }
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return MCT_OK;
}

}  // namespace

extern "C" int mct_grid_nearest_batch_device_noalloc(
    int d, int nchains, int ncell_max, const int *ncells, const double *points,
    const double *params, int nx, int ny, int nz, const double *grid_lo, const double *grid_step,
    const int *box, int *sites_id, double *vp, double *vs, double *rho, void *stream) {
  const char *name = "mct_grid_nearest_batch_device_noalloc";
  if ((d != 2 && d != 3) || nchains < 1 || ncell_max < 1 || nx < 1 || ny < 1 || (d == 3 && nz < 1)) {
    mct_set_error(name, "bad sizes", __FILE__, __LINE__);
    return MCT_ERR_ARG;
  }
  if (ncell_max > 12800) {
    mct_set_error(name, "ncell_max > 12800", __FILE__, __LINE__);
    return MCT_ERR_ARG;
  }
  const long nodes = (long)nx * ny * (d == 3 ? nz : 1);
  const size_t kd = kd_scratch_bytes(ncell_max);
  // same scratch layout as the allocating entry point
  const size_t need = carve_size({sizeof(int) * (size_t)nchains, sizeof(int) * (size_t)nchains * nodes,
                                  kd * nchains, sizeof(int)});
  if (need > kScratchBytes) {
    std::string why = "needs " + std::to_string(need) + " bytes of scratch; the fixed scratch holds " +
                      std::to_string(kScratchBytes) + " (use fewer chains per call or the allocating entry point)";
    mct_set_error(name, why.c_str(), __FILE__, __LINE__);
    return MCT_ERR_ARG;
  }
  void *scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Carve cv(scratch);
  GridJob job{};
  job.d = d; job.nx = nx; job.ny = ny; job.nz = d == 3 ? nz : 1;
  job.xmin = grid_lo[0]; job.ymin = grid_lo[1]; job.zmin = d == 3 ? grid_lo[2] : 0.0;
  job.dx = grid_step[0]; job.dy = grid_step[1]; job.dz = d == 3 ? grid_step[2] : 0.0;
  job.nchains = nchains; job.ncell_max = ncell_max; job.ncells = ncells;
  job.points = points; job.params = params; job.box = box;
  job.sites_id = sites_id; job.vp = vp; job.vs = vs; job.rho = rho;
  job.tie_count = cv.take<int>(nchains);
  job.tie_nodes = cv.take<int>((size_t)nchains * nodes);
  job.kd_scratch = cv.take<char>(kd * nchains);
  job.status = cv.take<int>(1);
  // Must start at zero: the error word (here) and the per-chain tie counters
  // (cleared by the launcher). Tie lists and kd-tree storage are written
  // before they are read.
  MCT_CUDA_TRY(cudaMemsetAsync(job.status, 0, sizeof(int), s));
  return launch_grid_nearest(job, s);
}
