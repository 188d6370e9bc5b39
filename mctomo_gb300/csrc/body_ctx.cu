// Batched body-wave (P and S) likelihood: the GPU replacement of
// likelihood() cases 0/1 (src/likelihood.f90:57-93) -> body_likelihood
// (src/likelihood_body.F90:151-337), with the kdtree_to_grid call the
// sampler makes before it.
//
// Per forward and chain: nearest-nucleus gridding of vp and vs; one 3D
// travel-time solve per station and phase when there are more events than
// stations (reciprocity, likelihood_body.F90:226-250), otherwise one per
// event; trilinear times at the other end of every path; then sigma and the
// misfit / -log L with the events' origin times (:284-333). The z axis is
// scaled by the grid's scaling factor as the reference's call does
// (dz/scaling, zmin/scaling).
#include "mct_common.cuh"
#include "eikonal3d.cuh"
#include "../../include/mctomo.h"
#include <vector>
#include <cfloat>
#include <climits>
#include <algorithm>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <mutex>
#include <string>
#include <system_error>
#include <thread>

namespace {

__global__ void body_material_kernel(int ncell_max, const int *ncells, const double *in, double *out) {
  const int c = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ncell_max; i += gridDim.x * blockDim.x) {
    size_t o = ((size_t)c * ncell_max + i) * 3;
    bool live = i < ncells[c];
    out[o] = live ? in[o] : 1.0; out[o + 1] = live ? in[o + 1] : 1.0; out[o + 2] = live ? in[o + 2] : 1.0;
  }
}

// Solve sources and receiver sets for every (chain, phase, station|event).
__global__ void body_geometry_kernel(int nchains, int nph, int nsrc, int nrev, int from_rev, const double *rev,
                                     const double *loc, double xmin, double ymin, double zmin_s, int nslots,
                                     double *src_out, int *grid_out, double *recv_out, int *recv_set) {
  const int per_chain = nph * (from_rev ? nrev : nsrc);
  const int total = nchains * per_chain;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += gridDim.x * blockDim.x) {
    int c = q / per_chain, r = q % per_chain;
    int ph = r / (from_rev ? nrev : nsrc), e = r % (from_rev ? nrev : nsrc);
    const double *p = from_rev ? rev + 3 * e : loc + ((size_t)c * nsrc + e) * 4;
    src_out[3 * q] = p[0] - xmin; src_out[3 * q + 1] = p[1] - ymin; src_out[3 * q + 2] = p[2] - zmin_s;
    grid_out[q] = ph == 0 ? c : nslots + c;      // vp grids, then vs grids
    recv_set[q] = c;
  }
  // receiver sets: per chain, the other end of every path
  const int nrecv = from_rev ? nsrc : nrev;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nchains * nrecv; q += gridDim.x * blockDim.x) {
    int c = q / nrecv, k = q % nrecv;
    const double *p = from_rev ? loc + ((size_t)c * nsrc + k) * 4 : rev + 3 * k;
    recv_out[3 * q] = p[0] - xmin; recv_out[3 * q + 1] = p[1] - ymin; recv_out[3 * q + 2] = p[2] - zmin_s;
  }
}

struct BodyDev {
  int nsrc, nrev, np, nrays, sigdep, from_rev;
  const int *raystat; const double *dtime, *dsigma;
};

// misfit with origin times (likelihood_body.F90:284-333), one block per chain
__global__ void body_misfit_kernel(BodyDev d, int nchains, const double *tt, const double *loc, const double *n0,
                                   const double *n1, double *ptime, double *out) {
  const int c = blockIdx.x;
  const int npairs = d.nsrc * d.nrev;
  const int nsol = d.from_rev ? d.nrev : d.nsrc, nrecv = d.from_rev ? d.nsrc : d.nrev;
  double like = 0, mis = 0, umis = 0, slog = 0;
  int bad = 0;
  for (int q = threadIdx.x; q < d.np * npairs; q += blockDim.x) {
    int p = q / npairs, r = q % npairs;
    int j = r / d.nrev, k = r % d.nrev;             // source j, receiver k (nrr = k + (j-1)*nrev)
    int sol = d.from_rev ? k : j, end = d.from_rev ? j : k;
    double t = tt[(((size_t)c * d.np + p) * nsol + sol) * nrecv + end];   // phaseTime(k,j,p)
    ptime[((size_t)c * d.np + p) * npairs + r] = t;
    bool used = d.raystat[(size_t)p * npairs + r] == 1;
    double sig = used ? (d.sigdep ? n0[(size_t)c * d.np + p] * t + n1[(size_t)c * d.np + p]
                                  : d.dsigma[(size_t)p * npairs + r]) : 1.0;
    if (used) {
      if (sig < 2.2250738585072014e-307) bad = 1;
      double res = t + loc[((size_t)c * d.nsrc + j) * 4 + 3] - d.dtime[(size_t)p * npairs + r];
      double r2 = res * res;
      like += r2 / (2 * (sig * sig));
      mis += r2 / (sig * sig);
      umis += r2;
    }
    slog += log(sig);
  }
  __shared__ double red[4][256];
  __shared__ int sbad;
  if (threadIdx.x == 0) sbad = 0;
  __syncthreads();
  if (bad) sbad = 1;
  red[0][threadIdx.x] = like; red[1][threadIdx.x] = mis; red[2][threadIdx.x] = umis; red[3][threadIdx.x] = slog;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      for (int k = 0; k < 4; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double PI2 = (double)6.283185f;
    double L = red[0][0] + red[3][0] + (double)((float)d.nrays / 2.0f) * log(PI2);
    out[(size_t)c * 4 + 0] = sbad ? DBL_MAX : L;
    out[(size_t)c * 4 + 1] = red[1][0];
    out[(size_t)c * 4 + 2] = red[2][0];
    out[(size_t)c * 4 + 3] = sbad ? 8.0 : 0.0;
  }
}

// Interpolate3d (src/likelihood_body.F90:976-1005) with point2idx
// (:1038-1054): the trilinear time of a field (nx, ny, nz; z fastest) at an
// event location, with the reference's cell clamp and REAL*4 1.0 weights.
__device__ double interpolate3d(const double *f, int nx, int ny, int nz, double xmin, double ymin, double zmin,
                                double dx, double dy, double dz, double scaling, const double *pt) {
  int ix = (int)floor((pt[0] - xmin) / dx) + 1;
  int iy = (int)floor((pt[1] - ymin) / dy) + 1;
  int iz = (int)floor((pt[2] - zmin / scaling) / (dz / scaling)) + 1;
  if (ix < 1) ix = 1;
  if (iy < 1) iy = 1;
  if (iz < 1) iz = 1;
  if (ix >= nx) ix = nx - 1;
  if (iy >= ny) iy = ny - 1;
  if (iz >= nz) iz = nz - 1;
  const double dsx = pt[0] - (xmin + (ix - 1) * dx);
  const double dsy = pt[1] - (ymin + (iy - 1) * dy);
  const double dsz = pt[2] - (zmin + (iz - 1) * dz) / scaling;
  double qv = 0;
  for (int i = 1; i <= 2; ++i)
    for (int j = 1; j <= 2; ++j)
      for (int k = 1; k <= 2; ++k) {
        const double w = (1.0 - fabs((i - 1) * dx - dsx) / dx) * (1.0 - fabs((j - 1) * dy - dsy) / dy) *
                         (1.0 - fabs((k - 1) * dz / scaling - dsz) / (dz / scaling));
        qv = qv + w * f[((size_t)(ix + i - 2) * ny + (iy + j - 2)) * nz + (iz + k - 2)];
      }
  return qv;
}

// body_location_likelihood (src/likelihood_body.F90:82-149): the committed
// fields of chain c (one per station and phase) read at the events' proposed
// locations, then the misfit with origin times and sigma = n0 * time + n1
// for every pair (unused pairs sigma 1); status 16 when nothing is committed.
__global__ void body_location_kernel(BodyDev d, mct_grid g, const double *cfield, const double *loc,
                                     const double *n0, const double *n1, const int *committed, double *ptime,
                                     double *out) {
  const int c = blockIdx.x;
  const int npairs = d.nsrc * d.nrev;
  const size_t nn = (size_t)g.nx * g.ny * g.nz;
  double like = 0, mis = 0, umis = 0, slog = 0;
  for (int q = threadIdx.x; q < d.np * npairs; q += blockDim.x) {
    const int p = q / npairs, r = q % npairs;
    const int j = r / d.nrev, k = r % d.nrev;       // event j, station k
    const double *f = cfield + (((size_t)c * d.np + p) * d.nrev + k) * nn;
    const double t = interpolate3d(f, g.nx, g.ny, g.nz, g.xmin, g.ymin, g.zmin, g.dx, g.dy, g.dz, g.scaling,
                                   loc + ((size_t)c * d.nsrc + j) * 4);
    ptime[((size_t)c * d.np + p) * npairs + r] = t;
    const bool used = d.raystat[(size_t)p * npairs + r] == 1;
    const double sig = used ? n0[(size_t)c * d.np + p] * t + n1[(size_t)c * d.np + p] : 1.0;
    if (used) {
      const double res = t + loc[((size_t)c * d.nsrc + j) * 4 + 3] - d.dtime[(size_t)p * npairs + r];
      const double r2 = res * res;
      like += r2 / (2 * (sig * sig));
      mis += r2 / (sig * sig);
      umis += r2;
    }
    slog += log(sig);
  }
  __shared__ double red[4][256];
  red[0][threadIdx.x] = like; red[1][threadIdx.x] = mis; red[2][threadIdx.x] = umis; red[3][threadIdx.x] = slog;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st)
      for (int m = 0; m < 4; ++m) red[m][threadIdx.x] += red[m][threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double PI2 = (double)6.283185f;
    const bool ok = committed[c] != 0;
    out[(size_t)c * 4 + 0] = ok ? red[0][0] + red[3][0] + (double)((float)d.nrays / 2.0f) * log(PI2) : DBL_MAX;
    out[(size_t)c * 4 + 1] = red[1][0];
    out[(size_t)c * 4 + 2] = red[2][0];
    out[(size_t)c * 4 + 3] = ok ? 0.0 : 16.0;
  }
}

// The fields of an accepted forward become its chain's committed fields.
__global__ void body_field_commit_kernel(size_t n, const int *accept, const double *out, const double *field,
                                         double *cfield) {
  const int c = blockIdx.y;
  if (!accept[c] || out[(size_t)c * 4 + 3] != 0.0) return;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
    cfield[(size_t)c * n + q] = field[(size_t)c * n + q];
}

// A location step's times become the chain's committed times.
__global__ void body_loc_commit_kernel(int n, const int *accept, const double *out, const double *lptime,
                                       double *cptime) {
  const int c = blockIdx.y;
  if (!accept[c] || out[(size_t)c * 4 + 3] != 0.0) return;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x)
    cptime[(size_t)c * n + q] = lptime[(size_t)c * n + q];
}

}  // namespace

// An accepted proposal becomes its chain's state (what the reference keeps
// in `like` after the Metropolis step; a rejected one is restored from the
// backup, src/mcmc_loc2.f90:456-465).
__global__ void body_commit_kernel(int n, const int *accept, const double *out, const double *ptime, double *cptime,
                                   int *committed) {
  const int c = blockIdx.y;
  if (!accept[c] || out[(size_t)c * 4 + 3] != 0.0) return;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x)
    cptime[(size_t)c * n + q] = ptime[(size_t)c * n + q];
  if (blockIdx.x == 0 && threadIdx.x == 0) committed[c] = 1;
}

// body_noise_likelihood (src/likelihood_body.F90:38-80): each chain's
// committed phase times re-reduced with new noise parameters and origin
// times, sigma = n0 * phase time + n1 for every pair, unused pairs with
// sigma = 1; status 16 when nothing is committed yet.
__global__ void body_noise_kernel(BodyDev d, const double *ptime, const double *loc, const double *n0,
                                  const double *n1, const int *committed, double *out) {
  const int c = blockIdx.x;
  const int npairs = d.nsrc * d.nrev;
  double like = 0, mis = 0, umis = 0, slog = 0;
  for (int q = threadIdx.x; q < d.np * npairs; q += blockDim.x) {
    const int p = q / npairs, r = q % npairs;
    const int j = r / d.nrev;
    const double t = ptime[((size_t)c * d.np + p) * npairs + r];
    const bool used = d.raystat[(size_t)p * npairs + r] == 1;
    const double sig = used ? n0[(size_t)c * d.np + p] * t + n1[(size_t)c * d.np + p] : 1.0;
    if (used) {
      const double res = t + loc[((size_t)c * d.nsrc + j) * 4 + 3] - d.dtime[(size_t)p * npairs + r];
      const double r2 = res * res;
      like += r2 / (2 * (sig * sig));
      mis += r2 / (sig * sig);
      umis += r2;
    }
    slog += log(sig);
  }
  __shared__ double red[4][256];
  red[0][threadIdx.x] = like; red[1][threadIdx.x] = mis; red[2][threadIdx.x] = umis; red[3][threadIdx.x] = slog;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st)
      for (int k = 0; k < 4; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double PI2 = (double)6.283185f;
    const bool ok = committed[c] != 0;
    out[(size_t)c * 4 + 0] = ok ? red[0][0] + red[3][0] + (double)((float)d.nrays / 2.0f) * log(PI2) : DBL_MAX;
    out[(size_t)c * 4 + 1] = red[1][0];
    out[(size_t)c * 4 + 2] = red[2][0];
    out[(size_t)c * 4 + 3] = ok ? 0.0 : 16.0;
  }
}

struct mct_body_ctx {
  mct_grid g{};
  int order = 0, np = 1, sigdep = 1, nslots = 0, ncell_max = 0;
  BodyDev dev{};
  cudaStream_t stream = nullptr;
  void *mem = nullptr;
  // device buffers
  int *ncells = nullptr; double *points = nullptr, *params_in = nullptr, *params = nullptr, *loc = nullptr;
  double *n0 = nullptr, *n1 = nullptr, *out = nullptr, *rev = nullptr;
  int *sites = nullptr; double *vel = nullptr; float *slow = nullptr;
  int *tie_count = nullptr, *tie_nodes = nullptr; void *kd = nullptr; int *gstatus = nullptr;
  double *esrc = nullptr, *erecv = nullptr, *ett = nullptr, *ptime = nullptr;
  double *cptime = nullptr, *nout = nullptr;          // committed times, noise-only results
  int *committed = nullptr, *accept = nullptr;
  int *gshift = nullptr;                              // [2 * nslots] fixed-point shift per grid
  int *egrid = nullptr, *eset = nullptr, *T = nullptr, *list = nullptr, *count = nullptr;
  unsigned char *flags = nullptr;
  // 3D solver and the heap march's scratch
  int method = EIK3_TILES;
  double2 *hvn = nullptr; void *hscratch = nullptr;
  int hchunk = 0; int *herr = nullptr;
  int last_nchains = 0, last_passes = 0;
  // dynamic (settings.dynamic): the travel-time fields of the last forward
  // and of each chain's committed model, [nslots][np][nrev][nodes] FP64
  // (the reference's like%field5d), the location step's times
  int dynamic = 0;
  double *field = nullptr, *cfield = nullptr, *lptime = nullptr, *lout = nullptr;
  // mct_body_submit / mct_body_poll: the forward waits on the host between
  // the 3D solver's passes, so a submitted batch runs on a worker thread of
  // the context (started by the first submit) with copies of the caller's
  // arrays; state 0 idle, 1 submitted, 2 finished (results in sub.out)
  int device = 0;
  std::thread worker;
  std::mutex mu;
  std::condition_variable cv;
  bool job_ready = false, quit = false;
  std::atomic<int> state{0};
  struct Submitted {
    int nchains = 0, rc = 0;
    std::vector<int> ncells;
    std::vector<double> points, params, loc, n0, n1, out;
    std::string err;
  } sub;
};

namespace {
int body_forward(mct_body_ctx *c, int nchains, const int *ncells, const double *points, const double *params,
                 const double *locations, const double *n0, const double *n1, double *out);

void body_worker(mct_body_ctx *c) {
  cudaSetDevice(c->device);
  std::unique_lock<std::mutex> lk(c->mu);
  for (;;) {
    c->cv.wait(lk, [c] { return c->job_ready || c->quit; });
    if (c->quit) return;
    c->job_ready = false;
    lk.unlock();
    mct_body_ctx::Submitted &j = c->sub;
    j.rc = body_forward(c, j.nchains, j.ncells.data(), j.points.data(), j.params.data(), j.loc.data(), j.n0.data(),
                        j.n1.data(), j.out.data());
    j.err = j.rc < 0 ? mct_last_error() : "";
    c->state.store(2, std::memory_order_release);
    lk.lock();
  }
}

// a submitted batch has not been polled: the blocking calls are refused
bool busy(const mct_body_ctx *c, const char *name) {
  if (c->state.load(std::memory_order_acquire) == 0) return false;
  mct_set_error(name, "a submitted batch is not polled yet", __FILE__, __LINE__);
  return true;
}
}  // namespace

extern "C" {

int mct_body_create(const mct_grid *g, const mct_body_settings *st, const mct_body_data *dat, int nslots,
                    int ncell_max, mct_body_ctx **out) {
  if (!g || !st || !dat || !out || nslots < 1 || ncell_max < 1 || ncell_max > 12800) return MCT_ERR_ARG;
  if (g->nx < 2 || g->ny < 2 || g->nz < 2 || !(g->dx > 0) || !(g->dy > 0) || !(g->dz > 0) || !(g->scaling > 0))
    return MCT_ERR_ARG;
  if (st->np != 1 && st->np != 2) return MCT_ERR_ARG;
  if (st->order != 0 && st->order != 1) return MCT_ERR_ARG;
  if (st->solver != 0 && st->solver != MCT_EIK3_TILES && st->solver != MCT_EIK3_HEAP) return MCT_ERR_ARG;
  if (st->dynamic != 0 && st->dynamic != 1) return MCT_ERR_ARG;
  if (dat->nsrc < 1 || dat->nrev < 1 || dat->np != st->np) return MCT_ERR_ARG;
  *out = nullptr;
  mct_body_ctx *c = new mct_body_ctx();
  c->g = *g; c->order = st->order; c->np = st->np; c->sigdep = st->sigdep; c->nslots = nslots; c->ncell_max = ncell_max;
  const int nsrc = dat->nsrc, nrev = dat->nrev, np = dat->np, npairs = nsrc * nrev;
  // likelihood_body.F90:204,226; with stored fields always from the
  // stations (:251-281), whose fields the location steps read
  const int from_rev = (nsrc > nrev || st->dynamic) ? 1 : 0;
  const int nsol = from_rev ? nrev : nsrc, nrecv = from_rev ? nsrc : nrev;
  const size_t nn = (size_t)g->nx * g->ny * g->nz;
  const size_t nsolve = (size_t)nslots * np * nsol;
  Eik3Job tmp{}; tmp.nx = g->nx; tmp.ny = g->ny; tmp.nz = g->nz;
  const int method = eik3_resolve_method(st->order, st->solver == MCT_EIK3_TILES ? EIK3_TILES
                                                    : st->solver == MCT_EIK3_HEAP ? EIK3_HEAP : EIK3_DEFAULT);
  const bool heap = method == EIK3_HEAP;
  if (heap && nn > (size_t)0x3FFFFFFF) { delete c; return MCT_ERR_ARG; }   // 30-bit node indices
  c->method = method;
  const size_t ntile = heap ? 0 : eik3_tiles(tmp);
  const size_t nT = heap ? 0 : nsolve * nn;
  // heap march: as many solves at once as fit in min(48 GiB, half the free
  // memory); the rest run in further equal chunks
  size_t hchunk = 0;
  if (heap) {
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) { delete c; return MCT_ERR_CUDA; }
    const size_t budget = std::min<size_t>(48ull << 30, fr / 2);
    hchunk = std::max<size_t>(1, std::min<size_t>(nsolve, budget / eik3_heap_bytes_per_solve(g->nx, g->ny, g->nz)));
  }
  const size_t kd = kd_scratch_bytes(ncell_max);
  std::vector<size_t> sz = {
      sizeof(int) * nslots, sizeof(double) * (size_t)nslots * ncell_max * 3 * 3, sizeof(double) * (size_t)nslots * nsrc * 4,
      sizeof(double) * 2 * (size_t)nslots * np, sizeof(double) * 4 * nslots, sizeof(double) * 3 * nrev,
      sizeof(int) * (size_t)nslots * nn, sizeof(double) * 2 * (size_t)nslots * nn, sizeof(float) * 2 * (size_t)nslots * nn,
      sizeof(int) * nslots, sizeof(int) * (size_t)nslots * nn, kd * nslots, sizeof(int) * 2,
      sizeof(double) * 3 * nsolve, sizeof(double) * 3 * (size_t)nslots * nrecv, sizeof(double) * nsolve * nrecv,
      sizeof(double) * (size_t)nslots * np * npairs, sizeof(int) * nsolve, sizeof(int) * nsolve,
      sizeof(int) * nT, ntile * nsolve, sizeof(int) * ntile * nsolve, sizeof(int),
      sizeof(int) * np * npairs, sizeof(double) * 2 * np * npairs,
      heap ? sizeof(double2) * 2 * (size_t)nslots * nn : 0,
      eik3_heap_scratch_bytes(g->nx, g->ny, g->nz, (int)hchunk), sizeof(int),
      sizeof(double) * (size_t)nslots * np * npairs, sizeof(int) * 2 * nslots, sizeof(double) * 4 * nslots,
      sizeof(int) * 2 * nslots,
      st->dynamic ? 2 * sizeof(double) * (size_t)nslots * np * nrev * nn : 0,
      st->dynamic ? sizeof(double) * (size_t)nslots * np * npairs : 0, st->dynamic ? sizeof(double) * 4 * nslots : 0};
  size_t total = 0;
  for (size_t s : sz) total = ((total + 255) & ~size_t(255)) + s;
  total += 256;
  if (cudaMalloc(&c->mem, total) != cudaSuccess) { delete c; return MCT_ERR_NOMEM; }
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaFree(c->mem); delete c; return MCT_ERR_CUDA;
  }
  Carve cv(c->mem);
  c->ncells = cv.take<int>(nslots);
  c->points = cv.take<double>((size_t)nslots * ncell_max * 9);
  c->params_in = c->points + (size_t)nslots * ncell_max * 3;
  c->params = c->params_in + (size_t)nslots * ncell_max * 3;
  c->loc = cv.take<double>((size_t)nslots * nsrc * 4);
  c->n0 = cv.take<double>((size_t)2 * nslots * np); c->n1 = c->n0 + (size_t)nslots * np;
  c->out = cv.take<double>((size_t)4 * nslots);
  c->rev = cv.take<double>((size_t)3 * nrev);
  c->sites = cv.take<int>((size_t)nslots * nn);
  c->vel = cv.take<double>((size_t)2 * nslots * nn);
  c->slow = cv.take<float>((size_t)2 * nslots * nn);
  c->tie_count = cv.take<int>(nslots);
  c->tie_nodes = cv.take<int>((size_t)nslots * nn);
  c->kd = cv.take<char>(kd * nslots);
  c->gstatus = cv.take<int>(2);
  c->esrc = cv.take<double>(3 * nsolve);
  c->erecv = cv.take<double>((size_t)3 * nslots * nrecv);
  c->ett = cv.take<double>(nsolve * nrecv);
  c->ptime = cv.take<double>((size_t)nslots * np * npairs);
  c->egrid = cv.take<int>(nsolve);
  c->eset = cv.take<int>(nsolve);
  c->T = cv.take<int>(nT);
  c->flags = cv.take<unsigned char>(ntile * nsolve);
  c->list = cv.take<int>(ntile * nsolve);
  c->count = cv.take<int>(1);
  int *rays = cv.take<int>((size_t)np * npairs);
  double *dt = cv.take<double>((size_t)2 * np * npairs);
  c->hvn = cv.take<double2>(heap ? 2 * (size_t)nslots * nn : 0);
  c->hscratch = cv.take<char>(eik3_heap_scratch_bytes(g->nx, g->ny, g->nz, (int)hchunk));
  c->herr = cv.take<int>(1);
  c->cptime = cv.take<double>((size_t)nslots * np * npairs);
  c->committed = cv.take<int>(2 * (size_t)nslots);
  c->accept = c->committed + nslots;
  c->nout = cv.take<double>(4 * (size_t)nslots);
  c->gshift = cv.take<int>(2 * (size_t)nslots);
  c->dynamic = st->dynamic;
  if (st->dynamic) {
    c->field = cv.take<double>(2 * (size_t)nslots * np * nrev * nn);
    c->cfield = c->field + (size_t)nslots * np * nrev * nn;
    c->lptime = cv.take<double>((size_t)nslots * np * npairs);
    c->lout = cv.take<double>(4 * (size_t)nslots);
  }
  cudaMemset(c->committed, 0, sizeof(int) * 2 * nslots);
  c->hchunk = (int)hchunk;
  std::vector<double> hs((size_t)np * npairs, 1.0);
  if (dat->sigma) for (size_t q = 0; q < hs.size(); ++q) hs[q] = dat->sigma[q];
  cudaMemcpy(c->rev, dat->rev, sizeof(double) * 3 * nrev, cudaMemcpyHostToDevice);
  cudaMemcpy(rays, dat->raystat, sizeof(int) * np * npairs, cudaMemcpyHostToDevice);
  cudaMemcpy(dt, dat->ttime, sizeof(double) * np * npairs, cudaMemcpyHostToDevice);
  cudaMemcpy(dt + (size_t)np * npairs, hs.data(), sizeof(double) * np * npairs, cudaMemcpyHostToDevice);
  if (cudaDeviceSynchronize() != cudaSuccess) { cudaFree(c->mem); cudaStreamDestroy(c->stream); delete c; return MCT_ERR_CUDA; }
  c->dev = BodyDev{nsrc, nrev, np, dat->nrays, st->sigdep, from_rev, rays, dt, dt + (size_t)np * npairs};
  cudaGetDevice(&c->device);
  *out = c;
  return MCT_OK;
}

int mct_body_set_priority(mct_body_ctx *c, int high) {
  if (!c || busy(c, "mct_body_set_priority")) return MCT_ERR_ARG;
  return mct_restream(&c->stream, high);
}

int mct_body_destroy(mct_body_ctx *c) {
  if (!c) return MCT_OK;
  if (c->worker.joinable()) {
    // the worker finishes a batch in flight before it sees quit
    { std::lock_guard<std::mutex> lk(c->mu); c->quit = true; }
    c->cv.notify_one();
    c->worker.join();
  }
  cudaStreamSynchronize(c->stream);
  cudaFree(c->mem);
  cudaStreamDestroy(c->stream);
  delete c;
  return MCT_OK;
}

int mct_body_forward(mct_body_ctx *c, int nchains, const int *ncells, const double *points, const double *params,
                     const double *locations, const double *n0, const double *n1, double *out) {
  if (!c || busy(c, "mct_body_forward") || nchains < 1 || nchains > c->nslots) return MCT_ERR_ARG;
  for (int i = 0; i < nchains; ++i) if (ncells[i] < 1 || ncells[i] > c->ncell_max) return MCT_ERR_ARG;
  return body_forward(c, nchains, ncells, points, params, locations, n0, n1, out);
}

int mct_body_submit(mct_body_ctx *c, int nchains, const int *ncells, const double *points, const double *params,
                    const double *locations, const double *n0, const double *n1) {
  if (!c || busy(c, "mct_body_submit") || nchains < 1 || nchains > c->nslots || !ncells || !points || !params ||
      !locations || !n0 || !n1)
    return MCT_ERR_ARG;
  for (int i = 0; i < nchains; ++i) if (ncells[i] < 1 || ncells[i] > c->ncell_max) return MCT_ERR_ARG;
  mct_body_ctx::Submitted &j = c->sub;
  const size_t pc = (size_t)nchains * c->ncell_max * 3, nl = (size_t)nchains * c->dev.nsrc * 4;
  const size_t nn = (size_t)nchains * c->dev.np;
  j.nchains = nchains;
  j.ncells.assign(ncells, ncells + nchains);
  j.points.assign(points, points + pc);
  j.params.assign(params, params + pc);
  j.loc.assign(locations, locations + nl);
  j.n0.assign(n0, n0 + nn);
  j.n1.assign(n1, n1 + nn);
  j.out.assign((size_t)4 * nchains, 0.0);
  if (!c->worker.joinable()) {
    try {
      c->worker = std::thread(body_worker, c);
    } catch (const std::system_error &e) {
      mct_set_error("mct_body_submit", e.what(), __FILE__, __LINE__);
      return MCT_ERR_INTERNAL;
    }
  }
  {
    std::lock_guard<std::mutex> lk(c->mu);
    c->state.store(1, std::memory_order_release);
    c->job_ready = true;
  }
  c->cv.notify_one();
  return MCT_OK;
}

int mct_body_poll(mct_body_ctx *c, double *out, int *done) {
  if (!c || !out || !done || c->state.load(std::memory_order_acquire) == 0) return MCT_ERR_ARG;
  *done = 0;
  if (c->state.load(std::memory_order_acquire) != 2) return MCT_OK;
  mct_body_ctx::Submitted &j = c->sub;
  std::memcpy(out, j.out.data(), sizeof(double) * 4 * j.nchains);
  const int rc = j.rc;
  if (rc < 0) mct_set_error("mct_body_poll", j.err.c_str(), __FILE__, __LINE__);
  c->state.store(0, std::memory_order_release);
  *done = 1;
  return rc;
}

}  // extern "C"

namespace {
int body_forward(mct_body_ctx *c, int nchains, const int *ncells, const double *points, const double *params,
                 const double *locations, const double *n0, const double *n1, double *out) {
  const mct_grid &g = c->g;
  const BodyDev &d = c->dev;
  cudaStream_t s = c->stream;
  const size_t nn = (size_t)g.nx * g.ny * g.nz;
  const size_t pc = (size_t)nchains * c->ncell_max * 3;
  MCT_CUDA_TRY(cudaMemcpyAsync(c->ncells, ncells, sizeof(int) * nchains, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(c->points, points, sizeof(double) * pc, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(c->params_in, params, sizeof(double) * pc, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(c->loc, locations, sizeof(double) * nchains * d.nsrc * 4, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(c->n0, n0, sizeof(double) * nchains * d.np, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(c->n1, n1, sizeof(double) * nchains * d.np, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemsetAsync(c->gstatus, 0, sizeof(int) * 2, s));
  body_material_kernel<<<dim3((c->ncell_max + 127) / 128, nchains), 128, 0, s>>>(c->ncell_max, c->ncells,
                                                                                   c->params_in, c->params);
  MCT_CUDA_TRY(cudaGetLastError());
  // gridding: vp into grids [0, nslots), vs into [nslots, 2 nslots)
  GridJob gj{};
  gj.d = 3; gj.nx = g.nx; gj.ny = g.ny; gj.nz = g.nz;
  gj.xmin = g.xmin; gj.ymin = g.ymin; gj.zmin = g.zmin; gj.dx = g.dx; gj.dy = g.dy; gj.dz = g.dz;
  gj.nchains = nchains; gj.ncell_max = c->ncell_max; gj.ncells = c->ncells;
  gj.points = c->points; gj.params = c->params; gj.box = nullptr;
  gj.sites_id = c->sites; gj.vp = c->vel; gj.vs = c->vel + (size_t)c->nslots * nn;
  gj.rho = reinterpret_cast<double *>(c->slow);   // density is not used by the body path: scratch target
  gj.tie_count = c->tie_count; gj.tie_nodes = c->tie_nodes; gj.kd_scratch = c->kd; gj.status = c->gstatus;
  int rc = launch_grid_nearest(gj, s); if (rc) return rc;
  // solves
  const int nsol = d.from_rev ? d.nrev : d.nsrc, nrecv = d.from_rev ? d.nsrc : d.nrev;
  const int nsolve = nchains * d.np * nsol;
  body_geometry_kernel<<<64, 256, 0, s>>>(nchains, d.np, d.nsrc, d.nrev, d.from_rev, c->rev, c->loc, g.xmin, g.ymin,
                                           g.zmin / g.scaling, c->nslots, c->esrc, c->egrid, c->erecv, c->eset);
  MCT_CUDA_TRY(cudaGetLastError());
  // velocity bound for the fixed-point scale (smallest nucleus velocity)
  std::vector<double> hp(pc);
  MCT_CUDA_TRY(cudaMemcpyAsync(hp.data(), c->params, sizeof(double) * pc, cudaMemcpyDeviceToHost, s));
  MCT_CUDA_TRY(cudaStreamSynchronize(s));
  // per chain, so that a chain's times do not depend on the other chains of
  // the call (its P and S grids share the chain's scale)
  const double dzs = g.dz / g.scaling;
  const double diag = sqrt(((g.nx - 1) * g.dx) * ((g.nx - 1) * g.dx) + ((g.ny - 1) * g.dy) * ((g.ny - 1) * g.dy) +
                           ((g.nz - 1) * dzs) * ((g.nz - 1) * dzs));
  double vmin = 1e300;
  std::vector<int> hshift((size_t)2 * c->nslots, 30);
  for (int ch = 0; ch < nchains; ++ch) {
    double vc = 1e300;
    for (int i = 0; i < ncells[ch]; ++i) {
      const double *q = &hp[((size_t)ch * c->ncell_max + i) * 3];
      if (q[0] > 0 && q[0] < vc) vc = q[0];
      if (d.np > 1 && q[1] > 0 && q[1] < vc) vc = q[1];
    }
    hshift[ch] = hshift[c->nslots + ch] = eik3_shift_for(4.0 * diag / vc);
    vmin = std::min(vmin, vc);
  }
  MCT_CUDA_TRY(cudaMemcpyAsync(c->gshift, hshift.data(), sizeof(int) * hshift.size(), cudaMemcpyHostToDevice, s));
  Eik3Job job{};
  job.nsolve = nsolve; job.nx = g.nx; job.ny = g.ny; job.nz = g.nz; job.dx = g.dx; job.dy = g.dy; job.dz = dzs;
  job.vel = c->vel; job.slow = c->slow; job.ngrids = 2 * c->nslots; job.solve_grid = c->egrid; job.src = c->esrc;
  job.order = c->order; job.method = c->method; job.shift = eik3_shift_for(4.0 * diag / vmin);
  job.grid_shift = c->gshift;
  job.T = c->T; job.flags = c->flags; job.list = c->list; job.count = c->count;
  job.hvn = c->hvn; job.herr = c->herr;
  if (c->method == EIK3_HEAP) {
    Carve hc(c->hscratch);
    eik3_heap_take(job, hc, c->hchunk);
  }
  job.nrev = nrecv; job.rev = c->erecv; job.rev_per_solve = 1; job.solve_rev = c->eset; job.ttime = c->ett;
  int passes = 0;
  rc = launch_eik3(job, s, 100000, &passes, c->dynamic ? c->field : nullptr); if (rc) return rc;
  c->last_passes = passes;
  body_misfit_kernel<<<nchains, 256, 0, s>>>(d, nchains, c->ett, c->loc, c->n0, c->n1, c->ptime, c->out);
  MCT_CUDA_TRY(cudaGetLastError());
  MCT_CUDA_TRY(cudaMemcpyAsync(out, c->out, sizeof(double) * 4 * nchains, cudaMemcpyDeviceToHost, s));
  int gst[2];
  MCT_CUDA_TRY(cudaMemcpyAsync(gst, c->gstatus, sizeof(int) * 2, cudaMemcpyDeviceToHost, s));
  MCT_CUDA_TRY(cudaStreamSynchronize(s));
  c->last_nchains = nchains;
  if (gst[0]) return gst[0];
  return MCT_OK;
}
}  // namespace

extern "C" {

int mct_body_commit(mct_body_ctx *c, int nchains, const int *accept) {
  if (!c || busy(c, "mct_body_commit") || nchains < 1 || nchains > c->last_nchains || !accept) return MCT_ERR_ARG;
  cudaStream_t s = c->stream;
  const int n = c->dev.np * c->dev.nsrc * c->dev.nrev;
  MCT_CUDA_TRY(cudaMemcpyAsync(c->accept, accept, sizeof(int) * nchains, cudaMemcpyHostToDevice, s));
  body_commit_kernel<<<dim3((n + 255) / 256, nchains), 256, 0, s>>>(n, c->accept, c->out, c->ptime, c->cptime,
                                                                    c->committed);
  MCT_CUDA_TRY(cudaGetLastError());
  if (c->dynamic) {
    const size_t nf = (size_t)c->dev.np * c->dev.nrev * c->g.nx * c->g.ny * c->g.nz;
    body_field_commit_kernel<<<dim3(1024, nchains), 256, 0, s>>>(nf, c->accept, c->out, c->field, c->cfield);
    MCT_CUDA_TRY(cudaGetLastError());
  }
  MCT_CUDA_TRY(cudaStreamSynchronize(s));
  return MCT_OK;
}

int mct_body_location_likelihood(mct_body_ctx *c, int nchains, const double *locations, const double *n0,
                                 const double *n1, double *out, double *phase_time) {
  if (!c || busy(c, "mct_body_location_likelihood") || nchains < 1 || nchains > c->nslots || !locations || !n0 ||
      !n1 || !out)
    return MCT_ERR_ARG;
  if (!c->dynamic) {
    mct_set_error("mct_body_location_likelihood", "the context keeps no fields (settings.dynamic = 0): "
                  "a location step is a full forward", __FILE__, __LINE__);
    return MCT_ERR_UNSUPPORTED;
  }
  cudaStream_t s = c->stream;
  const BodyDev &d = c->dev;
  MCT_CUDA_TRY(cudaMemcpyAsync(c->loc, locations, sizeof(double) * nchains * d.nsrc * 4, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(c->n0, n0, sizeof(double) * nchains * d.np, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(c->n1, n1, sizeof(double) * nchains * d.np, cudaMemcpyHostToDevice, s));
  body_location_kernel<<<nchains, 256, 0, s>>>(d, c->g, c->cfield, c->loc, c->n0, c->n1, c->committed, c->lptime,
                                              c->lout);
  MCT_CUDA_TRY(cudaGetLastError());
  MCT_CUDA_TRY(cudaMemcpyAsync(out, c->lout, sizeof(double) * 4 * nchains, cudaMemcpyDeviceToHost, s));
  const size_t npt = (size_t)d.np * d.nsrc * d.nrev;
  if (phase_time)
    MCT_CUDA_TRY(cudaMemcpyAsync(phase_time, c->lptime, sizeof(double) * npt * nchains, cudaMemcpyDeviceToHost, s));
  MCT_CUDA_TRY(cudaStreamSynchronize(s));
  return MCT_OK;
}

int mct_body_location_commit(mct_body_ctx *c, int nchains, const int *accept) {
  if (!c || busy(c, "mct_body_location_commit") || nchains < 1 || nchains > c->nslots || !accept) return MCT_ERR_ARG;
  if (!c->dynamic) return MCT_ERR_UNSUPPORTED;
  cudaStream_t s = c->stream;
  const int n = c->dev.np * c->dev.nsrc * c->dev.nrev;
  MCT_CUDA_TRY(cudaMemcpyAsync(c->accept, accept, sizeof(int) * nchains, cudaMemcpyHostToDevice, s));
  body_loc_commit_kernel<<<dim3((n + 255) / 256, nchains), 256, 0, s>>>(n, c->accept, c->lout, c->lptime,
                                                                        c->cptime);
  MCT_CUDA_TRY(cudaGetLastError());
  MCT_CUDA_TRY(cudaStreamSynchronize(s));
  return MCT_OK;
}

int mct_body_noise_likelihood(mct_body_ctx *c, int nchains, const double *locations, const double *n0,
                              const double *n1, double *out) {
  if (!c || busy(c, "mct_body_noise_likelihood") || nchains < 1 || nchains > c->nslots || !locations || !n0 || !n1 ||
      !out)
    return MCT_ERR_ARG;
  cudaStream_t s = c->stream;
  const BodyDev &d = c->dev;
  MCT_CUDA_TRY(cudaMemcpyAsync(c->loc, locations, sizeof(double) * nchains * d.nsrc * 4, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(c->n0, n0, sizeof(double) * nchains * d.np, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(c->n1, n1, sizeof(double) * nchains * d.np, cudaMemcpyHostToDevice, s));
  body_noise_kernel<<<nchains, 256, 0, s>>>(d, c->cptime, c->loc, c->n0, c->n1, c->committed, c->nout);
  MCT_CUDA_TRY(cudaGetLastError());
  MCT_CUDA_TRY(cudaMemcpyAsync(out, c->nout, sizeof(double) * 4 * nchains, cudaMemcpyDeviceToHost, s));
  MCT_CUDA_TRY(cudaStreamSynchronize(s));
  return MCT_OK;
}

int mct_body_phase_time(mct_body_ctx *c, int index, double *phase_time, int *passes) {
  if (!c || busy(c, "mct_body_phase_time") || index < 0 || index >= c->last_nchains) return MCT_ERR_ARG;
  const size_t n = (size_t)c->dev.np * c->dev.nsrc * c->dev.nrev;
  MCT_CUDA_TRY(cudaStreamSynchronize(c->stream));
  if (phase_time) MCT_CUDA_TRY(cudaMemcpy(phase_time, c->ptime + (size_t)index * n, sizeof(double) * n,
                                          cudaMemcpyDeviceToHost));
  if (passes) *passes = c->last_passes;
  return MCT_OK;
}

}  // extern "C"
