// Surface-wave likelihood context: device-resident chain slots and the C ABI
// around surf_forward / surf_commit (surf_pipeline.cu).
#include "mct_common.cuh"
#include "surf_pipeline.cuh"
#include <algorithm>
#include <cmath>
#include <vector>
#include <cstring>
#include <string>

struct mct_surf_ctx {
  SurfBatch b{};          // device pointers and sizes (inputs re-pointed per call)
  SurfPlan plan{};
  int nslots = 0;
  cudaStream_t stream = nullptr;
  void *mem = nullptr;    // one allocation for everything
  // device staging for host-pointer calls
  int *d_slots = nullptr, *d_ncells = nullptr, *d_accept = nullptr;
  double *d_points = nullptr, *d_params = nullptr, *d_n0 = nullptr, *d_n1 = nullptr, *d_out = nullptr;
  int last_nchains = 0;
  SurfProfile prof;
  size_t bytes = 0;       // device allocation
  // serving: one submitted batch in flight, pinned host staging, completion event
  int *h_ints = nullptr;              // [nslots] slots, [nslots] ncells, [2] device status
  double *h_dbl = nullptr;            // [nslots][ncell_max][3] points, params; [nslots][np] n0, n1; [nslots][4] out
  cudaEvent_t done = nullptr;
  int pending = 0;
  std::vector<char> in_use;           // slot allocator (mct_surf_admit / mct_surf_evict)
  // posterior statistics (mct_surf_stat_*), allocated by the first
  // mct_surf_stat_add: per slot the sums of vs, vs^2, vp, vp^2 over the
  // committed models added, and their count
  double *st_sum = nullptr;           // [nslots][4][nodes]
  int *st_slots = nullptr;            // [nslots] device copy of the call's slots
  std::vector<int> st_n;
};

namespace {
// stat_rti (src/mcmc_loc2.f90:1975-1978): aveS += vs, stdS += vs**2,
// aveP += vp, stdP += vp**2, node by node, for each listed slot's committed
// model
__global__ void stat_add_kernel(int nchains, const int *slots, size_t nodes, const double *cvp, const double *cvs,
                                double *sum) {
  const int slot = slots[blockIdx.y];
  const double *vp = cvp + (size_t)slot * nodes, *vs = cvs + (size_t)slot * nodes;
  double *s = sum + (size_t)slot * 4 * nodes;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < nodes; q += (size_t)gridDim.x * blockDim.x) {
    const double v = vs[q], p = vp[q];
    s[q] = s[q] + v;
    s[nodes + q] = s[nodes + q] + v * v;
    s[2 * nodes + q] = s[2 * nodes + q] + p;
    s[3 * nodes + q] = s[3 * nodes + q] + p * p;
  }
}
}  // namespace

namespace {
std::string &err() { static thread_local std::string e; return e; }
}

namespace {

// Builds a context; with dry set, only computes its device allocation.
int surf_create(const mct_grid *g, const mct_surf_settings *st, const mct_surf_data *dat, int nslots,
                int ncell_max, mct_surf_ctx **out, bool dry, size_t *bytes_out) {
  if (!g || !st || !dat || (!out && !dry) || nslots < 1 || ncell_max < 1 || ncell_max > 12800) return MCT_ERR_ARG;
  if (g->nx < 2 || g->ny < 2 || g->nz < 1 || !(g->dx > 0) || !(g->dy > 0) || !(g->dz > 0) || !(g->scaling > 0))
    return MCT_ERR_ARG;
  if (st->phase_group != 0 && st->phase_group != 1) return MCT_ERR_ARG;
  if (st->straight != 0 && st->straight != 1) return MCT_ERR_ARG;
  if (st->straight == 1) {
    // straight rays must stay inside the model (the reference's fatal
    // 'Straight ray out of area'); the model is a rectangle, so its stations must
    const double xmax = g->xmin + (double)(g->nx - 1) * g->dx, ymax = g->ymin + (double)(g->ny - 1) * g->dy;
    for (int i = 0; i < dat->nsrc; ++i)
      if (dat->src[2 * i] < g->xmin || dat->src[2 * i] > xmax || dat->src[2 * i + 1] < g->ymin ||
          dat->src[2 * i + 1] > ymax)
        return MCT_ERR_OUTSIDE;
    for (int i = 0; i < dat->nrev; ++i)
      if (dat->rev[2 * i] < g->xmin || dat->rev[2 * i] > xmax || dat->rev[2 * i + 1] < g->ymin ||
          dat->rev[2 * i + 1] > ymax)
        return MCT_ERR_OUTSIDE;
  }
  if (st->raylov != 0 && st->raylov != 1) return MCT_ERR_ARG;
  if (dat->np < 1 || dat->np > 60 || dat->nsrc < 1 || dat->nrev < 1) return MCT_ERR_ARG;
  if (!(st->dphase != 0.0)) return MCT_ERR_ARG;
  if (out) *out = nullptr;
  mct_surf_ctx *c = new mct_surf_ctx();
  SurfBatch &b = c->b;
  b.nx = g->nx; b.ny = g->ny; b.nz = g->nz;
  b.xmin = g->xmin; b.ymin = g->ymin; b.zmin = g->zmin; b.dx = g->dx; b.dy = g->dy; b.dz = g->dz;
  b.scaling = g->scaling; b.water_depth = g->water_depth;
  b.law = st->material_law; b.rho_value = st->rho_value;
  b.iwave = st->raylov == 1 ? 2 : 1; b.precision = st->precision; b.dphase = st->dphase;
  b.sigdep = st->sigdep;
  b.igr = st->phase_group; b.straight = st->straight;
  b.np = dat->np; b.nsrc = dat->nsrc; b.nrev = dat->nrev; b.nrays = dat->nrays;
  b.ncell_max = ncell_max;
  b.nl_max = g->nz + 1;
  c->nslots = nslots;
  const int np = dat->np, nsrc = dat->nsrc, nrev = dat->nrev, npairs = nsrc * nrev;
  const size_t nodes = (size_t)g->nx * g->ny * g->nz;
  const size_t ncol = (size_t)g->nx * g->ny;
  const size_t maps = (size_t)np * ncol;
  const size_t nvv = (size_t)(g->nx + 2) * (g->ny + 2);
  // fm2d plan and solve list for one chain (active sources per period)
  Fm2dJob &fj = c->plan.fm2d;
  fj.nvx = g->nx; fj.nvz = g->ny; fj.goxd = g->xmin; fj.gozd = g->ymin; fj.dvxd = g->dx; fj.dvzd = g->dy;
  fj.gdx = st->gridx; fj.gdz = st->gridy; fj.asgr = st->sgref; fj.sgdl = st->sgdic; fj.sgs = st->sgext;
  fj.fom = st->order; fj.nsrc = nsrc; fj.nrc = nrev; fj.srs_nmaps = np;
  fj.precision = (st->tt_precision >= 0 && st->tt_precision <= 2) ? st->tt_precision : 0;
  if (fj.gdx < 1 || fj.gdz < 1 || (fj.asgr == 1 && (fj.sgdl < 1 || fj.sgs < 1))) { delete c; return MCT_ERR_ARG; }
  int rc = fm2d_plan(fj, &c->plan.fm2d_plan);
  if (rc) { delete c; return MCT_ERR_ARG; }
  std::vector<int2> one;
  for (int p = 0; p < np; ++p)
    for (int i = 0; i < nsrc; ++i) {
      int any = 0;
      for (int j = 0; j < nrev; ++j) any |= dat->raystat[(size_t)p * npairs + (size_t)i * nrev + j] == 1;
      if (any || i == 0) one.push_back(make_int2(p, i));
    }
  const int spc = (int)one.size();
  c->plan.nsolve_per_chain = spc;
  std::vector<int2> all((size_t)spc * nslots);
  for (int ch = 0; ch < nslots; ++ch)
    for (int k = 0; k < spc; ++k) all[(size_t)ch * spc + k] = make_int2(ch * np + one[k].x, one[k].y);
  const Fm2dPlan &fp = c->plan.fm2d_plan;
  const size_t nsolve = all.size();
  const int nn = (g->nx - 1) * fj.gdx + 1, nz2 = (g->ny - 1) * fj.gdz + 1;
  // fm2d may reuse a committed refined box whose maps are unchanged
  const bool reuse = fj.asgr == 1 && !b.igr && !b.straight && fj.precision != 2;
  size_t kd = kd_scratch_bytes(ncell_max);
  std::vector<size_t> sz = {
      sizeof(double) * np, sizeof(int) * np * npairs, sizeof(double) * np * npairs, sizeof(double) * np * npairs,
      sizeof(double) * 2 * (nsrc + nrev), sizeof(int) * np * npairs, sizeof(int2) * nsolve,
      sizeof(double) * (size_t)fp.nref_map * np * nslots, sizeof(double) * (size_t)fp.map_tmp_max * nsolve,
      sizeof(short) * (size_t)fp.map_tmp_max * nsolve, sizeof(int) * (nsolve + 1),
      sizeof(double) * (size_t)nn * nz2 * np * nslots,
      sizeof(double) * (size_t)nn * nz2 * np * nslots,
      // batch working state
      sizeof(double) * (size_t)nslots * ncell_max * 3, sizeof(int) * (size_t)nslots * nodes,
      sizeof(double) * (size_t)nslots * nodes * 3, sizeof(int) * nslots, sizeof(int) * (size_t)nslots * nodes,
      kd * nslots, sizeof(int) * 2, sizeof(int) * nslots, sizeof(int), sizeof(int2) * nslots * ncol,
      sizeof(int) * nslots * ncol, sizeof(float) * 4 * (size_t)nslots * ncol * b.nl_max,
      sizeof(double) * 2 * (size_t)nslots * ncol * np, sizeof(int) * nslots * ncol, sizeof(unsigned long long) * 2,
      sizeof(double) * (size_t)nslots * maps, sizeof(double) * (size_t)nslots * np * nvv,
      sizeof(double) * (size_t)nslots * np * npairs,
      // committed state
      sizeof(int) * nslots, sizeof(double) * (size_t)nslots * nodes * 3, sizeof(double) * (size_t)nslots * maps,
      sizeof(double) * (size_t)nslots * np * npairs,
      // staging
      sizeof(int) * nslots * 3, sizeof(double) * (size_t)nslots * ncell_max * 6, sizeof(double) * 2 * nslots * np,
      sizeof(double) * 4 * nslots, sizeof(int),
      // group velocities, rays and straight rays
      sizeof(double) * (size_t)nslots * maps * (b.igr ? 2 : 0),
      sizeof(double) * 2 * (size_t)nslots * np * npairs * ((b.igr || b.straight) ? 1 : 0),
      sizeof(int) * (size_t)nslots * np, sizeof(double) * (size_t)npairs, sizeof(double) * 2 * (nsrc + nrev),
      sizeof(double) * (size_t)nslots * np * npairs,
      (b.igr && !b.straight) ? sizeof(double) * (size_t)fp.nref_max * nsolve : 0,
      (b.igr && !b.straight) ? sizeof(short) * (size_t)fp.nref_max * nsolve : 0,
      sizeof(int) * (size_t)nslots * ncol,
      // fm2d time-field slots
      fm2d_tws_bytes(fp, (long)nsolve),
      // committed refined-box results (reuse)
      reuse ? sizeof(double) * (size_t)nslots * np * nvv : 0,
      reuse ? sizeof(double) * nsolve * fp.map_tmp_max : 0, reuse ? sizeof(short) * nsolve * fp.map_tmp_max : 0,
      reuse ? sizeof(int) * ((size_t)nslots * np + nsolve + nsolve + 1) : 0};
  size_t total = 0;
  for (size_t s : sz) total = ((total + 255) & ~size_t(255)) + s;
  total += 256;
  if (dry) { *bytes_out = total; delete c; return MCT_OK; }
  c->bytes = total;
  if (cudaMalloc(&c->mem, total) != cudaSuccess) { err() = "cudaMalloc failed"; delete c; return MCT_ERR_NOMEM; }
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaFree(c->mem); delete c; return MCT_ERR_CUDA;
  }
  {
    const size_t ni = 2 * (size_t)nslots + 2;
    const size_t nd = 2 * (size_t)nslots * ncell_max * 3 + 2 * (size_t)nslots * np + 4 * (size_t)nslots;
    if (cudaMallocHost(&c->h_ints, sizeof(int) * ni) != cudaSuccess ||
        cudaMallocHost(&c->h_dbl, sizeof(double) * nd) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->done, cudaEventDisableTiming) != cudaSuccess) {
      if (c->h_ints) cudaFreeHost(c->h_ints);
      if (c->h_dbl) cudaFreeHost(c->h_dbl);
      cudaFree(c->mem); cudaStreamDestroy(c->stream); delete c; return MCT_ERR_NOMEM;
    }
    c->in_use.assign((size_t)nslots, 0);
  }
  Carve cv(c->mem);
  double *per = cv.take<double>(np);
  int *rays = cv.take<int>((size_t)np * npairs);
  double *dtime = cv.take<double>((size_t)np * npairs);
  double *dsig = cv.take<double>((size_t)np * npairs);
  double *xy = cv.take<double>(2 * (nsrc + nrev));
  int *srs = cv.take<int>((size_t)np * npairs);
  int2 *solves = cv.take<int2>(nsolve);
  fj.sref = cv.take<double>((size_t)fp.nref_map * np * nslots);
  fj.map_tmp_t = cv.take<double>((size_t)fp.map_tmp_max * nsolve);
  fj.map_tmp_s = cv.take<short>((size_t)fp.map_tmp_max * nsolve);
  fj.ovf_list = cv.take<int>(nsolve + 1);
  fj.ovf_count = fj.ovf_list + nsolve;
  fj.veln = cv.take<double>((size_t)nn * nz2 * np * nslots);
  fj.slon = cv.take<double>((size_t)nn * nz2 * np * nslots);
  b.params = cv.take<double>((size_t)nslots * ncell_max * 3);
  b.sites = cv.take<int>((size_t)nslots * nodes);
  b.vp = cv.take<double>((size_t)nslots * nodes * 3);
  b.vs = b.vp + (size_t)nslots * nodes; b.rho = b.vs + (size_t)nslots * nodes;
  b.tie_count = cv.take<int>(nslots);
  b.tie_nodes = cv.take<int>((size_t)nslots * nodes);
  b.kd_scratch = cv.take<char>(kd * nslots);
  b.dev_status = cv.take<int>(2);
  b.status = cv.take<int>(nslots);
  b.list_count = cv.take<int>(1);
  b.list = cv.take<int2>((size_t)nslots * ncol);
  b.lnl = cv.take<int>((size_t)nslots * ncol);
  b.lthk = cv.take<float>((size_t)4 * nslots * ncol * b.nl_max);
  b.lvp = b.lthk + (size_t)nslots * ncol * b.nl_max; b.lvs = b.lvp + (size_t)nslots * ncol * b.nl_max;
  b.lrho = b.lvs + (size_t)nslots * ncol * b.nl_max;
  b.lcp = cv.take<double>((size_t)2 * nslots * ncol * np);
  b.lcg = b.lcp + (size_t)nslots * ncol * np;
  b.lierr = cv.take<int>((size_t)nslots * ncol);
  b.ndltar = cv.take<unsigned long long>(2);
  b.pvel = cv.take<double>((size_t)nslots * maps);
  b.velv = cv.take<double>((size_t)nslots * np * nvv);
  b.ttime = cv.take<double>((size_t)nslots * np * npairs);
  b.committed = cv.take<int>(nslots);
  b.cvp = cv.take<double>((size_t)nslots * nodes * 3);
  b.cvs = b.cvp + (size_t)nslots * nodes; b.crho = b.cvs + (size_t)nslots * nodes;
  b.cpvel = cv.take<double>((size_t)nslots * maps);
  b.cttime = cv.take<double>((size_t)nslots * np * npairs);
  c->d_slots = cv.take<int>((size_t)nslots * 3);
  c->d_ncells = c->d_slots + nslots; c->d_accept = c->d_ncells + nslots;
  c->d_points = cv.take<double>((size_t)nslots * ncell_max * 6);
  c->d_params = c->d_points + (size_t)nslots * ncell_max * 3;
  c->d_n0 = cv.take<double>((size_t)2 * nslots * np);
  c->d_n1 = c->d_n0 + (size_t)nslots * np;
  c->d_out = cv.take<double>((size_t)4 * nslots);
  fj.vmin_bits = cv.take<int>(1);
  b.gvel = cv.take<double>((size_t)nslots * maps * (b.igr ? 1 : 0));
  b.cgvel = cv.take<double>((size_t)nslots * maps * (b.igr ? 1 : 0));
  b.gtime = cv.take<double>((size_t)nslots * np * npairs * ((b.igr || b.straight) ? 1 : 0));
  b.raylen = cv.take<double>((size_t)nslots * np * npairs * ((b.igr || b.straight) ? 1 : 0));
  b.crazy = cv.take<int>((size_t)nslots * np);
  double *sdist = cv.take<double>((size_t)npairs);
  double *sxy = cv.take<double>(2 * (size_t)(nsrc + nrev));
  b.csrd = cv.take<double>((size_t)nslots * np * npairs);
  fj.ref_t = cv.take<double>((b.igr && !b.straight) ? (size_t)fp.nref_max * nsolve : 0);
  fj.ref_s = cv.take<short>((b.igr && !b.straight) ? (size_t)fp.nref_max * nsolve : 0);
  b.lorder = cv.take<int>((size_t)nslots * ncol);
  fm2d_bind_tws(fj, fp, (long)nsolve, cv.take<char>(fm2d_tws_bytes(fp, (long)nsolve)));
  b.reuse = reuse ? 1 : 0;
  b.spc = spc;
  b.map_tmp_max = fp.map_tmp_max;
  b.map_tmp_t = fj.map_tmp_t;
  b.map_tmp_s = fj.map_tmp_s;
  b.cvelv = cv.take<double>(reuse ? (size_t)nslots * np * nvv : 0);
  b.cref_t = cv.take<double>(reuse ? nsolve * fp.map_tmp_max : 0);
  b.cref_s = cv.take<short>(reuse ? nsolve * fp.map_tmp_max : 0);
  b.cmap = cv.take<int>(reuse ? (size_t)nslots * np + 2 * nsolve + 1 : 0);
  b.csolve = b.cmap + (size_t)nslots * np;
  b.ref_list = b.csolve + nsolve;
  b.ref_count = b.ref_list + nsolve;
  b.sdist = sdist;
  c->plan.src_xy = sxy; c->plan.rev_xy = sxy + 2 * nsrc;
  {
    // setup_straightRays distances (likelihood_surf.F90:430-433) and the
    // stations as [n][2]
    std::vector<double> hd((size_t)npairs);
    for (int j = 0; j < nsrc; ++j)
      for (int k = 0; k < nrev; ++k) {
        const double ddx = dat->rev[2 * k] - dat->src[2 * j], ddy = dat->rev[2 * k + 1] - dat->src[2 * j + 1];
        hd[(size_t)j * nrev + k] = std::sqrt(ddx * ddx + ddy * ddy);
      }
    cudaMemcpy(sdist, hd.data(), sizeof(double) * npairs, cudaMemcpyHostToDevice);
    cudaMemcpy(sxy, dat->src, sizeof(double) * 2 * nsrc, cudaMemcpyHostToDevice);
    cudaMemcpy(sxy + 2 * nsrc, dat->rev, sizeof(double) * 2 * nrev, cudaMemcpyHostToDevice);
  }
  // static data
  std::vector<double> hper(np);
  for (int p = 0; p < np; ++p) hper[p] = 1.0 / dat->freqs[p];   // dble(1/freqs), surfmodes.f90:82
  std::vector<double> hxy(2 * (nsrc + nrev));
  for (int i = 0; i < nsrc; ++i) { hxy[i] = dat->src[2 * i]; hxy[nsrc + i] = dat->src[2 * i + 1]; }
  for (int i = 0; i < nrev; ++i) { hxy[2 * nsrc + i] = dat->rev[2 * i]; hxy[2 * nsrc + nrev + i] = dat->rev[2 * i + 1]; }
  std::vector<int> hr((size_t)np * npairs);
  for (size_t q = 0; q < hr.size(); ++q) hr[q] = dat->raystat[q] == 1 ? 1 : 0;
  std::vector<double> hs((size_t)np * npairs, 1.0);
  if (dat->sigma) for (size_t q = 0; q < hs.size(); ++q) hs[q] = dat->sigma[q];
  cudaMemcpy(per, hper.data(), sizeof(double) * np, cudaMemcpyHostToDevice);
  cudaMemcpy(rays, dat->raystat, sizeof(int) * np * npairs, cudaMemcpyHostToDevice);
  cudaMemcpy(srs, hr.data(), sizeof(int) * np * npairs, cudaMemcpyHostToDevice);
  cudaMemcpy(dtime, dat->ttime, sizeof(double) * np * npairs, cudaMemcpyHostToDevice);
  cudaMemcpy(dsig, hs.data(), sizeof(double) * np * npairs, cudaMemcpyHostToDevice);
  cudaMemcpy(xy, hxy.data(), sizeof(double) * hxy.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(solves, all.data(), sizeof(int2) * nsolve, cudaMemcpyHostToDevice);
  cudaMemset(b.committed, 0, sizeof(int) * nslots);
  cudaMemset(b.ttime, 0, sizeof(double) * (size_t)nslots * np * npairs);
  cudaMemset(b.cttime, 0, sizeof(double) * (size_t)nslots * np * npairs);
  cudaMemset(b.csrd, 0, sizeof(double) * (size_t)nslots * np * npairs);
  if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) {
    cudaFree(c->mem); cudaStreamDestroy(c->stream); delete c; return MCT_ERR_CUDA;
  }
  b.periods = per; b.raystat = rays; b.dtime = dtime; b.dsigma = dsig;
  fj.scx = xy; fj.scz = xy + nsrc; fj.rcx = xy + 2 * nsrc; fj.rcz = xy + 2 * nsrc + nrev;
  fj.srs = srs; fj.solves = solves;
  fj.nodes_max = fp.nodes_max; fj.nref_max = fp.nref_max; fj.map_tmp_max = fp.map_tmp_max;
  fj.nref_map = fp.nref_map;
  *out = c;
  return MCT_OK;
}

}  // namespace

extern "C" {

int mct_surf_create(const mct_grid *g, const mct_surf_settings *st, const mct_surf_data *dat, int nslots,
                    int ncell_max, mct_surf_ctx **out) {
  if (!out) return MCT_ERR_ARG;
  return surf_create(g, st, dat, nslots, ncell_max, out, false, nullptr);
}

int mct_surf_device_bytes(const mct_grid *g, const mct_surf_settings *st, const mct_surf_data *dat, int nslots,
                          int ncell_max, size_t *bytes) {
  if (!bytes) return MCT_ERR_ARG;
  return surf_create(g, st, dat, nslots, ncell_max, nullptr, true, bytes);
}

int mct_surf_set_priority(mct_surf_ctx *c, int high) {
  if (!c) return MCT_ERR_ARG;
  if (c->pending) return MCT_ERR_ARG;
  return mct_restream(&c->stream, high);
}

int mct_surf_set_sm_share(mct_surf_ctx *c, double share) {
  if (!c || !(share >= 0.0 && share <= 1.0)) return MCT_ERR_ARG;
  c->plan.fm2d_plan.sm_share = share;
  return MCT_OK;
}

int mct_surf_destroy(mct_surf_ctx *c) {
  if (!c) return MCT_OK;
  cudaStreamSynchronize(c->stream);
  if (c->done) cudaEventDestroy(c->done);
  if (c->h_ints) cudaFreeHost(c->h_ints);
  if (c->h_dbl) cudaFreeHost(c->h_dbl);
  if (c->prof.ev) {
    for (int i = 0; i < 5 * c->prof.max_steps; ++i) cudaEventDestroy(c->prof.ev[i]);
    delete[] c->prof.ev;
  }
  if (c->st_sum) cudaFree(c->st_sum);
  if (c->st_slots) cudaFree(c->st_slots);
  cudaFree(c->mem);
  cudaStreamDestroy(c->stream);
  delete c;
  return MCT_OK;
}

int mct_surf_forward_device(mct_surf_ctx *c, int nchains, const int *slots, const int *ncells,
                            const double *points, const double *params, const double *n0,
                            const double *n1, double *out, void *stream) {
  if (!c || nchains < 1 || nchains > c->nslots) return MCT_ERR_ARG;
  SurfBatch &b = c->b;
  b.nchains = nchains; b.slots = slots; b.ncells = ncells; b.points = points; b.params_in = params;
  b.n0 = n0; b.n1 = n1; b.out = out;
  c->last_nchains = nchains;
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c->stream;
  return surf_forward(b, c->plan, s, &c->prof);
}

int mct_surf_commit_device(mct_surf_ctx *c, const int *accept, void *stream) {
  if (!c || c->last_nchains < 1) return MCT_ERR_ARG;
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c->stream;
  c->prof.launches += c->b.reuse ? 2 : 1;
  return surf_commit(c->b, accept, s);
}

int mct_surf_forward(mct_surf_ctx *c, int nchains, const int *slots, const int *ncells, const double *points,
                     const double *params, const double *n0, const double *n1, double *out) {
  if (!c || nchains < 1 || nchains > c->nslots || c->pending) return MCT_ERR_ARG;
  for (int i = 0; i < nchains; ++i) {
    if (slots[i] < 0 || slots[i] >= c->nslots) return MCT_ERR_ARG;
    for (int j = 0; j < i; ++j) if (slots[j] == slots[i]) return MCT_ERR_ARG;
    if (ncells[i] < 1 || ncells[i] > c->b.ncell_max) return MCT_ERR_ARG;
  }
  cudaStream_t s = c->stream;
  const int np = c->b.np;
  const size_t pc = (size_t)nchains * c->b.ncell_max * 3;
  MCT_CUDA_TRY(cudaMemcpyAsync(c->d_slots, slots, sizeof(int) * nchains, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(c->d_ncells, ncells, sizeof(int) * nchains, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(c->d_points, points, sizeof(double) * pc, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(c->d_params, params, sizeof(double) * pc, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(c->d_n0, n0, sizeof(double) * nchains * np, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(c->d_n1, n1, sizeof(double) * nchains * np, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemsetAsync(c->b.dev_status, 0, sizeof(int) * 2, s));
  int rc = mct_surf_forward_device(c, nchains, c->d_slots, c->d_ncells, c->d_points, c->d_params, c->d_n0,
                                   c->d_n1, c->d_out, s);
  if (rc) return rc;
  MCT_CUDA_TRY(cudaMemcpyAsync(out, c->d_out, sizeof(double) * 4 * nchains, cudaMemcpyDeviceToHost, s));
  int dst[2];
  MCT_CUDA_TRY(cudaMemcpyAsync(dst, c->b.dev_status, sizeof(int) * 2, cudaMemcpyDeviceToHost, s));
  MCT_CUDA_TRY(cudaStreamSynchronize(s));
  if (dst[0]) return dst[0];
  return MCT_OK;
}

int mct_surf_commit(mct_surf_ctx *c, const int *accept) {
  if (!c || c->last_nchains < 1 || c->pending) return MCT_ERR_ARG;
  cudaStream_t s = c->stream;
  MCT_CUDA_TRY(cudaMemcpyAsync(c->d_accept, accept, sizeof(int) * c->last_nchains, cudaMemcpyHostToDevice, s));
  int rc = mct_surf_commit_device(c, c->d_accept, s);
  if (rc) return rc;
  MCT_CUDA_TRY(cudaStreamSynchronize(s));
  return MCT_OK;
}

int mct_surf_noise_likelihood(mct_surf_ctx *c, int nchains, const int *slots, const double *n0, const double *n1,
                              double *out) {
  if (!c || nchains < 1 || nchains > c->nslots || !slots || !n0 || !n1 || !out || c->pending) return MCT_ERR_ARG;
  for (int i = 0; i < nchains; ++i)
    if (slots[i] < 0 || slots[i] >= c->nslots) return MCT_ERR_ARG;
  cudaStream_t s = c->stream;
  const int np = c->b.np;
  // staging shared with forwards: calls on one context are ordered on its stream
  MCT_CUDA_TRY(cudaMemcpyAsync(c->d_slots, slots, sizeof(int) * nchains, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(c->d_n0, n0, sizeof(double) * nchains * np, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(c->d_n1, n1, sizeof(double) * nchains * np, cudaMemcpyHostToDevice, s));
  int rc = surf_noise(c->b, nchains, c->d_slots, c->d_n0, c->d_n1, c->d_out, s);
  if (rc) return rc;
  MCT_CUDA_TRY(cudaMemcpyAsync(out, c->d_out, sizeof(double) * 4 * nchains, cudaMemcpyDeviceToHost, s));
  MCT_CUDA_TRY(cudaStreamSynchronize(s));
  for (int i = 0; i < nchains; ++i)
    if (out[4 * i + 3] != 0.0) return MCT_MODEL_INVALID;
  return MCT_OK;
}

// Serving: the caller's arrays are copied into pinned staging before the
// call returns, the batch runs on the context's stream, and mct_surf_poll
// reports completion without blocking.
int mct_surf_submit(mct_surf_ctx *c, int nchains, const int *slots, const int *ncells, const double *points,
                    const double *params, const double *n0, const double *n1) {
  if (!c || nchains < 1 || nchains > c->nslots || c->pending || !slots || !ncells || !points || !params || !n0 ||
      !n1)
    return MCT_ERR_ARG;
  for (int i = 0; i < nchains; ++i) {
    if (slots[i] < 0 || slots[i] >= c->nslots) return MCT_ERR_ARG;
    for (int j = 0; j < i; ++j) if (slots[j] == slots[i]) return MCT_ERR_ARG;
    if (ncells[i] < 1 || ncells[i] > c->b.ncell_max) return MCT_ERR_ARG;
  }
  cudaStream_t s = c->stream;
  const int np = c->b.np, ns = c->nslots;
  const size_t pc = (size_t)nchains * c->b.ncell_max * 3, pmax = (size_t)ns * c->b.ncell_max * 3;
  int *hs = c->h_ints, *hn = c->h_ints + ns;
  double *hp = c->h_dbl, *hq = hp + pmax, *h0 = hq + pmax, *h1 = h0 + (size_t)ns * np;
  std::memcpy(hs, slots, sizeof(int) * nchains);
  std::memcpy(hn, ncells, sizeof(int) * nchains);
  std::memcpy(hp, points, sizeof(double) * pc);
  std::memcpy(hq, params, sizeof(double) * pc);
  std::memcpy(h0, n0, sizeof(double) * nchains * np);
  std::memcpy(h1, n1, sizeof(double) * nchains * np);
  MCT_CUDA_TRY(cudaMemcpyAsync(c->d_slots, hs, sizeof(int) * nchains, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(c->d_ncells, hn, sizeof(int) * nchains, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(c->d_points, hp, sizeof(double) * pc, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(c->d_params, hq, sizeof(double) * pc, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(c->d_n0, h0, sizeof(double) * nchains * np, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(c->d_n1, h1, sizeof(double) * nchains * np, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemsetAsync(c->b.dev_status, 0, sizeof(int) * 2, s));
  int rc = mct_surf_forward_device(c, nchains, c->d_slots, c->d_ncells, c->d_points, c->d_params, c->d_n0,
                                   c->d_n1, c->d_out, s);
  if (rc) return rc;
  double *ho = h1 + (size_t)ns * np;
  MCT_CUDA_TRY(cudaMemcpyAsync(ho, c->d_out, sizeof(double) * 4 * nchains, cudaMemcpyDeviceToHost, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(c->h_ints + 2 * ns, c->b.dev_status, sizeof(int) * 2, cudaMemcpyDeviceToHost, s));
  MCT_CUDA_TRY(cudaEventRecord(c->done, s));
  c->pending = nchains;
  return MCT_OK;
}

int mct_surf_poll(mct_surf_ctx *c, double *out, int *done) {
  if (!c || !out || !done || !c->pending) return MCT_ERR_ARG;
  *done = 0;
  const cudaError_t q = cudaEventQuery(c->done);
  if (q == cudaErrorNotReady) return MCT_OK;
  if (q != cudaSuccess) { mct_set_error("cudaEventQuery", cudaGetErrorString(q), __FILE__, __LINE__); return MCT_ERR_CUDA; }
  const int ns = c->nslots, np = c->b.np, n = c->pending;
  const double *ho = c->h_dbl + 2 * (size_t)ns * c->b.ncell_max * 3 + 2 * (size_t)ns * np;
  std::memcpy(out, ho, sizeof(double) * 4 * n);
  c->pending = 0;
  *done = 1;
  const int st = c->h_ints[2 * ns];
  return st ? st : MCT_OK;
}

int mct_surf_stat_add(mct_surf_ctx *c, int nchains, const int *slots) {
  if (!c || c->pending || nchains < 1 || nchains > c->nslots || !slots) return MCT_ERR_ARG;
  for (int i = 0; i < nchains; ++i) {
    if (slots[i] < 0 || slots[i] >= c->nslots) return MCT_ERR_ARG;
    for (int j = 0; j < i; ++j) if (slots[j] == slots[i]) return MCT_ERR_ARG;
  }
  const SurfBatch &b = c->b;
  const size_t nodes = (size_t)b.nx * b.ny * b.nz;
  if (!c->st_sum) {
    MCT_CUDA_TRY(cudaMalloc(&c->st_sum, sizeof(double) * 4 * nodes * c->nslots));
    MCT_CUDA_TRY(cudaMalloc(&c->st_slots, sizeof(int) * c->nslots));
    MCT_CUDA_TRY(cudaMemsetAsync(c->st_sum, 0, sizeof(double) * 4 * nodes * c->nslots, c->stream));
    c->st_n.assign((size_t)c->nslots, 0);
  }
  MCT_CUDA_TRY(cudaMemcpyAsync(c->st_slots, slots, sizeof(int) * nchains, cudaMemcpyHostToDevice, c->stream));
  stat_add_kernel<<<dim3((unsigned)std::min<size_t>((nodes + 255) / 256, 152), nchains), 256, 0, c->stream>>>(
      nchains, c->st_slots, nodes, b.cvp, b.cvs, c->st_sum);
  MCT_CUDA_TRY(cudaGetLastError());
  MCT_CUDA_TRY(cudaStreamSynchronize(c->stream));   // the slots array is the caller's
  for (int i = 0; i < nchains; ++i) ++c->st_n[(size_t)slots[i]];
  return MCT_OK;
}

int mct_surf_stat_read(mct_surf_ctx *c, int slot, double *mean_vp, double *mean_vs, double *msq_vp, double *msq_vs,
                       int *nthin) {
  if (!c || c->pending || slot < 0 || slot >= c->nslots) return MCT_ERR_ARG;
  const SurfBatch &b = c->b;
  const size_t nodes = (size_t)b.nx * b.ny * b.nz;
  const int n = c->st_sum ? c->st_n[(size_t)slot] : 0;
  if (nthin) *nthin = n;
  double *outs[4] = {mean_vs, msq_vs, mean_vp, msq_vp};
  std::vector<double> h(nodes);
  for (int k = 0; k < 4; ++k) {
    if (!outs[k]) continue;
    if (n == 0) { std::fill(outs[k], outs[k] + nodes, 0.0); continue; }
    MCT_CUDA_TRY(cudaMemcpyAsync(h.data(), c->st_sum + ((size_t)slot * 4 + k) * nodes, sizeof(double) * nodes,
                                 cudaMemcpyDeviceToHost, c->stream));
    MCT_CUDA_TRY(cudaStreamSynchronize(c->stream));
    // write_mean / write_var (src/read_write.f90:223-292): sums over nthin
    for (size_t q = 0; q < nodes; ++q) outs[k][q] = h[q] / n;
  }
  return MCT_OK;
}

}  // extern "C"

namespace {
int stat_reset_slot(mct_surf_ctx *c, int slot) {
  if (!c->st_sum) return MCT_OK;
  const size_t nodes = (size_t)c->b.nx * c->b.ny * c->b.nz;
  MCT_CUDA_TRY(cudaMemsetAsync(c->st_sum + (size_t)slot * 4 * nodes, 0, sizeof(double) * 4 * nodes, c->stream));
  c->st_n[(size_t)slot] = 0;
  return MCT_OK;
}
}  // namespace

extern "C" {

int mct_surf_stat_reset(mct_surf_ctx *c, int slot) {
  if (!c || c->pending || slot < 0 || slot >= c->nslots) return MCT_ERR_ARG;
  return stat_reset_slot(c, slot);
}

int mct_surf_admit(mct_surf_ctx *c, int *slot) {
  if (!c || !slot) return MCT_ERR_ARG;
  for (int i = 0; i < c->nslots; ++i) {
    if (c->in_use[(size_t)i]) continue;
    // a fresh chain: nothing committed, so its first forward computes every
    // column, and no posterior statistics
    MCT_CUDA_TRY(cudaMemsetAsync(c->b.committed + i, 0, sizeof(int), c->stream));
    int rc = stat_reset_slot(c, i);
    if (rc) return rc;
    c->in_use[(size_t)i] = 1;
    *slot = i;
    return MCT_OK;
  }
  mct_set_error("mct_surf_admit", "no free chain slot", __FILE__, __LINE__);
  return MCT_ERR_NOMEM;
}

int mct_surf_evict(mct_surf_ctx *c, int slot) {
  if (!c || slot < 0 || slot >= c->nslots || !c->in_use[(size_t)slot]) return MCT_ERR_ARG;
  MCT_CUDA_TRY(cudaMemsetAsync(c->b.committed + slot, 0, sizeof(int), c->stream));
  c->in_use[(size_t)slot] = 0;
  return MCT_OK;
}

int mct_surf_phase_time(mct_surf_ctx *c, int index, double *phase_time, double *phase_vel) {
  if (!c || index < 0 || index >= c->last_nchains) return MCT_ERR_ARG;
  const SurfBatch &b = c->b;
  const size_t npairs = (size_t)b.nsrc * b.nrev;
  MCT_CUDA_TRY(cudaStreamSynchronize(c->stream));
  // the likelihood's phaseTime: group times along the rays (or straight
  // rays) when those are used, otherwise the phase times
  const double *lt = (b.igr || b.straight) ? b.gtime : b.ttime;
  if (phase_time)
    MCT_CUDA_TRY(cudaMemcpy(phase_time, lt + (size_t)index * b.np * npairs, sizeof(double) * b.np * npairs,
                            cudaMemcpyDeviceToHost));
  if (phase_vel)
    MCT_CUDA_TRY(cudaMemcpy(phase_vel, b.pvel + (size_t)index * b.np * b.nx * b.ny,
                            sizeof(double) * b.np * b.nx * b.ny, cudaMemcpyDeviceToHost));
  return MCT_OK;
}

int mct_surf_profile_start(mct_surf_ctx *c, int max_steps) {
  if (!c || max_steps < 0) return MCT_ERR_ARG;
  SurfProfile &p = c->prof;
  if (p.ev) {
    for (int i = 0; i < 5 * p.max_steps; ++i) cudaEventDestroy(p.ev[i]);
    delete[] p.ev;
    p.ev = nullptr;
  }
  p.enabled = max_steps > 0; p.max_steps = max_steps; p.step = 0; p.launches = 0;
  if (max_steps > 0) {
    p.ev = new cudaEvent_t[5 * max_steps];
    for (int i = 0; i < 5 * max_steps; ++i) MCT_CUDA_TRY(cudaEventCreate(&p.ev[i]));
  }
  return MCT_OK;
}

int mct_surf_profile_read(mct_surf_ctx *c, double *stage_ms, int *steps, long long *launches) {
  if (!c) return MCT_ERR_ARG;
  SurfProfile &p = c->prof;
  for (int k = 0; k < 4; ++k) stage_ms[k] = 0.0;
  for (int i = 0; i < p.step; ++i) {
    MCT_CUDA_TRY(cudaEventSynchronize(p.ev[5 * i + 4]));
    for (int k = 0; k < 4; ++k) {
      float ms = 0.f;
      MCT_CUDA_TRY(cudaEventElapsedTime(&ms, p.ev[5 * i + k], p.ev[5 * i + k + 1]));
      stage_ms[k] += ms;
    }
  }
  if (steps) *steps = p.step;
  if (launches) *launches = p.launches;
  return MCT_OK;
}

int mct_surf_stream(mct_surf_ctx *c, void **stream) {
  if (!c || !stream) return MCT_ERR_ARG;
  *stream = c->stream;
  return MCT_OK;
}

}  // extern "C"
