// C-ABI entry points of libmctomo_gpu.so (declared in include/mctomo.h).
// Host-pointer calls stage their inputs into a grow-only device workspace on
// the library's own stream and wait for the result; _device calls launch on
// the caller's stream.
#include "mct_common.cuh"
#include "grt.cuh"
#include "fm2d.cuh"
#include "eikonal3d.cuh"
#include <cstring>
#include <climits>
#include <string>
#include <vector>
#include <algorithm>

static thread_local std::string g_last_error;

void mct_set_error(const char *what, const char *why, const char *file, int line) {
  char buf[512];
  snprintf(buf, sizeof(buf), "%s: %s (%s:%d)", what, why, file, line);
  g_last_error = buf;
}

int mct_smem_attr_raw(const void *func, int bytes) {
  int dev = 0;
  MCT_CUDA_TRY(cudaGetDevice(&dev));
  struct Rec { int dev; const void *func; int bytes; };
  static std::mutex mu;
  static std::vector<Rec> done;
  std::lock_guard<std::mutex> lk(mu);
  for (const Rec &r : done)
    if (r.dev == dev && r.func == func && r.bytes >= bytes) return MCT_OK;
  MCT_CUDA_TRY(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  done.push_back({dev, func, bytes});
  return MCT_OK;
}

namespace {

// Per host thread and device: the stream and grow-only workspace of the
// synchronous host-pointer calls. The reference calls its per-solve routines
// from OpenMP loops (src/likelihood_body.F90:204-224 over stations,
// src/likelihood_surf.F90:197-206 over columns), so calls from different
// threads run concurrently on their own streams, sharing nothing. A thread's
// buffers are released when the thread exits.
constexpr int kMaxDevices = 64;
struct ThreadDev {
  cudaStream_t stream = nullptr;
  DevBuf ws;
};
struct ThreadCtx {
  ThreadDev dev[kMaxDevices];
  ~ThreadCtx() {
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess) return;
    for (int d = 0; d < kMaxDevices; ++d) {
      if (!dev[d].stream && !dev[d].ws.p) continue;
      if (cudaSetDevice(d) != cudaSuccess) continue;
      if (dev[d].stream) cudaStreamDestroy(dev[d].stream);
      dev[d].ws.release();
    }
    cudaSetDevice(cur);
  }
};
thread_local ThreadCtx t_ctx;

int thread_dev(ThreadDev **out) {
  int d = -1;
  MCT_CUDA_TRY(cudaGetDevice(&d));
  if (d < 0 || d >= kMaxDevices) {
    mct_set_error("thread_dev", "device ordinal beyond 63", __FILE__, __LINE__);
    return MCT_ERR_ARG;
  }
  ThreadDev &td = t_ctx.dev[d];
  if (!td.stream) MCT_CUDA_TRY(cudaStreamCreateWithFlags(&td.stream, cudaStreamNonBlocking));
  *out = &td;
  return MCT_OK;
}

// the pop trace of one fm2d solve (diagnostics; the last traced call wins)
std::mutex g_trace_mu;
int g_trace_solve = -1;
std::vector<int> g_trace_i;
std::vector<double> g_trace_t;

int arg_error(const char *msg) {
  g_last_error = msg;
  return MCT_ERR_ARG;
}

int sync_and_check(cudaStream_t s, const int *d_status) {
  MCT_CUDA_TRY(cudaStreamSynchronize(s));
  if (d_status) {
    int st = 0;
    MCT_CUDA_TRY(cudaMemcpy(&st, d_status, sizeof(int), cudaMemcpyDeviceToHost));
    if (st != 0) { g_last_error = "device kernel reported an internal error"; return st; }
  }
  return MCT_OK;
}

}  // namespace

extern "C" {

const char *mct_version(void) { return "mctomo-gb300 0.1 (sm_103a)"; }

const char *mct_last_error(void) { return g_last_error.c_str(); }

// ---------------------------------------------------------------------------
// Gridding
// ---------------------------------------------------------------------------
int mct_grid_nearest_batch_device(int d, int nchains, int ncell_max, const int *ncells,
                                  const double *points, const double *params, int nx, int ny,
                                  int nz, const double *grid_lo, const double *grid_step,
                                  const int *box, int *sites_id, double *vp, double *vs,
                                  double *rho, void *stream) {
  if ((d != 2 && d != 3) || nchains < 1 || ncell_max < 1 || nx < 1 || ny < 1 || (d == 3 && nz < 1))
    return arg_error("mct_grid_nearest_batch_device: bad sizes");
  if (ncell_max > 12800) return arg_error("mct_grid_nearest_batch_device: ncell_max > 12800");
  // scratch owned per call site: allocate on the caller's stream ordering
  long nodes = (long)nx * ny * (d == 3 ? nz : 1);
  size_t kd = kd_scratch_bytes(ncell_max);
  size_t bytes = carve_size({sizeof(int) * (size_t)nchains, sizeof(int) * (size_t)nchains * nodes,
                             kd * nchains, sizeof(int)});
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  void *scratch = nullptr;
  MCT_CUDA_TRY(cudaMallocAsync(&scratch, bytes, s));
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
  MCT_CUDA_TRY(cudaMemsetAsync(job.status, 0, sizeof(int), s));
  int rc = launch_grid_nearest(job, s);
  cudaFreeAsync(scratch, s);
  return rc;
}

int mct_grid_status(void *stream, int *status) {
  if (!status) return arg_error("mct_grid_status: status is NULL");
  return grid_status_read(stream, status);
}

int mct_kdtree_to_grid(int d, int n, const double *points, const double *params, int nx, int ny,
                       int nz, const double *grid_lo, const double *grid_step, const int *box,
                       int *sites_id, double *vp, double *vs, double *rho) {
  if ((d != 2 && d != 3) || n < 1 || nx < 1 || ny < 1 || (d == 3 && nz < 1))
    return arg_error("mct_kdtree_to_grid: bad sizes");
  if (n > 12800) return arg_error("mct_kdtree_to_grid: more than 12800 nuclei");
  const int nzz = d == 3 ? nz : 1;
  int b[6] = {1, nx, 1, ny, 1, nzz};
  if (box) {
    for (int i = 0; i < 6; ++i) b[i] = box[i];
    if (d == 2) { b[4] = 1; b[5] = 1; }
    if (b[0] < 1 || b[1] > nx || b[2] < 1 || b[3] > ny || b[4] < 1 || b[5] > nzz ||
        b[0] > b[1] || b[2] > b[3] || b[4] > b[5])
      return arg_error("mct_kdtree_to_grid: box outside the grid");
  }
  ThreadDev *td = nullptr;
  int rc = thread_dev(&td); if (rc) return rc;
  size_t nodes = (size_t)nx * ny * nzz;
  size_t kd = kd_scratch_bytes(n);
  size_t bytes = carve_size({sizeof(double) * d * n, sizeof(double) * 3 * n, sizeof(int), sizeof(int) * 6,
                             sizeof(int) * nodes, sizeof(double) * nodes * 3, sizeof(int), sizeof(int) * nodes,
                             kd, sizeof(int)});
  rc = td->ws.reserve(bytes); if (rc) return rc;
  Carve cv(td->ws.p);
  double *d_pts = cv.take<double>((size_t)d * n);
  double *d_par = cv.take<double>((size_t)3 * n);
  int *d_n = cv.take<int>(1);
  int *d_box = cv.take<int>(6);
  int *d_sites = cv.take<int>(nodes);
  double *d_vel = cv.take<double>(nodes * 3);
  GridJob job{};
  job.tie_count = cv.take<int>(1);
  job.tie_nodes = cv.take<int>(nodes);
  job.kd_scratch = cv.take<char>(kd);
  job.status = cv.take<int>(1);
  cudaStream_t s = td->stream;
  MCT_CUDA_TRY(cudaMemcpyAsync(d_pts, points, sizeof(double) * d * n, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(d_par, params, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(d_n, &n, sizeof(int), cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(d_box, b, sizeof(int) * 6, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemsetAsync(job.status, 0, sizeof(int), s));
  // nodes outside the box keep the caller's values
  MCT_CUDA_TRY(cudaMemcpyAsync(d_sites, sites_id, sizeof(int) * nodes, cudaMemcpyHostToDevice, s));
  if (vp) {
    MCT_CUDA_TRY(cudaMemcpyAsync(d_vel, vp, sizeof(double) * nodes, cudaMemcpyHostToDevice, s));
    MCT_CUDA_TRY(cudaMemcpyAsync(d_vel + nodes, vs, sizeof(double) * nodes, cudaMemcpyHostToDevice, s));
    MCT_CUDA_TRY(cudaMemcpyAsync(d_vel + 2 * nodes, rho, sizeof(double) * nodes, cudaMemcpyHostToDevice, s));
  }
  job.d = d; job.nx = nx; job.ny = ny; job.nz = nzz;
  job.xmin = grid_lo[0]; job.ymin = grid_lo[1]; job.zmin = d == 3 ? grid_lo[2] : 0.0;
  job.dx = grid_step[0]; job.dy = grid_step[1]; job.dz = d == 3 ? grid_step[2] : 0.0;
  job.nchains = 1; job.ncell_max = n; job.ncells = d_n;
  job.points = d_pts; job.params = d_par; job.box = d_box;
  job.sites_id = d_sites;
  job.vp = vp ? d_vel : nullptr; job.vs = vp ? d_vel + nodes : nullptr; job.rho = vp ? d_vel + 2 * nodes : nullptr;
  rc = launch_grid_nearest(job, s); if (rc) return rc;
  MCT_CUDA_TRY(cudaMemcpyAsync(sites_id, d_sites, sizeof(int) * nodes, cudaMemcpyDeviceToHost, s));
  if (vp) {
    MCT_CUDA_TRY(cudaMemcpyAsync(vp, d_vel, sizeof(double) * nodes, cudaMemcpyDeviceToHost, s));
    MCT_CUDA_TRY(cudaMemcpyAsync(vs, d_vel + nodes, sizeof(double) * nodes, cudaMemcpyDeviceToHost, s));
    MCT_CUDA_TRY(cudaMemcpyAsync(rho, d_vel + 2 * nodes, sizeof(double) * nodes, cudaMemcpyDeviceToHost, s));
  }
  return sync_and_check(s, job.status);
}

// ---------------------------------------------------------------------------
// Dispersion
// ---------------------------------------------------------------------------
static int disp_args_ok(int ncol, int nl_max, int np, int iwave, int mode, int igr, double dphase) {
  if (ncol < 0 || nl_max < 1 || nl_max > 200) return 0;
  if (np < 1 || np > 60 || mode < 1 || mode > 20) return 0;
  if (iwave != 1 && iwave != 2) return 0;
  if (igr < 0) return 0;
  if (!(dphase != 0.0) || (float)dphase == 0.0f) return 0;
  return 1;
}

int mct_surfdisp_batch_device(int ncol, int nl_max, const int *nl, const float *thk, const float *vp,
                              const float *vs, const float *rho, int np, const double *periods,
                              int iwave, int mode, int igr, double dphase, int multimode,
                              int precision, double *cp, double *cg, int *ierr,
                              unsigned long long *ndltar, void *stream) {
  if (!disp_args_ok(ncol, nl_max, np, iwave, mode, igr, dphase))
    return arg_error("mct_surfdisp_batch_device: bad arguments");
  if (!multimode && mode != 1) return arg_error("surfdisp96 computes one mode; use multimode");
  DispJob job{};
  job.ncol = ncol; job.nl_max = nl_max; job.nl = nl;
  job.thk = thk; job.vp = vp; job.vs = vs; job.rho = rho;
  job.np = np; job.periods = periods; job.iwave = iwave; job.mode = mode; job.igr = igr;
  job.dphase = dphase; job.multimode = multimode; job.precision = precision ? 1 : 0;
  job.cp = cp; job.cg = cg; job.ierr = ierr; job.ndltar = ndltar;
  if (ncol == 0) return MCT_OK;
  // the column order scratch, on the caller's stream ordering
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  MCT_CUDA_TRY(cudaMallocAsync(&job.order, sizeof(int) * (size_t)ncol, s));
  const int rc = launch_surfdisp(job, s);
  cudaFreeAsync(job.order, s);
  return rc;
}

int mct_surfdisp_batch(int ncol, int nl_max, const int *nl, const float *thk, const float *vp,
                       const float *vs, const float *rho, int np, const double *periods, int iwave,
                       int mode, int igr, double dphase, int multimode, int precision, double *cp,
                       double *cg, int *ierr, unsigned long long *ndltar) {
  if (!disp_args_ok(ncol, nl_max, np, iwave, mode, igr, dphase))
    return arg_error("mct_surfdisp_batch: bad arguments");
  if (!multimode && mode != 1) return arg_error("surfdisp96 computes one mode; use multimode");
  if (ncol == 0) return MCT_OK;
  ThreadDev *td = nullptr;
  int rc = thread_dev(&td); if (rc) return rc;
  size_t lay = (size_t)ncol * nl_max;
  size_t outn = (size_t)ncol * mode * np;
  size_t bytes = carve_size({sizeof(int) * ncol, 4 * sizeof(float) * lay, sizeof(double) * np,
                             2 * sizeof(double) * outn, sizeof(int) * ncol, 2 * sizeof(unsigned long long),
                             sizeof(int) * ncol});
  rc = td->ws.reserve(bytes); if (rc) return rc;
  Carve cv(td->ws.p);
  int *d_nl = cv.take<int>(ncol);
  float *d_lay = cv.take<float>(4 * lay);
  double *d_per = cv.take<double>(np);
  double *d_out = cv.take<double>(2 * outn);
  int *d_ierr = cv.take<int>(ncol);
  unsigned long long *d_cnt = cv.take<unsigned long long>(2);
  int *d_order = cv.take<int>(ncol);
  cudaStream_t s = td->stream;
  MCT_CUDA_TRY(cudaMemcpyAsync(d_nl, nl, sizeof(int) * ncol, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(d_lay, thk, sizeof(float) * lay, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(d_lay + lay, vp, sizeof(float) * lay, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(d_lay + 2 * lay, vs, sizeof(float) * lay, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(d_lay + 3 * lay, rho, sizeof(float) * lay, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(d_per, periods, sizeof(double) * np, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemsetAsync(d_cnt, 0, 2 * sizeof(unsigned long long), s));
  DispJob job{};
  job.ncol = ncol; job.nl_max = nl_max; job.nl = d_nl;
  job.thk = d_lay; job.vp = d_lay + lay; job.vs = d_lay + 2 * lay; job.rho = d_lay + 3 * lay;
  job.np = np; job.periods = d_per; job.iwave = iwave; job.mode = mode; job.igr = igr;
  job.dphase = dphase; job.multimode = multimode; job.precision = precision ? 1 : 0;
  job.cp = d_out; job.cg = d_out + outn; job.ierr = d_ierr; job.ndltar = d_cnt; job.order = d_order;
  rc = launch_surfdisp(job, s); if (rc) return rc;
  MCT_CUDA_TRY(cudaMemcpyAsync(cp, d_out, sizeof(double) * outn, cudaMemcpyDeviceToHost, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(cg, d_out + outn, sizeof(double) * outn, cudaMemcpyDeviceToHost, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(ierr, d_ierr, sizeof(int) * ncol, cudaMemcpyDeviceToHost, s));
  unsigned long long cnt[2];
  MCT_CUDA_TRY(cudaMemcpyAsync(cnt, d_cnt, sizeof(cnt), cudaMemcpyDeviceToHost, s));
  rc = sync_and_check(s, nullptr);
  if (ndltar) { ndltar[0] = cnt[0]; ndltar[1] = cnt[1]; }
  return rc;
}

static int surfdisp_single(const float *thkm, const float *vpm, const float *vsm, const float *rhom,
                           int nlayer, int iflsph, int iwave, int mode, int igr, int kmax,
                           const double *t, double dphase, double *cp, double *cg, int *ierr,
                           int multimode) {
  if (iflsph != 0) { g_last_error = "spherical-earth flattening (iflsph=1) is not supported"; return MCT_ERR_UNSUPPORTED; }
  if (nlayer < 1 || nlayer > 200) return arg_error("surfdisp96: nlayer out of range");
  int nl = nlayer;
  int rc = mct_surfdisp_batch(1, nlayer, &nl, thkm, vpm, vsm, rhom, kmax, t, iwave, mode, igr, dphase,
                              multimode, 0, cp, cg, ierr, nullptr);
  return rc;
}

int mct_surfdisp96(const float *thkm, const float *vpm, const float *vsm, const float *rhom,
                   int nlayer, int iflsph, int iwave, int mode, int igr, int kmax, const double *t,
                   double dphase, double *cp, double *cg, int *ierr) {
  if (mode != 1) return arg_error("surfdisp96: mode must be 1 (use mct_surfdisp_mmodes)");
  return surfdisp_single(thkm, vpm, vsm, rhom, nlayer, iflsph, iwave, mode, igr, kmax, t, dphase,
                         cp, cg, ierr, 0);
}

int mct_surfdisp_mmodes(const float *thkm, const float *vpm, const float *vsm, const float *rhom,
                        int nlayer, int iflsph, int iwave, int mode, int igr, int kmax,
                        const double *t, double dphase, double *cp, double *cg, int *ierr) {
  return surfdisp_single(thkm, vpm, vsm, rhom, nlayer, iflsph, iwave, mode, igr, kmax, t, dphase,
                         cp, cg, ierr, 1);
}

// setup_grt's low-velocity-layer count (surfmodes.f90:320-450, nlvls1) that
// decides between surfdisp96 and the generalized R/T solver.
static int count_lvl(const double *vp, const double *vs, int nl, int modetype) {
  const double eps = (double)1e-6f;
  int ifs = 0;
  for (int i = 0; i < nl; ++i) if (!(std::fabs(vs[i]) > eps)) ifs++;
  int n = 0;
  if (ifs > 0 && modetype == 1) {
    double vss1 = vs[ifs < nl ? ifs : nl - 1];
    for (int i = 1; i < nl - 1; ++i) if (i + 1 > ifs && vs[i] < vss1) n++;
    return n;
  }
  double vs1 = (modetype == 1) ? vs[0] : vs[ifs < nl ? ifs : nl - 1];
  for (int i = 1; i < nl - 1; ++i) {
    if (vp[i] < vp[i + 1] && vp[i] < vp[i - 1]) {
      if (ifs == 0) { if (vs[i] < vs1) n++; }
      else if (vs[i] > 0.) { if (vs[i] < vs1) n++; }
    }
  }
  return n;
}

static bool modes_para_ok(const mct_modes_para *p) {
  return p && (p->modetype == 0 || p->modetype == 1) && (p->phase_group == 0 || p->phase_group == 1) &&
         p->tolmin > 0 && p->tolmax > 0 && p->smin_min > 0 && p->smin_max > 0 && p->dc > 0;
}

int mct_grt_batch_device(int ncol, int nl_max, const int *nl, const double *thk, const double *vp,
                         const double *vs, const double *rho, int np, const double *freqs,
                         const mct_modes_para *paras, double *phase, double *group, int *ierr,
                         unsigned long long *nevals, void *stream) {
  if (ncol < 0 || nl_max < 2 || nl_max > 200 || np < 1 || np > 100 || !modes_para_ok(paras) ||
      (ncol > 0 && (!nl || !thk || !vp || !vs || !rho || !freqs || !phase || !group || !ierr)))
    return arg_error("mct_grt_batch_device: bad arguments");
  if (ncol == 0) return MCT_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t lay = (size_t)ncol * nl_max;
  const size_t nscr = grt_scratch_doubles(ncol, paras->modetype);
  double *w = nullptr;
  MCT_CUDA_TRY(cudaMallocAsync(&w, sizeof(double) * (7 * lay + nscr + 1), s));
  GrtJob J{};
  J.ncol = ncol; J.nl_max = nl_max; J.np = np; J.modetype = paras->modetype; J.phase_group = paras->phase_group;
  J.nl = nl; J.freqs = freqs;
  J.tolmin = paras->tolmin; J.tolmax = paras->tolmax; J.smin_min = paras->smin_min; J.smin_max = paras->smin_max;
  J.dc = paras->dc;
  J.mu = w + 4 * lay; J.v = w + 5 * lay; J.scratch = w + 7 * lay;
  J.cols = nullptr; J.n = ncol;
  J.next = reinterpret_cast<unsigned *>(w + 7 * lay + nscr);
  J.phase = phase; J.group = group; J.ierr = ierr; J.nevals = nevals;
  const double *rows[4] = {thk, vp, vs, rho};
  const int rc = launch_grt(J, rows, w, s);
  cudaFreeAsync(w, s);
  return rc;
}

int mct_grt_batch(int ncol, int nl_max, const int *nl, const double *thk, const double *vp, const double *vs,
                  const double *rho, int np, const double *freqs, const mct_modes_para *paras, double *phase,
                  double *group, int *ierr, unsigned long long *nevals) {
  if (ncol < 0 || nl_max < 2 || nl_max > 200 || np < 1 || np > 100 || !modes_para_ok(paras))
    return arg_error("mct_grt_batch: bad arguments");
  for (int c = 0; c < ncol; ++c)
    if (nl[c] < 2 || nl[c] > nl_max) return arg_error("mct_grt_batch: layer count outside 2..nl_max");
  if (ncol == 0) return MCT_OK;
  ThreadDev *td = nullptr;
  int rc = thread_dev(&td); if (rc) return rc;
  const size_t lay = (size_t)ncol * nl_max, outn = (size_t)ncol * np;
  size_t bytes = carve_size({sizeof(int) * ncol, 4 * sizeof(double) * lay, sizeof(double) * np,
                             2 * sizeof(double) * outn, sizeof(int) * ncol, sizeof(unsigned long long)});
  rc = td->ws.reserve(bytes); if (rc) return rc;
  Carve cv(td->ws.p);
  int *d_nl = cv.take<int>(ncol);
  double *d_lay = cv.take<double>(4 * lay);
  double *d_f = cv.take<double>(np);
  double *d_out = cv.take<double>(2 * outn);
  int *d_ierr = cv.take<int>(ncol);
  unsigned long long *d_cnt = cv.take<unsigned long long>(1);
  cudaStream_t s = td->stream;
  MCT_CUDA_TRY(cudaMemcpyAsync(d_nl, nl, sizeof(int) * ncol, cudaMemcpyHostToDevice, s));
  const double *src[4] = {thk, vp, vs, rho};
  for (int a = 0; a < 4; ++a)
    MCT_CUDA_TRY(cudaMemcpyAsync(d_lay + a * lay, src[a], sizeof(double) * lay, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(d_f, freqs, sizeof(double) * np, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemsetAsync(d_cnt, 0, sizeof(unsigned long long), s));
  rc = mct_grt_batch_device(ncol, nl_max, d_nl, d_lay, d_lay + lay, d_lay + 2 * lay, d_lay + 3 * lay, np, d_f,
                            paras, d_out, d_out + outn, d_ierr, d_cnt, s);
  if (rc) return rc;
  MCT_CUDA_TRY(cudaMemcpyAsync(phase, d_out, sizeof(double) * outn, cudaMemcpyDeviceToHost, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(group, d_out + outn, sizeof(double) * outn, cudaMemcpyDeviceToHost, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(ierr, d_ierr, sizeof(int) * ncol, cudaMemcpyDeviceToHost, s));
  unsigned long long cnt = 0;
  MCT_CUDA_TRY(cudaMemcpyAsync(&cnt, d_cnt, sizeof(cnt), cudaMemcpyDeviceToHost, s));
  rc = sync_and_check(s, nullptr);
  if (nevals) *nevals = cnt;
  return rc;
}

int mct_surfmodes_route(int ncol, int nl_max, const int *nl, const double *vp, const double *vs, int modetype,
                        int *route) {
  if (ncol < 0 || nl_max < 1 || nl_max > 200 || (modetype != 0 && modetype != 1) ||
      (ncol > 0 && (!nl || !vp || !vs || !route)))
    return arg_error("mct_surfmodes_route: bad arguments");
  for (int c = 0; c < ncol; ++c) {
    const int n = nl[c];
    if (n < 1 || n > nl_max) return arg_error("mct_surfmodes_route: layer count outside 1..nl_max");
    const double *a = vp + (size_t)c * nl_max, *b = vs + (size_t)c * nl_max;
    int r = count_lvl(a, b, n, modetype) > 0 ? 1 : 0;
    if (r)
      for (int i = 0; i < n; ++i)
        if (!(std::fabs(b[i]) > (double)1e-6f)) { r = -2; break; }
    route[c] = r;
  }
  return MCT_OK;
}

int mct_surfmodes_para(const double *thick, const double *vp, const double *vs, const double *rho,
                       int nlayers, const double *freqs, int np, const mct_modes_para *paras, double *phase,
                       double *group, int *ierr) {
  if (nlayers < 1 || nlayers > 200 || np < 1 || np > 60 || !modes_para_ok(paras))
    return arg_error("mct_surfmodes_para: bad arguments");
  if (count_lvl(vp, vs, nlayers, paras->modetype) > 0) {
    for (int i = 0; i < nlayers; ++i)
      if (!(std::fabs(vs[i]) > (double)1e-6f)) {
        g_last_error = "low-velocity layer under a fluid layer (the Stoneley-mode path)";
        return MCT_ERR_UNSUPPORTED;
      }
    if (nlayers < 2) return arg_error("mct_surfmodes_para: one layer");
    int nl = nlayers;
    return mct_grt_batch(1, nlayers, &nl, thick, vp, vs, rho, np, freqs, paras, phase, group, ierr, nullptr);
  }
  std::vector<float> t4(nlayers), a4(nlayers), b4(nlayers), r4(nlayers);
  std::vector<double> per(np);
  for (int i = 0; i < nlayers; ++i) {
    t4[i] = (float)thick[i]; a4[i] = (float)vp[i]; b4[i] = (float)vs[i]; r4[i] = (float)rho[i];
  }
  for (int i = 0; i < np; ++i) per[i] = 1.0 / freqs[i];
  return mct_surfdisp96(t4.data(), a4.data(), b4.data(), r4.data(), nlayers, 0, paras->modetype == 1 ? 2 : 1,
                        1, paras->phase_group, np, per.data(), paras->dc, phase, group, ierr);
}

int mct_surfmodes(const double *thick, const double *vp, const double *vs, const double *rho,
                  int nlayers, const double *freqs, int np, int modetype, int phase_group,
                  double dc, double *phase, double *group, int *ierr) {
  mct_modes_para p{};
  p.modetype = modetype; p.nmodes = 1; p.phase_group = phase_group;
  p.tolmin = 1e-6; p.tolmax = 1e-5; p.smin_min = (double)1e-3f; p.smin_max = (double)5e-3f;
  p.dc = p.dcm = p.dc1 = p.dc2 = dc;
  if (modetype != 0 && modetype != 1) return arg_error("mct_surfmodes: modetype must be 0 or 1");
  return mct_surfmodes_para(thick, vp, vs, rho, nlayers, freqs, np, &p, phase, group, ierr);
}


// ---------------------------------------------------------------------------
// 2D travel times (fm2d modrays)
// ---------------------------------------------------------------------------
}  // extern "C"

namespace {
// modrays over many maps; with gvel set (rays), also the ray-path group
// delays and lengths of every path (modrays uar = 0 + CalGroupTime).
int modrays_batch(int nmaps, int nsrc, const double *scx, const double *scz, int nrc,
                  const double *rcx, const double *rcz, int srs_nmaps, const int *srs, int nvx,
                  int nvz, double goxd, double gozd, double dvxd, double dvzd,
                  const double *velv, int gdx, int gdz, int asgr, int sgdl, int sgs, int fom,
                  double *ttime, double *tfield, int precision, const double *gvel, double *gtime,
                  double *raylen, int *crazy) {
  const bool rays = gvel != nullptr;
  if (nmaps < 1 || nsrc < 1 || nrc < 1 || nvx < 2 || nvz < 2 || gdx < 1 || gdz < 1 ||
      srs_nmaps < 1 || (asgr == 1 && (sgdl < 1 || sgs < 1)) || (fom != 0 && fom != 1) ||
      !(dvxd > 0) || !(dvzd > 0))
    return arg_error("mct_modrays_batch: bad arguments");
  Fm2dJob job{};
  job.nmaps = nmaps; job.nvx = nvx; job.nvz = nvz;
  job.goxd = goxd; job.gozd = gozd; job.dvxd = dvxd; job.dvzd = dvzd;
  job.gdx = gdx; job.gdz = gdz; job.asgr = asgr; job.sgdl = sgdl; job.sgs = sgs; job.fom = fom;
  job.nsrc = nsrc; job.nrc = nrc; job.srs_nmaps = srs_nmaps;
  job.precision = (precision >= 0 && precision <= 2) ? precision : 0;
  Fm2dPlan plan;
  int rc = fm2d_plan(job, &plan);
  if (rc) return arg_error("mct_modrays_batch: grid too large for the shared-memory solver");
  // active solves: a source with no paths is skipped unless it is the first
  // (fm2dray_cartesian.f90:213-215)
  std::vector<int2> solves;
  for (int m = 0; m < nmaps; ++m) {
    const int *f = srs + (size_t)(m % srs_nmaps) * nsrc * nrc;
    for (int i = 0; i < nsrc; ++i) {
      int any = 0;
      for (int j = 0; j < nrc; ++j) any |= f[(size_t)i * nrc + j];
      if (any || i == 0) solves.push_back(make_int2(m, i));
    }
  }
  const int nnx = (nvx - 1) * gdx + 1, nnz = (nvz - 1) * gdz + 1;
  const size_t nv = (size_t)(nvx + 2) * (nvz + 2);
  const size_t ns = solves.size();
  ThreadDev *td = nullptr;
  rc = thread_dev(&td); if (rc) return rc;
  size_t bytes = carve_size({sizeof(double) * nv * nmaps, sizeof(double) * (size_t)nnx * nnz * nmaps,
                             sizeof(double) * (size_t)nnx * nnz * nmaps,
                             sizeof(double) * (size_t)plan.nref_map * nmaps, sizeof(double) * (size_t)plan.map_tmp_max * ns,
                             sizeof(short) * (size_t)plan.map_tmp_max * ns, sizeof(int) * (ns + 1),
                             sizeof(double) * 2 * (nsrc + nrc),
                             sizeof(int) * (size_t)srs_nmaps * nsrc * nrc, sizeof(int2) * ns,
                             sizeof(double) * (size_t)nmaps * nsrc * nrc,
                             tfield ? sizeof(double) * (size_t)nmaps * nsrc * nnx * nnz : 0, sizeof(int),
                             sizeof(int),
                             rays ? sizeof(double) * (size_t)nmaps * nvx * nvz : 0,
                             rays ? sizeof(double) * 2 * (size_t)nmaps * nsrc * nrc : 0,
                             rays ? sizeof(int) * (size_t)nmaps : 0,
                             rays ? sizeof(double) * (size_t)plan.nref_max * ns : 0,
                             rays ? sizeof(short) * (size_t)plan.nref_max * ns : 0,
                             fm2d_tws_bytes(plan, (long)ns)});
  rc = td->ws.reserve(bytes); if (rc) return rc;
  Carve cv(td->ws.p);
  double *d_velv = cv.take<double>(nv * nmaps);
  job.veln = cv.take<double>((size_t)nnx * nnz * nmaps);
  job.slon = cv.take<double>((size_t)nnx * nnz * nmaps);
  job.sref = cv.take<double>((size_t)plan.nref_map * nmaps);
  job.map_tmp_t = cv.take<double>((size_t)plan.map_tmp_max * ns);
  job.map_tmp_s = cv.take<short>((size_t)plan.map_tmp_max * ns);
  job.ovf_list = cv.take<int>(ns + 1);
  job.ovf_count = job.ovf_list + ns;
  double *d_xy = cv.take<double>(2 * (nsrc + nrc));
  int *d_srs = cv.take<int>((size_t)srs_nmaps * nsrc * nrc);
  int2 *d_solves = cv.take<int2>(ns);
  double *d_tt = cv.take<double>((size_t)nmaps * nsrc * nrc);
  double *d_tf = tfield ? cv.take<double>((size_t)nmaps * nsrc * nnx * nnz) : nullptr;
  int *d_status = cv.take<int>(1);
  job.vmin_bits = cv.take<int>(1);
  double *d_gvel = nullptr, *d_gt = nullptr;
  int *d_crazy = nullptr;
  if (rays) {
    d_gvel = cv.take<double>((size_t)nmaps * nvx * nvz);
    d_gt = cv.take<double>(2 * (size_t)nmaps * nsrc * nrc);
    d_crazy = cv.take<int>((size_t)nmaps);
    job.ref_t = cv.take<double>((size_t)plan.nref_max * ns);
    job.ref_s = cv.take<short>((size_t)plan.nref_max * ns);
    job.rays = 1; job.gvel = d_gvel; job.gtime = d_gt; job.raylen = d_gt + (size_t)nmaps * nsrc * nrc;
    job.crazy = d_crazy;
  }
  fm2d_bind_tws(job, plan, (long)ns, cv.take<char>(fm2d_tws_bytes(plan, (long)ns)));
  cudaStream_t s = td->stream;
  if (rays) {
    MCT_CUDA_TRY(cudaMemcpyAsync(d_gvel, gvel, sizeof(double) * (size_t)nmaps * nvx * nvz, cudaMemcpyHostToDevice, s));
    MCT_CUDA_TRY(cudaMemsetAsync(d_gt, 0, sizeof(double) * 2 * (size_t)nmaps * nsrc * nrc, s));
    MCT_CUDA_TRY(cudaMemsetAsync(d_crazy, 0, sizeof(int) * (size_t)nmaps, s));
  }
  MCT_CUDA_TRY(cudaMemcpyAsync(d_velv, velv, sizeof(double) * nv * nmaps, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(d_xy, scx, sizeof(double) * nsrc, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(d_xy + nsrc, scz, sizeof(double) * nsrc, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(d_xy + 2 * nsrc, rcx, sizeof(double) * nrc, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(d_xy + 2 * nsrc + nrc, rcz, sizeof(double) * nrc, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(d_srs, srs, sizeof(int) * (size_t)srs_nmaps * nsrc * nrc, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(d_solves, solves.data(), sizeof(int2) * ns, cudaMemcpyHostToDevice, s));
  // paths that are not computed keep the caller's values
  MCT_CUDA_TRY(cudaMemcpyAsync(d_tt, ttime, sizeof(double) * (size_t)nmaps * nsrc * nrc, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemsetAsync(d_status, 0, sizeof(int), s));
  job.velv = d_velv;
  job.scx = d_xy; job.scz = d_xy + nsrc; job.rcx = d_xy + 2 * nsrc; job.rcz = d_xy + 2 * nsrc + nrc;
  job.srs = d_srs; job.nsolve = (int)ns; job.solves = d_solves;
  job.ttime = d_tt; job.tfield = d_tf; job.status = d_status;
  job.nodes_max = plan.nodes_max; job.nref_max = plan.nref_max; job.map_tmp_max = plan.map_tmp_max;
  job.nref_map = plan.nref_map;
  job.precision = (precision >= 0 && precision <= 2) ? precision : 0;
  int *d_ti = nullptr; double *d_trt = nullptr;
  int trace_solve;
  {
    std::lock_guard<std::mutex> lk(g_trace_mu);
    trace_solve = g_trace_solve;
  }
  if (trace_solve >= 0) {
    job.trace_solve = trace_solve; job.trace_max = 20000;
    MCT_CUDA_TRY(cudaMalloc(&d_ti, sizeof(int) * 3 * job.trace_max));
    MCT_CUDA_TRY(cudaMalloc(&d_trt, sizeof(double) * job.trace_max));
    MCT_CUDA_TRY(cudaMemset(d_ti, 0xff, sizeof(int) * 3 * job.trace_max));
    job.trace_i = d_ti; job.trace_t = d_trt;
  }
  rc = launch_fm2d(job, plan, s); if (rc) return rc;
  if (d_ti) {
    MCT_CUDA_TRY(cudaStreamSynchronize(s));
    std::lock_guard<std::mutex> lk(g_trace_mu);
    g_trace_i.resize(3 * job.trace_max); g_trace_t.resize(job.trace_max);
    MCT_CUDA_TRY(cudaMemcpy(g_trace_i.data(), d_ti, sizeof(int) * 3 * job.trace_max, cudaMemcpyDeviceToHost));
    MCT_CUDA_TRY(cudaMemcpy(g_trace_t.data(), d_trt, sizeof(double) * job.trace_max, cudaMemcpyDeviceToHost));
    cudaFree(d_ti); cudaFree(d_trt);
  }
  MCT_CUDA_TRY(cudaMemcpyAsync(ttime, d_tt, sizeof(double) * (size_t)nmaps * nsrc * nrc, cudaMemcpyDeviceToHost, s));
  if (tfield)
    MCT_CUDA_TRY(cudaMemcpyAsync(tfield, d_tf, sizeof(double) * (size_t)nmaps * nsrc * nnx * nnz, cudaMemcpyDeviceToHost, s));
  if (rays) {
    MCT_CUDA_TRY(cudaMemcpyAsync(gtime, d_gt, sizeof(double) * (size_t)nmaps * nsrc * nrc, cudaMemcpyDeviceToHost, s));
    MCT_CUDA_TRY(cudaMemcpyAsync(raylen, d_gt + (size_t)nmaps * nsrc * nrc, sizeof(double) * (size_t)nmaps * nsrc * nrc,
                                 cudaMemcpyDeviceToHost, s));
    MCT_CUDA_TRY(cudaMemcpyAsync(crazy, d_crazy, sizeof(int) * (size_t)nmaps, cudaMemcpyDeviceToHost, s));
  }
  rc = sync_and_check(s, d_status);
  return rc;
}
}  // namespace

extern "C" {

int mct_modrays_batch(int nmaps, int nsrc, const double *scx, const double *scz, int nrc,
                      const double *rcx, const double *rcz, int srs_nmaps, const int *srs, int nvx,
                      int nvz, double goxd, double gozd, double dvxd, double dvzd,
                      const double *velv, int gdx, int gdz, int asgr, int sgdl, int sgs, int fom,
                      double *ttime, double *tfield, int precision) {
  return modrays_batch(nmaps, nsrc, scx, scz, nrc, rcx, rcz, srs_nmaps, srs, nvx, nvz, goxd, gozd, dvxd, dvzd,
                       velv, gdx, gdz, asgr, sgdl, sgs, fom, ttime, tfield, precision, nullptr, nullptr, nullptr,
                       nullptr);
}

int mct_modrays_group_batch(int nmaps, int nsrc, const double *scx, const double *scz, int nrc,
                            const double *rcx, const double *rcz, int srs_nmaps, const int *srs, int nvx,
                            int nvz, double goxd, double gozd, double dvxd, double dvzd,
                            const double *velv, const double *gvel, int gdx, int gdz, int asgr, int sgdl,
                            int sgs, int fom, double *ttime, double *gtime, double *raylen, int *crazy,
                            int precision) {
  if (!gvel || !gtime || !raylen || !crazy) return arg_error("mct_modrays_group_batch: null output");
  return modrays_batch(nmaps, nsrc, scx, scz, nrc, rcx, rcz, srs_nmaps, srs, nvx, nvz, goxd, gozd, dvxd, dvzd,
                       velv, gdx, gdz, asgr, sgdl, sgs, fom, ttime, nullptr, precision, gvel, gtime, raylen, crazy);
}

int mct_modrays(int nsrc, const double *scx, const double *scz, int nrc, const double *rcx,
                const double *rcz, const int *srsin, int wrgf, int nvx, int nvz, double goxd,
                double gozd, double dvxd, double dvzd, const double *velvin, int gdx, int gdz,
                int asgr, int sgdl, int sgs, double earth, int fom, double snb, double *ttime,
                int uar, int *crazyray, double *tfield) {
  (void)earth; (void)snb;
  if (wrgf != 0) { g_last_error = "writing ray geometries to file (wrgf) is not supported"; return MCT_ERR_UNSUPPORTED; }
  if (uar == 0) { g_last_error = "ray paths (uar=0, group velocity) are not supported"; return MCT_ERR_UNSUPPORTED; }
  if (crazyray) *crazyray = 0;
  return mct_modrays_batch(1, nsrc, scx, scz, nrc, rcx, rcz, 1, srsin, nvx, nvz, goxd, gozd, dvxd,
                           dvzd, velvin, gdx, gdz, asgr, sgdl, sgs, fom, ttime, tfield, 0);
}


// Diagnostics (not part of the public header): record the marching order of
// one solve of the next mct_modrays_batch call.
int mct_debug_fm2d_trace(int solve, int *idx_out, double *t_out, int max) {
  std::lock_guard<std::mutex> lk(g_trace_mu);
  if (solve >= -1 && idx_out == nullptr) { g_trace_solve = solve; return MCT_OK; }
  int n = std::min<int>(max, (int)g_trace_t.size());
  for (int i = 0; i < n; ++i) { idx_out[3 * i] = g_trace_i[3 * i]; idx_out[3 * i + 1] = g_trace_i[3 * i + 1]; idx_out[3 * i + 2] = g_trace_i[3 * i + 2]; t_out[i] = g_trace_t[i]; }
  return n;
}



// ---------------------------------------------------------------------------
// 3D travel times (fastMarching3D)
// ---------------------------------------------------------------------------
int mct_eikonal3d_batch(int nsolve, int nx, int ny, int nz, double dx, double dy, double dz, double xmin,
                        double ymin, double zmin, int ngrids, const double *vel, const int *solve_grid,
                        const double *src, int nrev, const double *rev, int order, double *ttime,
                        double *tfield, int *passes) {
  const int ord = order & 0xF, mflag = order & ~0xF;
  if (nsolve < 1 || nx < 2 || ny < 2 || nz < 2 || ngrids < 1 || nrev < 0 || !(dx > 0) || !(dy > 0) ||
      !(dz > 0) || (ord != 0 && ord != 1) ||
      (mflag != 0 && mflag != MCT_EIK3_TILES && mflag != MCT_EIK3_HEAP))
    return arg_error("mct_eikonal3d_batch: bad arguments");
  const int method = eik3_resolve_method(ord, mflag == MCT_EIK3_TILES ? EIK3_TILES
                                              : mflag == MCT_EIK3_HEAP ? EIK3_HEAP : EIK3_DEFAULT);
  const size_t nn = (size_t)nx * ny * nz;
  if (method == EIK3_HEAP && nn > (size_t)0x3FFFFFFF) return arg_error("mct_eikonal3d_batch: grid too large");
  double vmin = 1e300;
  for (size_t q = 0; q < nn * ngrids; ++q)
    if (vel[q] >= 2.220446049250313e-11 && vel[q] < vmin) vmin = vel[q];
  if (!(vmin < 1e300)) return arg_error("mct_eikonal3d_batch: no positive velocity");
  for (int sI = 0; sI < nsolve; ++sI)
    if (solve_grid[sI] < 0 || solve_grid[sI] >= ngrids) return arg_error("mct_eikonal3d_batch: bad grid index");
  const double diag = sqrt(((nx - 1) * dx) * ((nx - 1) * dx) + ((ny - 1) * dy) * ((ny - 1) * dy) +
                           ((nz - 1) * dz) * ((nz - 1) * dz));
  ThreadDev *td = nullptr;
  int rc = thread_dev(&td); if (rc) return rc;
  Eik3Job job{};
  job.nsolve = nsolve; job.nx = nx; job.ny = ny; job.nz = nz; job.dx = dx; job.dy = dy; job.dz = dz;
  job.ngrids = ngrids; job.order = ord; job.method = method; job.nrev = nrev; job.rev_per_solve = 0;
  job.shift = eik3_shift_for(4.0 * diag / vmin);
  const bool heap = method == EIK3_HEAP;
  const size_t ntile = heap ? 0 : eik3_tiles(job);
  const size_t nT = heap ? 0 : nn * nsolve;
  // heap march: as many solves at once as 16 GiB of scratch holds
  const size_t per_solve = eik3_heap_bytes_per_solve(nx, ny, nz);
  const int hchunk = heap ? (int)std::max<size_t>(1, std::min<size_t>(nsolve, (16ull << 30) / per_solve)) : 0;
  size_t bytes = carve_size({sizeof(double) * nn * ngrids, sizeof(float) * nn * ngrids, sizeof(int) * nsolve,
                             sizeof(double) * 3 * nsolve, sizeof(int) * nT, ntile * nsolve,
                             sizeof(int) * ntile * nsolve, sizeof(int), sizeof(double) * 3 * (nrev + 1),
                             sizeof(double) * (size_t)nsolve * (nrev + 1),
                             tfield ? sizeof(double) * nn * nsolve : 0,
                             heap ? sizeof(double2) * nn * ngrids : 0,
                             eik3_heap_scratch_bytes(nx, ny, nz, hchunk), sizeof(int)});
  rc = td->ws.reserve(bytes); if (rc) return rc;
  Carve cv(td->ws.p);
  double *d_vel = cv.take<double>(nn * ngrids);
  job.slow = cv.take<float>(nn * ngrids);
  int *d_sg = cv.take<int>(nsolve);
  double *d_src = cv.take<double>(3 * (size_t)nsolve);
  job.T = cv.take<int>(nT);
  job.flags = cv.take<unsigned char>(ntile * nsolve);
  job.list = cv.take<int>(ntile * nsolve);
  job.count = cv.take<int>(1);
  double *d_rev = cv.take<double>(3 * (size_t)(nrev + 1));
  double *d_tt = cv.take<double>((size_t)nsolve * (nrev + 1));
  double *d_tf = tfield ? cv.take<double>(nn * nsolve) : nullptr;
  if (heap) {
    job.hvn = cv.take<double2>(nn * ngrids);
    Carve hc(cv.take<char>(eik3_heap_scratch_bytes(nx, ny, nz, hchunk)));
    eik3_heap_take(job, hc, hchunk);
  }
  job.herr = cv.take<int>(1);
  std::vector<double> hsrc(3 * (size_t)nsolve), hrev(3 * (size_t)nrev);
  for (int q = 0; q < nsolve; ++q) {
    hsrc[3 * q] = src[3 * q] - xmin; hsrc[3 * q + 1] = src[3 * q + 1] - ymin; hsrc[3 * q + 2] = src[3 * q + 2] - zmin;
  }
  for (int q = 0; q < nrev; ++q) {
    hrev[3 * q] = rev[3 * q] - xmin; hrev[3 * q + 1] = rev[3 * q + 1] - ymin; hrev[3 * q + 2] = rev[3 * q + 2] - zmin;
  }
  cudaStream_t s = td->stream;
  MCT_CUDA_TRY(cudaMemcpyAsync(d_vel, vel, sizeof(double) * nn * ngrids, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(d_sg, solve_grid, sizeof(int) * nsolve, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(d_src, hsrc.data(), sizeof(double) * 3 * nsolve, cudaMemcpyHostToDevice, s));
  if (nrev) MCT_CUDA_TRY(cudaMemcpyAsync(d_rev, hrev.data(), sizeof(double) * 3 * nrev, cudaMemcpyHostToDevice, s));
  job.vel = d_vel; job.solve_grid = d_sg; job.src = d_src; job.rev = d_rev; job.ttime = d_tt;
  int np_ = 0;
  rc = launch_eik3(job, s, 100000, &np_, d_tf);
  if (rc) return rc;
  if (nrev) MCT_CUDA_TRY(cudaMemcpyAsync(ttime, d_tt, sizeof(double) * nsolve * nrev, cudaMemcpyDeviceToHost, s));
  if (tfield) MCT_CUDA_TRY(cudaMemcpyAsync(tfield, d_tf, sizeof(double) * nn * nsolve, cudaMemcpyDeviceToHost, s));
  rc = sync_and_check(s, nullptr);
  if (passes) *passes = np_;
  return rc;
}

int mct_fast_marching3d(int nx, int ny, int nz, double dx, double dy, double dz, double xmin, double ymin,
                        double zmin, const double *vel, const double *src, const double *rev, int nrev, int order,
                        double *ttime, double *tfield) {
  const int g = 0;
  // the reference: order 1 -> second order, anything else first order
  // (fastMarching.cpp:76-80); a solver-selection flag may be added
  const int flags = order & ~0xF;
  const int ord = (flags == MCT_EIK3_TILES || flags == MCT_EIK3_HEAP) ? ((order & 0xF) == 1 ? 1 : 0) | flags
                                                                       : (order == 1 ? 1 : 0);
  return mct_eikonal3d_batch(1, nx, ny, nz, dx, dy, dz, xmin, ymin, zmin, 1, vel, &g, src, nrev, rev, ord,
                             ttime, tfield, nullptr);
}

}  // extern "C"

