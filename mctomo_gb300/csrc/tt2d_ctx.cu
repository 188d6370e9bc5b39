// Batched 2D travel-time likelihood: the GPU replacement of the 2D code's
// likelihood call (mcmc2d/likelihood_joint.f90:56) -> body_likelihood
// (mcmc2d/likelihood_dd.F90:349-529), with the kdtree_to_grid call the
// sampler makes before it (mcmc2d/mcmc.f90:1469-1525) and the noise-only
// likelihood (mcmc2d/likelihood_dd.F90:32-106).
//
// Per forward and chain: nearest-nucleus gridding of the velocity
// (parameters(1,:)) on the (ny, nx) grid; the padded vertex grid
// (likelihood_dd.F90:413-423); modrays from every source with any path
// (fm2d, the same kernels as the surface-wave path; y divided by the grid's
// scaling as the reference's call does), or straight rays
// (setup_straightRays / IntegrateRays, :732-806); then sigma and the
// misfit / -log L (:455-499) and, for datatype 1, the differential times of
// every source pair (:467-476, :501-522).
//
// Reference quirks kept:
//  * the differential-time test reads dat%dtime(ddindex,k,1) (indices
//    swapped against the dtime(k,ddindex,1) it then uses), i.e. element
//    ddindex + k*nrev of the column-major array; creation is refused where
//    that read would leave the array;
//  * eps is the REAL*4 literal 0.000000001 (utils/utils.f90:58), PI2 the
//    REAL*4 literal 6.283185, nrays/2.0 and ndtime/2.0 REAL*4;
//  * the noise-only likelihood keeps the differential sigma log-sum in an
//    INTEGER (likelihood_dd.F90:41), truncating after every term, and does
//    not touch the unweighted misfit;
//  * the noise-only likelihood takes sigma = n0 * srdist + n1 whatever
//    sigdep is: srdist is the last forward's times when sigdep != 0 (:457),
//    else the straight-ray distances (:743-753) or, for fm2d, the initial
//    norm2 source-receiver distances (likelihood_ddsettings.f90:112-120);
//  * the 2D GetVelocity divides the y offset by dy and then by the scaling
//    (:829) while its weights use dy/scaling (:838).
// Paths without data are never computed and keep time 0, as the
// reference's phaseTime does; the differential times read them.
#include "mct_common.cuh"
#include "fm2d.cuh"
#include "../../include/mctomo.h"
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

namespace {

constexpr double kPI2 = (double)6.283185f;
constexpr double kEps = (double)0.000000001f;

// REAL*8 to INTEGER assignment as the reference's x86 build does it
// (truncation toward zero; out of range and NaN give -2^31).
__device__ __forceinline__ int fortran_int(double x) {
  if (!(x > -2147483649.0 && x < 2147483648.0)) return INT_MIN;
  return (int)x;
}

struct Tt2dDev {
  int nx, ny;
  double xmin, ymin, dx, dy, scaling;
  int nsrc, nrev, nrays, sigdep, datatype, straight, ndd, ndtime;
  const int *raystat;      // [nsrc*nrev]
  const double *tobs;      // [nsrc*nrev] observed times
  const double *tsig;      // [nsrc*nrev] data sigma
  const double *dtime;     // [ndd][nrev] observed differential times (column-major (nrev, ndd))
  const double *dcc;       // same layout
  const int2 *pairs;       // [ndd] (i, j), i < j
  const double *srd0;      // [nsrc*nrev] srdist when sigdep == 0 (noise-only likelihood)
  const double *sdist;     // [nsrc*nrev] straight-ray distances
  const double *src_xy;    // [nsrc][2]
  const double *rev_xy;    // [nrev][2]
};

// Padded vertex grid (likelihood_dd.F90:413-423): ext_vel(2:ny+1,2:nx+1) =
// vel, then the first and last columns and rows copied from their
// neighbours, i.e. every edge node takes the nearest interior value.
__global__ void tt2d_pad_kernel(int nx, int ny, const double *vel, double *velv) {
  const int c = blockIdx.y;
  const int nvx = nx + 2, nvz = ny + 2;
  const double *v = vel + (size_t)c * nx * ny;
  double *o = velv + (size_t)c * nvx * nvz;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nvx * nvz; q += gridDim.x * blockDim.x) {
    const int jj = q % nvz, ii = q / nvz;
    const int j = min(max(jj, 1), ny) - 1, i = min(max(ii, 1), nx) - 1;
    o[q] = v[(size_t)i * ny + j];
  }
}

// GetVelocity of the 2D code (likelihood_dd.F90:815-841), vel (ny, nx)
// column-major = [nx][ny].
__device__ double velocity_2d(const Tt2dDev &d, const double *vel, double px, double py) {
  const double ymin_s = d.ymin / d.scaling, dy_s = d.dy / d.scaling;
  int ix = (int)floor((px - d.xmin) / d.dx) + 1;
  int iy = (int)floor((py - ymin_s) / d.dy / d.scaling) + 1;
  if (ix < 1) ix = 1;
  if (iy < 1) iy = 1;
  if (ix >= d.nx) ix = d.nx - 1;
  if (iy >= d.ny) iy = d.ny - 1;
  const double dsx = px - (d.xmin + (double)(ix - 1) * d.dx);
  const double dsy = py - (ymin_s + (double)(iy - 1) * d.dy / d.scaling);
  double qv = 0;
  for (int i = 1; i <= 2; ++i)
    for (int j = 1; j <= 2; ++j) {
      const double weight = (1.0 - fabs((double)(i - 1) * d.dx - dsx) / d.dx) *
                            (1.0 - fabs((double)(j - 1) * d.dy / d.scaling - dsy) / dy_s);
      qv = qv + weight * vel[(size_t)(ix + i - 2) * d.ny + (iy + j - 2)];
    }
  return qv;
}

// setup_straightRays + IntegrateRays (likelihood_dd.F90:732-806), one thread
// per (chain, path): points every min(dx, dy/scaling)/2 from the source,
// the receiver last; 'Straight ray out of area' is MCT_ERR_OUTSIDE.
__global__ void tt2d_straight_kernel(Tt2dDev d, const double *vel_all, double *tt, int *dev_status) {
  const int npairs = d.nsrc * d.nrev;
  const int c = blockIdx.y;
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= npairs) return;
  double *t = tt + (size_t)c * npairs;
  t[n] = 0;
  if (d.raystat[n] != 1) return;
  const int j = n / d.nrev, k = n % d.nrev;
  const double *vel = vel_all + (size_t)c * d.nx * d.ny;
  const double sx = d.src_xy[2 * j], sy = d.src_xy[2 * j + 1], rx = d.rev_xy[2 * k], ry = d.rev_xy[2 * k + 1];
  const double ddx = rx - sx, ddy = ry - sy;
  const double ds = sqrt(ddx * ddx + ddy * ddy);
  const double dl = fmin(d.dx, d.dy / d.scaling) / 2;
  const int npts = (int)floor(ds / dl) + 1;
  const double b1 = d.xmin, b2 = d.xmin + (double)(d.nx - 1) * d.dx;
  const double b3 = d.ymin / d.scaling, b4 = (d.ymin + (double)(d.ny - 1) * d.dy) / d.scaling;
  double px = sx, py = sy, vhead = 0, acc = 0;
  for (int l = 1; l <= npts; ++l) {
    double qx, qy;
    if (l < npts) {
      qx = sx + (double)(l - 1) * dl * ddx / ds;
      qy = sy + (double)(l - 1) * dl * ddy / ds;
      if (qx < b1 || qx > b2 || qy < b3 || qy > b4) {
        atomicExch(dev_status, MCT_ERR_OUTSIDE);
        return;
      }
    } else {
      qx = rx; qy = ry;
    }
    const double v = velocity_2d(d, vel, qx, qy);
    if (l > 1) {
      double dist = (qx - px) * (qx - px) + (qy - py) * (qy - py);
      dist = sqrt(dist);
      acc = acc + dist * 2 / (vhead + v);
    }
    vhead = v; px = qx; py = qy;
  }
  t[n] = acc;
}

__device__ __forceinline__ void block_sum(double *v, int nv, double (*red)[256]) {
  for (int k = 0; k < nv; ++k) red[k][threadIdx.x] = v[k];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      for (int k = 0; k < nv; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + s];
    __syncthreads();
  }
}

// One differential-time term (likelihood_dd.F90:467-476, 501-522), q =
// ddindex * nrev + k: adds to like, misfit, unweighted misfit and the
// log-sum of dsigma when the reference's test lets it in.
__device__ void dd_terms(const Tt2dDev &d, const double *T, double n0, double n1, int q, double &like, double &mis,
                         double &umis, double &sdl) {
  const int dd = q / d.nrev, k = q % d.nrev;
  const int2 ij = d.pairs[dd];
  const double dt = T[(size_t)ij.y * d.nrev + k] - T[(size_t)ij.x * d.nrev + k];
  const double ds = n0 * (1 - d.dcc[(size_t)dd * d.nrev + k]) + n1;
  // dat%dtime(ddindex,k,1): column-major element (ddindex-1) + (k-1)*nrev
  if (fabs(d.dtime[(size_t)dd + (size_t)k * d.nrev]) > kEps) {
    const double r = dt - d.dtime[(size_t)dd * d.nrev + k];
    const double r2 = r * r;
    like += r2 / (2 * (ds * ds));
    mis += r2 / (ds * ds);
    umis += r2;
    sdl += log(ds);
  }
}

// sigma and the misfit / -log L of every chain, one block per chain.
__global__ void tt2d_misfit_kernel(Tt2dDev d, const double *tt, const double *n0, const double *n1, double *out,
                                   double *umis_keep) {
  const int c = blockIdx.x;
  const int npairs = d.nsrc * d.nrev;
  const double *T = tt + (size_t)c * npairs;           // [src][rev] = phaseTime(k,j,1)
  double v[7] = {0, 0, 0, 0, 0, 0, 0};                  // like, mis, umis, slog, dd like, dd mis+umis share, sdl
  double dmis = 0, dumis = 0;
  int bad = 0;
  for (int q = threadIdx.x; q < npairs; q += blockDim.x) {
    const bool used = d.raystat[q] == 1;
    double sig = 1.0;
    if (used) sig = d.sigdep ? n0[2 * c] * T[q] + n1[2 * c] : d.tsig[q];
    if (used) {
      if (sig == 0.0) bad = 1;                          // 'The noise level is 0!'
      const double res = T[q] - d.tobs[q];
      const double r2 = res * res;
      v[0] += r2 / (2 * (sig * sig));
      v[1] += r2 / (sig * sig);
      v[2] += r2;
    }
    v[3] += log(sig);
  }
  if (d.datatype == 1)
    for (int q = threadIdx.x; q < d.ndd * d.nrev; q += blockDim.x)
      dd_terms(d, T, n0[2 * c + 1], n1[2 * c + 1], q, v[4], dmis, dumis, v[6]);
  v[1] += dmis; v[2] += dumis;
  __shared__ double red[7][256];
  __shared__ int sbad;
  if (threadIdx.x == 0) sbad = 0;
  __syncthreads();
  if (bad) sbad = 1;
  block_sum(v, 7, red);
  if (threadIdx.x == 0) {
    double L = red[0][0] + red[3][0] + (double)((float)d.nrays / 2.0f) * log(kPI2);
    if (d.datatype == 1) L = L + red[4][0] + red[6][0] + (double)((float)d.ndtime / 2.0f) * log(kPI2);
    out[(size_t)c * 4 + 0] = sbad ? DBL_MAX : L;
    out[(size_t)c * 4 + 1] = red[1][0];
    out[(size_t)c * 4 + 2] = red[2][0];
    out[(size_t)c * 4 + 3] = sbad ? 8.0 : 0.0;
    umis_keep[c] = red[2][0];
  }
}

// Noise-only likelihood (likelihood_dd.F90:32-106) on the last forward's
// times; the differential sigma log-sum is an INTEGER there, truncated
// after every term, so one thread adds it in the reference's order.
__global__ void tt2d_noise_kernel(Tt2dDev d, const double *tt, const double *n0, const double *n1,
                                  const double *umis_keep, const int *committed, double *out) {
  const int c = blockIdx.x;
  const int npairs = d.nsrc * d.nrev;
  const double *T = tt + (size_t)c * npairs;
  double v[5] = {0, 0, 0, 0, 0};                        // like, mis, slog, dd like, dd mis
  double dumis = 0, dsl = 0;
  int bad = 0;
  for (int q = threadIdx.x; q < npairs; q += blockDim.x) {
    const double srd = d.sigdep ? T[q] : d.srd0[q];
    double sig = n0[2 * c] * srd + n1[2 * c];
    if (d.raystat[q] == 1) {
      if (sig == 0.0) bad = 1;
      const double res = T[q] - d.tobs[q];
      const double r2 = res * res;
      v[0] += r2 / (2 * (sig * sig));
      v[1] += r2 / (sig * sig);
    } else {
      sig = 1.0;
    }
    if (sig < kEps) bad = 1;                            // any(like%sigma < EPS)
    v[2] += log(sig);
  }
  if (d.datatype == 1)
    for (int q = threadIdx.x; q < d.ndd * d.nrev; q += blockDim.x)
      dd_terms(d, T, n0[2 * c + 1], n1[2 * c + 1], q, v[3], v[4], dumis, dsl);
  __shared__ double red[5][256];
  __shared__ int sbad;
  if (threadIdx.x == 0) sbad = 0;
  __syncthreads();
  if (bad) sbad = 1;
  block_sum(v, 5, red);
  if (threadIdx.x == 0) {
    double L = red[0][0] + red[2][0] + (double)((float)d.nrays / 2.0f) * log(kPI2);
    double mis = red[1][0];
    if (d.datatype == 1) {
      int sumdsigma = 0;
      for (int q = 0; q < d.ndd * d.nrev; ++q) {
        const int dd = q / d.nrev, k = q % d.nrev;
        if (fabs(d.dtime[(size_t)dd + (size_t)k * d.nrev]) > kEps) {
          const double ds = n0[2 * c + 1] * (1 - d.dcc[(size_t)dd * d.nrev + k]) + n1[2 * c + 1];
          sumdsigma = fortran_int((double)sumdsigma + log(ds));
        }
      }
      L = L + red[3][0] + (double)sumdsigma + (double)((float)d.ndtime / 2.0f) * log(kPI2);
      mis += red[4][0];
    }
    const int stt = (sbad ? 8 : 0) | (committed[c] ? 0 : 16);
    out[(size_t)c * 4 + 0] = stt ? DBL_MAX : L;
    out[(size_t)c * 4 + 1] = mis;
    out[(size_t)c * 4 + 2] = umis_keep[c];
    out[(size_t)c * 4 + 3] = (double)stt;
  }
}

// Source-receiver distance as gfortran's NORM2 computes it (the scaled sum
// of squares of LAPACK's dnrm2: scale by the largest magnitude so far),
// which the 2D code's setup uses as the initial srdist.
double norm2_fortran(double a, double b) {
  double scale = 1.0, ssq = 0.0;
  for (double x : {a, b}) {
    if (x != 0.0) {
      const double ax = std::fabs(x);
      if (scale < ax) {
        const double v = scale / ax;
        ssq = 1.0 + ssq * v * v;
        scale = ax;
      } else {
        const double v = ax / scale;
        ssq += v * v;
      }
    }
  }
  return scale * std::sqrt(ssq);
}

// An accepted proposal becomes its chain's state: times and unweighted
// misfit (what the reference keeps in `like` after the Metropolis step).
__global__ void tt2d_commit_kernel(int npairs, const int *accept, const double *out, const double *tt,
                                   const double *umis, double *ctt, double *cumis, int *committed) {
  const int c = blockIdx.y;
  if (!accept[c] || out[(size_t)c * 4 + 3] != 0.0) return;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < npairs; q += gridDim.x * blockDim.x)
    ctt[(size_t)c * npairs + q] = tt[(size_t)c * npairs + q];
  if (blockIdx.x == 0 && threadIdx.x == 0) { cumis[c] = umis[c]; committed[c] = 1; }
}

// Committed counterparts of the forward's maps and solves for fm2d's reuse
// of refined boxes (chain c is slot c; -1 while nothing is committed).
__global__ void tt2d_reuse_index_kernel(int nchains, int spc, const int *committed, int *cmap, int *csolve) {
  const int stride = gridDim.x * blockDim.x, i0 = blockIdx.x * blockDim.x + threadIdx.x;
  for (int m = i0; m < nchains; m += stride) cmap[m] = committed[m] ? m : -1;
  for (int q = i0; q < nchains * spc; q += stride) csolve[q] = committed[q / spc] ? q : -1;
}

// An accepted forward's padded map and refined-box mappings become the
// chain's committed ones.
__global__ void tt2d_commit_ref_kernel(const int *accept, const double *out, size_t nvv, const double *velv,
                                       double *cvelv, size_t nref, const double *map_t, const short *map_s,
                                       double *cref_t, short *cref_s) {
  const int c = blockIdx.y;
  if (!accept[c] || out[(size_t)c * 4 + 3] != 0.0) return;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < nvv; q += (size_t)gridDim.x * blockDim.x)
    cvelv[(size_t)c * nvv + q] = velv[(size_t)c * nvv + q];
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < nref; q += (size_t)gridDim.x * blockDim.x) {
    cref_t[(size_t)c * nref + q] = map_t[(size_t)c * nref + q];
    cref_s[(size_t)c * nref + q] = map_s[(size_t)c * nref + q];
  }
}

}  // namespace

struct mct_tt2d_ctx {
  mct_grid g{};
  mct_tt2d_settings st{};
  int nslots = 0, ncell_max = 0, spc = 0, last_nchains = 0;
  Tt2dDev dev{};
  Fm2dJob fj{};
  Fm2dPlan fp{};
  cudaStream_t stream = nullptr;
  void *mem = nullptr;
  int *ncells = nullptr; double *points = nullptr, *params = nullptr;
  double *n0 = nullptr, *n1 = nullptr, *out = nullptr, *umis = nullptr;
  int *sites = nullptr, *tie_count = nullptr, *tie_nodes = nullptr, *gstatus = nullptr;
  void *kd = nullptr;
  double *vel = nullptr, *velv = nullptr, *tt = nullptr;
  double *ctt = nullptr, *cumis = nullptr;     // committed state per slot
  int *committed = nullptr, *accept = nullptr;
  // fm2d's reuse of committed refined boxes (refined source boxes only)
  int reuse = 0;
  double *cvelv = nullptr, *cref_t = nullptr; short *cref_s = nullptr;
  int *cmap = nullptr, *csolve = nullptr, *ref_list = nullptr;
  // mct_tt2d_submit / mct_tt2d_poll: pinned staging (allocated by the first
  // submit), the completion event and the batch in flight
  int *h_ints = nullptr;       // [nslots] ncells, [2] device status
  double *h_dbl = nullptr;     // points [nslots][ncell_max][2], params [..][3], n0, n1 [nslots][2], out [nslots][4]
  cudaEvent_t done = nullptr;
  int pending = 0;
};

namespace {
bool tt2d_busy(const mct_tt2d_ctx *c, const char *name);
}

extern "C" {

int mct_tt2d_create(const mct_grid *g, const mct_tt2d_settings *st, const mct_tt2d_data *dat, int nslots,
                    int ncell_max, mct_tt2d_ctx **out) {
  const char *name = "mct_tt2d_create";
  if (out) *out = nullptr;
  if (!g || !st || !dat || !out || nslots < 1 || ncell_max < 1 || ncell_max > 12800 || g->nx < 2 || g->ny < 2 ||
      !(g->dx > 0) || !(g->dy > 0) || !(g->scaling > 0) || dat->nsrc < 1 || dat->nrev < 1 || !dat->src ||
      !dat->rev || !dat->raystat || !dat->ttime || (st->sigdep == 0 && !dat->sigma) ||
      (st->datatype != 0 && st->datatype != 1) || (st->straight != 0 && st->straight != 1) ||
      (st->precision != 0 && st->precision != 1)) {
    mct_set_error(name, "bad arguments", __FILE__, __LINE__);
    return MCT_ERR_ARG;
  }
  const int nsrc = dat->nsrc, nrev = dat->nrev, npairs = nsrc * nrev;
  const int ndd = st->datatype == 1 ? nsrc * (nsrc - 1) / 2 : 0;
  if (ndd > 0) {
    // the swapped-index test reads element ddindex + k*nrev of dtime(:,:,1)
    if (!dat->dtime || !dat->dcc ||
        (long long)(ndd - 1) + (long long)(nrev - 1) * nrev >= (long long)ndd * nrev) {
      mct_set_error(name, "differential times: the reference's test would read outside dtime", __FILE__, __LINE__);
      return MCT_ERR_ARG;
    }
  }
  mct_tt2d_ctx *c = new mct_tt2d_ctx();
  c->g = *g; c->st = *st; c->nslots = nslots; c->ncell_max = ncell_max;
  const int nx = g->nx, ny = g->ny;
  const size_t nodes = (size_t)nx * ny, nvv = (size_t)(nx + 2) * (ny + 2);
  // fm2d: vertex grid = the model grid, y over the scaling (likelihood_dd.F90:438-446)
  Fm2dJob &fj = c->fj;
  fj.nvx = nx; fj.nvz = ny; fj.goxd = g->xmin; fj.gozd = g->ymin / g->scaling; fj.dvxd = g->dx;
  fj.dvzd = g->dy / g->scaling;
  fj.gdx = st->gridx; fj.gdz = st->gridy; fj.asgr = st->sgref; fj.sgdl = st->sgdic; fj.sgs = st->sgext;
  fj.fom = st->order; fj.nsrc = nsrc; fj.nrc = nrev; fj.srs_nmaps = 1; fj.precision = st->precision;
  std::vector<int2> all;
  if (!st->straight) {
    if (fj.gdx < 1 || fj.gdz < 1 || (fj.asgr == 1 && (fj.sgdl < 1 || fj.sgs < 1)) || (fj.fom != 0 && fj.fom != 1) ||
        fm2d_plan(fj, &c->fp)) {
      delete c;
      mct_set_error(name, "fm2d settings or grid size", __FILE__, __LINE__);
      return MCT_ERR_ARG;
    }
    // a source with no path is skipped unless it is the first
    // (fm2dray_cartesian.f90:213-215)
    std::vector<int> act;
    for (int i = 0; i < nsrc; ++i) {
      int any = 0;
      for (int k = 0; k < nrev; ++k) any |= dat->raystat[(size_t)i * nrev + k] == 1;
      if (any || i == 0) act.push_back(i);
    }
    c->spc = (int)act.size();
    for (int ch = 0; ch < nslots; ++ch)
      for (int i : act) all.push_back(make_int2(ch, i));
  }
  const size_t nsolve = all.size();
  const int nnx = (nx - 1) * std::max(fj.gdx, 1) + 1, nnz = (ny - 1) * std::max(fj.gdz, 1) + 1;
  const size_t kd = kd_scratch_bytes(ncell_max);
  const bool fm = !st->straight;
  // fm2d may reuse a committed refined box whose map is unchanged
  const bool reuse = fm && fj.asgr == 1 && fj.precision != 2;
  std::vector<size_t> sz = {
      sizeof(int) * nslots, sizeof(double) * (size_t)nslots * ncell_max * 5, sizeof(double) * 4 * nslots,
      sizeof(double) * 8 * nslots, sizeof(double) * nslots,
      sizeof(int) * nslots * nodes, sizeof(int) * nslots, sizeof(int) * nslots * nodes, kd * nslots, sizeof(int) * 2,
      sizeof(double) * 3 * nslots * nodes, sizeof(double) * nslots * nvv, sizeof(double) * (size_t)nslots * npairs,
      sizeof(double) * (size_t)nslots * (npairs + 1), sizeof(int) * 2 * nslots,
      // data
      sizeof(int) * npairs, sizeof(double) * 5 * (size_t)npairs, sizeof(double) * 2 * (size_t)ndd * nrev,
      sizeof(int2) * (size_t)std::max(ndd, 1), sizeof(double) * 2 * (nsrc + nrev), sizeof(double) * 2 * (nsrc + nrev),
      // fm2d scratch
      fm ? sizeof(int2) * nsolve : 0, fm ? sizeof(double) * (size_t)c->fp.nref_map * nslots : 0,
      fm ? sizeof(double) * (size_t)c->fp.map_tmp_max * nsolve : 0,
      fm ? sizeof(short) * (size_t)c->fp.map_tmp_max * nsolve : 0, sizeof(int) * (nsolve + 1),
      fm ? sizeof(double) * 2 * (size_t)nnx * nnz * nslots : 0, sizeof(int),
      fm ? fm2d_tws_bytes(c->fp, (long)nsolve) : 0,
      reuse ? sizeof(double) * nslots * nvv : 0, reuse ? sizeof(double) * (size_t)c->fp.map_tmp_max * nsolve : 0,
      reuse ? sizeof(short) * (size_t)c->fp.map_tmp_max * nsolve : 0,
      reuse ? sizeof(int) * ((size_t)nslots + 2 * nsolve + 1) : 0};
  size_t total = 0;
  for (size_t b : sz) total = ((total + 255) & ~size_t(255)) + b;
  total += 256;
  if (cudaMalloc(&c->mem, total) != cudaSuccess) {
    delete c;
    mct_set_error(name, "cudaMalloc failed", __FILE__, __LINE__);
    return MCT_ERR_NOMEM;
  }
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaFree(c->mem); delete c; return MCT_ERR_CUDA;
  }
  Carve cv(c->mem);
  c->ncells = cv.take<int>(nslots);
  c->points = cv.take<double>((size_t)nslots * ncell_max * 5);
  c->params = c->points + (size_t)nslots * ncell_max * 2;
  c->n0 = cv.take<double>((size_t)4 * nslots); c->n1 = c->n0 + 2 * (size_t)nslots;
  c->out = cv.take<double>((size_t)8 * nslots);     // forward results, then noise-only results
  c->umis = cv.take<double>(nslots);
  c->sites = cv.take<int>(nslots * nodes);
  c->tie_count = cv.take<int>(nslots);
  c->tie_nodes = cv.take<int>(nslots * nodes);
  c->kd = cv.take<char>(kd * nslots);
  c->gstatus = cv.take<int>(2);
  c->vel = cv.take<double>(3 * nslots * nodes);
  c->velv = cv.take<double>(nslots * nvv);
  c->tt = cv.take<double>((size_t)nslots * npairs);
  c->ctt = cv.take<double>((size_t)nslots * (npairs + 1));
  c->cumis = c->ctt + (size_t)nslots * npairs;
  c->committed = cv.take<int>(2 * nslots);
  c->accept = c->committed + nslots;
  int *d_rays = cv.take<int>(npairs);
  double *d_pd = cv.take<double>(5 * (size_t)npairs);
  double *d_dd = cv.take<double>(2 * (size_t)ndd * nrev);
  int2 *d_pairs = cv.take<int2>((size_t)std::max(ndd, 1));
  double *d_xy = cv.take<double>(2 * (size_t)(nsrc + nrev));
  double *d_sep = cv.take<double>(2 * (size_t)(nsrc + nrev));
  int2 *d_solves = cv.take<int2>(fm ? nsolve : 0);
  fj.sref = cv.take<double>(fm ? (size_t)c->fp.nref_map * nslots : 0);
  fj.map_tmp_t = cv.take<double>(fm ? (size_t)c->fp.map_tmp_max * nsolve : 0);
  fj.map_tmp_s = cv.take<short>(fm ? (size_t)c->fp.map_tmp_max * nsolve : 0);
  fj.ovf_list = cv.take<int>(nsolve + 1);
  fj.ovf_count = fj.ovf_list + nsolve;
  fj.veln = cv.take<double>(fm ? 2 * (size_t)nnx * nnz * nslots : 0);
  fj.slon = fj.veln + (size_t)nnx * nnz * nslots;
  fj.vmin_bits = cv.take<int>(1);
  if (fm) fm2d_bind_tws(fj, c->fp, (long)nsolve, cv.take<char>(fm2d_tws_bytes(c->fp, (long)nsolve)));
  c->reuse = reuse ? 1 : 0;
  c->cvelv = cv.take<double>(reuse ? (size_t)nslots * nvv : 0);
  c->cref_t = cv.take<double>(reuse ? (size_t)c->fp.map_tmp_max * nsolve : 0);
  c->cref_s = cv.take<short>(reuse ? (size_t)c->fp.map_tmp_max * nsolve : 0);
  c->cmap = cv.take<int>(reuse ? (size_t)nslots + 2 * nsolve + 1 : 0);
  c->csolve = c->cmap + nslots;
  c->ref_list = c->csolve + nsolve;
  // data in the reference's layouts
  std::vector<double> pd(5 * (size_t)npairs, 1.0), xy(2 * (size_t)(nsrc + nrev)), sep(2 * (size_t)(nsrc + nrev));
  std::vector<int2> pairs((size_t)std::max(ndd, 1), make_int2(0, 0));
  for (int j = 0; j < nsrc; ++j)
    for (int k = 0; k < nrev; ++k) {
      const size_t n = (size_t)j * nrev + k;
      const double sx = dat->src[2 * j], sy = dat->src[2 * j + 1], rx = dat->rev[2 * k], ry = dat->rev[2 * k + 1];
      pd[n] = dat->ttime[n];
      pd[npairs + n] = dat->sigma ? dat->sigma[n] : 1.0;
      const double dx = rx - sx, dy = ry - sy;
      pd[4 * (size_t)npairs + n] = std::sqrt(dx * dx + dy * dy);          // setup_straightRays
      pd[2 * (size_t)npairs + n] = st->straight ? pd[4 * (size_t)npairs + n] : norm2_fortran(sx - rx, sy - ry);
    }
  for (int j = 0; j < nsrc; ++j) {
    xy[2 * j] = dat->src[2 * j]; xy[2 * j + 1] = dat->src[2 * j + 1];
    sep[j] = dat->src[2 * j]; sep[nsrc + j] = dat->src[2 * j + 1];
  }
  for (int k = 0; k < nrev; ++k) {
    xy[2 * (nsrc + k)] = dat->rev[2 * k]; xy[2 * (nsrc + k) + 1] = dat->rev[2 * k + 1];
    sep[2 * nsrc + k] = dat->rev[2 * k]; sep[2 * nsrc + nrev + k] = dat->rev[2 * k + 1];
  }
  {
    int q = 0;
    for (int i = 0; i < nsrc; ++i)
      for (int j = i + 1; j < nsrc && ndd > 0; ++j) pairs[q++] = make_int2(i, j);
  }
  bool ok = cudaMemcpy(d_rays, dat->raystat, sizeof(int) * npairs, cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemcpy(d_pd, pd.data(), sizeof(double) * pd.size(), cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemcpy(d_pairs, pairs.data(), sizeof(int2) * pairs.size(), cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemcpy(d_xy, xy.data(), sizeof(double) * xy.size(), cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemcpy(d_sep, sep.data(), sizeof(double) * sep.size(), cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemset(c->tt, 0, sizeof(double) * (size_t)nslots * npairs) == cudaSuccess &&
            cudaMemset(c->umis, 0, sizeof(double) * nslots) == cudaSuccess &&
            cudaMemset(c->ctt, 0, sizeof(double) * (size_t)nslots * (npairs + 1)) == cudaSuccess &&
            cudaMemset(c->committed, 0, sizeof(int) * 2 * nslots) == cudaSuccess;
  if (ok && ndd > 0)
    ok = cudaMemcpy(d_dd, dat->dtime, sizeof(double) * (size_t)ndd * nrev, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(d_dd + (size_t)ndd * nrev, dat->dcc, sizeof(double) * (size_t)ndd * nrev,
                    cudaMemcpyHostToDevice) == cudaSuccess;
  if (ok && fm)
    ok = cudaMemcpy(d_solves, all.data(), sizeof(int2) * nsolve, cudaMemcpyHostToDevice) == cudaSuccess;
  if (!ok || cudaDeviceSynchronize() != cudaSuccess) {
    cudaFree(c->mem); cudaStreamDestroy(c->stream); delete c;
    mct_set_error(name, "upload failed", __FILE__, __LINE__);
    return MCT_ERR_CUDA;
  }
  Tt2dDev &d = c->dev;
  d.nx = nx; d.ny = ny; d.xmin = g->xmin; d.ymin = g->ymin; d.dx = g->dx; d.dy = g->dy; d.scaling = g->scaling;
  d.nsrc = nsrc; d.nrev = nrev; d.nrays = dat->nrays; d.sigdep = st->sigdep; d.datatype = st->datatype;
  d.straight = st->straight; d.ndd = ndd; d.ndtime = dat->ndtime;
  d.raystat = d_rays; d.tobs = d_pd; d.tsig = d_pd + npairs; d.srd0 = d_pd + 2 * (size_t)npairs;
  d.sdist = d_pd + 4 * (size_t)npairs; d.dtime = d_dd; d.dcc = d_dd + (size_t)ndd * nrev; d.pairs = d_pairs;
  d.src_xy = d_xy; d.rev_xy = d_xy + 2 * nsrc;
  fj.scx = d_sep; fj.scz = d_sep + nsrc; fj.rcx = d_sep + 2 * nsrc; fj.rcz = d_sep + 2 * nsrc + nrev;
  fj.srs = d_rays; fj.solves = d_solves;
  fj.nodes_max = c->fp.nodes_max; fj.nref_max = c->fp.nref_max; fj.map_tmp_max = c->fp.map_tmp_max;
  fj.nref_map = c->fp.nref_map;
  *out = c;
  return MCT_OK;
}

int mct_tt2d_set_priority(mct_tt2d_ctx *c, int high) {
  if (!c || tt2d_busy(c, "mct_tt2d_set_priority")) return MCT_ERR_ARG;
  return mct_restream(&c->stream, high);
}

int mct_tt2d_set_sm_share(mct_tt2d_ctx *c, double share) {
  if (!c || !(share >= 0.0 && share <= 1.0)) return MCT_ERR_ARG;
  c->fp.sm_share = share;
  return MCT_OK;
}

int mct_tt2d_destroy(mct_tt2d_ctx *c) {
  if (!c) return MCT_OK;
  cudaStreamSynchronize(c->stream);
  if (c->h_ints) cudaFreeHost(c->h_ints);
  if (c->h_dbl) cudaFreeHost(c->h_dbl);
  if (c->done) cudaEventDestroy(c->done);
  cudaFree(c->mem);
  cudaStreamDestroy(c->stream);
  delete c;
  return MCT_OK;
}

}  // extern "C"

namespace {
bool tt2d_busy(const mct_tt2d_ctx *c, const char *name) {
  if (!c->pending) return false;
  mct_set_error(name, "a submitted batch is not polled yet", __FILE__, __LINE__);
  return true;
}

int tt2d_check(const mct_tt2d_ctx *c, int nchains, const int *ncells, const double *points, const double *params,
               const double *n0, const double *n1, const char *name) {
  if (!c || tt2d_busy(c, name)) return MCT_ERR_ARG;
  if (nchains < 1 || nchains > c->nslots || !ncells || !points || !params || !n0 || !n1) {
    mct_set_error(name, "bad arguments", __FILE__, __LINE__);
    return MCT_ERR_ARG;
  }
  for (int i = 0; i < nchains; ++i)
    if (ncells[i] < 1 || ncells[i] > c->ncell_max) {
      mct_set_error(name, "cell count outside [1, ncell_max]", __FILE__, __LINE__);
      return MCT_ERR_ARG;
    }
  return MCT_OK;
}

// The forward's work on the context's stream: the inputs copied from host
// arrays, the results and the two device status words copied to out and gst
// (host arrays; pinned ones make the copies asynchronous).
int tt2d_enqueue(mct_tt2d_ctx *c, int nchains, const int *ncells, const double *points, const double *params,
                 const double *n0, const double *n1, double *out, int *gst) {
  const mct_grid &g = c->g;
  const Tt2dDev &d = c->dev;
  cudaStream_t s = c->stream;
  const size_t nodes = (size_t)g.nx * g.ny;
  const size_t npc = (size_t)nchains * c->ncell_max;
  MCT_CUDA_TRY(cudaMemcpyAsync(c->ncells, ncells, sizeof(int) * nchains, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(c->points, points, sizeof(double) * npc * 2, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(c->params, params, sizeof(double) * npc * 3, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(c->n0, n0, sizeof(double) * 2 * nchains, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(c->n1, n1, sizeof(double) * 2 * nchains, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemsetAsync(c->gstatus, 0, sizeof(int) * 2, s));
  // gridding (mcmc2d/mcmc.f90:1469-1525): velocity = parameters(1, nearest)
  GridJob gj{};
  gj.d = 2; gj.nx = g.nx; gj.ny = g.ny; gj.nz = 1;
  gj.xmin = g.xmin; gj.ymin = g.ymin; gj.zmin = 0.0; gj.dx = g.dx; gj.dy = g.dy; gj.dz = 0.0;
  gj.nchains = nchains; gj.ncell_max = c->ncell_max; gj.ncells = c->ncells;
  gj.points = c->points; gj.params = c->params; gj.box = nullptr;
  gj.sites_id = c->sites; gj.vp = c->vel; gj.vs = c->vel + c->nslots * nodes; gj.rho = c->vel + 2 * c->nslots * nodes;
  gj.tie_count = c->tie_count; gj.tie_nodes = c->tie_nodes; gj.kd_scratch = c->kd; gj.status = c->gstatus;
  int rc = launch_grid_nearest(gj, s); if (rc) return rc;
  const int npairs = d.nsrc * d.nrev;
  if (d.straight) {
    tt2d_straight_kernel<<<dim3((npairs + 127) / 128, nchains), 128, 0, s>>>(d, c->vel, c->tt, c->gstatus + 1);
    MCT_CUDA_TRY(cudaGetLastError());
  } else {
    tt2d_pad_kernel<<<dim3(8, nchains), 256, 0, s>>>(g.nx, g.ny, c->vel, c->velv);
    MCT_CUDA_TRY(cudaGetLastError());
    Fm2dJob fj = c->fj;
    fj.nmaps = nchains; fj.velv = c->velv; fj.nsolve = c->spc * nchains;
    fj.ttime = c->tt; fj.tfield = nullptr; fj.status = c->gstatus + 1;
    if (c->reuse) {
      tt2d_reuse_index_kernel<<<64, 256, 0, s>>>(nchains, c->spc, c->committed, c->cmap, c->csolve);
      MCT_CUDA_TRY(cudaGetLastError());
      fj.cvelv = c->cvelv; fj.cmap = c->cmap; fj.csolve = c->csolve; fj.cref_t = c->cref_t; fj.cref_s = c->cref_s;
      fj.ref_list = c->ref_list; fj.ref_count = c->ref_list + (size_t)c->spc * c->nslots;
    }
    rc = launch_fm2d(fj, c->fp, s); if (rc) return rc;
  }
  tt2d_misfit_kernel<<<nchains, 256, 0, s>>>(d, c->tt, c->n0, c->n1, c->out, c->umis);
  MCT_CUDA_TRY(cudaGetLastError());
  MCT_CUDA_TRY(cudaMemcpyAsync(out, c->out, sizeof(double) * 4 * nchains, cudaMemcpyDeviceToHost, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(gst, c->gstatus, sizeof(int) * 2, cudaMemcpyDeviceToHost, s));
  return MCT_OK;
}

// The call's status from the device status words (gridding, fm2d).
int tt2d_status(const int *gst, const char *name) {
  if (gst[0]) return gst[0];
  if (gst[1]) {
    mct_set_error(name, gst[1] == MCT_ERR_OUTSIDE ? "ray or source outside the grid" : "fm2d status", __FILE__,
                  __LINE__);
    return gst[1] < 0 ? gst[1] : MCT_ERR_INTERNAL;
  }
  return MCT_OK;
}
}  // namespace

extern "C" {

int mct_tt2d_forward(mct_tt2d_ctx *c, int nchains, const int *ncells, const double *points, const double *params,
                     const double *n0, const double *n1, double *out) {
  int rc = tt2d_check(c, nchains, ncells, points, params, n0, n1, "mct_tt2d_forward");
  if (rc) return rc;
  if (!out) return MCT_ERR_ARG;
  int gst[2] = {0, 0};
  rc = tt2d_enqueue(c, nchains, ncells, points, params, n0, n1, out, gst);
  if (rc) return rc;
  MCT_CUDA_TRY(cudaStreamSynchronize(c->stream));
  c->last_nchains = nchains;
  return tt2d_status(gst, "mct_tt2d_forward");
}

int mct_tt2d_submit(mct_tt2d_ctx *c, int nchains, const int *ncells, const double *points, const double *params,
                    const double *n0, const double *n1) {
  int rc = tt2d_check(c, nchains, ncells, points, params, n0, n1, "mct_tt2d_submit");
  if (rc) return rc;
  const int ns = c->nslots;
  const size_t pmax = (size_t)ns * c->ncell_max;
  if (!c->h_ints) {
    MCT_CUDA_TRY(cudaHostAlloc(&c->h_ints, sizeof(int) * (ns + 2), cudaHostAllocDefault));
    MCT_CUDA_TRY(cudaHostAlloc(&c->h_dbl, sizeof(double) * (pmax * 5 + (size_t)ns * 8), cudaHostAllocDefault));
    MCT_CUDA_TRY(cudaEventCreateWithFlags(&c->done, cudaEventDisableTiming));
  }
  const size_t npc = (size_t)nchains * c->ncell_max;
  int *hn = c->h_ints, *hg = c->h_ints + ns;
  double *hp = c->h_dbl, *hq = hp + pmax * 2, *h0 = hq + pmax * 3, *h1 = h0 + (size_t)ns * 2, *ho = h1 + (size_t)ns * 2;
  std::memcpy(hn, ncells, sizeof(int) * nchains);
  std::memcpy(hp, points, sizeof(double) * npc * 2);
  std::memcpy(hq, params, sizeof(double) * npc * 3);
  std::memcpy(h0, n0, sizeof(double) * 2 * nchains);
  std::memcpy(h1, n1, sizeof(double) * 2 * nchains);
  rc = tt2d_enqueue(c, nchains, hn, hp, hq, h0, h1, ho, hg);
  if (rc) return rc;
  MCT_CUDA_TRY(cudaEventRecord(c->done, c->stream));
  c->pending = nchains;
  return MCT_OK;
}

int mct_tt2d_poll(mct_tt2d_ctx *c, double *out, int *done) {
  if (!c || !out || !done || !c->pending) return MCT_ERR_ARG;
  *done = 0;
  const cudaError_t q = cudaEventQuery(c->done);
  if (q == cudaErrorNotReady) return MCT_OK;
  if (q != cudaSuccess) { mct_set_error("cudaEventQuery", cudaGetErrorString(q), __FILE__, __LINE__); return MCT_ERR_CUDA; }
  const int ns = c->nslots, n = c->pending;
  const size_t pmax = (size_t)ns * c->ncell_max;
  const double *ho = c->h_dbl + pmax * 5 + (size_t)ns * 4;
  std::memcpy(out, ho, sizeof(double) * 4 * n);
  c->pending = 0;
  c->last_nchains = n;
  *done = 1;
  return tt2d_status(c->h_ints + ns, "mct_tt2d_poll");
}

int mct_tt2d_commit(mct_tt2d_ctx *c, int nchains, const int *accept) {
  if (!c || tt2d_busy(c, "mct_tt2d_commit")) return MCT_ERR_ARG;
  if (nchains < 1 || nchains > c->last_nchains || !accept) {
    mct_set_error("mct_tt2d_commit", "bad arguments (commit follows a forward of at least nchains)", __FILE__,
                  __LINE__);
    return MCT_ERR_ARG;
  }
  cudaStream_t s = c->stream;
  const int npairs = c->dev.nsrc * c->dev.nrev;
  MCT_CUDA_TRY(cudaMemcpyAsync(c->accept, accept, sizeof(int) * nchains, cudaMemcpyHostToDevice, s));
  if (c->reuse) {
    // before tt2d_commit_kernel sets the chains' committed flags
    const size_t nvv = (size_t)(c->g.nx + 2) * (c->g.ny + 2), nref = (size_t)c->spc * c->fp.map_tmp_max;
    tt2d_commit_ref_kernel<<<dim3(32, nchains), 256, 0, s>>>(c->accept, c->out, nvv, c->velv, c->cvelv, nref,
                                                            c->fj.map_tmp_t, c->fj.map_tmp_s, c->cref_t, c->cref_s);
    MCT_CUDA_TRY(cudaGetLastError());
  }
  tt2d_commit_kernel<<<dim3((npairs + 255) / 256, nchains), 256, 0, s>>>(npairs, c->accept, c->out, c->tt, c->umis,
                                                                         c->ctt, c->cumis, c->committed);
  MCT_CUDA_TRY(cudaGetLastError());
  MCT_CUDA_TRY(cudaStreamSynchronize(s));
  return MCT_OK;
}

int mct_tt2d_noise_likelihood(mct_tt2d_ctx *c, int nchains, const double *n0, const double *n1, double *out) {
  if (!c || tt2d_busy(c, "mct_tt2d_noise_likelihood")) return MCT_ERR_ARG;
  if (nchains < 1 || nchains > c->nslots || !n0 || !n1 || !out) {
    mct_set_error("mct_tt2d_noise_likelihood", "bad arguments", __FILE__, __LINE__);
    return MCT_ERR_ARG;
  }
  cudaStream_t s = c->stream;
  MCT_CUDA_TRY(cudaMemcpyAsync(c->n0, n0, sizeof(double) * 2 * nchains, cudaMemcpyHostToDevice, s));
  MCT_CUDA_TRY(cudaMemcpyAsync(c->n1, n1, sizeof(double) * 2 * nchains, cudaMemcpyHostToDevice, s));
  double *nout = c->out + 4 * (size_t)c->nslots;   // the forward's results stay for commit
  tt2d_noise_kernel<<<nchains, 256, 0, s>>>(c->dev, c->ctt, c->n0, c->n1, c->cumis, c->committed, nout);
  MCT_CUDA_TRY(cudaGetLastError());
  MCT_CUDA_TRY(cudaMemcpyAsync(out, nout, sizeof(double) * 4 * nchains, cudaMemcpyDeviceToHost, s));
  MCT_CUDA_TRY(cudaStreamSynchronize(s));
  return MCT_OK;
}

int mct_tt2d_phase_time(mct_tt2d_ctx *c, int index, double *phase_time) {
  if (!c || tt2d_busy(c, "mct_tt2d_phase_time") || index < 0 || index >= c->last_nchains || !phase_time) return MCT_ERR_ARG;
  const size_t npairs = (size_t)c->dev.nsrc * c->dev.nrev;
  MCT_CUDA_TRY(cudaMemcpyAsync(phase_time, c->tt + (size_t)index * npairs, sizeof(double) * npairs,
                               cudaMemcpyDeviceToHost, c->stream));
  MCT_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return MCT_OK;
}

}  // extern "C"
