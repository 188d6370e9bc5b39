// Batched surface-wave likelihood with device-resident chain state: the GPU
// replacement of likelihood() case 2 (src/likelihood.f90:57-93) ->
// surf_likelihood (src/likelihood_surf.F90:110-410), together with the
// kdtree_to_grid call the sampler makes before it.
//
// One forward evaluates a proposal for each of many chains:
//   1. nearest-nucleus gridding of every chain's Voronoi model;
//   2. material laws vs -> vp (1.73 vs) and vp -> rho (1.74 vp^0.25) or a
//      fixed density (src/likelihood.f90:75-76, src/utils.f90:98-135);
//   3. check_model (likelihood_surf.F90:631-646);
//   4. the columns whose (vp, vs, rho) differ from the chain's committed
//      state are layered (convert_to_layer, :523-629) and get new dispersion
//      curves (surfmodes/surfdisp96); the rest reuse the committed curves.
//      This replaces the CGAL bounding box (:155-170) with an exact
//      changed-column mask: the curves are identical;
//   5. phase-velocity maps padded by edge copies (:259-264) feed fm2d for
//      every (period, source) (:295-320);
//   6. sigma and the misfit / -log L reductions (:356-404).
// commit() makes a proposal the chain's state (the sampler's accept);
// otherwise the next forward starts again from the committed state (reject).
#include "mct_common.cuh"
#include "fm2d.cuh"
#include "surf_pipeline.cuh"
#include <cfloat>
#include <vector>
#include <algorithm>

namespace {

__global__ void material_kernel(int nchains, int ncell_max, const int *ncells, const double *params_in,
                                double *params_out, int law, double rho_value) {
  const int c = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ncell_max; i += gridDim.x * blockDim.x) {
    size_t o = ((size_t)c * ncell_max + i) * 3;
    if (i >= ncells[c]) { params_out[o] = params_out[o + 1] = params_out[o + 2] = 1.0; continue; }
    double vs = params_in[o + 1];
    double vp, rho;
    if (law == MCT_LAW_EXPLICIT) {
      vp = params_in[o]; rho = params_in[o + 2];
    } else {
      vp = vs * (double)1.730f;                           // vs2vp_3d
      rho = (law == MCT_LAW_REFERENCE) ? (double)1.74f * pow(vp, 0.25) : rho_value;   // vp2rho_3d
    }
    params_out[o] = vp; params_out[o + 1] = vs; params_out[o + 2] = rho;
  }
}

// check_model + changed-column list. One thread per (chain, column).
__global__ void columns_kernel(SurfBatch b) {
  const int c = blockIdx.y;
  const int ncol = b.nx * b.ny;
  const int slot = b.slots[c];
  const size_t nodes = (size_t)ncol * b.nz;
  for (int col = blockIdx.x * blockDim.x + threadIdx.x; col < ncol; col += gridDim.x * blockDim.x) {
    const size_t o = (size_t)c * nodes + (size_t)col * b.nz;
    const double *vs = b.vs + o, *vp = b.vp + o, *rho = b.rho + o;
    bool bad = false;
    for (int k = 1; k < b.nz; ++k) if (vs[k] < vs[0]) bad = true;
    if (bad) atomicOr(&b.status[c], 1);
    bool changed = !b.committed[slot];
    if (!changed) {
      const size_t co = (size_t)slot * nodes + (size_t)col * b.nz;
      for (int k = 0; k < b.nz && !changed; ++k)
        changed = vs[k] != b.cvs[co + k] || vp[k] != b.cvp[co + k] || rho[k] != b.crho[co + k];
    }
    if (changed) {
      int pos = atomicAdd(b.list_count, 1);
      b.list[pos] = make_int2(c, col);
    }
  }
}

// convert_to_layer (likelihood_surf.F90:523-629) for listed columns, cast to
// REAL*4 as surfmodes does (surfmodes.f90:81).
__global__ void layer_kernel(SurfBatch b) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= *b.list_count) return;
  const int2 e = b.list[q];
  const size_t nodes = (size_t)b.nx * b.ny * b.nz;
  const size_t o = (size_t)e.x * nodes + (size_t)e.y * b.nz;
  const double *vp = b.vp + o, *vs = b.vs + o, *rho = b.rho + o;
  const double EPS = 1.0E-10;
  float *thk = b.lthk + (size_t)q * b.nl_max, *a = b.lvp + (size_t)q * b.nl_max;
  float *bb = b.lvs + (size_t)q * b.nl_max, *r = b.lrho + (size_t)q * b.nl_max;
  int nl = 0;
  double wd = b.water_depth;
  if (wd > EPS) { nl = 1; a[0] = (float)(double)1.5f; bb[0] = 0.f; r[0] = 1.f; thk[0] = (float)wd; }
  double last_vp = vp[0], last_vs = vs[0], last_rho = rho[0];
  int last_k = 1;
  for (int k = 2; k <= b.nz; ++k) {
    if (fabs(vs[k - 1] - last_vs) > EPS) {
      nl = nl + 1;
      a[nl - 1] = (float)last_vp; bb[nl - 1] = (float)last_vs; r[nl - 1] = (float)last_rho;
      thk[nl - 1] = (float)(((double)(k - last_k) * b.dz) / b.scaling);
      last_vp = vp[k - 1]; last_vs = vs[k - 1]; last_rho = rho[k - 1];
      last_k = k;
    }
  }
  nl = nl + 1;
  a[nl - 1] = (float)vp[b.nz - 1]; bb[nl - 1] = (float)vs[b.nz - 1]; r[nl - 1] = (float)rho[b.nz - 1];
  thk[nl - 1] = 0.f;
  if (wd > 0) thk[0] = (float)wd;
  b.lnl[q] = nl;
}

// Proposal phase maps: committed maps updated with the recomputed columns.
// pvel layout [chain][period][nx][ny] (Fortran (ny,nx) per period).
__global__ void scatter_kernel(SurfBatch b) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= *b.list_count) return;
  const int2 e = b.list[q];
  const int ncol = b.nx * b.ny;
  if (b.lierr[q]) atomicOr(&b.status[e.x], 2);
  for (int p = 0; p < b.np; ++p)
    b.pvel[((size_t)e.x * b.np + p) * ncol + e.y] = b.lcp[(size_t)q * b.np + p];
  if (b.igr)
    for (int p = 0; p < b.np; ++p)
      b.gvel[((size_t)e.x * b.np + p) * ncol + e.y] = b.lcg[(size_t)q * b.np + p];
}

// Padded fm2d vertex grids (likelihood_surf.F90:259-264): interior = phase
// map, edges copied from the nearest interior node.
__global__ void pad_kernel(SurfBatch b) {
  const int map = blockIdx.y;        // chain * np + period
  const int nvx = b.nx + 2, nvz = b.ny + 2;
  const double *pv = b.pvel + (size_t)map * b.nx * b.ny;
  double *v = b.velv + (size_t)map * nvx * nvz;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nvx * nvz; q += gridDim.x * blockDim.x) {
    int jj = q % nvz, ii = q / nvz;            // 0-based padded row (y) and column (x)
    int j = min(max(jj, 1), b.ny) - 1, i = min(max(ii, 1), b.nx) - 1;
    v[q] = pv[(size_t)i * b.ny + j];
  }
}

// sigma and the misfit / -log L (likelihood_surf.F90:356-404), one block per
// chain, FP64 block reduction.
// The likelihood's phaseTime and srdist by mode (likelihood_surf.F90:233-329):
// phase times and srdist = phase time; group times along the rays and
// srdist = ray length; straight-ray times and srdist = the distance.
__device__ __forceinline__ const double *like_times(const SurfBatch &b) {
  return (b.igr || b.straight) ? b.gtime : b.ttime;
}
__device__ __forceinline__ double like_srdist(const SurfBatch &b, size_t q, int r) {
  return b.straight ? b.sdist[r] : (b.igr ? b.raylen[q] : b.ttime[q]);
}

__global__ void misfit_kernel(SurfBatch b) {
  const int c = blockIdx.x;
  const int npairs = b.nsrc * b.nrev;
  const double *pt = like_times(b) + (size_t)c * b.np * npairs;   // [p][src][rev] = phaseTime(k,j,p)
  if (b.igr && !b.straight && threadIdx.x < b.np && b.crazy[(size_t)c * b.np + threadIdx.x] > 0)
    atomicOr(&b.status[c], 4);     // crazyray: like = huge
  double like = 0, mis = 0, umis = 0, slog = 0;
  for (int q = threadIdx.x; q < b.np * npairs; q += blockDim.x) {
    int p = q / npairs, r = q % npairs;
    double sig;
    bool used = b.raystat[(size_t)p * npairs + r] == 1;
    const double srd = like_srdist(b, (size_t)c * b.np * npairs + q, r);
    if (b.sigdep != 0) sig = used ? b.n0[(size_t)c * b.np + p] * srd + b.n1[(size_t)c * b.np + p] : 1.0;
    else sig = used ? b.dsigma[(size_t)p * npairs + r] : 1.0;
    if (used) {
      if (sig < 1.0E-10) atomicOr(&b.status[c], 8);
      double res = pt[q] - b.dtime[(size_t)p * npairs + r];
      double r2 = res * res;
      like += r2 / (2 * (sig * sig));
      mis += r2 / (sig * sig);
      umis += r2;
    }
    slog += log(sig);
  }
  __shared__ double red[4][256];
  red[0][threadIdx.x] = like; red[1][threadIdx.x] = mis; red[2][threadIdx.x] = umis; red[3][threadIdx.x] = slog;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      for (int k = 0; k < 4; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double PI2 = (double)6.283185f;
    double L = red[0][0] + red[3][0] + (double)((float)b.nrays / 2.0f) * log(PI2);
    int st = b.status[c];
    b.out[(size_t)c * 4 + 0] = st ? DBL_MAX : L;
    b.out[(size_t)c * 4 + 1] = red[1][0];
    b.out[(size_t)c * 4 + 2] = red[2][0];
    b.out[(size_t)c * 4 + 3] = (double)st;
  }
}

// Copy a chain's proposal into its slot's committed state.
// Committed counterparts of this forward's maps and solves (-1: the slot
// holds no committed state), for the reuse test of the refined stage.
__global__ void reuse_index_kernel(SurfBatch b, int nch) {
  const int stride = gridDim.x * blockDim.x, i0 = blockIdx.x * blockDim.x + threadIdx.x;
  for (int m = i0; m < nch * b.np; m += stride) {
    const int slot = b.slots[m / b.np];
    b.cmap[m] = b.committed[slot] ? slot * b.np + m % b.np : -1;
  }
  for (int q = i0; q < nch * b.spc; q += stride) {
    const int slot = b.slots[q / b.spc];
    b.csolve[q] = b.committed[slot] ? slot * b.spc + q % b.spc : -1;
  }
}

// An accepted forward's padded maps and refined-box mappings become the
// slot's committed ones (beside commit_kernel's state).
__global__ void commit_ref_kernel(SurfBatch b, const int *accept) {
  const int c = blockIdx.y;
  if (!accept[c] || b.status[c]) return;
  const int slot = b.slots[c];
  const size_t nvv = (size_t)(b.nx + 2) * (b.ny + 2) * b.np;
  for (size_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nvv; q += (size_t)gridDim.x * blockDim.x)
    b.cvelv[(size_t)slot * nvv + q] = b.velv[(size_t)c * nvv + q];
  const size_t nt = (size_t)b.spc * b.map_tmp_max;
  for (size_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nt; q += (size_t)gridDim.x * blockDim.x) {
    b.cref_t[(size_t)slot * nt + q] = b.map_tmp_t[(size_t)c * nt + q];
    b.cref_s[(size_t)slot * nt + q] = b.map_tmp_s[(size_t)c * nt + q];
  }
}

__global__ void commit_kernel(SurfBatch b, const int *accept) {
  const int c = blockIdx.y;
  if (!accept[c] || b.status[c]) return;
  const int slot = b.slots[c];
  const size_t nodes = (size_t)b.nx * b.ny * b.nz;
  const size_t maps = (size_t)b.np * b.nx * b.ny;
  for (size_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nodes; q += (size_t)gridDim.x * blockDim.x) {
    b.cvp[(size_t)slot * nodes + q] = b.vp[(size_t)c * nodes + q];
    b.cvs[(size_t)slot * nodes + q] = b.vs[(size_t)c * nodes + q];
    b.crho[(size_t)slot * nodes + q] = b.rho[(size_t)c * nodes + q];
  }
  for (size_t q = blockIdx.x * blockDim.x + threadIdx.x; q < maps; q += (size_t)gridDim.x * blockDim.x)
    b.cpvel[(size_t)slot * maps + q] = b.pvel[(size_t)c * maps + q];
  if (b.igr)
    for (size_t q = blockIdx.x * blockDim.x + threadIdx.x; q < maps; q += (size_t)gridDim.x * blockDim.x)
      b.cgvel[(size_t)slot * maps + q] = b.gvel[(size_t)c * maps + q];
  const size_t nt = (size_t)b.np * b.nsrc * b.nrev;
  const int npairs = b.nsrc * b.nrev;
  const double *lt = like_times(b);
  for (size_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nt; q += (size_t)gridDim.x * blockDim.x) {
    b.cttime[(size_t)slot * nt + q] = lt[(size_t)c * nt + q];
    b.csrd[(size_t)slot * nt + q] = like_srdist(b, (size_t)c * nt + q, (int)(q % npairs));
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) b.committed[slot] = 1;
}

// surf_noise_likelihood (src/likelihood_surf.F90:56-99): the committed phase
// times re-reduced with new noise parameters, sigma = n0 * srdist + n1 with
// the committed srdist (phase time, ray length or distance by mode), for
// every pair; unused pairs count with sigma = 1.
// A sigma below 1e-10 is the reference's fatal 'noise level is 0' (status 8).
__global__ void noise_kernel(SurfBatch b, const int *slots, const double *n0, const double *n1, double *out) {
  const int c = blockIdx.x;
  const int slot = slots[c];
  const int npairs = b.nsrc * b.nrev;
  const double *pt = b.cttime + (size_t)slot * b.np * npairs;
  double like = 0, mis = 0, umis = 0, slog = 0;
  int bad = 0;
  for (int q = threadIdx.x; q < b.np * npairs; q += blockDim.x) {
    const int p = q / npairs, r = q % npairs;
    const bool used = b.raystat[(size_t)p * npairs + r] == 1;
    const double srd = b.csrd[(size_t)slot * b.np * npairs + q];
    double sig = n0[(size_t)c * b.np + p] * srd + n1[(size_t)c * b.np + p];
    if (used) {
      if (sig == 0.0) bad = 1;
      const double res = pt[q] - b.dtime[(size_t)p * npairs + r];
      const double r2 = res * res;
      like += r2 / (2 * (sig * sig));
      mis += r2 / (sig * sig);
      umis += r2;
    } else {
      sig = 1.0;
    }
    if (sig < 1.0E-10) bad = 1;
    slog += log(sig);
  }
  __shared__ double red[4][256];
  __shared__ int sbad;
  if (threadIdx.x == 0) sbad = 0;
  __syncthreads();
  if (bad) sbad = 1;
  red[0][threadIdx.x] = like; red[1][threadIdx.x] = mis; red[2][threadIdx.x] = umis; red[3][threadIdx.x] = slog;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st)
      for (int k = 0; k < 4; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double PI2 = (double)6.283185f;
    const double L = red[0][0] + red[3][0] + (double)((float)b.nrays / 2.0f) * log(PI2);
    const int stt = (sbad ? 8 : 0) | (b.committed[slot] ? 0 : 16);
    out[(size_t)c * 4 + 0] = stt ? DBL_MAX : L;
    out[(size_t)c * 4 + 1] = red[1][0];
    out[(size_t)c * 4 + 2] = red[2][0];
    out[(size_t)c * 4 + 3] = (double)stt;
  }
}

__global__ void gather_committed_maps(SurfBatch b) {
  const int c = blockIdx.y;
  const int slot = b.slots[c];
  const size_t maps = (size_t)b.np * b.nx * b.ny;
  for (size_t q = blockIdx.x * blockDim.x + threadIdx.x; q < maps; q += (size_t)gridDim.x * blockDim.x)
    b.pvel[(size_t)c * maps + q] = b.committed[slot] ? b.cpvel[(size_t)slot * maps + q] : 0.0;
  if (b.igr)
    for (size_t q = blockIdx.x * blockDim.x + threadIdx.x; q < maps; q += (size_t)gridDim.x * blockDim.x)
      b.gvel[(size_t)c * maps + q] = b.committed[slot] ? b.cgvel[(size_t)slot * maps + q] : 0.0;
}

// setup_straightRays + CalGroupTime (likelihood_surf.F90:412-494), one thread
// per (chain, period, path): points every min(dx, dy)/2 from the source, the
// receiver last, delay on the group maps (phase maps for phaseGroup = 0).
__device__ double grid_velocity(const SurfBatch &b, const double *vel, double px, double py) {
  int ix = (int)floor((px - b.xmin) / b.dx) + 1;
  int iy = (int)floor((py - b.ymin) / b.dy) + 1;
  if (ix < 1) ix = 1;
  if (iy < 1) iy = 1;
  if (ix >= b.nx) ix = b.nx - 1;
  if (iy >= b.ny) iy = b.ny - 1;
  const double dsx = px - (b.xmin + (double)(ix - 1) * b.dx);
  const double dsy = py - (b.ymin + (double)(iy - 1) * b.dy);
  double qv = 0;
  for (int i = 1; i <= 2; ++i)
    for (int j = 1; j <= 2; ++j) {
      const double weight = (1.0 - fabs((double)(i - 1) * b.dx - dsx) / b.dx) *
                            (1.0 - fabs((double)(j - 1) * b.dy - dsy) / b.dy);
      qv = qv + weight * vel[(size_t)(ix + i - 2) * b.ny + (iy + j - 2)];
    }
  return qv;
}

__global__ void straight_kernel(SurfBatch b, const double *src, const double *rev) {
  const int npairs = b.nsrc * b.nrev;
  const int map = blockIdx.y;                 // chain * np + period
  const int p = map % b.np;
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= npairs) return;
  double *t = b.gtime + (size_t)map * npairs;
  t[n] = 0;
  if (b.raystat[(size_t)p * npairs + n] != 1) return;
  const int j = n / b.nrev, k = n % b.nrev;
  const double *vel = (b.igr ? b.gvel : b.pvel) + (size_t)map * b.nx * b.ny;
  const double sx = src[2 * j], sy = src[2 * j + 1], rx = rev[2 * k], ry = rev[2 * k + 1];
  const double ddx = rx - sx, ddy = ry - sy;
  const double ds = sqrt(ddx * ddx + ddy * ddy);
  const double dl = fmin(b.dx, b.dy) / 2;
  const int npts = (int)floor(ds / dl) + 1;
  const double xmax = b.xmin + (double)(b.nx - 1) * b.dx, ymax = b.ymin + (double)(b.ny - 1) * b.dy;
  double px = sx, py = sy, vhead = 0, tt = 0;
  for (int l = 1; l <= npts; ++l) {
    double qx, qy;
    if (l < npts) {
      qx = sx + (double)(l - 1) * dl * ddx / ds;
      qy = sy + (double)(l - 1) * dl * ddy / ds;
      if (qx < b.xmin || qx > xmax || qy < b.ymin || qy > ymax) {   // 'Straight ray out of area'
        atomicExch(&b.dev_status[0], MCT_ERR_OUTSIDE);
        return;
      }
    } else {
      qx = rx; qy = ry;
    }
    const double v = grid_velocity(b, vel, qx, qy);
    if (l > 1) {
      double dist = (qx - px) * (qx - px) + (qy - py) * (qy - py);
      dist = sqrt(dist);
      tt = tt + dist * 2 / (vhead + v);
    }
    vhead = v; px = qx; py = qy;
  }
  t[n] = tt;
}

}  // namespace

int surf_forward(SurfBatch &b, const SurfPlan &plan, cudaStream_t s, SurfProfile *prof) {
  const int nch = b.nchains;
  cudaEvent_t *ev = nullptr;
  if (prof && prof->enabled && prof->step < prof->max_steps) ev = prof->ev + 5 * prof->step++;
  if (ev) MCT_CUDA_TRY(cudaEventRecord(ev[0], s));
  if (prof) {
    // the kernels of one forward: material, gridding (3), layering and
    // dispersion (4), the committed maps' gather and scatter, the misfit,
    // and the travel-time stage's
    const Fm2dJob &f = plan.fm2d;
    const Fm2dPlan &fp = plan.fm2d_plan;
    int n = 11;
    if (b.straight) n += 1;
    else n += 3 + (f.precision == 2 ? 1 : 0) + (f.asgr == 1 ? 2 + (fp.ref_heap_cap < fp.nref_max ? 1 : 0) : 0) +
              (b.reuse ? 2 : 0);
    prof->launches += n;
  }
  const int ncol = b.nx * b.ny;
  MCT_CUDA_TRY(cudaMemsetAsync(b.status, 0, sizeof(int) * nch, s));
  MCT_CUDA_TRY(cudaMemsetAsync(b.list_count, 0, sizeof(int), s));
  MCT_CUDA_TRY(cudaMemsetAsync(b.dev_status, 0, sizeof(int) * 2, s));
  // 1-2: material laws then gridding
  material_kernel<<<dim3((b.ncell_max + 127) / 128, nch), 128, 0, s>>>(nch, b.ncell_max, b.ncells, b.params_in,
                                                                         b.params, b.law, b.rho_value);
  MCT_CUDA_TRY(cudaGetLastError());
  GridJob gj{};
  gj.d = 3; gj.nx = b.nx; gj.ny = b.ny; gj.nz = b.nz;
  gj.xmin = b.xmin; gj.ymin = b.ymin; gj.zmin = b.zmin; gj.dx = b.dx; gj.dy = b.dy; gj.dz = b.dz;
  gj.nchains = nch; gj.ncell_max = b.ncell_max; gj.ncells = b.ncells;
  gj.points = b.points; gj.params = b.params; gj.box = nullptr;
  gj.sites_id = b.sites; gj.vp = b.vp; gj.vs = b.vs; gj.rho = b.rho;
  gj.tie_count = b.tie_count; gj.tie_nodes = b.tie_nodes; gj.kd_scratch = b.kd_scratch; gj.status = b.dev_status;
  int rc = launch_grid_nearest(gj, s); if (rc) return rc;
  if (ev) MCT_CUDA_TRY(cudaEventRecord(ev[1], s));
  // 3-4: model check, changed columns, layering, dispersion, scatter
  columns_kernel<<<dim3((ncol + 127) / 128, nch), 128, 0, s>>>(b);
  MCT_CUDA_TRY(cudaGetLastError());
  const int maxlist = nch * ncol;
  layer_kernel<<<(maxlist + 127) / 128, 128, 0, s>>>(b);
  MCT_CUDA_TRY(cudaGetLastError());
  DispJob dj{};
  dj.ncol = maxlist; dj.ncol_dev = b.list_count; dj.nl_max = b.nl_max; dj.nl = b.lnl;
  dj.thk = b.lthk; dj.vp = b.lvp; dj.vs = b.lvs; dj.rho = b.lrho;
  dj.np = b.np; dj.periods = b.periods; dj.iwave = b.iwave; dj.mode = 1; dj.igr = b.igr;
  dj.dphase = b.dphase; dj.multimode = 0; dj.precision = b.precision;
  dj.cp = b.lcp; dj.cg = b.lcg; dj.ierr = b.lierr; dj.ndltar = b.ndltar; dj.order = b.lorder;
  rc = launch_surfdisp(dj, s); if (rc) return rc;
  gather_committed_maps<<<dim3(64, nch), 256, 0, s>>>(b);
  MCT_CUDA_TRY(cudaGetLastError());
  scatter_kernel<<<(maxlist + 127) / 128, 128, 0, s>>>(b);
  MCT_CUDA_TRY(cudaGetLastError());
  if (ev) MCT_CUDA_TRY(cudaEventRecord(ev[2], s));
  // 5: padded maps and fm2d
  if (b.straight) {
    const int npairs = b.nsrc * b.nrev;
    straight_kernel<<<dim3((npairs + 127) / 128, nch * b.np), 128, 0, s>>>(b, plan.src_xy, plan.rev_xy);
    MCT_CUDA_TRY(cudaGetLastError());
  } else {
    pad_kernel<<<dim3(8, nch * b.np), 256, 0, s>>>(b);
    MCT_CUDA_TRY(cudaGetLastError());
    Fm2dJob fj = plan.fm2d;
    fj.nmaps = nch * b.np;
    fj.velv = b.velv;
    fj.nsolve = plan.nsolve_per_chain * nch;
    fj.ttime = b.ttime;
    fj.tfield = nullptr;
    fj.status = b.dev_status;
    if (b.igr) {
      fj.rays = 1; fj.gvel = b.gvel; fj.gtime = b.gtime; fj.raylen = b.raylen; fj.crazy = b.crazy;
      MCT_CUDA_TRY(cudaMemsetAsync(b.crazy, 0, sizeof(int) * (size_t)nch * b.np, s));
    }
    if (b.reuse) {
      reuse_index_kernel<<<64, 256, 0, s>>>(b, nch);
      MCT_CUDA_TRY(cudaGetLastError());
      fj.cvelv = b.cvelv; fj.cmap = b.cmap; fj.csolve = b.csolve; fj.cref_t = b.cref_t; fj.cref_s = b.cref_s;
      fj.ref_list = b.ref_list; fj.ref_count = b.ref_count;
    }
    rc = launch_fm2d(fj, plan.fm2d_plan, s); if (rc) return rc;
  }
  if (ev) MCT_CUDA_TRY(cudaEventRecord(ev[3], s));
  // 6: misfit
  misfit_kernel<<<nch, 256, 0, s>>>(b);
  MCT_CUDA_TRY(cudaGetLastError());
  if (ev) MCT_CUDA_TRY(cudaEventRecord(ev[4], s));
  return MCT_OK;
}

int surf_noise(const SurfBatch &b, int nchains, const int *slots, const double *n0, const double *n1, double *out,
               cudaStream_t s) {
  noise_kernel<<<nchains, 256, 0, s>>>(b, slots, n0, n1, out);
  MCT_CUDA_TRY(cudaGetLastError());
  return MCT_OK;
}

int surf_commit(SurfBatch &b, const int *accept_dev, cudaStream_t s) {
  if (b.reuse) {
    commit_ref_kernel<<<dim3(64, b.nchains), 256, 0, s>>>(b, accept_dev);
    MCT_CUDA_TRY(cudaGetLastError());
  }
  commit_kernel<<<dim3(64, b.nchains), 256, 0, s>>>(b, accept_dev);
  MCT_CUDA_TRY(cudaGetLastError());
  return MCT_OK;
}
