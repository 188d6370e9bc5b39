// Voronoi -> grid map (nearest nucleus per grid node), the GPU replacement of
// kdtree_to_grid (src/mcmc_loc2.f90:2002-2082, mcmc2d/mcmc.f90:1469-1525) and
// its kdtree2 search (src/kdtree2.f90).
//
// The output must equal kdtree2's, including which of several equidistant
// nuclei wins. kdtree2 keeps the last visited point whose squared distance is
// <= the best so far (process_terminal_node, kdtree2.f90:1530-1592), with the
// squared distance summed over coordinates left to right without FMA
// (kdtree2.f90:1534-1538). So:
//   1. every node finds its nearest nucleus by brute force over nuclei staged
//      in shared memory, in FP32 on coordinates shifted to the grid origin;
//   2. the nuclei within a rigorous FP32 error margin of that minimum are
//      re-scored with the exact FP64 squared distance (__dmul_rn/__dadd_rn);
//   3. a unique FP64 minimum is the answer; nodes with an exact or near tie
//      (relative gap <= 1e-13) are queued and resolved by running the kdtree2
//      build and search on the device for that chain, so ties break as in the
//      reference.
#include "mct_common.cuh"
#include <cfloat>

namespace {

constexpr int BUCKET = 12;          // kdtree2.f90:516 bucket_size
constexpr int KD_STACK = 96;
constexpr int GRID_THREADS = 256;

struct KdNode {
  int cut_dim, l, u, left, right, pad;
  double cut_val, cut_val_left, cut_val_right;
  double lo[3], hi[3];
};

struct KdTree {
  int d, n;
  const double *data;   // [n][d] original order, 1-based index i -> data[(i-1)*d]
  int *ind;             // [n] 1-based permutation
  double *rdata;        // [n][d] rearranged
  KdNode *nodes;
  int nnodes, root;
};

__device__ __forceinline__ double kv(const KdTree &t, int c, int pos) {
  return t.data[(size_t)(t.ind[pos - 1] - 1) * t.d + c];
}

__device__ void kd_spread(const KdTree &t, int c, int l, int u, double &lo, double &hi) {
  double smin = kv(t, c, l), smax = smin;
  for (int i = l + 1; i <= u; ++i) {
    double x = kv(t, c, i);
    if (smin > x) smin = x;
    if (smax < x) smax = x;
  }
  lo = smin; hi = smax;
}

// kdtree2.f90:843-895 select_on_coordinate_value
__device__ int kd_select(KdTree &t, int c, double alpha, int li, int ui) {
  int lb = li, rb = ui;
  while (lb < rb) {
    if (kv(t, c, lb) <= alpha) lb = lb + 1;
    else { int tmp = t.ind[lb - 1]; t.ind[lb - 1] = t.ind[rb - 1]; t.ind[rb - 1] = tmp; rb = rb - 1; }
  }
  return (kv(t, c, lb) <= alpha) ? lb : lb - 1;
}

struct BuildFrame { int l, u, parent, id, m, stage, slot_owner, slot; };

// kdtree2.f90:704-840 build_tree_for_range, iterative. Returns 0 or -1 on
// stack/node overflow.
__device__ int kd_build(KdTree &t, int max_nodes) {
  BuildFrame st[KD_STACK];
  int sp = 0;
  t.nnodes = 0; t.root = -1;
  st[sp++] = {1, t.n, -1, -1, 0, 0, -1, 0};
  while (sp > 0) {
    BuildFrame &f = st[sp - 1];
    if (f.stage == 0) {
      int result = -1;
      bool done = true;
      if (f.u >= f.l) {
        if (t.nnodes >= max_nodes) return -1;
        int id = t.nnodes++;
        KdNode &r = t.nodes[id];
        r.left = r.right = -1;
        r.cut_val_left = r.cut_val_right = 0.0;
        r.l = f.l; r.u = f.u;
        if ((f.u - f.l) <= BUCKET) {
          for (int i = 0; i < t.d; ++i) kd_spread(t, i, f.l, f.u, r.lo[i], r.hi[i]);
          r.cut_dim = 0; r.cut_val = 0.0;
          result = id;
        } else {
          for (int i = 0; i < t.d; ++i) {
            bool recompute = !(f.parent >= 0 && i != t.nodes[f.parent].cut_dim);
            if (recompute) kd_spread(t, i, f.l, f.u, r.lo[i], r.hi[i]);
            else { r.lo[i] = t.nodes[f.parent].lo[i]; r.hi[i] = t.nodes[f.parent].hi[i]; }
          }
          int c = 0;
          double best = r.hi[0] - r.lo[0];
          for (int i = 1; i < t.d; ++i) {
            double s = r.hi[i] - r.lo[i];
            if (s > best) { best = s; c = i; }
          }
          double sum = 0.0;
          for (int i = f.l; i <= f.u; ++i) sum = __dadd_rn(sum, kv(t, c, i));
          double average = __ddiv_rn(sum, (double)(f.u - f.l + 1));
          r.cut_val = average;
          r.cut_dim = c;
          f.m = kd_select(t, c, average, f.l, f.u);
          f.id = id;
          f.stage = 1;
          done = false;
          if (sp >= KD_STACK) return -1;
          st[sp++] = {f.l, f.m, id, -1, 0, 0, id, 0};
        }
      }
      if (done) {
        int owner = f.slot_owner, slot = f.slot;
        --sp;
        if (owner < 0) t.root = result;
        else if (slot == 0) t.nodes[owner].left = result;
        else t.nodes[owner].right = result;
      }
    } else if (f.stage == 1) {
      f.stage = 2;
      if (sp >= KD_STACK) return -1;
      int id = f.id, m = f.m, u = f.u;
      st[sp++] = {m + 1, u, id, -1, 0, 0, id, 1};
    } else {
      KdNode &r = t.nodes[f.id];
      int c = r.cut_dim;
      if (r.right < 0) {
        const KdNode &L = t.nodes[r.left];
        for (int i = 0; i < t.d; ++i) { r.lo[i] = L.lo[i]; r.hi[i] = L.hi[i]; }
        r.cut_val_left = L.hi[c];
        r.cut_val = r.cut_val_left;
      } else if (r.left < 0) {
        const KdNode &R = t.nodes[r.right];
        for (int i = 0; i < t.d; ++i) { r.lo[i] = R.lo[i]; r.hi[i] = R.hi[i]; }
        r.cut_val_right = R.lo[c];
        r.cut_val = r.cut_val_right;
      } else {
        const KdNode &L = t.nodes[r.left];
        const KdNode &R = t.nodes[r.right];
        r.cut_val_right = R.lo[c];
        r.cut_val_left = L.hi[c];
        r.cut_val = __ddiv_rn(__dadd_rn(r.cut_val_left, r.cut_val_right), 2.0);
        for (int i = 0; i < t.d; ++i) {
          r.hi[i] = fmax(L.hi[i], R.hi[i]);
          r.lo[i] = fmin(L.lo[i], R.lo[i]);
        }
      }
      int owner = f.slot_owner, slot = f.slot, id = f.id;
      --sp;
      if (owner < 0) t.root = id;
      else if (slot == 0) t.nodes[owner].left = id;
      else t.nodes[owner].right = id;
    }
  }
  for (int i = 0; i < t.n; ++i)
    for (int k = 0; k < t.d; ++k) t.rdata[(size_t)i * t.d + k] = t.data[(size_t)(t.ind[i] - 1) * t.d + k];
  return 0;
}

__device__ __forceinline__ double dis2_from_bnd(double x, double amin, double amax) {
  if (x > amax) { double e = __dsub_rn(x, amax); return __dmul_rn(e, e); }
  if (x < amin) { double e = __dsub_rn(amin, x); return __dmul_rn(e, e); }
  return 0.0;
}

struct SearchFrame { int node, stage, farther; double dis; };

// kdtree2.f90:1369-1443 search + 1496-1599 process_terminal_node (nn = 1).
__device__ int kd_nearest(const KdTree &t, const double *qv, int *err) {
  double ballsize = (double)FLT_MAX;   // huge(1.0)
  int best = 0;
  SearchFrame st[64];
  int sp = 0;
  st[sp++] = {t.root, 0, -1, 0.0};
  while (sp > 0) {
    SearchFrame &f = st[sp - 1];
    const KdNode &node = t.nodes[f.node];
    if (f.stage == 0) {
      if (!(node.left >= 0 && node.right >= 0)) {
        for (int i = node.l; i <= node.u; ++i) {
          double sd = 0.0;
          bool skip = false;
          for (int k = 0; k < t.d; ++k) {
            double df = __dsub_rn(t.rdata[(size_t)(i - 1) * t.d + k], qv[k]);
            sd = __dadd_rn(sd, __dmul_rn(df, df));
            if (sd > ballsize) { skip = true; break; }
          }
          if (skip) continue;
          best = t.ind[i - 1];
          ballsize = sd;
        }
        --sp;
        continue;
      }
      int cd = node.cut_dim;
      double qval = qv[cd];
      int closer;
      if (qval < node.cut_val) {
        closer = node.left; f.farther = node.right;
        double e = __dsub_rn(node.cut_val_right, qval); f.dis = __dmul_rn(e, e);
      } else {
        closer = node.right; f.farther = node.left;
        double e = __dsub_rn(node.cut_val_left, qval); f.dis = __dmul_rn(e, e);
      }
      f.stage = 1;
      if (closer >= 0) {
        if (sp >= 64) { *err = 1; return best; }
        st[sp++] = {closer, 0, -1, 0.0};
      }
    } else if (f.stage == 1) {
      f.stage = 2;
      bool go = false;
      if (f.farther >= 0 && f.dis <= ballsize) {
        double dis = f.dis;
        go = true;
        for (int i = 0; i < t.d; ++i) {
          if (i != node.cut_dim) {
            dis = __dadd_rn(dis, dis2_from_bnd(qv[i], node.lo[i], node.hi[i]));
            if (dis > ballsize) { go = false; break; }
          }
        }
      }
      if (go) {
        if (sp >= 64) { *err = 1; return best; }
        st[sp++] = {f.farther, 0, -1, 0.0};
      } else {
        --sp;
      }
    } else {
      --sp;
    }
  }
  return best;
}

__device__ __forceinline__ double node_coord(double origin, int i1, double step) {
  return __dadd_rn(origin, __dmul_rn((double)(i1 - 1), step));
}

struct BoxIdx { int ix0, ix1, iy0, iy1, iz0, iz1; };

// The chain's box clipped to the grid. Returns false for an empty or
// inverted box (the chain is then skipped and the call's status set).
__device__ __forceinline__ bool chain_box(const GridJob &job, int c, BoxIdx &b) {
  if (job.box) {
    const int *p = job.box + 6 * c;
    b = {max(p[0], 1), min(p[1], job.nx), max(p[2], 1), min(p[3], job.ny), max(p[4], 1), min(p[5], job.nz)};
  } else {
    b = {1, job.nx, 1, job.ny, 1, job.nz};
  }
  if (job.d == 2) { b.iz0 = 1; b.iz1 = 1; }
  return b.ix0 <= b.ix1 && b.iy0 <= b.iy1 && b.iz0 <= b.iz1;
}

// The chain's nucleus count, or -1 when it lies outside [1, ncell_max]
// (the chain is then skipped and the call's status set).
__device__ __forceinline__ int chain_cells(const GridJob &job, int c) {
  const int n = job.ncells[c];
  return (n >= 1 && n <= job.ncell_max) ? n : -1;
}

// Error word that outlives the calls: every launch folds its own status into
// it (the first nonzero code stays until read by mct_grid_status).
__device__ int g_grid_status;

__global__ void fold_status_kernel(const int *status) {
  const int st = *status;
  if (st != 0) atomicCAS(&g_grid_status, 0, st);
}

__global__ void __launch_bounds__(GRID_THREADS)
grid_nearest_kernel(GridJob job) {
  extern __shared__ float4 nuc[];
  __shared__ float s_scale;
  const int c = blockIdx.y;
  const int n = chain_cells(job, c);
  BoxIdx b;
  const bool box_ok = chain_box(job, c, b);
  if (n < 0 || !box_ok) {
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicExch(job.status, MCT_ERR_ARG);
    return;
  }
  const int d = job.d;
  const double *pts = job.points + (size_t)c * job.ncell_max * d;
  const double *par = job.params + (size_t)c * job.ncell_max * 3;
  if (threadIdx.x == 0) s_scale = 0.f;
  __syncthreads();
  float lmax = 0.f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    float x = (float)__dsub_rn(pts[(size_t)i * d + 0], job.xmin);
    float y = (float)__dsub_rn(pts[(size_t)i * d + 1], job.ymin);
    float z = d == 3 ? (float)__dsub_rn(pts[(size_t)i * d + 2], job.zmin) : 0.f;
    nuc[i] = make_float4(x, y, z, 0.f);
    lmax = fmaxf(lmax, fmaxf(fabsf(x), fmaxf(fabsf(y), fabsf(z))));
  }
  // shifted coordinates are non-negative finite floats: compare as ints
  atomicMax(reinterpret_cast<int *>(&s_scale), __float_as_int(lmax));
  __syncthreads();
  const int bnx = b.ix1 - b.ix0 + 1, bny = b.iy1 - b.iy0 + 1, bnz = b.iz1 - b.iz0 + 1;
  const long nbox = (long)bnx * bny * bnz;
  const float ext = fmaxf(s_scale, fmaxf((float)((job.nx - 1) * job.dx),
                          fmaxf((float)((job.ny - 1) * job.dy), (float)((job.nz - 1) * job.dz))));
  // Each FP32 squared distance is within 21*2^-24*d*ext^2 of the exact one;
  // twice that (two distances compared) times a safety factor of 4.
  const float margin = 1.0e-5f * (float)d * ext * ext;
  const long nodes_total = (long)job.nx * job.ny * (d == 3 ? job.nz : 1);
  for (long li = (long)blockIdx.x * blockDim.x + threadIdx.x; li < nbox;
       li += (long)gridDim.x * blockDim.x) {
    int kk = (int)(li % bnz);
    long r = li / bnz;
    int jj = (int)(r % bny);
    int ii = (int)(r / bny);
    int i = b.ix0 + ii, j = b.iy0 + jj, k = b.iz0 + kk;
    double qx = node_coord(job.xmin, i, job.dx);
    double qy = node_coord(job.ymin, j, job.dy);
    double qz = d == 3 ? node_coord(job.zmin, k, job.dz) : 0.0;
    float fx = (float)__dmul_rn((double)(i - 1), job.dx);
    float fy = (float)__dmul_rn((double)(j - 1), job.dy);
    float fz = d == 3 ? (float)__dmul_rn((double)(k - 1), job.dz) : 0.f;
    float best32 = FLT_MAX;
    for (int p = 0; p < n; ++p) {
      float4 q = nuc[p];
      float ex = __fsub_rn(q.x, fx), ey = __fsub_rn(q.y, fy), ez = __fsub_rn(q.z, fz);
      float s = __fadd_rn(__fadd_rn(__fmul_rn(ex, ex), __fmul_rn(ey, ey)), __fmul_rn(ez, ez));
      best32 = fminf(best32, s);
    }
    const float thr = best32 + margin;
    double bsd = DBL_MAX, second = DBL_MAX;
    int bidx = -1;
    bool tie = false;
    for (int p = 0; p < n; ++p) {
      float4 q = nuc[p];
      float ex = __fsub_rn(q.x, fx), ey = __fsub_rn(q.y, fy), ez = __fsub_rn(q.z, fz);
      float s = __fadd_rn(__fadd_rn(__fmul_rn(ex, ex), __fmul_rn(ey, ey)), __fmul_rn(ez, ez));
      if (s > thr) continue;
      const double *pp = pts + (size_t)p * d;
      double dx = __dsub_rn(pp[0], qx), dy = __dsub_rn(pp[1], qy);
      double sd = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
      if (d == 3) { double dz = __dsub_rn(pp[2], qz); sd = __dadd_rn(sd, __dmul_rn(dz, dz)); }
      if (sd < bsd) { second = bsd; bsd = sd; bidx = p; }
      else if (sd < second) second = sd;
    }
    if (second <= bsd * (1.0 + 1e-13)) tie = true;
    size_t o = (size_t)c * nodes_total + (size_t)(k - 1) +
               (size_t)(d == 3 ? job.nz : 1) * ((size_t)(j - 1) + (size_t)job.ny * (i - 1));
    if (tie || bidx < 0) {
      int slot = atomicAdd(&job.tie_count[c], 1);
      job.tie_nodes[(size_t)c * nodes_total + slot] = (int)((size_t)o - (size_t)c * nodes_total);
      continue;
    }
    job.sites_id[o] = bidx + 1;
    if (job.vp) {
      job.vp[o] = par[(size_t)bidx * 3 + 0];
      job.vs[o] = par[(size_t)bidx * 3 + 1];
      job.rho[o] = par[(size_t)bidx * 3 + 2];
    }
  }
}

// One block per chain with queued tie nodes: build the chain's kd-tree once
// (thread 0) and resolve those nodes with the kdtree2 search.
__global__ void kd_resolve_kernel(GridJob job, size_t scratch_stride) {
  const int c = blockIdx.x;
  const int n = chain_cells(job, c);
  BoxIdx bx;
  if (n < 0 || !chain_box(job, c, bx)) return;   // skipped by grid_nearest_kernel
  const int cnt = job.tie_count[c];
  if (cnt == 0) return;
  const int d = job.d;
  char *base = static_cast<char *>(job.kd_scratch) + (size_t)c * scratch_stride;
  KdTree t;
  t.d = d; t.n = n;
  t.data = job.points + (size_t)c * job.ncell_max * d;
  t.ind = reinterpret_cast<int *>(base);
  t.rdata = reinterpret_cast<double *>(base + (((size_t)job.ncell_max * sizeof(int) + 255) & ~size_t(255)));
  t.nodes = reinterpret_cast<KdNode *>(reinterpret_cast<char *>(t.rdata) +
                                       (((size_t)job.ncell_max * 3 * sizeof(double) + 255) & ~size_t(255)));
  const int max_nodes = 2 * job.ncell_max + 16;
  __shared__ int s_ok, s_root, s_nn;
  if (threadIdx.x == 0) {
    for (int i = 0; i < n; ++i) t.ind[i] = i + 1;
    s_ok = kd_build(t, max_nodes) == 0;
    s_root = t.root; s_nn = t.nnodes;
  }
  __syncthreads();
  t.root = s_root; t.nnodes = s_nn;
  const double *par = job.params + (size_t)c * job.ncell_max * 3;
  const int nzz = d == 3 ? job.nz : 1;
  const long nodes_total = (long)job.nx * job.ny * nzz;
  for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
    int o = job.tie_nodes[(size_t)c * nodes_total + q];
    int k = o % nzz + 1;
    int rest = o / nzz;
    int j = rest % job.ny + 1;
    int i = rest / job.ny + 1;
    double qv[3] = {node_coord(job.xmin, i, job.dx), node_coord(job.ymin, j, job.dy),
                    d == 3 ? node_coord(job.zmin, k, job.dz) : 0.0};
    int err = 0;
    int idx = s_ok ? kd_nearest(t, qv, &err) : 0;
    size_t oo = (size_t)c * nodes_total + o;
    if (!s_ok || err || idx < 1) {
      // the kd-tree could not be built or searched (its depth exceeds the
      // fixed stacks): the node gets the documented failure value
      atomicExch(job.status, MCT_ERR_INTERNAL);
      job.sites_id[oo] = 0;
      if (job.vp) { job.vp[oo] = 0.0; job.vs[oo] = 0.0; job.rho[oo] = 0.0; }
      continue;
    }
    job.sites_id[oo] = idx;
    if (job.vp) {
      job.vp[oo] = par[(size_t)(idx - 1) * 3 + 0];
      job.vs[oo] = par[(size_t)(idx - 1) * 3 + 1];
      job.rho[oo] = par[(size_t)(idx - 1) * 3 + 2];
    }
  }
}

}  // namespace

size_t kd_scratch_bytes(int ncell_max) {
  size_t a = ((size_t)ncell_max * sizeof(int) + 255) & ~size_t(255);
  size_t b = ((size_t)ncell_max * 3 * sizeof(double) + 255) & ~size_t(255);
  size_t c = (size_t)(2 * ncell_max + 16) * sizeof(KdNode);
  return (a + b + c + 255) & ~size_t(255);
}

int launch_grid_nearest(const GridJob &job, cudaStream_t s) {
  if (job.nchains < 1 || job.ncell_max < 1 || (job.d != 2 && job.d != 3)) return MCT_ERR_ARG;
  size_t smem = (size_t)job.ncell_max * sizeof(float4);
  if (smem > 200 * 1024) return MCT_ERR_ARG;
  if (smem > 48 * 1024) {
    const int rc = mct_smem_attr(grid_nearest_kernel, 200 * 1024);
    if (rc) return rc;
  }
  long nodes = (long)job.nx * job.ny * (job.d == 3 ? job.nz : 1);
  MCT_CUDA_TRY(cudaMemsetAsync(job.tie_count, 0, sizeof(int) * job.nchains, s));
  int bx = (int)std::min<long>((nodes + GRID_THREADS - 1) / GRID_THREADS, 1024);
  dim3 grid(bx, job.nchains);
  grid_nearest_kernel<<<grid, GRID_THREADS, smem, s>>>(job);
  MCT_CUDA_TRY(cudaGetLastError());
  kd_resolve_kernel<<<job.nchains, 128, 0, s>>>(job, kd_scratch_bytes(job.ncell_max));
  MCT_CUDA_TRY(cudaGetLastError());
  fold_status_kernel<<<1, 1, 0, s>>>(job.status);
  MCT_CUDA_TRY(cudaGetLastError());
  return MCT_OK;
}

int grid_status_read(void *stream, int *status) {
  MCT_CUDA_TRY(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
  int st = 0;
  MCT_CUDA_TRY(cudaMemcpyFromSymbol(&st, g_grid_status, sizeof(int)));
  const int zero = 0;
  MCT_CUDA_TRY(cudaMemcpyToSymbol(g_grid_status, &zero, sizeof(int)));
  *status = st;
  return MCT_OK;
}
