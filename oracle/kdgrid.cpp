// ORACLE (test infrastructure only): CPU restatement of the kdtree2 nearest
// neighbour search (src/kdtree2.f90) and of kdtree_to_grid
// (src/mcmc_loc2.f90:2002-2082 for 3D, mcmc2d/mcmc.f90:1469-1525 for 2D),
// used as the parity checker for the GPU gridding kernel. Never linked into
// the product.
//
// Parity status: unpinned by reference execution (Fortran, no compiler on this
// image); pinned by brute-force nearest neighbour on tie-free inputs and by the
// tie rule of the restated search on constructed ties.
//
// The tie rule matters: kdtree2 replaces the current best whenever a later
// visited point has a squared distance <= the best (process_terminal_node,
// kdtree2.f90:1530-1592), so which of several equidistant nuclei wins depends
// on the tree's visiting order. The squared distance is summed over
// coordinates left to right without FMA (kdtree2.f90:1534-1538).
#include <cmath>
#include <vector>
#include <limits>
#include "oracle.h"

namespace {

const int BUCKET = 12;  // kdtree2.f90:516

struct Node {
  int cut_dim;
  double cut_val, cut_val_left, cut_val_right;
  int l, u;          // 1-based inclusive range into ind
  int left, right;   // child node ids, -1 = none
  double lo[3], hi[3];
};

struct Tree {
  int d, n;
  const double *data;   // data[(i-1)*d + k], i 1-based point index
  std::vector<int> ind; // 1-based permutation, ind[pos-1]
  std::vector<Node> nodes;
  std::vector<double> rdata;  // rearranged copy, rdata[(pos-1)*d + k]
  int root;
  double v(int c, int pos) const { return data[(ind[pos - 1] - 1) * d + c]; }
};

// kdtree2.f90:944-987 spread_in_coordinate (min/max are exact)
void spread(const Tree &t, int c, int l, int u, double &lo, double &hi) {
  double smin = t.v(c, l), smax = smin;
  for (int i = l + 1; i <= u; ++i) {
    double x = t.v(c, i);
    if (smin > x) smin = x;
    if (smax < x) smax = x;
  }
  lo = smin; hi = smax;
}

// kdtree2.f90:843-895 select_on_coordinate_value
int select_value(Tree &t, int c, double alpha, int li, int ui) {
  int lb = li, rb = ui;
  while (lb < rb) {
    if (t.v(c, lb) <= alpha) lb = lb + 1;
    else { std::swap(t.ind[lb - 1], t.ind[rb - 1]); rb = rb - 1; }
  }
  return (t.v(c, lb) <= alpha) ? lb : lb - 1;
}

// kdtree2.f90:704-840 build_tree_for_range
int build(Tree &t, int l, int u, int parent) {
  if (u < l) return -1;
  int id = (int)t.nodes.size();
  t.nodes.push_back(Node());
  Node res;
  res.left = res.right = -1;
  if ((u - l) <= BUCKET) {
    for (int i = 0; i < t.d; ++i) spread(t, i, l, u, res.lo[i], res.hi[i]);
    res.cut_dim = 0; res.cut_val = 0.0;
    res.cut_val_left = res.cut_val_right = 0.0;
    res.l = l; res.u = u;
    t.nodes[id] = res;
    return id;
  }
  for (int i = 0; i < t.d; ++i) {
    bool recompute = true;
    if (parent >= 0 && i != t.nodes[parent].cut_dim) recompute = false;
    if (recompute) spread(t, i, l, u, res.lo[i], res.hi[i]);
    else { res.lo[i] = t.nodes[parent].lo[i]; res.hi[i] = t.nodes[parent].hi[i]; }
  }
  int c = 0;
  double best = res.hi[0] - res.lo[0];
  for (int i = 1; i < t.d; ++i) {
    double s = res.hi[i] - res.lo[i];
    if (s > best) { best = s; c = i; }
  }
  double sum = 0.0;
  for (int i = l; i <= u; ++i) sum = sum + t.v(c, i);
  double average = sum / (double)(u - l + 1);
  res.cut_val = average;
  res.cut_val_left = res.cut_val_right = 0.0;
  int m = select_value(t, c, average, l, u);
  res.cut_dim = c; res.l = l; res.u = u;
  t.nodes[id] = res;   // children read this approximate box
  int left = build(t, l, m, id);
  int right = build(t, m + 1, u, id);
  Node &r = t.nodes[id];
  r.left = left; r.right = right;
  if (right < 0) {
    for (int i = 0; i < t.d; ++i) { r.lo[i] = t.nodes[left].lo[i]; r.hi[i] = t.nodes[left].hi[i]; }
    r.cut_val_left = t.nodes[left].hi[c];
    r.cut_val = r.cut_val_left;
  } else if (left < 0) {
    for (int i = 0; i < t.d; ++i) { r.lo[i] = t.nodes[right].lo[i]; r.hi[i] = t.nodes[right].hi[i]; }
    r.cut_val_right = t.nodes[right].lo[c];
    r.cut_val = r.cut_val_right;
  } else {
    r.cut_val_right = t.nodes[right].lo[c];
    r.cut_val_left = t.nodes[left].hi[c];
    r.cut_val = (r.cut_val_left + r.cut_val_right) / 2;
    for (int i = 0; i < t.d; ++i) {
      r.hi[i] = std::fmax(t.nodes[left].hi[i], t.nodes[right].hi[i]);
      r.lo[i] = std::fmin(t.nodes[left].lo[i], t.nodes[right].lo[i]);
    }
  }
  return id;
}

void create(Tree &t, const double *pts, int d, int n) {
  t.d = d; t.n = n; t.data = pts;
  t.ind.resize(n);
  for (int j = 0; j < n; ++j) t.ind[j] = j + 1;
  t.nodes.clear();
  t.nodes.reserve(2 * n / BUCKET + 8);
  t.root = build(t, 1, n, -1);
  t.rdata.resize((size_t)n * d);
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < d; ++k) t.rdata[(size_t)i * d + k] = pts[(size_t)(t.ind[i] - 1) * d + k];
}

struct Search {
  const Tree *t;
  const double *qv;
  double ballsize;
  int nfound;
  int best_idx;
};

inline double dis2_from_bnd(double x, double amin, double amax) {
  if (x > amax) return (x - amax) * (x - amax);
  if (x < amin) return (amin - x) * (amin - x);
  return 0.0;
}

// kdtree2.f90:1496-1599 process_terminal_node for nn = 1
void terminal(Search &s, const Node &node) {
  const Tree &t = *s.t;
  double ballsize = s.ballsize;
  for (int i = node.l; i <= node.u; ++i) {
    double sd = 0.0;
    bool skip = false;
    for (int k = 0; k < t.d; ++k) {
      double df = t.rdata[(size_t)(i - 1) * t.d + k] - s.qv[k];
      sd = sd + df * df;
      if (sd > ballsize) { skip = true; break; }
    }
    if (skip) continue;
    int indexofi = t.ind[i - 1];
    if (s.nfound < 1) {
      s.nfound = 1;
      s.best_idx = indexofi;
      ballsize = sd;
    } else {
      s.best_idx = indexofi;   // pq_replace_max with a one-element queue
      ballsize = sd;
    }
  }
  s.ballsize = ballsize;
}

// kdtree2.f90:1369-1443 search
void search(Search &s, int nid) {
  const Tree &t = *s.t;
  const Node &node = t.nodes[nid];
  if (!(node.left >= 0 && node.right >= 0)) { terminal(s, node); return; }
  int cut_dim = node.cut_dim;
  double qval = s.qv[cut_dim];
  int ncloser, nfarther;
  double dis;
  if (qval < node.cut_val) {
    ncloser = node.left; nfarther = node.right;
    dis = (node.cut_val_right - qval) * (node.cut_val_right - qval);
  } else {
    ncloser = node.right; nfarther = node.left;
    dis = (node.cut_val_left - qval) * (node.cut_val_left - qval);
  }
  if (ncloser >= 0) search(s, ncloser);
  if (nfarther >= 0) {
    double ballsize = s.ballsize;
    if (dis <= ballsize) {
      for (int i = 0; i < t.d; ++i) {
        if (i != cut_dim) {
          dis = dis + dis2_from_bnd(s.qv[i], node.lo[i], node.hi[i]);
          if (dis > ballsize) return;
        }
      }
      search(s, nfarther);
    }
  }
}

int nearest(const Tree &t, const double *qv) {
  Search s;
  s.t = &t; s.qv = qv;
  s.ballsize = (double)std::numeric_limits<float>::max();  // huge(1.0)
  s.nfound = 0; s.best_idx = 0;
  search(s, t.root);
  return s.best_idx;
}

}  // namespace

extern "C" {

// kdtree_to_grid for one chain. points: (d, n) column-major (Fortran
// RTI%points(:,1:ncells)); params: (3, n) = vp, vs, rho per nucleus.
// Box indices are 1-based inclusive, already clamped to the grid.
// sites_id/vp/vs/rho: Fortran (nz,ny,nx) for d=3, (ny,nx) for d=2.
// Nodes outside the box are left untouched.
int orc_kdtree_to_grid(int d, int n, const double *points, const double *params,
                       int nx, int ny, int nz, double xmin, double ymin,
                       double zmin, double dx, double dy, double dz, int ix0,
                       int ix1, int iy0, int iy1, int iz0, int iz1,
                       int *sites_id, double *vp, double *vs, double *rho) {
  if (n < 1 || (d != 2 && d != 3)) return -1;
  Tree t;
  create(t, points, d, n);
  if (d == 2) { nz = 1; iz0 = iz1 = 1; }
  double qv[3];
  for (int i = ix0; i <= ix1; ++i)
    for (int j = iy0; j <= iy1; ++j)
      for (int k = iz0; k <= iz1; ++k) {
        qv[0] = xmin + (double)(i - 1) * dx;
        qv[1] = ymin + (double)(j - 1) * dy;
        qv[2] = zmin + (double)(k - 1) * dz;
        int idx = nearest(t, qv);
        size_t o = (size_t)(k - 1) + (size_t)nz * ((size_t)(j - 1) + (size_t)ny * (i - 1));
        sites_id[o] = idx;
        vp[o] = params[3 * (idx - 1) + 0];
        vs[o] = params[3 * (idx - 1) + 1];
        rho[o] = params[3 * (idx - 1) + 2];
      }
  return 0;
}

// Single nearest-nucleus query (1-based index), for tests.
int orc_kdtree_nearest(int d, int n, const double *points, const double *qv) {
  Tree t;
  create(t, points, d, n);
  return nearest(t, qv);
}

}  // extern "C"
