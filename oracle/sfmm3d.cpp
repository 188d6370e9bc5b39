// ORACLE (test infrastructure only): CPU restatement of the reference's 3D
// eikonal entry point fastMarching3D (fastmarching/fastMarching.cpp:26-129):
// SFMM = FMM with a std::priority_queue-style binary heap that re-pushes on
// improvement (fmm/fmm.hpp:92-158, fmm/fmdata/fmpriorityqueue.hpp:23-88),
// first-order solveEikonal / mixed second-order highAccuracySolveEikonal
// (fmm/eikonalsolver.hpp:50-145,292-368), 8-corner source initialisation
// (fmm/solver.hpp:72-107) and trilinear receiver read-out
// (ndgridmap/ndgridmap.hpp:158-191,433-490). Used as the parity checker for
// the GPU 3D eikonal kernel and as the timed CPU baseline on hosts where the
// reference itself is not compiled. Never linked into the product.
//
// Parity status: PINNED. tests/ compare this restatement bit-for-bit with the
// reference's own fastMarching3D compiled from its sources (oracle/_ref) on
// random media, in this container.
//
// The heap holds cell indices and compares the cells' live arrival times
// (FMCompare reads getTotalValue() at comparison time), so a decreased key
// leaves a stale entry in place. The push/pop steps reproduce libstdc++'s
// std::push_heap / std::pop_heap (hole-moving sift with "larger child wins"),
// which boost::heap::priority_queue delegates to.
#include <cmath>
#include <vector>
#include <limits>
#include <algorithm>
#include "oracle.h"

namespace {

const double COMP_MARGIN = std::numeric_limits<double>::epsilon() * 1e5;
const unsigned UMAX = std::numeric_limits<unsigned>::max();
const double INF = std::numeric_limits<double>::infinity();
const double DMAX = std::numeric_limits<double>::max();

enum State : unsigned char { OPEN = 0, NARROW = 1, FROZEN = 2 };

struct Grid {
  unsigned nx, ny, nz, n;
  unsigned d[3];   // d_[0]=nx, d_[1]=nx*ny, d_[2]=nx*ny*nz
  double h[3];
  std::vector<double> vel, t;
  std::vector<unsigned char> st;
};

// ---- libstdc++ heap algorithm on a vector of cell ids ------------------
// comp(a, b) == "a has lower priority than b" == t[a] > t[b]  (min-heap)
struct Heap {
  std::vector<unsigned> c;
  const std::vector<double> *t;
  bool comp(unsigned a, unsigned b) const { return (*t)[a] > (*t)[b]; }
  void push_up(long hole, long top, unsigned value) {
    long parent = (hole - 1) / 2;
    while (hole > top && comp(c[parent], value)) {
      c[hole] = c[parent];
      hole = parent;
      parent = (hole - 1) / 2;
    }
    c[hole] = value;
  }
  void push(unsigned v) {
    c.push_back(v);
    push_up((long)c.size() - 1, 0, v);
  }
  void adjust(long hole, long len, unsigned value) {
    const long top = hole;
    long second = hole;
    while (second < (len - 1) / 2) {
      second = 2 * (second + 1);
      if (comp(c[second], c[second - 1])) second--;
      c[hole] = c[second];
      hole = second;
    }
    if ((len & 1) == 0 && second == (len - 2) / 2) {
      second = 2 * (second + 1);
      c[hole] = c[second - 1];
      hole = second - 1;
    }
    push_up(hole, top, value);
  }
  unsigned pop() {
    unsigned top = c[0];
    long n = (long)c.size();
    if (n > 1) {
      unsigned value = c[n - 1];
      c[n - 1] = c[0];
      adjust(0, n - 1, value);
    }
    c.pop_back();
    return top;
  }
};

// ndgridmap.hpp getNeighborsInDim (4-connectivity pair in one dimension)
inline int neigh_in_dim(const Grid &g, unsigned idx, unsigned dim, unsigned out[2]) {
  unsigned c1, c2;
  if (dim == 0) { c1 = idx - 1; c2 = idx + 1; }
  else { c1 = idx - g.d[dim - 1]; c2 = idx + g.d[dim - 1]; }
  int n = 0;
  if (c1 / g.d[dim] == idx / g.d[dim]) out[n++] = c1;
  if (c2 / g.d[dim] == idx / g.d[dim]) out[n++] = c2;
  return n;
}

// ndgridmap.hpp getNeighborsInDim (pairs: 1 and 2 steps away)
inline void neigh2_in_dim(const Grid &g, unsigned idx, unsigned dim, unsigned o[4]) {
  unsigned c1a, c1b, c2a, c2b;
  if (dim == 0) { c1a = idx - 1; c1b = c1a - 1; c2a = idx + 1; c2b = c2a + 1; }
  else {
    c1a = idx - g.d[dim - 1]; c1b = c1a - g.d[dim - 1];
    c2a = idx + g.d[dim - 1]; c2b = c2a + g.d[dim - 1];
  }
  if (!(c1a / g.d[dim] == idx / g.d[dim])) c1a = UMAX;
  if (!(c1b / g.d[dim] == idx / g.d[dim])) c1b = UMAX;
  if (c2a >= g.n || c2a / g.d[dim] != idx / g.d[dim]) c2a = UMAX;
  if (c2b >= g.n || c2b / g.d[dim] != idx / g.d[dim]) c2b = UMAX;
  o[0] = c1a; o[1] = c1b; o[2] = c2a; o[3] = c2b;
}

inline double min_value_in_dim(const Grid &g, unsigned idx, unsigned dim) {
  unsigned nb[2];
  int n = neigh_in_dim(g, idx, dim, nb);
  if (n == 1) return g.t[nb[0]];
  return (g.t[nb[0]] < g.t[nb[1]]) ? g.t[nb[0]] : g.t[nb[1]];
}

// eikonalsolver.hpp:50-80 solveEikonal (first order)
double solve_first(const Grid &g, unsigned idx) {
  double tv[3]; unsigned td[3]; unsigned a = 3, cnt = 0;
  for (unsigned dim = 0; dim < 3; ++dim) {
    double m = min_value_in_dim(g, idx, dim);
    if (!std::isinf(m) && m < g.t[idx]) { tv[cnt] = m; td[cnt] = dim; cnt++; }
    else a -= 1;
  }
  if (a == 0) return INF;
  // std::sort of <= 3 elements is an insertion sort (stable for equal keys)
  for (unsigned i = 1; i < cnt; ++i) {
    double v = tv[i]; unsigned dd = td[i]; unsigned j = i;
    if (v < tv[0]) {
      for (; j > 0; --j) { tv[j] = tv[j - 1]; td[j] = td[j - 1]; }
    } else {
      while (v < tv[j - 1]) { tv[j] = tv[j - 1]; td[j] = td[j - 1]; --j; }
    }
    tv[j] = v; td[j] = dd;
  }
  double vel = g.vel[idx];
  double updated = 0;
  for (unsigned i = 1; i <= a; ++i) {
    if (i == 1) {
      updated = tv[0] + g.h[td[0]] / vel;
    } else {
      double A = 0.0, B = 0.0, C = -1.0 / (vel * vel);
      for (unsigned q = 0; q < i; ++q) {
        double alpha = 1.0 / (g.h[td[q]] * g.h[td[q]]);
        C += tv[q] * tv[q] * alpha;
        B += -2.0 * tv[q] * alpha;
        A += alpha;
      }
      double quad = B * B - 4 * A * C;
      updated = (quad < 0) ? INF : (-B + std::sqrt(quad)) / (2 * A);
    }
    if (i == a || (updated - tv[i]) < COMP_MARGIN) break;
  }
  return updated;
}

// eikonalsolver.hpp:83-145 highAccuracySolveEikonal (mixed second order)
double solve_high(const Grid &g, unsigned idx) {
  double t1[3], t2[3]; unsigned td[3]; unsigned a = 3, cnt = 0;
  double cur = g.t[idx];
  for (unsigned dim = 0; dim < 3; ++dim) {
    unsigned nb[4];
    neigh2_in_dim(g, idx, dim, nb);
    double minT = DMAX, minT2 = DMAX;
    for (int s = 0; s < 2; ++s) {
      unsigned first = nb[2 * s], second = nb[2 * s + 1];
      if (first < UMAX) {
        double tvalue = g.t[first];
        if (!std::isinf(tvalue) && tvalue < minT) {
          minT = tvalue;
          minT2 = DMAX;
          if (second < UMAX) {
            double tvalue2 = g.t[second];
            if (!std::isinf(tvalue2) && tvalue2 <= tvalue) minT2 = tvalue2;
          }
        }
      }
    }
    if (minT2 < DMAX && minT < cur) { t1[cnt] = minT; t2[cnt] = minT2; td[cnt] = dim; cnt++; }
    else if (minT < DMAX && minT < cur) { t1[cnt] = minT; t2[cnt] = INF; td[cnt] = dim; cnt++; }
    else a -= 1;
  }
  if (a == 0) return cur;
  for (unsigned i = 1; i < cnt; ++i) {
    double v = t1[i], v2 = t2[i]; unsigned dd = td[i]; unsigned j = i;
    if (v < t1[0]) {
      for (; j > 0; --j) { t1[j] = t1[j - 1]; t2[j] = t2[j - 1]; td[j] = td[j - 1]; }
    } else {
      while (v < t1[j - 1]) { t1[j] = t1[j - 1]; t2[j] = t2[j - 1]; td[j] = td[j - 1]; --j; }
    }
    t1[j] = v; t2[j] = v2; td[j] = dd;
  }
  double vel = g.vel[idx];
  double updated = INF;
  for (unsigned i = a; i >= 1; --i) {
    double cand;
    if (i == 1) {
      cand = t1[0] + g.h[td[0]] / vel;
    } else {
      double A = 0.0, B = 0.0, C = -1.0 / (vel * vel);
      for (unsigned q = 0; q < i; ++q) {
        double hj = g.h[td[q]];
        if (!std::isinf(t2[q])) {
          double alpha = 9.0 / 4.0 / (hj * hj);
          double tt = (4.0 * t1[q] - t2[q]) / 3.0;
          C += tt * tt * alpha;
          B += -2.0 * tt * alpha;
          A += alpha;
        } else if (t1[q] < DMAX) {
          double alpha = 1.0 / (hj * hj);
          C += t1[q] * t1[q] * alpha;
          B += -2.0 * t1[q] * alpha;
          A += alpha;
        }
      }
      double quad = B * B - 4 * A * C;
      cand = (quad < 0) ? INF : (-B + std::sqrt(quad)) / (2 * A);
    }
    if (!std::isinf(cand) && (cand - t1[i - 1]) > COMP_MARGIN) { updated = cand; break; }
  }
  return updated;
}

inline void idx2coord(const Grid &g, unsigned idx, unsigned c[3]) {
  c[2] = idx / g.d[1];
  unsigned aux = idx - c[2] * g.d[1];
  c[1] = aux / g.d[0];
  aux -= c[1] * g.d[0];
  c[0] = aux;
}

inline void point_coord(const Grid &g, const double p[3], unsigned c[3]) {
  unsigned dims[3] = {g.nx, g.ny, g.nz};
  for (int k = 0; k < 3; ++k) {
    int ci = (int)(p[k] / g.h[k]);
    if (ci < 0) ci = 0;
    else if (ci >= (int)dims[k]) ci = (int)dims[k] - 1;
    c[k] = (unsigned)ci;
  }
}

inline void corners(const Grid &g, const double p[3], unsigned nb[8]) {
  unsigned c[3];
  point_coord(g, p, c);
  unsigned dims[3] = {g.nx, g.ny, g.nz};
  for (int v = 0; v < 8; ++v) {
    unsigned vc[3];
    for (int dim = 0; dim < 3; ++dim) {
      unsigned vi = (v >> (3 - dim - 1)) & 1;
      vc[dim] = c[dim] + vi;
      if (vc[dim] >= dims[dim]) vc[dim] = dims[dim] - 1;
    }
    nb[v] = vc[0] + vc[1] * g.d[0] + vc[2] * g.d[1];
  }
}

// ndgridmap.hpp getVel/getTime: trilinear with the max-face clamp quirk
double trilinear(const Grid &g, const double p[3], const std::vector<double> &f) {
  unsigned pc[3];
  point_coord(g, p, pc);
  unsigned nb[8];
  corners(g, p, nb);
  double acc = 0;
  for (int i = 0; i < 8; ++i) {
    unsigned c[3];
    idx2coord(g, nb[i], c);
    double w = 1.0;
    for (int j = 0; j < 3; ++j) {
      unsigned di = c[j] - pc[j];
      double s = p[j] - g.h[j] * pc[j];
      double wj = std::fabs(di * g.h[j] - g.h[j] + s);
      w = w * wj / g.h[j];
    }
    acc = acc + w * f[nb[i]];
  }
  return acc;
}

}  // namespace

extern "C" {

// Same contract as the reference's fastMarching3D, returning 0; -1 when a
// computed arrival time is infinite (where the reference asserts).
int orc_fast_marching3d(int nx, int ny, int nz, double dx, double dy, double dz,
                        double xmin, double ymin, double zmin, const double *vel,
                        const double *src, const double *rev, int nrev,
                        int order, double *ttime, double *tfield) {
  Grid g;
  g.nx = nx; g.ny = ny; g.nz = nz; g.n = (unsigned)nx * ny * nz;
  g.d[0] = nx; g.d[1] = nx * ny; g.d[2] = g.n;
  g.h[0] = dx; g.h[1] = dy; g.h[2] = dz;
  g.vel.resize(g.n); g.t.assign(g.n, INF); g.st.assign(g.n, OPEN);
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j < ny; ++j)
      for (int k = 0; k < nz; ++k)
        g.vel[i + j * nx + k * nx * ny] = vel[((size_t)i * ny + j) * nz + k];
  double sp[3] = {src[0] - xmin, src[1] - ymin, src[2] - zmin};
  // solver.hpp:72-92 setInitialPoints
  double v = trilinear(g, sp, g.vel);
  unsigned nb[8];
  corners(g, sp, nb);
  double it[8];
  for (int i = 0; i < 8; ++i) {
    unsigned c[3];
    idx2coord(g, nb[i], c);
    double dist = 0;
    for (int k = 0; k < 3; ++k) {
      double pk = c[k] * g.h[k];
      double xi = (pk - sp[k]) * (pk - sp[k]);
      dist = dist + xi;
    }
    dist = std::sqrt(dist);
    it[i] = dist * 2 / (v + g.vel[nb[i]]);
  }
  Heap heap; heap.t = &g.t; heap.c.reserve(g.n);
  for (int i = 0; i < 8; ++i) {
    g.t[nb[i]] = it[i];
    g.st[nb[i]] = NARROW;
    heap.push(nb[i]);
  }
  bool high = (order == 1);
  int status = 0;
  while (!heap.c.empty()) {
    unsigned idxMin = heap.pop();
    unsigned nbs[6]; int nn = 0;
    for (unsigned dim = 0; dim < 3; ++dim) {
      unsigned o[2]; int m = neigh_in_dim(g, idxMin, dim, o);
      for (int q = 0; q < m; ++q) nbs[nn++] = o[q];
    }
    g.st[idxMin] = FROZEN;
    if (std::isinf(g.t[idxMin])) status = -1;
    for (int s = 0; s < nn; ++s) {
      unsigned j = nbs[s];
      if (g.st[j] == FROZEN || g.vel[j] < COMP_MARGIN) continue;
      double nt = high ? solve_high(g, j) : solve_first(g, j);
      if (g.st[j] == NARROW) {
        if (nt + COMP_MARGIN < g.t[j]) { g.t[j] = nt; heap.push(j); }
      } else {
        g.st[j] = NARROW; g.t[j] = nt; heap.push(j);
      }
    }
  }
  for (int i = 0; i < nrev; ++i) {
    double goal[3] = {rev[3 * i] - xmin, rev[3 * i + 1] - ymin, rev[3 * i + 2] - zmin};
    ttime[i] = trilinear(g, goal, g.t);
  }
  if (tfield) {
    for (int i = 0; i < nx; ++i)
      for (int j = 0; j < ny; ++j)
        for (int k = 0; k < nz; ++k)
          tfield[((size_t)i * ny + j) * nz + k] = g.t[i + j * nx + k * nx * ny];
  }
  return status;
}

}  // extern "C"
