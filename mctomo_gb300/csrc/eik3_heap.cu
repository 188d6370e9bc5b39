// Exact 3D heap march: the reference's fastMarching3D
// (fastmarching/fastMarching.cpp:26-129) run step for step on the GPU, so
// that its results are the reference's bit for bit, for the first-order and
// the mixed second-order scheme alike.
//
// The reference's solver is SFMM (fmm/fmm.hpp:92-158): a binary heap of
// node indices that compares the nodes' live arrival times
// (fmm/fmdata/fmpriorityqueue.hpp:23-88 over boost::heap, whose push/pop are
// libstdc++'s push_heap/pop_heap: hole-moving sifts, the larger child wins
// ties), re-pushes a node when its time improves by more than COMP_MARGIN
// (fmm/utils/utils.h:27-34) and leaves the old entry in place (its key is
// the node's live time, so it moves with the improvement), and freezes
// whatever it pops, stale entries included. The mixed second-order update
// (fmm/eikonalsolver.hpp:83-145) reads every finite neighbour, frozen or
// not, so the result depends on the order in which nodes are accepted; only
// the same sequence of pops, with the same floating-point operations, gives
// the same times. That sequence is inherently serial, so here the
// parallelism is across solves: one group of G lanes marches one solve, and
// the lanes of a group share the work of each step:
//
//  * pop: the hole-moving sift-down needs, per level, the two children's
//    node indices and then their times (two dependent loads). The G lanes
//    fetch a whole subtree of depth log2(G) below the hole at once (indices,
//    then times: two memory round trips for log2(G) levels), and the group
//    leader walks it in shared memory. The final sift-up of the moved last
//    element runs along the path just walked, whose entries are known.
//  * update: lanes 0..5 take the six neighbours of the popped node (x-, x+,
//    y-, y+, z-, z+), load their whole stencils (up to 12 times, state,
//    velocity) in one round trip and evaluate the reference's update in
//    FP64 with its exact operation order. Neighbours on different axes do
//    not read each other; the + neighbour of an axis can read the -
//    neighbour (two steps away in the second-order stencil), so it is
//    evaluated again with the new value in the rare case that value enters
//    its stencil (it is at most the popped time).
//  * accept: the leader applies the results in the reference's order (write
//    the time, then push, for each neighbour in turn), so every comparison
//    in every push sees exactly the live times the reference's push sees.
//
// Comparisons between times are integer comparisons of the IEEE bit
// patterns (all times are >= 0 or +inf), which are exact and keep them off
// the FP64 pipe; the arithmetic of the update is the reference's, FP64,
// without contraction (the library is built with -fmad=false).
//
// Loops are bounded: the march stops with an error bit after 8 * nodes
// pops (every pop matches one push; a node is pushed once when reached and
// again per improvement, a handful of times at most), and a push beyond
// the heap capacity stops that solve with an error bit; no lane waits on
// another lane outside __syncwarp.
#include "mct_common.cuh"
#include "eikonal3d.cuh"
#include "eik3_common.cuh"
#include <cfloat>
#include <climits>
#include <string>

namespace {

constexpr double kMargin = DBL_EPSILON * 1e5;   // COMP_MARGIN
constexpr unsigned char kOpen = 0, kNarrow = 1, kFrozen = 2;
constexpr long long kInfBits = 0x7FF0000000000000LL;
constexpr int kBlock = 128;
constexpr int kMaxDepth = 33;
constexpr unsigned kFull = 0xffffffffu;

enum HeapErr { HERR_INF = 1, HERR_OVERFLOW = 2, HERR_STEPS = 4, HERR_INDEX = 8 };

// Non-negative doubles (and +inf) order like their bit patterns.
__device__ __forceinline__ long long bits(double x) { return __double_as_longlong(x); }
__device__ __forceinline__ bool is_inf(double x) { return bits(x) == kInfBits; }
__device__ __forceinline__ bool lt(double a, double b) { return bits(a) < bits(b); }
__device__ __forceinline__ bool le(double a, double b) { return bits(a) <= bits(b); }
__device__ __forceinline__ bool gt(double a, double b) { return bits(a) > bits(b); }

// Constants of the update per axis: h, 1/h^2 and 9/4/h^2 (the reference
// evaluates 1.0/(h*h) and 9.0/4.0/(h*h) in place; same values).
struct Axes {
  double h[3], a1[3], a2[3];
};

__device__ __forceinline__ double sel3(const double v[3], int i) { return i == 0 ? v[0] : (i == 1 ? v[1] : v[2]); }
__device__ __forceinline__ int seli(const int v[3], int i) { return i == 0 ? v[0] : (i == 1 ? v[1] : v[2]); }

// The stencil of a node: times at -1, -2, +1, +2 along each axis, which of
// them exist, and the node's own time.
struct Stencil {
  double v[3][4];
  unsigned pres;   // bit 4*axis + slot
  double cur;
};

// Stable sort of three (t1, t2, axis) slots by t1 (std::sort of <= 3
// elements is an insertion sort: equal times keep axis order); unused slots
// hold +inf and sort last.
__device__ __forceinline__ void sort3(double t1[3], double t2[3], int dm[3]) {
  auto cswap = [&](int i, int j) {
    if (lt(t1[j], t1[i])) {
      double v = t1[i]; t1[i] = t1[j]; t1[j] = v;
      v = t2[i]; t2[i] = t2[j]; t2[j] = v;
      int w = dm[i]; dm[i] = dm[j]; dm[j] = w;
    }
  };
  cswap(0, 1); cswap(1, 2); cswap(0, 1);
}

// solveEikonal (fmm/eikonalsolver.hpp:50-80): first order.
__device__ double solve_first(const Stencil &S, double vel, double nis, const Axes &ax) {
  double tv[3]; double dummy[3]; int dm[3];
  int cnt = 0;
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    // getMinValueInDim: the one neighbour, or (v0 < v1) ? v0 : v1
    const bool p0 = (S.pres >> (4 * e)) & 1, p1 = (S.pres >> (4 * e + 2)) & 1;
    double m;
    if (p0 && p1) m = lt(S.v[e][0], S.v[e][2]) ? S.v[e][0] : S.v[e][2];
    else m = p0 ? S.v[e][0] : S.v[e][2];
    const bool use = !is_inf(m) && lt(m, S.cur);
    tv[e] = use ? m : __longlong_as_double(kInfBits);
    dummy[e] = 0.0;
    dm[e] = e;
    cnt += use ? 1 : 0;
  }
  if (cnt == 0) return __longlong_as_double(kInfBits);
  sort3(tv, dummy, dm);
  // prefix sums of the quadratic's terms, in the reference's order
  double A = 0.0, B = 0.0, C = nis;
  double updated = 0.0;
  bool done = false;
#pragma unroll
  for (int i = 1; i <= 3; ++i) {
    if (done || i > cnt) continue;
    const double alpha = sel3(ax.a1, dm[i - 1]);
    C += tv[i - 1] * tv[i - 1] * alpha;
    B += -2.0 * tv[i - 1] * alpha;
    A += alpha;
    if (i == 1) {
      updated = tv[0] + sel3(ax.h, dm[0]) / vel;
    } else {
      const double quad = B * B - 4 * A * C;
      updated = (quad < 0) ? __longlong_as_double(kInfBits) : (-B + sqrt(quad)) / (2 * A);
    }
    if (i == cnt) done = true;
    else if ((updated - tv[i < 3 ? i : 2]) < kMargin) done = true;
  }
  return updated;
}

// highAccuracySolveEikonal (fmm/eikonalsolver.hpp:83-145): mixed second
// order, the largest number of axes first.
__device__ double solve_high(const Stencil &S, double vel, double nis, const Axes &ax) {
  const double INF = __longlong_as_double(kInfBits);
  double t1[3], t2[3]; int dm[3];
  int cnt = 0;
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    double minT = DBL_MAX, minT2 = DBL_MAX;
#pragma unroll
    for (int sd = 0; sd < 2; ++sd) {
      const bool pf = (S.pres >> (4 * e + 2 * sd)) & 1, ps = (S.pres >> (4 * e + 2 * sd + 1)) & 1;
      if (pf) {
        const double tval = S.v[e][2 * sd];
        if (!is_inf(tval) && lt(tval, minT)) {
          minT = tval;
          minT2 = DBL_MAX;
          if (ps) {
            const double tval2 = S.v[e][2 * sd + 1];
            if (!is_inf(tval2) && le(tval2, tval)) minT2 = tval2;
          }
        }
      }
    }
    bool use = false;
    double u1 = INF, u2 = INF;
    if (lt(minT2, DBL_MAX) && lt(minT, S.cur)) { use = true; u1 = minT; u2 = minT2; }
    else if (lt(minT, DBL_MAX) && lt(minT, S.cur)) { use = true; u1 = minT; u2 = INF; }
    t1[e] = u1; t2[e] = u2; dm[e] = e;
    cnt += use ? 1 : 0;
  }
  if (cnt == 0) return S.cur;
  sort3(t1, t2, dm);
  // per-slot terms (identical for every candidate that includes the slot)
  double cC[3], cB[3], cA[3];
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    cC[q] = 0.0; cB[q] = 0.0; cA[q] = 0.0;
    if (q >= cnt) continue;
    if (!is_inf(t2[q])) {
      const double alpha = sel3(ax.a2, dm[q]);
      const double tt = (4.0 * t1[q] - t2[q]) / 3.0;
      cC[q] = tt * tt * alpha; cB[q] = -2.0 * tt * alpha; cA[q] = alpha;
    } else {
      const double alpha = sel3(ax.a1, dm[q]);
      cC[q] = t1[q] * t1[q] * alpha; cB[q] = -2.0 * t1[q] * alpha; cA[q] = alpha;
    }
  }
  // the candidate with i axes uses the sums over slots 0..i-1
  double Cs[3], Bs[3], As[3];
  {
    double A = 0.0, B = 0.0, C = nis;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      C += cC[q]; B += cB[q]; A += cA[q];
      Cs[q] = C; Bs[q] = B; As[q] = A;
    }
  }
  double updated = INF;
  bool done = false;
#pragma unroll
  for (int i = 3; i >= 1; --i) {
    if (done || i > cnt) continue;
    double cand;
    if (i == 1) {
      cand = t1[0] + sel3(ax.h, dm[0]) / vel;
    } else {
      const double A = As[i - 1], B = Bs[i - 1], C = Cs[i - 1];
      const double quad = B * B - 4 * A * C;
      cand = (quad < 0) ? INF : (-B + sqrt(quad)) / (2 * A);
    }
    if (!is_inf(cand) && (cand - t1[i - 1]) > kMargin) { updated = cand; done = true; }
  }
  return updated;
}

template <int G>
struct alignas(16) GroupSmem {
  // subtree below the hole: entries 0..2G-3 by level
  unsigned sub_id[2 * G];
  double sub_t[2 * G];
  // sift-down path: position, node and time of each element moved up
  unsigned path_pos[kMaxDepth];
  unsigned path_id[kMaxDepth];
  double path_t[kMaxDepth];
  // neighbour results
  double nb_t[6];
  unsigned nb_j[6];
  int nb_act[6];          // 0 none, 1 OPEN -> NARROW, 2 improved
  // walk state
  unsigned size, len, hole, second, sub_root, top, val;
  double ttop, tval;
  int lv, depth, need, active;
};

template <int G>
struct Lg { static constexpr int value = G == 8 ? 3 : (G == 16 ? 4 : 5); };

// One group of G lanes per solve; kBlock / G solves per block.
template <int G>
__global__ void __launch_bounds__(kBlock) heap_march_kernel(Eik3Job job, int s0, int nsol) {
  // at least six lanes: one per neighbour in the update step
  static_assert(G == 8 || G == 16 || G == 32, "group size");
  constexpr int D = Lg<G>::value;          // subtree levels fetched per round trip
  constexpr int E = 2 * G - 2;             // subtree entries
  __shared__ GroupSmem<G> sm_all[kBlock / G];
  const int gi = threadIdx.x / G, gl = threadIdx.x % G;
  GroupSmem<G> &sm = sm_all[gi];
  const int sl = blockIdx.x * (kBlock / G) + gi;          // solve within the chunk
  const bool live = sl < nsol;
  const int s = s0 + (live ? sl : 0);
  const E3Dims d{job.nx, job.ny, job.nz};
  const unsigned n = (unsigned)job.nx * job.ny * job.nz;
  const int strideA[3] = {job.ny * job.nz, job.nz, 1};
  const int dimA[3] = {job.nx, job.ny, job.nz};
  double *t = job.ht + (size_t)(live ? sl : 0) * n;
  unsigned char *st = job.hst + (size_t)(live ? sl : 0) * n;
  unsigned *heap = job.hheap + (size_t)(live ? sl : 0) * job.hcap;
  const double2 *vn = job.hvn + (size_t)job.solve_grid[s] * n;
  Axes ax;
  {
    const double h[3] = {job.dx, job.dy, job.dz};
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      ax.h[q] = h[q];
      ax.a1[q] = 1.0 / (h[q] * h[q]);
      ax.a2[q] = 9.0 / 4.0 / (h[q] * h[q]);
    }
  }
  const bool high = job.order == 1;
  int err = 0;

  // ---- source: 8 corners with times dist*2/(v_src + v_corner), pushed in
  // corner order (solver.hpp:72-92 setInitialPoints, fmm.hpp:103-115)
  if (gl == 0) {
    sm.size = 0; sm.active = live ? 1 : 0;
    if (live) {
      const double hh[3] = {job.dx, job.dy, job.dz};
      const double sp[3] = {job.src[3 * s], job.src[3 * s + 1], job.src[3 * s + 2]};
      auto vget = [&](int i, int j, int k) { return vn[e3_nidx(d, i, j, k)].x; };
      const double v = e3_trilinear(d, hh, sp, vget);
      int pc[3];
      e3_point_cell(d, hh, sp, pc);
      unsigned size = 0;
      for (int c = 0; c < 8; ++c) {
        int vc[3];
        e3_corner(d, pc, c, vc);
        double dist = 0;
        for (int q = 0; q < 3; ++q) {
          const double pk = (double)(unsigned)vc[q] * hh[q];
          const double xi = (pk - sp[q]) * (pk - sp[q]);
          dist = dist + xi;
        }
        dist = sqrt(dist);
        const unsigned id = (unsigned)e3_nidx(d, vc[0], vc[1], vc[2]);
        const double tv = dist * 2 / (v + vn[id].x);
        t[id] = tv;
        st[id] = kNarrow;
        // push_heap
        unsigned hole = size++;
        while (hole > 0) {
          const unsigned parent = (hole - 1) / 2;
          const unsigned pid = heap[parent];
          if (!gt(t[pid], tv)) break;
          heap[hole] = pid;
          hole = parent;
        }
        heap[hole] = id;
      }
      sm.size = size;
    }
  }
  __syncwarp();

  const long long max_pops = 8LL * n + 64;
  for (long long it = 0;; ++it) {
    // ---------------- pop: start the walk at the root
    if (gl == 0 && sm.active) {
      if (sm.size == 0 || it >= max_pops) {
        if (sm.size != 0) err |= HERR_STEPS;
        sm.active = 0;
      } else {
        sm.len = sm.size - 1;
        sm.hole = 0; sm.second = 0; sm.sub_root = 0; sm.lv = 0; sm.depth = 0;
        sm.need = 1;
      }
    }
    __syncwarp();
    const bool act = sm.active != 0;
    if (!__any_sync(kFull, act)) break;
    bool first = true;
    for (;;) {
      const bool need = act && sm.need;
      if (!__any_sync(kFull, need)) break;
      if (need) {
        const unsigned R = sm.sub_root, len = sm.len;
        // round 1: node indices of the subtree (and root / last on the first)
        unsigned ida = UINT_MAX, idb = UINT_MAX, idx_extra = UINT_MAX;
        int ea = gl, eb = gl + G;
        auto pos_of = [&](int e) -> unsigned long long {
          const int L = 31 - __clz(e + 2);
          const unsigned long long o = (unsigned long long)(e + 2 - (1 << L));
          return (((unsigned long long)R + 1) << L) - 1 + o;
        };
        if (ea < E) { const unsigned long long p = pos_of(ea); if (p < len) ida = heap[p]; }
        if (eb < E) { const unsigned long long p = pos_of(eb); if (p < len) idb = heap[p]; }
        if (first && gl == G - 2) idx_extra = heap[0];
        if (first && gl == G - 1 && len > 0) idx_extra = heap[len];
        // round 2: their times
        auto tload = [&](unsigned id) -> double {
          if (id == UINT_MAX) return 0.0;
          if (id >= n) { err |= HERR_INDEX; return 0.0; }
          return t[id];
        };
        const double ta = tload(ida), tb = tload(idb), tx = tload(idx_extra);
        if (ea < E) { sm.sub_id[ea] = ida; sm.sub_t[ea] = ta; }
        if (eb < E) { sm.sub_id[eb] = idb; sm.sub_t[eb] = tb; }
        if (first && gl == G - 2) { sm.top = idx_extra < n ? idx_extra : 0; sm.ttop = tx; }
        if (first && gl == G - 1) { sm.val = idx_extra < n ? idx_extra : 0; sm.tval = tx; }
      }
      __syncwarp();
      if (need && gl == 0) {
        // walk the subtree: adjust() of libstdc++'s pop_heap
        const unsigned len = sm.len, limit = (len - 1) / 2;   // len >= 1 here (else no loop)
        unsigned hole = sm.hole, second = sm.second, R = sm.sub_root;
        int lv = sm.lv, depth = sm.depth;
        bool finished = false, reload = false;
        if (len == 0) finished = true;
        while (!finished && !reload) {
          const bool two = second < limit;
          const bool odd = !two && (len & 1) == 0 && second == (len - 2) / 2;
          if (!two && !odd) { finished = true; break; }
          if (lv + 1 > D) { reload = true; break; }
          const unsigned right = 2 * (second + 1), left = right - 1;
          const unsigned long long base = (((unsigned long long)R + 1) << (lv + 1)) - 1;
          const int eL = (1 << (lv + 1)) - 2 + (int)(left - base);
          unsigned pick; int ep;
          if (two) {
            const int eR = eL + 1;
            if (gt(sm.sub_t[eR], sm.sub_t[eL])) { pick = left; ep = eL; } else { pick = right; ep = eR; }
          } else {
            pick = left; ep = eL;
          }
          const unsigned id = sm.sub_id[ep];
          heap[hole] = id;
          if (depth < kMaxDepth) { sm.path_pos[depth] = hole; sm.path_id[depth] = id; sm.path_t[depth] = sm.sub_t[ep]; }
          ++depth;
          second = pick; hole = pick; ++lv;
          if (odd) { finished = true; break; }
        }
        if (reload) {
          sm.sub_root = hole; sm.lv = 0;
        }
        sm.hole = hole; sm.second = second; sm.depth = depth;
        if (finished) {
          sm.need = 0;
          // push_up of the last element from the hole along the path
          if (sm.size > 1) {
            const unsigned val = sm.val; const double tval = sm.tval;
            int k = depth - 1;
            while (hole > 0 && k >= 0 && k < kMaxDepth && gt(sm.path_t[k], tval)) {
              heap[hole] = sm.path_id[k];
              hole = sm.path_pos[k];
              --k;
            }
            heap[hole] = val;
          }
          sm.size = sm.size - 1;
        }
      }
      first = false;
      __syncwarp();
    }

    // ---------------- update the six neighbours of the popped node
    const unsigned top = sm.top;
    const double ttop = sm.ttop;
    if (act && gl == 0) {
      st[top] = kFrozen;
      if (is_inf(ttop)) err |= HERR_INF;
    }
    int ci[3];
    {
      const unsigned k = top % (unsigned)job.nz, r = top / (unsigned)job.nz;
      ci[2] = (int)k; ci[1] = (int)(r % (unsigned)job.ny); ci[0] = (int)(r / (unsigned)job.ny);
    }
    Stencil S;
    double nt = 0.0, vel = 0.0, nis = 0.0;
    bool valid = false;
    int act_code = 0;
    unsigned char sj = kFrozen;
    unsigned j = 0;
    const int q = gl, ax_q = q >> 1, side = q & 1;
    if (act && q < 6) {
      const int cq = seli(ci, ax_q) + (side ? 1 : -1);
      if (cq >= 0 && cq < seli(dimA, ax_q)) {
        const unsigned sq = (unsigned)seli(strideA, ax_q);
        j = side ? top + sq : top - sq;
        int cj[3];
#pragma unroll
        for (int e = 0; e < 3; ++e) cj[e] = e == ax_q ? cq : ci[e];
        // all loads of the stencil at once
        sj = st[j];
        const double2 v2 = vn[j];
        S.cur = t[j];
        S.pres = 0;
#pragma unroll
        for (int e = 0; e < 3; ++e) {
          const int off[4] = {-1, -2, 1, 2};
#pragma unroll
          for (int m = 0; m < 4; ++m) {
            S.v[e][m] = 0.0;
            if (!high && (m == 1 || m == 3)) continue;
            const int c = cj[e] + off[m];
            if (c >= 0 && c < dimA[e]) {
              S.pres |= 1u << (4 * e + m);
              S.v[e][m] = t[(long long)j + (long long)off[m] * strideA[e]];
            }
          }
        }
        vel = v2.x; nis = v2.y;
        valid = sj != kFrozen && !(vel < kMargin);
        if (valid) {
          nt = high ? solve_high(S, vel, nis, ax) : solve_first(S, vel, nis, ax);
          if (sj == kNarrow) act_code = (nt + kMargin < S.cur) ? 2 : 0;   // isTimeBetterThan
          else act_code = 1;
        }
      }
      sm.nb_act[q] = act_code; sm.nb_t[q] = nt; sm.nb_j[q] = j;
    }
    __syncwarp();
    if (high) {
      // the + neighbour of an axis reads the - neighbour two steps away:
      // evaluate again when the new value of the - neighbour enters its
      // stencil (only possible when that value is <= the popped time)
      bool redo = false;
      if (act && q < 6 && side == 1 && valid && sm.nb_act[q - 1] != 0) {
        const double t1new = sm.nb_t[q - 1];
        if (!is_inf(t1new) && le(t1new, ttop)) {
#pragma unroll
          for (int e = 0; e < 3; ++e)
            if (e == ax_q) S.v[e][1] = t1new;
          redo = true;
        }
      }
      if (__any_sync(kFull, redo)) {
        if (redo) {
          nt = solve_high(S, vel, nis, ax);
          const int code = (sj == kNarrow) ? ((nt + kMargin < S.cur) ? 2 : 0) : 1;
          sm.nb_act[q] = code; sm.nb_t[q] = nt;
        }
        __syncwarp();
      }
    }
    // ---------------- apply in the reference's order: time, state, push
    if (act && gl == 0) {
      unsigned size = sm.size;
      bool stop = false;
      for (int r = 0; r < 6 && !stop; ++r) {
        const int code = sm.nb_act[r];
        if (code == 0) continue;
        const unsigned jj = sm.nb_j[r];
        const double tv = sm.nb_t[r];
        t[jj] = tv;
        if (code == 1) st[jj] = kNarrow;
        if (size >= job.hcap) { err |= HERR_OVERFLOW; stop = true; break; }
        unsigned hole = size++;
        while (hole > 0) {
          const unsigned parent = (hole - 1) / 2;
          const unsigned pid = heap[parent];
          if (pid >= n) { err |= HERR_INDEX; break; }
          if (!gt(t[pid], tv)) break;
          heap[hole] = pid;
          hole = parent;
        }
        heap[hole] = jj;
      }
      sm.size = size;
      if (stop) sm.active = 0;
      // clear for the next step (lanes 0..5 rewrite them when active)
      for (int r = 0; r < 6; ++r) sm.nb_act[r] = 0;
    }
    __syncwarp();
  }
  if (err) atomicOr(job.herr, err);
}

__global__ void vn_kernel(const double *vel, double2 *vn, size_t n) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
    const double v = vel[q];
    vn[q] = make_double2(v, -1.0 / (v * v));
  }
}

__global__ void heap_fill_kernel(double *t, unsigned char *st, size_t n) {
  const double INF = __longlong_as_double(kInfBits);
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
    t[q] = INF;
    st[q] = kOpen;
  }
}

// Receiver read-out on the FP64 field (ndgridmap.hpp:462-490).
__global__ void heap_readout_kernel(Eik3Job job, int s0, int nsol) {
  const int sl = blockIdx.y;
  if (sl >= nsol) return;
  const int s = s0 + sl;
  const E3Dims d{job.nx, job.ny, job.nz};
  const size_t nn = (size_t)d.nx * d.ny * d.nz;
  const double *t = job.ht + (size_t)sl * nn;
  const double h[3] = {job.dx, job.dy, job.dz};
  const int rs = job.solve_rev ? job.solve_rev[s] : (job.rev_per_solve ? s : 0);
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < job.nrev; r += gridDim.x * blockDim.x) {
    const double *p = job.rev + ((size_t)rs * job.nrev + r) * 3;
    const double pt[3] = {p[0], p[1], p[2]};
    auto tget = [&](int i, int j, int k) { return t[e3_nidx(d, i, j, k)]; };
    job.ttime[(size_t)s * job.nrev + r] = e3_trilinear(d, h, pt, tget);
  }
}

int g_group = 8;
int g_chunk_cap = 0;     // diagnostics: solves per launch at most (0: no cap)

template <int G>
int launch_group(const Eik3Job &job, int s0, int nsol, cudaStream_t s) {
  constexpr int per_block = kBlock / G;
  heap_march_kernel<G><<<(nsol + per_block - 1) / per_block, kBlock, 0, s>>>(job, s0, nsol);
  MCT_CUDA_TRY(cudaGetLastError());
  return MCT_OK;
}

}  // namespace

int eik3_resolve_method(int order, int method) {
  if (method == EIK3_TILES || method == EIK3_HEAP) return method;
  return order == 1 ? EIK3_HEAP : EIK3_TILES;
}

unsigned eik3_heap_cap(int nx, int ny, int nz) {
  // the reference reserves one entry per node; the live narrow band with
  // its stale entries stays far below that
  return (unsigned)((size_t)nx * ny * nz);
}

size_t eik3_heap_bytes_per_solve(int nx, int ny, int nz) {
  const size_t nn = (size_t)nx * ny * nz;
  return carve_size({sizeof(double) * nn, nn, sizeof(unsigned) * (size_t)eik3_heap_cap(nx, ny, nz)});
}

int launch_eik3_heap(Eik3Job &job, cudaStream_t s, double *tfield) {
  const size_t nn = (size_t)job.nx * job.ny * job.nz;
  if (nn >= (size_t)UINT_MAX / 2 || job.hchunk < 1 || job.hcap < 8) {
    mct_set_error("launch_eik3_heap", "grid too large or no heap scratch", __FILE__, __LINE__);
    return MCT_ERR_ARG;
  }
  MCT_CUDA_TRY(cudaMemsetAsync(job.herr, 0, sizeof(int), s));
  vn_kernel<<<1024, 256, 0, s>>>(job.vel, job.hvn, nn * job.ngrids);
  MCT_CUDA_TRY(cudaGetLastError());
  // equal chunks (a short last chunk would run alone at the latency of one
  // whole march)
  const int maxc = g_chunk_cap > 0 ? std::min(g_chunk_cap, job.hchunk) : job.hchunk;
  const int nchunks = (job.nsolve + maxc - 1) / maxc;
  const int per = (job.nsolve + nchunks - 1) / nchunks;
  for (int s0 = 0; s0 < job.nsolve; s0 += per) {
    const int nsol = std::min(per, job.nsolve - s0);
    heap_fill_kernel<<<1024, 256, 0, s>>>(job.ht, job.hst, nn * nsol);
    MCT_CUDA_TRY(cudaGetLastError());
    int rc = g_group == 32 ? launch_group<32>(job, s0, nsol, s)
           : g_group == 16 ? launch_group<16>(job, s0, nsol, s)
           : launch_group<8>(job, s0, nsol, s);
    if (rc) return rc;
    if (job.nrev > 0) {
      heap_readout_kernel<<<dim3((job.nrev + 127) / 128, nsol), 128, 0, s>>>(job, s0, nsol);
      MCT_CUDA_TRY(cudaGetLastError());
    }
    if (tfield)
      MCT_CUDA_TRY(cudaMemcpyAsync(tfield + (size_t)s0 * nn, job.ht, sizeof(double) * nn * nsol,
                                   cudaMemcpyDeviceToDevice, s));
  }
  int herr = 0;
  MCT_CUDA_TRY(cudaMemcpyAsync(&herr, job.herr, sizeof(int), cudaMemcpyDeviceToHost, s));
  MCT_CUDA_TRY(cudaStreamSynchronize(s));
  if (herr & HERR_INDEX) { mct_set_error("heap march", "corrupt heap entry", __FILE__, __LINE__); return MCT_ERR_INTERNAL; }
  if (herr & HERR_OVERFLOW) { mct_set_error("heap march", "heap capacity exceeded", __FILE__, __LINE__); return MCT_ERR_NOMEM; }
  if (herr & HERR_STEPS) { mct_set_error("heap march", "step limit reached", __FILE__, __LINE__); return MCT_ERR_TIMEOUT; }
  if (herr & HERR_INF) {
    // the reference asserts on an infinite accepted time (fmm.hpp:123)
    mct_set_error("heap march", "unreachable node (infinite arrival time accepted)", __FILE__, __LINE__);
    return MCT_ERR_INTERNAL;
  }
  return MCT_OK;
}

// Diagnostics (not part of the public header): lanes per solve of the heap
// march (8, 16 or 32); returns the previous value.
extern "C" int mct_debug_eik3_heap_group(int g) {
  const int old = g_group;
  if (g == 8 || g == 16 || g == 32) g_group = g;
  return old;
}

// Diagnostics (not part of the public header): at most n solves per heap
// march launch (0: no cap); returns the previous value.
extern "C" int mct_debug_eik3_heap_chunk(int n) {
  const int old = g_chunk_cap;
  g_chunk_cap = n > 0 ? n : 0;
  return old;
}
