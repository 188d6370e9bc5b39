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
// parallelism is across solves: one group of G lanes (8 or 32) marches one
// solve, and the lanes of a group share the work of each step:
//
//  * pop: the heap keeps each entry's key beside its node index (kept equal
//    to the node's live time, see the heap section below), so one round
//    trip fetches the keys of a whole subtree of D levels below the hole.
//    Every lane decides the walk's step at its internal nodes of the
//    subtree, a ballot gathers the decisions, all lanes follow them to the
//    same path, and the lanes holding the path's entries move them up; the
//    final sift-up of the last element along the path is one more ballot.
//  * update: lanes 0..5 take the six neighbours of the popped node (x-, x+,
//    y-, y+, z-, z+), issue the loads of their whole stencils (up to 12
//    times, state, velocity) while the pop runs, and evaluate the
//    reference's update in FP64 with its exact operation order. Neighbours
//    on different axes do not read each other; the + neighbour of an axis
//    can read the - neighbour (two steps away in the second-order stencil),
//    so it is evaluated again with the new value in the rare case that
//    value enters its stencil (it is at most the popped time).
//  * accept: the leader applies the results in the reference's order (write
//    the time, update the keys of the node's older entries, push), so every
//    comparison in every push sees exactly the keys the reference's push
//    sees.
//
// Comparisons between times are integer comparisons of the IEEE bit
// patterns (all times are >= 0 or +inf), which are exact and keep them off
// the FP64 pipe; the arithmetic of the update is the reference's, FP64,
// without contraction (the library is built with -fmad=false), except that
// divisions by divisors known in advance take Markstein's FMA correction,
// which returns the same correctly rounded quotient in fewer steps.
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

// ---------------------------------------------------------------------------
// The same updates with fewer and shorter FP64 steps. On this GPU a
// dependent FP64 add or multiply costs ~64 cycles and a division or square
// root ~550, and the FP64 pipe is shared by the whole SM, so the update's
// dependent chain bounds each pop and its instruction count bounds many
// solves at once. Divisions by divisors known in advance (3, and 2A, which
// takes one of 108 values per launch: the axes of the slots in sorted order
// and which of them are second order) use Markstein's correction step
// (P. Markstein, "Computation of elementary functions on the IBM RISC
// System/6000 processor", IBM J. Res. Dev. 34(1), 1990): with yinv = RN(1/y),
// q = RN(x*yinv), r = x - q*y (exact with a fused multiply-add) and
// RN(q + r*yinv) is the correctly rounded x/y, so the results are the same
// bits as the reference's divisions. Comparisons use the integer order of
// the bit patterns. Every other operation is the reference's, in its order.
// ---------------------------------------------------------------------------
struct Combo {
  double four_a, two_a, rtwo_a, pad;
};
constexpr int kCombos = 36 + 72;   // i = 2: 9 slot-axis pairs x 4 flag sets; i = 3: 9 x 8
constexpr double kThird = 1.0 / 3.0;

// Correctly rounded x / y given yinv = RN(1/y) (Markstein's correction).
__device__ __forceinline__ double div_known(double x, double y, double yinv) {
  const double q = __dmul_rn(x, yinv);
  const double r = __fma_rn(-q, y, x);
  return __fma_rn(r, yinv, q);
}

// A of the reference's quadratic for every candidate shape, summed in the
// reference's order (0.0 + alpha of slot 0 + alpha of slot 1 [+ slot 2]),
// with 4A, 2A and RN(1/(2A)).
__device__ void build_combos(Combo *tab, const Axes &ax, int tid, int nthreads) {
  for (int c = tid; c < kCombos; c += nthreads) {
    const int i = c < 36 ? 2 : 3;
    const int pair = c < 36 ? c / 4 : (c - 36) / 8, flags = c < 36 ? c % 4 : (c - 36) % 8;
    const int d0 = pair / 3, d1 = pair % 3, d2 = 3 - d0 - d1;
    Combo cb{0.0, 0.0, 0.0, 0.0};
    if (d0 != d1) {
      const int dd[3] = {d0, d1, d2};
      double A = 0.0;
      for (int q = 0; q < i; ++q) A += ((flags >> q) & 1) ? ax.a2[dd[q]] : ax.a1[dd[q]];
      cb.four_a = 4 * A; cb.two_a = 2 * A; cb.rtwo_a = 1.0 / (2 * A);
    }
    tab[c] = cb;
  }
}

__device__ __forceinline__ int combo_index(int i, int pair, int flags) {
  return i == 2 ? pair * 4 + (flags & 3) : 36 + pair * 8 + flags;
}

// quad < 0 on the bit pattern (quad is never NaN here; -0 is not < 0)
__device__ __forceinline__ bool negative(double x) {
  const long long b = bits(x);
  return b < 0 && b != (long long)0x8000000000000000ULL;
}

__device__ double solve_first_fast(const Stencil &S, double vel, double nis, const Axes &ax, const Combo *tab) {
  const double INF = __longlong_as_double(kInfBits);
  double tv[3]; double dummy[3]; int dm[3];
  int cnt = 0;
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    const bool p0 = (S.pres >> (4 * e)) & 1, p1 = (S.pres >> (4 * e + 2)) & 1;
    double m;
    if (p0 && p1) m = lt(S.v[e][0], S.v[e][2]) ? S.v[e][0] : S.v[e][2];
    else m = p0 ? S.v[e][0] : S.v[e][2];
    const bool use = !is_inf(m) && lt(m, S.cur);
    tv[e] = use ? m : INF;
    dummy[e] = 0.0;
    dm[e] = e;
    cnt += use ? 1 : 0;
  }
  if (cnt == 0) return INF;
  sort3(tv, dummy, dm);
  const int pair = dm[0] * 3 + dm[1];
  double B = 0.0, C = nis;
  double updated = 0.0;
  bool done = false;
#pragma unroll
  for (int i = 1; i <= 3; ++i) {
    if (done || i > cnt) continue;
    const double alpha = sel3(ax.a1, dm[i - 1]);
    C += tv[i - 1] * tv[i - 1] * alpha;
    B += -2.0 * tv[i - 1] * alpha;
    if (i == 1) {
      updated = tv[0] + sel3(ax.h, dm[0]) / vel;
    } else {
      const Combo &cb = tab[combo_index(i, pair, 0)];
      const double quad = B * B - cb.four_a * C;
      updated = negative(quad) ? INF : div_known(-B + sqrt(quad), cb.two_a, cb.rtwo_a);
    }
    if (i == cnt) done = true;
    else if (lt(updated - tv[i < 3 ? i : 2], kMargin)) done = true;
  }
  return updated;
}

__device__ double solve_high_fast(const Stencil &S, double vel, double nis, const Axes &ax, const Combo *tab) {
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
  double cC[3], cB[3];
  int fl = 0;
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    cC[q] = 0.0; cB[q] = 0.0;
    if (q >= cnt) continue;
    if (!is_inf(t2[q])) {
      const double alpha = sel3(ax.a2, dm[q]);
      const double tt = div_known(4.0 * t1[q] - t2[q], 3.0, kThird);
      cC[q] = tt * tt * alpha; cB[q] = -2.0 * tt * alpha;
      fl |= 1 << q;
    } else {
      const double alpha = sel3(ax.a1, dm[q]);
      cC[q] = t1[q] * t1[q] * alpha; cB[q] = -2.0 * t1[q] * alpha;
    }
  }
  double Cs[3], Bs[3];
  {
    double B = 0.0, C = nis;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      C += cC[q]; B += cB[q];
      Cs[q] = C; Bs[q] = B;
    }
  }
  const int pair = dm[0] * 3 + dm[1];
  double updated = INF;
  bool done = false;
#pragma unroll
  for (int i = 3; i >= 1; --i) {
    if (done || i > cnt) continue;
    double cand;
    if (i == 1) {
      cand = t1[0] + sel3(ax.h, dm[0]) / vel;
    } else {
      const Combo &cb = tab[combo_index(i, pair, fl)];
      const double B = Bs[i - 1], C = Cs[i - 1];
      const double quad = B * B - cb.four_a * C;
      cand = negative(quad) ? INF : div_known(-B + sqrt(quad), cb.two_a, cb.rtwo_a);
    }
    if (!is_inf(cand) && gt(cand - t1[i - 1], kMargin)) { updated = cand; done = true; }
  }
  return updated;
}

// ---------------------------------------------------------------------------
// The heap. Entries are (key, node) pairs in two arrays, hkey[] and hid[],
// so that the entries of one heap level are contiguous. The reference's key
// is the node's live time; it is kept in hkey[] by updating, in place and
// without a sift, every entry of a node whose time changes (exactly what the
// reference's comparisons see: the old entry's key drops with the node's
// time). For that, each node records the heap positions of its first two
// entries (hpos[2*node + slot], rewritten on every move; hid[] carries the
// slot in its top two bits). A node that gets a third entry (measured: ~0.3%
// of nodes) switches to "live" keys: its entries' hkey hold a marker and
// comparisons read the node's time instead.
// ---------------------------------------------------------------------------
constexpr unsigned kNone = 0xFFFFFFFFu;       // hpos: no entry in this slot
constexpr unsigned kLiveFlag = 0xFFFFFFFEu;   // hpos: node uses live keys
constexpr unsigned kIdMask = 0x3FFFFFFFu;
constexpr unsigned kUntracked = 3u;           // slot bits of a live-key entry
constexpr long long kLiveBits = (long long)0xFFF8000000000001ULL;   // sign set: not a time

__device__ __forceinline__ bool is_live(double k) { return bits(k) < 0; }

struct Heap {
  double *t;
  unsigned char *st;
  double *hkey;
  unsigned *hid;
  unsigned *hpos;
  unsigned n, cap;
};

// Write entry (key, idw) at position p and record the move.
__device__ __forceinline__ void put(const Heap &H, unsigned p, double key, unsigned idw) {
  H.hkey[p] = key;
  H.hid[p] = idw;
  const unsigned slot = idw >> 30;
  if (slot < 2) H.hpos[2 * (idw & kIdMask) + slot] = p;
}

__device__ __forceinline__ double resolve(const Heap &H, double key, unsigned idw) {
  return is_live(key) ? H.t[idw & kIdMask] : key;
}

// push_heap of an entry whose live key is tv.
__device__ __forceinline__ void heap_push(const Heap &H, unsigned &size, double key, unsigned idw, double tv,
                                          int &err) {
  if (size >= H.cap) { err |= HERR_OVERFLOW; return; }
  unsigned hole = size++;
  while (hole > 0) {
    const unsigned parent = (hole - 1) / 2;
    const double pk = H.hkey[parent];
    const unsigned pid = H.hid[parent];
    if ((pid & kIdMask) >= H.n) { err |= HERR_INDEX; break; }
    if (!gt(resolve(H, pk, pid), tv)) break;
    put(H, hole, pk, pid);
    hole = parent;
  }
  put(H, hole, key, idw);
}

// t[j] = tv, then push j (fmm.hpp:103-115 for the source, :138-148 for the
// updates). fresh: j has no entry yet (it was OPEN).
__device__ void assign_push(const Heap &H, unsigned &size, unsigned j, double tv, bool fresh, int &err) {
  H.t[j] = tv;
  double key = tv;
  unsigned slot = 0;
  if (!fresh) {
    const uint2 hp = reinterpret_cast<const uint2 *>(H.hpos)[j];
    if (hp.x == kLiveFlag) {
      key = __longlong_as_double(kLiveBits); slot = kUntracked;
    } else if (hp.x == kNone) {
      slot = 0;
    } else if (hp.y == kNone) {
      H.hkey[hp.x] = tv;
      slot = 1;
    } else {
      const double live = __longlong_as_double(kLiveBits);
      H.hkey[hp.x] = live; H.hid[hp.x] = j | (kUntracked << 30);
      H.hkey[hp.y] = live; H.hid[hp.y] = j | (kUntracked << 30);
      reinterpret_cast<uint2 *>(H.hpos)[j] = make_uint2(kLiveFlag, kLiveFlag);
      key = live; slot = kUntracked;
    }
  }
  heap_push(H, size, key, j | (slot << 30), tv, err);
}

template <int E>
struct alignas(16) GroupSmem {
  // subtree below the hole, entries by level: stored key, live key, node
  double sub_raw[E];
  double sub_res[E];
  unsigned sub_id[E];
  // sift-down path: position, stored key, live key and node of the element
  // moved up into each level
  unsigned path_pos[kMaxDepth];
  unsigned path_id[kMaxDepth];
  double path_raw[kMaxDepth];
  double path_res[kMaxDepth];
  // neighbour results
  double nb_t[6];
  unsigned nb_j[6];
  int nb_act[6];          // 0 none, 1 OPEN -> NARROW, 2 improved
  unsigned size, top, val;
  double ttop, val_raw, val_res;
  int active;
};

// Position of subtree entry e (levels 1.. below the subtree root R, level
// order) in the heap.
__device__ __forceinline__ unsigned long long sub_pos(unsigned R, int e) {
  const int L = 31 - __clz(e + 2);
  return (((unsigned long long)R + 1) << L) - 1 + (unsigned long long)(e + 2 - (1 << L));
}

// One group of G lanes per solve, kBlock / G solves per block; the pop
// walks subtrees of D levels (2^(D+1) - 2 entries) per round trip.
//
// The pop (libstdc++'s pop_heap: adjust, then push_up of the last element)
// runs on all lanes of the group at once: after one round trip fetches a
// subtree's keys, each lane decides for its internal nodes of the subtree
// which child the walk would take (the larger key loses; ties go right;
// the reference's end-of-heap cases), a ballot gathers the decisions, every
// lane follows them from the root to get the same path, and the lanes that
// hold the path's entries move them up. The final push_up of the last
// element along the path is one more ballot (which path entries are larger)
// and parallel moves.
template <int G, int D>
__global__ void __launch_bounds__(kBlock) heap_march_kernel(Eik3Job job, int s0, int nsol) {
  // at least six lanes: one per neighbour in the update step
  static_assert(G == 8 || G == 16 || G == 32, "group size");
  static_assert(D >= 2 && D <= 5, "subtree depth");
  constexpr int E = (2 << D) - 2;             // subtree entries
  constexpr int NI = (1 << D) - 1;            // internal nodes of a subtree (<= 31)
  constexpr int PER = (E + G - 1) / G;        // entries per lane
  constexpr int PERI = (NI + G - 1) / G;      // internal nodes per lane
  constexpr int PERD = (kMaxDepth + G - 1) / G;       // path levels per lane
  static_assert((PERI - 1) * G < 32 && (PERD - 1) * G < 64, "decision masks fit their words");
  __shared__ GroupSmem<E> sm_all[kBlock / G];
  __shared__ Combo tab[kCombos];
  const int gi = threadIdx.x / G, gl = threadIdx.x % G;
  const int gshift = (threadIdx.x % 32) / G * G;      // the group's first lane in the warp
  const unsigned gmask_bits = G == 32 ? 0xffffffffu : ((1u << G) - 1);
  GroupSmem<E> &sm = sm_all[gi];
  const int sl = blockIdx.x * (kBlock / G) + gi;          // solve within the chunk
  const bool live = sl < nsol;
  const int s = s0 + (live ? sl : 0);
  const E3Dims d{job.nx, job.ny, job.nz};
  const unsigned n = (unsigned)job.nx * job.ny * job.nz;
  const int strideA[3] = {job.ny * job.nz, job.nz, 1};
  const int dimA[3] = {job.nx, job.ny, job.nz};
  const size_t so = (size_t)(live ? sl : 0);
  Heap H;
  H.t = job.ht + so * n;
  H.st = job.hst + so * n;
  H.hkey = job.hkey + so * job.hcap;
  H.hid = job.hid + so * job.hcap;
  H.hpos = job.hpos + so * 2 * (size_t)n;
  H.n = n; H.cap = job.hcap;
  double *t = H.t;
  unsigned char *st = H.st;
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
  build_combos(tab, ax, threadIdx.x, blockDim.x);
  __syncthreads();
  const bool high = job.order == 1;
  int err = 0;

  // ---- source: 8 corners with times dist*2/(v_src + v_corner), assigned
  // and pushed in corner order (solver.hpp:72-92 setInitialPoints,
  // fmm.hpp:103-115); a corner clamped onto another is assigned again
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
        const bool fresh = st[id] == kOpen;
        st[id] = kNarrow;
        assign_push(H, size, id, tv, fresh, err);
      }
      sm.size = size;
    }
  }
  __syncwarp();

  const long long max_pops = 8LL * n + 64;
  for (long long it = 0;; ++it) {
    // ---------------- pop
    if (gl == 0 && sm.active && (sm.size == 0 || it >= max_pops || err)) {
      if (sm.size != 0 && !err) err |= HERR_STEPS;
      sm.active = 0;
    }
    __syncwarp();
    const bool act = sm.active != 0;
    if (!__any_sync(kFull, act)) break;
    const unsigned size = sm.size;
    const unsigned len = act ? size - 1 : 0;
    const unsigned limit = len > 0 ? (len - 1) / 2 : 0;
    const bool even = (len & 1) == 0;
    const unsigned last_parent = len >= 2 ? (len - 2) / 2 : kNone;   // the odd case's node
    unsigned R = 0, hole = 0;
    int depth = 0;
    bool need = act;

    // stencil of this lane's neighbour of the popped node, loaded while the
    // walk runs (times do not change during a pop)
    Stencil S;
    S.pres = 0; S.cur = 0.0;
    unsigned char sj = kFrozen;
    double2 v2 = make_double2(0.0, 0.0);
    unsigned j = 0;
    bool has = false;
    const int q = gl, ax_q = q >> 1, side = q & 1;

    for (int iter = 0;; ++iter) {
      if (!__any_sync(kFull, need)) break;
      double kraw[PER], kres[PER]; unsigned kid[PER];
      if (need) {
        // one round trip: keys and nodes of the whole subtree (and the root
        // and last entry on the first)
#pragma unroll
        for (int u = 0; u < PER; ++u) {
          const int e = gl + u * G;
          kraw[u] = 0.0; kid[u] = kNone;
          if (e < E) {
            const unsigned long long p = sub_pos(R, e);
            if (p < len) { kraw[u] = H.hkey[p]; kid[u] = H.hid[p]; }
          }
        }
        double xr = 0.0; unsigned xi = kNone;
        if (iter == 0 && gl == G - 2) { xr = H.hkey[0]; xi = H.hid[0]; }
        if (iter == 0 && gl == G - 1 && len > 0) { xr = H.hkey[len]; xi = H.hid[len]; }
#pragma unroll
        for (int u = 0; u < PER; ++u) {
          const int e = gl + u * G;
          kres[u] = kraw[u];
          if (kid[u] != kNone) {
            if ((kid[u] & kIdMask) >= n) { err |= HERR_INDEX; kid[u] = kNone; }
            else if (is_live(kraw[u])) kres[u] = t[kid[u] & kIdMask];   // live key (rare)
          }
          if (e < E) { sm.sub_raw[e] = kraw[u]; sm.sub_res[e] = kres[u]; sm.sub_id[e] = kid[u]; }
        }
        if (xi != kNone) {
          double xres = xr;
          if ((xi & kIdMask) >= n) { err |= HERR_INDEX; xi = 0; xres = 0.0; }
          else if (is_live(xr)) xres = t[xi & kIdMask];
          if (gl == G - 2) { sm.top = xi & kIdMask; sm.ttop = xres; }
          else { sm.val = xi; sm.val_raw = xr; sm.val_res = xres; }
        }
      }
      __syncwarp();
      if (iter == 0 && act && q < 6) {
        // issue the stencil loads now; they are consumed after the walk
        const unsigned top = sm.top;
        int ci[3];
        {
          const unsigned k = top % (unsigned)job.nz, r = top / (unsigned)job.nz;
          ci[2] = (int)k; ci[1] = (int)(r % (unsigned)job.ny); ci[0] = (int)(r / (unsigned)job.ny);
        }
        const int cq = seli(ci, ax_q) + (side ? 1 : -1);
        if (cq >= 0 && cq < seli(dimA, ax_q)) {
          has = true;
          const unsigned sq = (unsigned)seli(strideA, ax_q);
          j = side ? top + sq : top - sq;
          int cj[3];
#pragma unroll
          for (int e = 0; e < 3; ++e) cj[e] = e == ax_q ? cq : ci[e];
          sj = st[j];
          v2 = vn[j];
          S.cur = t[j];
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
        }
      }
      // the walk's decision at each internal node of the subtree
      unsigned m_two = 0, m_odd = 0, m_right = 0;
#pragma unroll
      for (int u = 0; u < PERI; ++u) {
        const int k = gl + u * G;
        bool two = false, odd = false, right = false;
        if (need && k < NI) {
          const unsigned long long pk = k == 0 ? R : sub_pos(R, k - 1);
          if (k == 0 || pk < len) {
            two = pk < limit;
            odd = !two && even && pk == last_parent;
            if (two) right = !gt(sm.sub_res[2 * k + 1], sm.sub_res[2 * k]);
          }
        }
        const unsigned b2 = (__ballot_sync(kFull, two) >> gshift) & gmask_bits;
        const unsigned bo = (__ballot_sync(kFull, odd) >> gshift) & gmask_bits;
        const unsigned br = (__ballot_sync(kFull, right) >> gshift) & gmask_bits;
        m_two |= b2 << (u * G); m_odd |= bo << (u * G); m_right |= br << (u * G);
      }
      if (need) {
        // follow the decisions from the subtree root (same on every lane)
        int k = 0, steps = 0, lastc = -1;
        bool ended = false;
        unsigned long long chosen = 0;
#pragma unroll
        for (int lvl = 0; lvl < D; ++lvl) {
          if (ended) continue;
          int c;
          if ((m_two >> k) & 1) c = 2 * k + (int)((m_right >> k) & 1);
          else if ((m_odd >> k) & 1) { c = 2 * k; ended = true; }
          else { ended = true; continue; }
          chosen |= 1ull << c; lastc = c; ++steps;
          k = c + 1;
        }
        // the lanes holding the path's entries move them up one level
#pragma unroll
        for (int u = 0; u < PER; ++u) {
          const int e = gl + u * G;
          if (e < E && ((chosen >> e) & 1)) {
            const unsigned p = (unsigned)sub_pos(R, e);
            const unsigned parent = (p - 1) / 2;
            put(H, parent, kraw[u], kid[u]);
            const int dl = depth + (31 - __clz(e + 2)) - 1;
            if (dl < kMaxDepth) {
              sm.path_pos[dl] = parent; sm.path_id[dl] = kid[u]; sm.path_raw[dl] = kraw[u]; sm.path_res[dl] = kres[u];
            }
          }
        }
        depth += steps;
        if (steps > 0) hole = (unsigned)sub_pos(R, lastc);
        if (ended) {
          need = false;
        } else {
          // D levels walked: continue below the new hole if it has children
          const bool more = hole < limit || (even && hole == last_parent);
          if (more) R = hole; else need = false;
        }
      }
      __syncwarp();
    }

    // push_up of the last element from the hole along the path
    const bool up = act && size > 1;
    unsigned long long bmask = 0;     // bit k: path entry k is larger than the last element
    {
      const double vres = up ? sm.val_res : 0.0;
#pragma unroll
      for (int u = 0; u < PERD; ++u) {
        const int k = gl + u * G;
        const bool b = up && k < depth && k < kMaxDepth && gt(sm.path_res[k], vres);
        bmask |= (unsigned long long)((__ballot_sync(kFull, b) >> gshift) & gmask_bits) << (u * G);
      }
    }
    if (up) {
      const int dd = depth < kMaxDepth ? depth : kMaxDepth;
      const unsigned long long valid = (1ull << dd) - 1;   // dd <= 33
      const unsigned long long F = ~bmask & valid;
      const int m = F == 0 ? 0 : 64 - __clzll(F);        // entries m..depth-1 move down one level
#pragma unroll
      for (int u = 0; u < PERD; ++u) {
        const int k = gl + u * G;
        if (k >= m && k < dd) {
          const unsigned to = k + 1 < dd ? sm.path_pos[k + 1] : hole;
          put(H, to, sm.path_raw[k], sm.path_id[k]);
        }
      }
      if (gl == 0) put(H, m < dd ? sm.path_pos[m] : hole, sm.val_raw, sm.val);
    }
    if (act && gl == 0) sm.size = size - 1;
    __syncwarp();

    // ---------------- update the six neighbours of the popped node
    const unsigned top = sm.top;
    const double ttop = sm.ttop;
    if (act && gl == 0) {
      st[top] = kFrozen;
      if (is_inf(ttop)) err |= HERR_INF;
    }
    double nt = 0.0;
    bool valid = false;
    int act_code = 0;
    if (act && q < 6) {
      if (has) {
        const double vel = v2.x, nis = v2.y;
        valid = sj != kFrozen && !(vel < kMargin);
        if (valid) {
          nt = high ? solve_high_fast(S, vel, nis, ax, tab) : solve_first_fast(S, vel, nis, ax, tab);
          if (sj == kNarrow) act_code = lt(nt + kMargin, S.cur) ? 2 : 0;   // isTimeBetterThan
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
          nt = solve_high_fast(S, v2.x, v2.y, ax, tab);
          const int code = (sj == kNarrow) ? (lt(nt + kMargin, S.cur) ? 2 : 0) : 1;
          sm.nb_act[q] = code; sm.nb_t[q] = nt;
        }
        __syncwarp();
      }
    }
    // ---------------- apply in the reference's order: time, state, push
    if (act && gl == 0) {
      unsigned sz = sm.size;
      for (int r = 0; r < 6 && !err; ++r) {
        const int code = sm.nb_act[r];
        if (code == 0) continue;
        const unsigned jj = sm.nb_j[r];
        if (code == 1) st[jj] = kNarrow;
        assign_push(H, sz, jj, sm.nb_t[r], code == 1, err);
      }
      sm.size = sz;
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

__global__ void heap_fill_kernel(double *t, unsigned char *st, uint2 *hpos, size_t n) {
  const double INF = __longlong_as_double(kInfBits);
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
    t[q] = INF;
    st[q] = kOpen;
    hpos[q] = make_uint2(kNone, kNone);
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

int g_variant = -1;      // diagnostics: lane-group / subtree-depth variant (-1: by batch size)
int g_chunk_cap = 0;     // diagnostics: solves per launch at most (0: no cap)

template <int G, int D>
int launch_variant(const Eik3Job &job, int s0, int nsol, cudaStream_t s) {
  constexpr int per_block = kBlock / G;
  heap_march_kernel<G, D><<<(nsol + per_block - 1) / per_block, kBlock, 0, s>>>(job, s0, nsol);
  MCT_CUDA_TRY(cudaGetLastError());
  return MCT_OK;
}

int launch_march(const Eik3Job &job, int s0, int nsol, cudaStream_t s) {
  // Few solves: the march's latency decides, and 32 lanes per solve give
  // the shortest steps. Many solves: the SM's shared FP64 pipe decides, and
  // 8-lane groups let four solves share each FP64 instruction (measured on
  // 101x101x51: 3.7 s vs 4.4 s for one solve, 7.6 s vs 11.2 s for 3840).
  const int v = g_variant >= 0 ? g_variant : (nsol >= 4 * 152 ? 1 : 3);
  switch (v) {
    case 1: return launch_variant<8, 4>(job, s0, nsol, s);
    case 2: return launch_variant<16, 5>(job, s0, nsol, s);
    case 3: return launch_variant<32, 5>(job, s0, nsol, s);
    case 4: return launch_variant<16, 4>(job, s0, nsol, s);
    case 5: return launch_variant<8, 3>(job, s0, nsol, s);
    default: return launch_variant<8, 5>(job, s0, nsol, s);
  }
}

// Random stencils shaped like a marching front (times near a base time,
// some neighbours unreached or outside the grid) for the update check.
__device__ unsigned long long mix64(unsigned long long x) {
  x ^= x >> 33; x *= 0xff51afd7ed558ccdULL; x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ULL; x ^= x >> 33;
  return x;
}
__device__ double unit(unsigned long long &rs) {
  rs = mix64(rs + 0x9E3779B97F4A7C15ULL);
  return (double)(rs >> 11) * (1.0 / 9007199254740992.0);
}

__global__ void update_check_kernel(int order, Axes ax, unsigned long long count, unsigned long long seed,
                                    unsigned long long *out) {
  __shared__ Combo tab[kCombos];
  build_combos(tab, ax, threadIdx.x, blockDim.x);
  __syncthreads();
  const double INF = __longlong_as_double(kInfBits);
  for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < count;
       k += (unsigned long long)gridDim.x * blockDim.x) {
    unsigned long long rs = mix64(k * 7 + seed);
    Stencil S;
    const double T = 0.2 + 30.0 * unit(rs);
    S.pres = 0;
    for (int e = 0; e < 3; ++e)
      for (int m = 0; m < 4; ++m) {
        S.v[e][m] = 0.0;
        if (order == 0 && (m == 1 || m == 3)) continue;
        if (unit(rs) < 0.1) continue;
        S.pres |= 1u << (4 * e + m);
        const double spread = (m == 1 || m == 3) ? 0.5 : 0.25;
        const double v = unit(rs) < 0.25 ? INF : T + spread * (2 * unit(rs) - 1);
        S.v[e][m] = v < 0 ? 0.0 : v;
      }
    S.cur = unit(rs) < 0.4 ? INF : T + 0.3 * unit(rs);
    const double vel = 1.0 + 7.0 * unit(rs);
    const double nis = -1.0 / (vel * vel);
    const double a = order ? solve_high(S, vel, nis, ax) : solve_first(S, vel, nis, ax);
    const double b = order ? solve_high_fast(S, vel, nis, ax, tab) : solve_first_fast(S, vel, nis, ax, tab);
    if (bits(a) != bits(b)) atomicAdd(out, 1ULL);
    if (!is_inf(a)) atomicAdd(out + 1, 1ULL);
  }
}

}  // namespace

int eik3_resolve_method(int order, int method) {
  if (method == EIK3_TILES || method == EIK3_HEAP) return method;
  return order == 1 ? EIK3_HEAP : EIK3_TILES;
}

unsigned eik3_heap_cap(int nx, int ny, int nz) {
  // the live narrow band with its stale entries stays far below half the
  // nodes (measured: under 3% on 101x101x51 grids); overflow is an error
  const size_t nn = (size_t)nx * ny * nz;
  return (unsigned)std::max<size_t>(64, nn / 2);
}

size_t eik3_heap_bytes_per_solve(int nx, int ny, int nz) {
  const size_t nn = (size_t)nx * ny * nz;
  const size_t cap = eik3_heap_cap(nx, ny, nz);
  return carve_size({sizeof(double) * nn, nn, sizeof(double) * cap, sizeof(unsigned) * cap,
                     2 * sizeof(unsigned) * nn});
}

void eik3_heap_take(Eik3Job &job, Carve &cv, int chunk) {
  const size_t nn = (size_t)job.nx * job.ny * job.nz;
  const size_t cap = eik3_heap_cap(job.nx, job.ny, job.nz);
  const size_t c = chunk > 0 ? (size_t)chunk : 0;
  job.ht = cv.take<double>(nn * c);
  job.hst = cv.take<unsigned char>(nn * c);
  job.hkey = cv.take<double>(cap * c);
  job.hid = cv.take<unsigned>(cap * c);
  job.hpos = cv.take<unsigned>(2 * nn * c);
  job.hchunk = chunk; job.hcap = (unsigned)cap;
}

size_t eik3_heap_scratch_bytes(int nx, int ny, int nz, int chunk) {
  const size_t nn = (size_t)nx * ny * nz;
  const size_t cap = eik3_heap_cap(nx, ny, nz);
  const size_t c = chunk > 0 ? (size_t)chunk : 0;
  return carve_size({sizeof(double) * nn * c, nn * c, sizeof(double) * cap * c, sizeof(unsigned) * cap * c,
                     2 * sizeof(unsigned) * nn * c});
}

int launch_eik3_heap(Eik3Job &job, cudaStream_t s, double *tfield) {
  const size_t nn = (size_t)job.nx * job.ny * job.nz;
  if (nn > (size_t)kIdMask || job.hchunk < 1 || job.hcap < 8) {
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
    heap_fill_kernel<<<1024, 256, 0, s>>>(job.ht, job.hst, reinterpret_cast<uint2 *>(job.hpos), nn * nsol);
    MCT_CUDA_TRY(cudaGetLastError());
    int rc = launch_march(job, s0, nsol, s);
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

// Diagnostics (not part of the public header): lane-group / subtree-depth
// variant of the heap march (0: 8 lanes, 5 levels; 1: 8/4; 2: 16/5; 3: 32/5;
// 4: 16/4; 5: 8/3; -1: chosen by the number of solves); returns the previous
// value.
extern "C" int mct_debug_eik3_heap_variant(int v) {
  const int old = g_variant;
  if (v >= -1 && v <= 5) g_variant = v;
  return old;
}

// Diagnostics (not part of the public header): at most n solves per heap
// march launch (0: no cap); returns the previous value.
extern "C" int mct_debug_eik3_heap_chunk(int n) {
  const int old = g_chunk_cap;
  g_chunk_cap = n > 0 ? n : 0;
  return old;
}

// Diagnostics (not part of the public header): evaluates count random
// front-like stencils with both the reference-order FP64 update and the
// update the march uses (Markstein divisions, integer comparisons) and
// counts results whose bits differ (out[0]) and finite results (out[1]).
extern "C" int mct_debug_eik3_update_check(int order, double dx, double dy, double dz, unsigned long long count,
                                           unsigned long long seed, unsigned long long *out) {
  Axes ax;
  const double h[3] = {dx, dy, dz};
  for (int q = 0; q < 3; ++q) {
    ax.h[q] = h[q];
    ax.a1[q] = 1.0 / (h[q] * h[q]);
    ax.a2[q] = 9.0 / 4.0 / (h[q] * h[q]);
  }
  unsigned long long *d = nullptr;
  MCT_CUDA_TRY(cudaMalloc(&d, 2 * sizeof(unsigned long long)));
  MCT_CUDA_TRY(cudaMemset(d, 0, 2 * sizeof(unsigned long long)));
  update_check_kernel<<<152 * 8, 256>>>(order, ax, count, seed, d);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(out, d, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  cudaFree(d);
  MCT_CUDA_TRY(e);
  return MCT_OK;
}
