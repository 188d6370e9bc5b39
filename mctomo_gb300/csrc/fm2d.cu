// 2D first-arrival travel times: the GPU replacement of fm2d's modrays
// (fm2d/fm2dray_cartesian.f90:67-480) with gridder (491-600), bsplrefine
// (608-674), srtimes (682-797) and the fast marching core travel / fouds1 /
// fouds2 / addtree / downtree / updtree (fm2d/fm2d_ttime.f90:41-680).
//
// fm2d's mixed-order scheme (fouds2) consults only "alive" neighbours, so its
// result depends on the order in which the narrow band is accepted. To give
// the reference's travel times rather than a different discretisation, each
// solve runs the reference's own marching order: one warp per (velocity map,
// source), the narrow band kept in the reference's binary heap in shared
// memory (lane 0 performs the sifts in the reference's sequence, so ties break
// identically), and the up-to-four neighbour updates of each accepted node
// computed by 16 lanes at once, one stencil combination each (they read only
// accepted nodes and are independent). The refined source grid with its early exit at the box edge,
// the refined-to-coarse mapping and the narrow-band repair follow modrays.
// Arithmetic follows the Fortran expression order; the file is built with
// -fmad=false so nothing is fused.
#include "mct_common.cuh"
#include "fm2d.cuh"
#include "exact_sqrt.cuh"
#include <algorithm>
#include <climits>
#include <type_traits>
#include <utility>
#include <vector>

namespace {


struct Grid2 {
  int nnx, nnz, ld;
  double gox, goz, dnx, dnz;
};

// Per-solve shared-memory state. TT is double (FP64 times, precision 0 and 1)
// or int (fixed-point times in units of 2^-shift s, precision 2).
struct CaseTab;
template <class TT> struct WarpStateT {
  TT *T;              // [ld * cols]
  CaseTab *tab;       // [8] per-case constants of the FP64 update (precision 0)
  short *S;           // node status: -1 far, 0 alive, >0 heap position
  unsigned short *H;  // heap, 1-based: H[p] = packed node ((ix-1) << 8) | (iz-1)
  int ntr;
  int ld;
  int cap;            // heap capacity (entries)
  bool overflow;      // a node did not fit: the solve is abandoned and redone
};
using WarpState = WarpStateT<double>;

__device__ __forceinline__ int lin(const Grid2 &g, int iz, int ix) { return (iz - 1) + g.ld * (ix - 1); }
__device__ __forceinline__ unsigned short pack(int iz, int ix) { return (unsigned short)(((ix - 1) << 8) | (iz - 1)); }
template <class TT> __device__ __forceinline__ int plin(const WarpStateT<TT> &w, int p) { return (p & 255) + w.ld * (p >> 8); }

// Travel times are finite and non-negative, so the IEEE bit patterns of the
// FP64 times order exactly like the values: the heap compares them on the
// integer pipe. Fixed-point times compare directly.
__device__ __forceinline__ bool tlt(double a, double b) { return __double_as_longlong(a) < __double_as_longlong(b); }
__device__ __forceinline__ bool tlt(int a, int b) { return a < b; }
// double-float times (hi, lo) are normalised, so they order lexicographically
__device__ __forceinline__ bool tlt(float2 a, float2 b) { return a.x < b.x || (a.x == b.x && a.y < b.y); }

// ---- binary heap (fm2d_ttime.f90:527-680), lane 0 only --------------------
// The reference swaps the moving node with its parent (addtree, updtree) or
// its smaller child (downtree) level by level. Moving a hole instead and
// writing the node once at its final position visits the same positions with
// the same comparisons (the moving node's time is fixed during a sift), so
// the heap ends in the identical state; the moving node's time stays in a
// register and the two child ids are read with one 32-bit load.
template <class TT>
__device__ __forceinline__ void sift_up(WarpStateT<TT> &w, int me, unsigned short pm, int pos, TT tme) {
  int tpc = pos, tpp = tpc >> 1;
  while (tpp > 0) {
    const int pp = w.H[tpp];
    const int pn = plin(w, pp);
    if (!tlt(tme, w.T[pn])) break;
    w.H[tpc] = (unsigned short)pp;
    w.S[pn] = (short)tpc;
    tpc = tpp; tpp = tpc >> 1;
  }
  w.H[tpc] = pm;
  w.S[me] = (short)tpc;
}

// addtree: a far node joins the heap with time tme (already stored in T)
template <class TT>
__device__ __forceinline__ void addtree(WarpStateT<TT> &w, const Grid2 &g, int iz, int ix, TT tme) {
  if (w.ntr >= w.cap) { w.overflow = true; return; }
  w.ntr = w.ntr + 1;
  sift_up(w, lin(g, iz, ix), pack(iz, ix), w.ntr, tme);
}
template <class TT>
__device__ __forceinline__ void addtree(WarpStateT<TT> &w, const Grid2 &g, int iz, int ix) {
  addtree(w, g, iz, ix, w.T[lin(g, iz, ix)]);
}

// updtree: a close node's time decreased to tme
template <class TT>
__device__ __forceinline__ void updtree(WarpStateT<TT> &w, const Grid2 &g, int iz, int ix, TT tme) {
  const int me = lin(g, iz, ix);
  sift_up(w, me, pack(iz, ix), w.S[me], tme);
}

// downtree: remove the root (already marked alive by the caller). The ids
// of both possible next-level child pairs are fetched (one 64-bit load)
// while the current children's times are compared.
template <class TT>
__device__ void downtree(WarpStateT<TT> &w) {
  if (w.ntr == 1) { w.ntr = 0; return; }
  const int lastp = w.H[w.ntr];
  const int ln = plin(w, lastp);
  w.ntr = w.ntr - 1;
  const int ntr = w.ntr;
  const TT key = w.T[ln];
  int hole = 1, c = 2;
  unsigned pair = c < ntr ? reinterpret_cast<const unsigned *>(w.H)[1] : 0u;   // H[2], H[3]
  while (c < ntr) {
    const int p1 = (int)(pair & 0xffffu), p2 = (int)(pair >> 16);
    const int n1 = plin(w, p1), n2 = plin(w, p2);
    const TT k1 = w.T[n1], k2 = w.T[n2];
    // H[2c], H[2c+1] (children of c) and H[2c+2], H[2c+3] (children of c+1)
    const unsigned long long quad =
        2 * c < ntr ? reinterpret_cast<const unsigned long long *>(w.H)[c >> 1] : 0ull;
    const bool right = tlt(k2, k1);
    const int cp = right ? p2 : p1, cn = right ? n2 : n1, cc = c + (right ? 1 : 0);
    if (!tlt(right ? k2 : k1, key)) { c = ntr + 1; break; }
    w.H[hole] = (unsigned short)cp;
    w.S[cn] = (short)hole;
    hole = cc; c = 2 * hole;
    pair = right ? (unsigned)(quad >> 32) : (unsigned)quad;
  }
  if (c == ntr) {
    const int cp = w.H[c];
    const int cn = plin(w, cp);
    if (tlt(w.T[cn], key)) {
      w.H[hole] = (unsigned short)cp;
      w.S[cn] = (short)hole;
      hole = c;
    }
  }
  w.H[hole] = (unsigned short)lastp;
  w.S[ln] = (short)hole;
}

// Shared-memory layout of one solve: S [n], H [cap + 2] (1-based heap of at
// most cap entries), each array starting on a 16-byte boundary. The solve's
// time field T [n] lives in global memory (a slot of Fm2dJob::tws_ref / tws
// per resident solve), where it stays in L1/L2: with 8 of every 10 bytes per
// node out of shared memory, twice as many solves fit on an SM, and the
// march is bound by the per-solve latency, which more solves per SM hide.
__host__ __device__ __forceinline__ int align16(int b) { return (b + 15) & ~15; }
// ... then the 8 per-case constant records of the FP64 update (CaseTab, 64 B
// each).
constexpr int CASE_TAB_BYTES = 8 * 64;
constexpr int MAILBOX_BYTES = 128;   // ... and the solve's mailbox (last 128 B, see march)
struct SolveLayout { int offS, offH, offTab, bytes; };
__host__ __device__ __forceinline__ SolveLayout solve_layout(int n, int cap, bool sglobal) {
  SolveLayout L;
  L.offS = 0;
  L.offH = sglobal ? 0 : L.offS + align16(2 * n);
  L.offTab = L.offH + align16(2 * (cap + 2));
  L.bytes = L.offTab + CASE_TAB_BYTES + MAILBOX_BYTES;
  return L;
}
// A time-field slot of n nodes: the times (elements of T bytes), then, when
// the node states are kept in global memory too, the states (int16).
__host__ __device__ __forceinline__ size_t slot_bytes(int n, int tbytes, bool sglobal) {
  return (((size_t)n * tbytes + 15) & ~size_t(15)) + (sglobal ? (((size_t)n * 2 + 15) & ~size_t(15)) : 0);
}
// Heap capacity of the refined source-box stage. The heap holds the narrow
// band, a closed front around the source (a few hundred nodes on the largest
// box), so a capacity well below the node count frees shared memory for more
// resident solves; a solve whose band outgrows it is redone with a full-size
// heap (see the overflow pass below).
constexpr int REFINED_HEAP_CAP = 1024;

// ---- upwind arithmetic ------------------------------------------------------

// Double-float variant (precision == 1): times are unevaluated sums of two
// FP32 numbers (hi + lo, |lo| <= ulp(hi)/2) and every operation of the
// reference's update is carried out in that format with error-free
// transformations (Knuth's two-sum, the two-product via fmaf, division and
// square root from a hardware reciprocal / reciprocal-square-root estimate
// refined by exact remainders), giving about 2^-46 relative precision on the
// FP32 pipe. Results agree with the FP64 reference to ~1e-12 s, so the
// acceptance order only differs on ties closer than that.
struct DF { float hi, lo; };
__device__ __forceinline__ DF df(float a) { return DF{a, 0.f}; }
__device__ __forceinline__ DF df_from(double d) { float h = (float)d; return DF{h, (float)(d - (double)h)}; }
__device__ __forceinline__ DF two_sum(float a, float b) {
  float s = a + b, bb = s - a;
  return DF{s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ DF quick_two_sum(float a, float b) {
  float s = a + b;
  return DF{s, b - (s - a)};
}
__device__ __forceinline__ DF dadd(DF a, DF b) {
  DF s = two_sum(a.hi, b.hi), t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = quick_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return quick_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ DF dneg(DF a) { return DF{-a.hi, -a.lo}; }
__device__ __forceinline__ DF dsub(DF a, DF b) { return dadd(a, dneg(b)); }
__device__ __forceinline__ DF dmul(DF a, DF b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return quick_two_sum(p, e);
}
__device__ __forceinline__ DF dmulf(DF a, float f) {
  const float p = a.hi * f;
  float e = fmaf(a.hi, f, -p);
  e = fmaf(a.lo, f, e);
  return quick_two_sum(p, e);
}
// a / b: quotient digits from an approximate reciprocal of b.hi (relative
// error ~2^-22), each followed by the exact remainder a - b*q; three digits
// reach double-float accuracy.
__device__ __forceinline__ DF ddiv(DF a, DF b) {
  const float r = __fdividef(1.f, b.hi);
  const float q1 = a.hi * r;
  DF rem = dsub(a, dmulf(b, q1));
  const float q2 = rem.hi * r;
  rem = dsub(rem, dmulf(b, q2));
  const float q3 = rem.hi * r;
  return dadd(quick_two_sum(q1, q2), df(q3));
}
// sqrt(a): the correctly rounded FP32 root of a.hi plus one correction
// (a - y^2) / (2y) from the exact remainder, the halved reciprocal square
// root standing in for 1 / (2y).
__device__ __forceinline__ DF dsqrt(DF a) {
  const bool pos = a.hi > 0.f;
  const float x = pos ? a.hi : 1.f;
  const float y = sqrtf(x);
  const float h = 0.5f * rsqrtf(x);
  const float p = y * y, e = fmaf(y, y, -p);
  const DF rem = dsub(pos ? a : df(1.f), DF{p, e});
  const DF r = quick_two_sum(y, rem.hi * h);
  return pos ? r : df(0.f);
}
__device__ __forceinline__ DF f2df(float2 v) { return DF{v.x, v.y}; }



// Fixed-point variant (precision == 2): times are int32 in units of
// 2^-shift s, each update's quadratic is solved in FP32 on the neighbours'
// times relative to a nearby accepted time, and the result is rounded back to
// the fixed-point grid. The stencils and case selection are fouds1/fouds2's.
struct Fx { float scale, inv; };

template <class TT> __device__ __forceinline__ TT from_double(double t, const Fx &fx);
template <> __device__ __forceinline__ double from_double<double>(double t, const Fx &) { return t; }
template <> __device__ __forceinline__ float2 from_double<float2>(double t, const Fx &) {
  float h = (float)t; return make_float2(h, (float)(t - (double)h));
}
template <> __device__ __forceinline__ int from_double<int>(double t, const Fx &fx) {
  return (int)min(llrint(t * (double)fx.scale), (long long)INT_MAX - 1);
}
__device__ __forceinline__ double to_double(double t, const Fx &) { return t; }
__device__ __forceinline__ double to_double(float2 t, const Fx &) { return (double)t.x + (double)t.y; }
__device__ __forceinline__ double to_double(int t, const Fx &fx) { return (double)t * (double)fx.inv; }

// ---- upwind updates (fm2d_ttime.f90:248-518) ------------------------------
// fouds1 / fouds2 give the node being updated the minimum, over its four
// (x-neighbour j, z-neighbour k) combinations, of the solution of that
// combination's local stencil. The combinations are independent of each other
// and of the order of evaluation, so a warp evaluates the 16 combinations of
// an accepted node's four neighbours at once (one per lane) and takes the
// minimum over each group of four lanes: the minimum of the same candidate
// values, hence the reference's result.
//
// Per combination, X = 2 if the x term is second order (j and the next node
// j2 beyond it are accepted and T(j2) < T(j)), 1 if only j is accepted, 0
// otherwise; Z likewise along z (second order only with fom = 1). Every
// two-term case of fouds1/fouds2 solves
//     a = vv + m*uu,  b = (kb*em)*uu,  c = uu*(em*em - s^2*vv)
// with (uu, vv, m, kb, em, tref, tdiv) set per case, and every one-term case
// a = 1, b = 0, c = -(uu*s^2); the operand order below is the reference's
// (scaling by 2 and negation are exact, so (2*em)*uu with em = Tj - Tk is
// bit-identical to the reference's -(2*uu*em) with em = Tk - Tj).
template <class TT> struct Stencil {
  int X, Z;                 // order of the x and z terms (0, 1, 2)
  TT Tj, Tj2, Tk, Tk2;      // times of nodes j, j2 (along x) and k, k2 (along z)
};

// Combination cmb (0..3) of node (iz, ix): j = ix -/+ 1, k = iz -/+ 1.
// Returns false when the reference skips it (j or k off the grid, neither
// accepted). Node curl (the node being accepted, which the heap warp may not
// have marked yet) counts as accepted with time tcur; it can only be j or k.
// A second-order node's time is used only when that node is accepted; the
// times of unused nodes are not read.
template <class TT>
__device__ __forceinline__ bool combo_stencil(const WarpStateT<TT> &w, const Grid2 &g, int iz, int ix, int cmb,
                                              int fom, int curl, TT tcur, Stencil<TT> &s) {
  const int dj = cmb < 2 ? -1 : 1, dk = (cmb & 1) ? 1 : -1;
  const int j = ix + dj, k = iz + dk;
  if (j < 1 || j > g.nnx || k < 1 || k > g.nnz) return false;
  const int lj = lin(g, iz, j), lk = lin(g, k, ix);
  const bool jcur = lj == curl, kcur = lk == curl;
  const bool jal = jcur || w.S[lj] == 0, kal = kcur || w.S[lk] == 0;
  if (!jal && !kal) return false;
  s.X = jal ? 1 : 0; s.Z = kal ? 1 : 0;
  s.Tj = jal ? (jcur ? tcur : w.T[lj]) : TT();
  s.Tk = kal ? (kcur ? tcur : w.T[lk]) : TT();
  s.Tj2 = s.Tj; s.Tk2 = s.Tk;
  if (fom == 1) {
    const int j2 = j + dj, k2 = k + dk;
    if (jal && j2 >= 1 && j2 <= g.nnx) {
      const int l2 = lin(g, iz, j2);
      if (w.S[l2] == 0) {
        const TT t2 = w.T[l2];
        if (tlt(t2, s.Tj)) { s.X = 2; s.Tj2 = t2; }
      }
    }
    if (kal && k2 >= 1 && k2 <= g.nnz) {
      const int l2 = lin(g, k2, ix);
      if (w.S[l2] == 0) {
        const TT t2 = w.T[l2];
        if (tlt(t2, s.Tk)) { s.Z = 2; s.Tk2 = t2; }
      }
    }
  }
  return true;
}


// Node slowness as each mode consumes it: FP64 (precision 0), an FP32 pair
// (precision 1) or FP32 (precision 2), stored in the same 8-byte slots.
template <class TT> struct SlowOf { using type = double; };
template <> struct SlowOf<float2> { using type = float2; };
template <> struct SlowOf<int> { using type = float; };
template <class TT> using SlowT = typename SlowOf<TT>::type;
__device__ __forceinline__ void store_slowness(double *base, size_t i, double s, int precision) {
  if (precision == 1) {
    const float h = (float)s;
    reinterpret_cast<float2 *>(base)[i] = make_float2(h, (float)(s - (double)h));
  } else if (precision == 2) {
    reinterpret_cast<float *>(base)[i] = (float)s;
  } else {
    base[i] = s;
  }
}

// Per-march constants of the reduced-precision updates. Every two-term case
// is a W^2 + 2 B W + c = 0 with a = vv + m uu fixed by the grid spacing, so a
// and 1/a are computed once per march for the four cases (X, Z) = (2, 2),
// (2, 1), (1, 2), (1, 1); the root is then (-B + sqrt(B^2 - a c)) / a with
// no division. A one-term case (alpha T - R)^2 / h^2 = s^2 has the root
// T = (R + h s) / alpha, again without a division or a square root.
template <class TT> struct UpdConst {
  __device__ void init(const Grid2 &) {}
};
// FP64 (precision 0). Every case of fouds1 / fouds2 is evaluated by one
// straight-line sequence, so the 16 lanes of a warp run the FP64 operations
// once whatever mix of cases they hold (GB300 issues two FP64 lanes per cycle
// per SM and charges an FP64 warp instruction the same whatever its active
// lanes). The sequence performs, for each case, exactly the reference's FP64
// operations in its order, with per-case operands from a table (CaseTab) in
// the solve's shared memory:
//   P = A1 B1 - C1            (4 Tj - Tj2, 3 Tk, 3 Tj, Tj, 4 Tk - Tk2, Tk)
//   em = (P - Q) + R          (two-term cases; 0 otherwise)
//   b = (kb em) uu,  c = uu (em em - ss vv),  rd1 = b b - (4a) c
//   t = tref + (-b + sqrt(max(rd1, 0))) / (2a),  t / 3 for second-order
//   one-term cases
// with a = vv + m uu per two-term case and a = 1 for one-term cases, whose
// c = -(uu ss) the same sequence gives as uu (0 - ss 1). Multiplying by 1 or
// subtracting 0 is exact, so P and em equal the reference's tref / em.
// Divisions by 2a and by 3 take Markstein's correction (P. Markstein,
// "Computation of elementary functions on the IBM RISC System/6000
// processor", IBM J. Res. Dev. 34(1), 1990): with yinv = RN(1/y),
// q = RN(x yinv), r = x - q y (exact with a fused multiply-add), RN(q + r
// yinv) is the correctly rounded x / y. The square root is exact_sqrt_rn
// (integer and FP32 pipes, the same bits as the library's).
struct CaseTab {
  double uu, vv, kb, fa, ta, ra;   // uu, vv, kb; 4a, 2a, RN(1/(2a))
  int third;                       // the result is divided by 3
  int pad[3];
};
// Case codes: two-term (X, Z) = (2, 2) 0, (2, 1) 1, (1, 2) 2, (1, 1) 3;
// one-term X = 2: 4, X = 1: 5, Z = 2: 6, Z = 1: 7.
__device__ __forceinline__ void build_case_tab(CaseTab *tab, const Grid2 &g, int lane) {
  if (lane < 8) {
    const double u2x = 2.0 * g.dnx, u2z = 2.0 * g.dnz;
    const double hx1 = g.dnx * g.dnx, hz1 = g.dnz * g.dnz, hx2 = u2x * u2x, hz2 = u2z * u2z;
    CaseTab t;
    switch (lane) {   // uu, vv of fm2d_ttime.f90's cases
      case 0: t.uu = hx2; t.vv = hz2; break;
      case 1: t.uu = hz1; t.vv = hx2; break;
      case 2: t.uu = hx1; t.vv = hz2; break;
      case 3: t.uu = hx1; t.vv = hz1; break;
      case 4: t.uu = hx2; t.vv = 1.0; break;
      case 5: t.uu = hx1; t.vv = 1.0; break;
      case 6: t.uu = hz2; t.vv = 1.0; break;
      default: t.uu = hz1; t.vv = 1.0; break;
    }
    const bool m9 = lane == 1 || lane == 2;
    t.kb = m9 ? 6.0 : 2.0;
    const double a = lane < 4 ? t.vv + (m9 ? 9.0 : 1.0) * t.uu : 1.0;
    t.fa = 4.0 * a; t.ta = 2.0 * a; t.ra = 1.0 / (2.0 * a);
    t.third = (lane == 0 || lane == 4 || lane == 6) ? 1 : 0;
    t.pad[0] = t.pad[1] = t.pad[2] = 0;
    tab[lane] = t;
  }
}
template <> struct UpdConst<double> {
  __device__ void init(const Grid2 &) {}
};
__device__ __forceinline__ double div_known(double x, double y, double yinv) {
  const double q = __dmul_rn(x, yinv);
  const double r = __fma_rn(-q, y, x);
  return __fma_rn(r, yinv, q);
}
template <> struct UpdConst<float2> {
  DF dnx, dnz, hx1, hz1, a[4], ia[4];
  __device__ void init(const Grid2 &g) {
    dnx = df_from(g.dnx); dnz = df_from(g.dnz);
    hx1 = dmul(dnx, dnx); hz1 = dmul(dnz, dnz);
    const DF hx2 = dmulf(hx1, 4.f), hz2 = dmulf(hz1, 4.f);
    a[0] = dadd(hz2, hx2);
    a[1] = dadd(hx2, dmulf(hz1, 9.f));
    a[2] = dadd(hz2, dmulf(hx1, 9.f));
    a[3] = dadd(hz1, hx1);
#pragma unroll
    for (int i = 0; i < 4; ++i) ia[i] = ddiv(df(1.f), a[i]);
  }
};
template <> struct UpdConst<int> {
  float dnx, dnz, a[4], ia[4];
  __device__ void init(const Grid2 &g) {
    dnx = (float)g.dnx; dnz = (float)g.dnz;
    const float hx1 = dnx * dnx, hz1 = dnz * dnz;
    a[0] = 4.f * hz1 + 4.f * hx1;
    a[1] = 4.f * hx1 + 9.f * hz1;
    a[2] = 4.f * hz1 + 9.f * hx1;
    a[3] = hz1 + hx1;
#pragma unroll
    for (int i = 0; i < 4; ++i) ia[i] = 1.f / a[i];
  }
};

// FP64, the reference's arithmetic (precision 0). slown is the node's
// slowness 1/V, precomputed per node with the reference's division.
__device__ double combo_time(const WarpStateT<double> &w, const Grid2 &g, const Stencil<double> &s, double slown,
                             int fom, const Fx &, const UpdConst<double> &) {
  const double ss = slown * slown;
  const double Tj = s.Tj, Tk = s.Tk, Tj2 = s.Tj2, Tk2 = s.Tk2;
  const int X = s.X, Z = s.Z;
  const bool two = X != 0 && Z != 0;
  const int cc = two ? ((X == 2) ? (Z == 2 ? 0 : 1) : (Z == 2 ? 2 : 3)) : (X ? (X == 2 ? 4 : 5) : (Z == 2 ? 6 : 7));
  const CaseTab &t = w.tab[cc];
  // P = A1 B1 - C1: 0, 4: 4 Tj - Tj2; 1: 3 Tk; 2: 3 Tj; 3, 5: Tj; 6: 4 Tk - Tk2; 7: Tk
  const double A1 = (cc == 0 || cc == 4 || cc == 6) ? 4.0 : ((cc == 1 || cc == 2) ? 3.0 : 1.0);
  const double B1 = (cc == 1 || cc >= 6) ? Tk : Tj;
  const double C1 = (cc == 0 || cc == 4) ? Tj2 : (cc == 6 ? Tk2 : 0.0);
  const double P = A1 * B1 - C1;
  // em = (P - Q) + R: 0: 4 Tk, Tk2; 1: 4 Tj, Tj2; 2: 4 Tk, Tk2; 3: Tk, 0
  const double Q = two ? (cc == 3 ? 1.0 : 4.0) * (cc == 1 ? Tj : Tk) : 0.0;
  const double R = two ? (cc == 1 ? Tj2 : (cc == 3 ? 0.0 : Tk2)) : 0.0;
  const double em = ((two ? P : 0.0) - Q) + R;
  const double tref = cc == 1 ? Tk : ((cc == 2 || cc == 3) ? Tj : P);
  const double b = (t.kb * em) * t.uu;
  double c = t.uu * (em * em - ss * t.vv);
  if (fom == 0 && cc == 7) {   // first-order z-only stencil of fouds1
    const double sd = slown * g.dnz;
    c = -(sd * sd);
  }
  double rd1 = b * b - t.fa * c;
  if (__double_as_longlong(rd1) < 0) rd1 = 0.0;   // rd1 < 0 (rd1 is never -0 or NaN)
  const double tt = tref + div_known(-b + exact_sqrt_rn(rd1), t.ta, t.ra);
  const double t3 = div_known(tt, 3.0, 1.0 / 3.0);
  return t.third ? t3 : tt;
}

// Double-float (precision 1): the same cases and stencils in FP32-pair
// arithmetic, written as one branch-free formula so that the 16 lanes do not
// serialise over the cases. With R = 4 T1 - T2 (second order, alpha = 3) or
// R = T1 (first order, alpha = 1) per axis, the pivot axis p is x unless x is
// unused or x is second order and z first order; W = alpha_p T - R_p solves
//   a W^2 + 2 B W + c = 0,  B = k e uu,  c = uu (e^2 - s^2 vv),  e = k R_p - R_q,
// k = alpha_q / alpha_p (0 for one term, whose a = vv = 1), uu and vv the
// squared stencil spacings of p and q; T = (R_p + W) / alpha_p.
__device__ float2 combo_time(const WarpStateT<float2> &, const Grid2 &, const Stencil<float2> &s, float2 sl, int,
                             const Fx &, const UpdConst<float2> &K) {
  const DF slown = f2df(sl);
  const DF Tj = f2df(s.Tj), Tk = f2df(s.Tk);
  const DF Rx2 = dsub(dmulf(Tj, 4.f), f2df(s.Tj2));
  const DF Rz2 = dsub(dmulf(Tk, 4.f), f2df(s.Tk2));
  const DF Rx = s.X == 2 ? Rx2 : Tj, Rz = s.Z == 2 ? Rz2 : Tk;
  const bool two = s.X != 0 && s.Z != 0;
  const bool pz = s.X == 0 || (s.X == 2 && s.Z == 1);
  const int op = pz ? s.Z : s.X;
  const DF Rp = pz ? Rz : Rx, Rq = pz ? Rx : Rz;
  const DF hx = s.X == 2 ? dmulf(K.hx1, 4.f) : K.hx1, hz = s.Z == 2 ? dmulf(K.hz1, 4.f) : K.hz1;
  const DF uu = pz ? hz : hx;
  const DF vv = two ? (pz ? hx : hz) : df(1.f);
  const float k = two ? (s.X == s.Z ? 1.f : 3.f) : 0.f;
  const int ci = (s.X == 2) ? (s.Z == 2 ? 0 : 1) : (s.Z == 2 ? 2 : 3);
  const DF A = !two ? df(1.f) : ci == 0 ? K.a[0] : ci == 1 ? K.a[1] : ci == 2 ? K.a[2] : K.a[3];
  const DF IA = !two ? df(1.f) : ci == 0 ? K.ia[0] : ci == 1 ? K.ia[1] : ci == 2 ? K.ia[2] : K.ia[3];
  const DF e = two ? dsub(dmulf(Rp, k), Rq) : df(0.f);
  const DF B = dmulf(dmul(e, uu), k);
  // B^2 - A c with A = vv + k^2 uu (every case's a) and c = uu (e^2 - s^2 vv)
  // is uu vv (A s^2 - e^2): the same discriminant without the cancellation
  // of B^2 against A c, and a shorter dependent chain
  DF disc = dmul(dmul(uu, vv), dsub(dmul(A, dmul(slown, slown)), dmul(e, e)));
  if (disc.hi < 0.f) disc = df(0.f);
  DF trav = dadd(Rp, dmul(dsub(dsqrt(disc), B), IA));
  trav = dmul(trav, op == 2 ? df_from(1.0 / 3.0) : df(1.f));
  return make_float2(trav.hi, trav.lo);
}

// Fixed point (precision 2): the same cases in FP32 on times taken relative
// to the combination's first accepted neighbour, rounded back to the
// fixed-point grid.
__device__ int combo_time(const WarpStateT<int> &, const Grid2 &, const Stencil<int> &s, float sl, int,
                          const Fx &fx, const UpdConst<int> &K) {
  const float slown = sl;
  const int base = s.X ? s.Tj : s.Tk;
  auto sh = [&](int t) { return (float)(t - base) * fx.inv; };
  const float Tj = sh(s.Tj), Tk = sh(s.Tk);
  float trav;
  bool third = false;
  if (s.X && s.Z) {
    float uu, vv, em, tref, A, IA, k = 1.f;
    const float hx1 = K.dnx * K.dnx, hz1 = K.dnz * K.dnz;
    if (s.X == 2 && s.Z == 2) {
      tref = 4.f * Tj - sh(s.Tj2);
      em = (tref - 4.f * Tk) + sh(s.Tk2);
      uu = 4.f * hx1; vv = 4.f * hz1; A = K.a[0]; IA = K.ia[0]; third = true;
    } else if (s.X == 2) {
      em = (3.f * Tk - 4.f * Tj) + sh(s.Tj2);
      uu = hz1; vv = 4.f * hx1; k = 3.f; A = K.a[1]; IA = K.ia[1]; tref = Tk;
    } else if (s.Z == 2) {
      em = (3.f * Tj - 4.f * Tk) + sh(s.Tk2);
      uu = hx1; vv = 4.f * hz1; k = 3.f; A = K.a[2]; IA = K.ia[2]; tref = Tj;
    } else {
      em = Tj - Tk;
      uu = hx1; vv = hz1; A = K.a[3]; IA = K.ia[3]; tref = Tj;
    }
    const float B = k * (em * uu);
    const float c = uu * (em * em - (slown * slown) * vv);
    float disc = B * B - A * c;
    if (disc < 0.f) disc = 0.f;
    trav = tref + (sqrtf(disc) - B) * IA;
  } else {
    float tref, h;
    if (s.X) {
      if (s.X == 2) { tref = 4.f * Tj - sh(s.Tj2); h = 2.f * K.dnx; third = true; }
      else { tref = Tj; h = K.dnx; }
    } else {
      if (s.Z == 2) { tref = 4.f * Tk - sh(s.Tk2); h = 2.f * K.dnz; third = true; }
      else { tref = Tk; h = K.dnz; }
    }
    trav = tref + h * slown;
  }
  if (third) trav = trav * (1.f / 3.f);
  long long r = (long long)base + llrintf(trav * fx.scale);
  return (int)min(max(r, 0LL), (long long)INT_MAX - 1);
}

// "no candidate" value for the group minimum, above every time
__device__ __forceinline__ double time_inf(double) { return __longlong_as_double(0x7ff0000000000000LL); }
__device__ __forceinline__ float2 time_inf(float2) { return make_float2(__int_as_float(0x7f800000), 0.f); }
__device__ __forceinline__ int time_inf(int) { return INT_MAX; }
__device__ __forceinline__ double shfl_xor_time(unsigned mk, double v, int m) { return __shfl_xor_sync(mk, v, m); }
__device__ __forceinline__ int shfl_xor_time(unsigned mk, int v, int m) { return __shfl_xor_sync(mk, v, m); }
__device__ __forceinline__ float2 shfl_xor_time(unsigned mk, float2 v, int m) {
  return make_float2(__shfl_xor_sync(mk, v.x, m), __shfl_xor_sync(mk, v.y, m));
}
__device__ __forceinline__ double shfl_time(unsigned mk, double v, int src) { return __shfl_sync(mk, v, src); }
__device__ __forceinline__ int shfl_time(unsigned mk, int v, int src) { return __shfl_sync(mk, v, src); }
__device__ __forceinline__ float2 shfl_time(unsigned mk, float2 v, int src) {
  return make_float2(__shfl_sync(mk, v.x, src), __shfl_sync(mk, v.y, src));
}

// Exact 8-byte round trip of a time through the mapping scratch.
__device__ __forceinline__ double bit_store(double t) { return t; }
__device__ __forceinline__ double bit_store(int t) { return (double)t; }
__device__ __forceinline__ double bit_store(float2 t) {
  return __longlong_as_double(((long long)__float_as_uint(t.y) << 32) | __float_as_uint(t.x));
}
template <class TT> __device__ __forceinline__ TT bit_load(double v);
template <> __device__ __forceinline__ double bit_load<double>(double v) { return v; }
template <> __device__ __forceinline__ int bit_load<int>(double v) { return (int)v; }
template <> __device__ __forceinline__ float2 bit_load<float2>(double v) {
  unsigned long long b = (unsigned long long)__double_as_longlong(v);
  return make_float2(__uint_as_float((unsigned)(b & 0xffffffffu)), __uint_as_float((unsigned)(b >> 32)));
}

// fm2d_ttime.f90:682-711 bilinear
__device__ __forceinline__ double bilinear(const double nv[2][2], double dsx, double dsz, double dnx, double dnz) {
  double biv = 0.0;
  for (int i = 1; i <= 2; ++i)
    for (int j = 1; j <= 2; ++j) {
      double produ = (1.0 - fabs(((double)(i - 1) * dnx - dsx) / dnx)) *
                     (1.0 - fabs(((double)(j - 1) * dnz - dsz) / dnz));
      biv = biv + nv[i - 1][j - 1] * produ;
    }
  return biv;
}

// The marching loop of travel (fm2d_ttime.f90:137-237), run by a pair of
// warps per solve: the heap warp and the update warp.
//
// Per accepted node the reference pops the heap root, restores the heap
// (downtree), computes the new times of the root's up-to-four neighbours
// (fouds1/fouds2, which read only accepted nodes) and sifts them into the
// heap (addtree/updtree). Here the heap warp does all heap work (one lane per
// solve, in the reference's order, so ties break identically) while the
// update warp computes the neighbours' times (16 lanes per solve, one stencil
// combination each). The two overlap: while the heap warp sifts node i's
// neighbours and pops and restores the heap for node i+1, the update warp
// already evaluates node i+1's neighbours, for the node that it predicts will
// be the next root (the root left by downtree unless a sifted neighbour is
// strictly earlier). The heap warp then reports the node it actually popped;
// a wrong prediction (possible because fouds2 replaces, rather than lowers, a
// close node's time, which can leave the heap out of order) is recomputed
// before its results are used. The update warp writes nothing but the
// mailbox; the heap warp is the only writer of the times and states, and it
// changes no accepted node's time, so the update warp's reads (accepted
// nodes, plus the node being accepted, whose time comes with the
// prediction) see final values.
//
// Per step the warps exchange through the solve's mailbox and two named
// barriers (64 threads): bar1 after the heap warp's pop (node, new root,
// end flag), bar2 after the update warp's times. With two solves per pair
// (SPW = 2) the pair marches them in lockstep: heap lanes 0 and 16, update
// lanes 0-15 and 16-31, so the update's FP64 instructions serve both.
struct Trace { int *ti; double *tt; int max; int n; };

template <class TT> struct Mailbox {
  TT tn[4];     // update warp -> heap warp: new times of the accepted node's neighbours
  TT rkey;      // heap warp -> update warp: time of the heap root after the removal
  int cd[4];    // 1: neighbour k (x-1, x+1, z-1, z+1) takes tn[k]
  int cur;      // heap warp -> update warp: the node accepted in this step
  int root;     // the heap root after the removal, -1 if the heap is empty
  int stop;     // 0 marching, 1 ended, 2 ended by a heap overflow
};
constexpr int PAIRS_MAX = 7;   // named barriers 1..14: two per warp pair

__device__ __forceinline__ void pair_sync(int id) { asm volatile("bar.sync %0, 64;" ::"r"(id) : "memory"); }
__device__ __forceinline__ void pair_arrive(int id) { asm volatile("bar.arrive %0, 64;" ::"r"(id) : "memory"); }

// New times of the up-to-four neighbours of node cur (packed; its time tcur)
// by the 16 lanes of this half-warp: lane hl handles neighbour q = hl / 4 in
// the reference's order (x-1, x+1, z-1, z+1) and stencil combination hl % 4;
// the minimum over a neighbour's four lanes is fouds1/fouds2's result. On
// return every lane of the half holds tn[4] and cd[4] (cd 1: a neighbour on
// the grid that is not accepted).
template <class TT>
__device__ __forceinline__ void update_neighbours(const WarpStateT<TT> &w, const Grid2 &g, const SlowT<TT> *SL,
                                                  int sld, int fom, const Fx &fx, const UpdConst<TT> &K, int lane,
                                                  int cur, TT tcur, TT *tn, int *cd) {
  const int hl = lane & 15, hbase = lane & 16;
  const unsigned hmask = 0xFFFFu << hbase;
  const int q = hl >> 2, cmb = hl & 3;
  const int dqx = q == 0 ? -1 : (q == 1 ? 1 : 0), dqz = q == 2 ? -1 : (q == 3 ? 1 : 0);
  const int iz = (cur & 255) + 1, ix = (cur >> 8) + 1;
  const int curl = lin(g, iz, ix);
  const int nx_ = ix + dqx, nz_ = iz + dqz;
  const bool valid = nx_ >= 1 && nx_ <= g.nnx && nz_ >= 1 && nz_ <= g.nnz;
  bool open = false, have = false;
  TT cand = time_inf(TT());
  if (valid) {
    open = w.S[lin(g, nz_, nx_)] != 0;
    Stencil<TT> sc;
    if (open && combo_stencil(w, g, nz_, nx_, cmb, fom, curl, tcur, sc)) {
      have = true;
      cand = combo_time(w, g, sc, SL[(nz_ - 1) + (size_t)sld * (nx_ - 1)], fom, fx, K);
    }
  }
  const unsigned hb = __ballot_sync(hmask, have);
#pragma unroll
  for (int m = 1; m <= 2; m <<= 1) {
    const TT o = shfl_xor_time(hmask, cand, m);
    if (tlt(o, cand)) cand = o;
  }
  // a node with no usable combination gets 0, the reference's initial travm
  if (((hb >> (lane & ~3)) & 0xFu) == 0u) cand = TT();
  const int code = (valid && open) ? 1 : 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    cd[k] = __shfl_sync(hmask, code, hbase + 4 * k);
    tn[k] = shfl_time(hmask, cand, hbase + 4 * k);
  }
}

// march (fm2d_ttime.f90:137-237) for this thread's solve (state w, mailbox
// mb; active false without a solve), called by all threads of both warps of
// the pair. Only the halves with marches set (both with two solves per pair,
// the first with one) work on the solve. urg == 1 adds the refined-box exit
// test; vnr/vnb are compared with the current (refined) grid size exactly as
// the reference's module variables are at that point. Returns the end flag
// (2: heap overflow) to every thread of an active solve.
template <class TT>
__device__ int march(WarpStateT<TT> &w, Mailbox<TT> *mb, bool active, bool marches, const Grid2 &g,
                     const SlowT<TT> *SL, int sld, int fom, int urg, int vnl, int vnr, int vnt, int vnb, const Fx &fx,
                     int bar1, int bar2, Trace *tr) {
  const int t64 = threadIdx.x & 63, lane = t64 & 31, hbase = lane & 16;
  const bool leader = (lane & 15) == 0;
  UpdConst<TT> K;
  K.init(g);
  bool live = active && marches;
  if (t64 < 32) {
    // ---- heap warp: lanes 0 and 16 hold the solves' heaps
    for (;;) {
      if (leader && live) {
        int st = 0, cur = -1;
        if (w.overflow) {
          st = 2;
        } else if (w.ntr == 0) {
          st = 1;
        } else {
          const int top = w.H[1];
          const int iz = (top & 255) + 1, ix = (top >> 8) + 1;
          int swrg = 0;
          if (urg == 1) {
            if (ix == 1 && vnl != 1) swrg = 1;
            if (ix == g.nnx && vnr != g.nnx) swrg = 1;
            if (iz == 1 && vnt != 1) swrg = 1;
            if (iz == g.nnz && vnb != g.nnz) swrg = 1;
          }
          if (!swrg && tr && tr->n < tr->max) {
            tr->ti[3 * tr->n] = urg; tr->ti[3 * tr->n + 1] = lin(g, iz, ix); tr->ti[3 * tr->n + 2] = w.ntr;
            tr->tt[tr->n] = to_double(w.T[lin(g, iz, ix)], fx); tr->n++;
          }
          w.S[lin(g, iz, ix)] = 0;
          if (swrg) {
            st = 1;
          } else {
            downtree(w);
            cur = top;
          }
        }
        const int root = (st == 0 && w.ntr > 0) ? (int)w.H[1] : -1;
        mb->cur = cur;
        mb->root = root;
        mb->rkey = root >= 0 ? w.T[plin(w, root)] : TT();
        mb->stop = st;
        live = st == 0;
      }
      live = __shfl_sync(0xffffffffu, live, hbase);
      const bool any = __any_sync(0xffffffffu, live);
      pair_arrive(bar1);
      if (!any) break;
      pair_sync(bar2);
      if (leader && live) {
        const int cur = mb->cur;
        const int iz = (cur & 255) + 1, ix = (cur >> 8) + 1;
        const int qz[4] = {iz, iz, iz - 1, iz + 1}, qx[4] = {ix - 1, ix + 1, ix, ix};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          if (mb->cd[k] == 0) continue;
          const TT t = mb->tn[k];
          const int l = lin(g, qz[k], qx[k]);
          w.T[l] = t;
          if (w.S[l] == -1) addtree(w, g, qz[k], qx[k], t);
          else updtree(w, g, qz[k], qx[k], t);
        }
      }
      __syncwarp();
    }
  } else {
    // ---- update warp: lanes 0-15 and 16-31 evaluate the solves' updates
    if constexpr (std::is_same<TT, double>::value) {
      if (live) build_case_tab(w.tab, g, lane & 15);
      __syncwarp();
    }
    int pred = -1;
    TT tpred = TT();
    TT tn[4];
    int cd[4];
    for (;;) {
      // speculative: the predicted node's neighbours, while the heap warp
      // sifts the previous node's neighbours and pops
      if (live && pred >= 0) update_neighbours(w, g, SL, sld, fom, fx, K, lane, pred, tpred, tn, cd);
      pair_sync(bar1);
      int st = 1, cur = -1, root = -1;
      TT rkey = TT();
      if (live) { st = mb->stop; cur = mb->cur; root = mb->root; rkey = mb->rkey; }
      if (st != 0) live = false;
      if (!__any_sync(0xffffffffu, live)) break;
      if (live && cur != pred) update_neighbours(w, g, SL, sld, fom, fx, K, lane, cur, w.T[plin(w, cur)], tn, cd);
      pred = -1;
      if (live) {
        if (leader) {
#pragma unroll
          for (int k = 0; k < 4; ++k) { mb->tn[k] = tn[k]; mb->cd[k] = cd[k]; }
        }
        // the next root: the root left by downtree unless a sifted neighbour
        // is strictly earlier (or the root itself is updated)
        const int iz = (cur & 255) + 1, ix = (cur >> 8) + 1;
        const int qz[4] = {iz, iz, iz - 1, iz + 1}, qx[4] = {ix - 1, ix + 1, ix, ix};
        int r = root;
        TT rk = rkey;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          if (cd[k] == 0) continue;
          const int pq = (int)pack(qz[k], qx[k]);
          if (r < 0 || pq == r || tlt(tn[k], rk)) { r = pq; rk = tn[k]; }
        }
        pred = r; tpred = rk;
      }
      __syncwarp();
      pair_arrive(bar2);
    }
  }
  pair_sync(bar2);   // both warps: the solve's times and states are complete
  return active ? mb->stop : 1;
}

// Source initialisation of travel (fm2d_ttime.f90:95-127), lane 0. vel(iz, ix)
// gives the node velocities of the grid g.
template <class TT, class Vel>
__device__ void init_source(WarpStateT<TT> &w, const Grid2 &g, Vel vel, double scx, double scz, const Fx &fx) {
  int isx = (int)((scx - g.gox) / g.dnx) + 1;
  int isz = (int)((scz - g.goz) / g.dnz) + 1;
  if (isx == g.nnx) isx = isx - 1;
  if (isz == g.nnz) isz = isz - 1;
  double vss[2][2];
  for (int i = 1; i <= 2; ++i)
    for (int j = 1; j <= 2; ++j) vss[i - 1][j - 1] = vel(isz - 1 + j, isx - 1 + i);
  double dsx = (scx - g.gox) - (double)(isx - 1) * g.dnx;
  double dsz = (scz - g.goz) - (double)(isz - 1) * g.dnz;
  double vsrc = bilinear(vss, dsx, dsz, g.dnx, g.dnz);
  w.ntr = 0;
  for (int i = 1; i <= 2; ++i)
    for (int j = 1; j <= 2; ++j) {
      double ex = dsx - (double)(i - 1) * g.dnx;
      double ez = dsz - (double)(j - 1) * g.dnz;
      double ds = sqrt(ex * ex + ez * ez);
      const double t0 = 2.0 * ds / (vss[i - 1][j - 1] + vsrc);
      w.T[lin(g, isz - 1 + j, isx - 1 + i)] = from_double<TT>(t0, fx);
      addtree(w, g, isz - 1 + j, isx - 1 + i);
    }
}

__device__ __forceinline__ double bsw(int q, double u) {
  double om = 1.0 - u;
  switch (q) {
    case 0: return om * om * om / 6.0;
    case 1: return (4.0 - 6.0 * (u * u) + 3.0 * (u * u * u)) / 6.0;
    case 2: return (1.0 + 3.0 * u + 3.0 * (u * u) - 3.0 * (u * u * u)) / 6.0;
    default: return (u * u * u) / 6.0;
  }
}

__global__ void set_int_kernel(int *p, int v) { *p = v; }

// gridder (fm2dray_cartesian.f90:491-600): one block per map.
__global__ void gridder_kernel(Fm2dJob job) {
  const int map = blockIdx.x;
  const int nnx = (job.nvx - 1) * job.gdx + 1, nnz = (job.nvz - 1) * job.gdz + 1;
  const int ldv = job.nvz + 2;
  const double *velv = job.velv + (size_t)map * (job.nvx + 2) * ldv;
  double *veln = job.veln + (size_t)map * nnx * nnz;
  if (job.vmin_bits) {
    float vm = 3.0e38f;
    for (int q = threadIdx.x; q < (job.nvx + 2) * ldv; q += blockDim.x) vm = fminf(vm, (float)velv[q] * 0.999f);
    if (vm > 0.f) atomicMin(job.vmin_bits, __float_as_int(vm));
  }
  for (int node = threadIdx.x; node < nnx * nnz; node += blockDim.x) {
    int stz = node % nnz + 1, stx = node / nnz + 1;
    // invert stz = gdz*(i-1)+l (l in 1..gdz, or gdz+1 in the last cell)
    int i = (stz - 1) / job.gdz + 1; if (i > job.nvz - 1) i = job.nvz - 1;
    int l = stz - job.gdz * (i - 1);
    int j = (stx - 1) / job.gdx + 1; if (j > job.nvx - 1) j = job.nvx - 1;
    int m = stx - job.gdx * (j - 1);
    double u = (double)(m - 1) / (double)job.gdx;
    double v = (double)(l - 1) / (double)job.gdz;
    double sumi = 0.0;
    for (int i1 = 1; i1 <= 4; ++i1) {
      double sumj = 0.0;
      for (int j1 = 1; j1 <= 4; ++j1)
        sumj = sumj + bsw(j1 - 1, u) * velv[(size_t)(j - 2 + j1) * ldv + (i - 2 + i1)];
      sumi = sumi + bsw(i1 - 1, v) * sumj;
    }
    veln[(size_t)(stx - 1) * nnz + (stz - 1)] = sumi;
    store_slowness(job.slon, (size_t)map * nnx * nnz + (size_t)(stx - 1) * nnz + (stz - 1), 1.0 / sumi,
                   job.precision);
  }
}

// bsplrefine (fm2dray_cartesian.f90:608-674) over the whole map: the refined
// grid of every source box is a window of one grid, (nvx-1) gdx sgdl + 1 by
// (nvz-1) gdz sgdl + 1 nodes, and the velocity of a refined node depends only
// on its position in that grid. So the slowness 1 / v of every refined node
// is computed once per map (blockIdx.y), with the B-spline weights of the
// nrxr + 1 (nrzr + 1) positions in a cell tabulated in shared memory, in the
// operation order of refined_velocity below.
__global__ void refine_slowness_kernel(Fm2dJob job) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int map = blockIdx.y;
  const int sgdl = job.sgdl;
  const int nrxr = job.gdx * sgdl, nrzr = job.gdz * sgdl;
  const int nrgx = (job.nvx - 1) * nrxr + 1, nrgz = (job.nvz - 1) * nrzr + 1;
  double *wu = reinterpret_cast<double *>(smem), *wv = wu + 4 * (nrxr + 1);
  for (int q = threadIdx.x; q < 4 * (nrxr + 1) + 4 * (nrzr + 1); q += blockDim.x) {
    const bool alx = q < 4 * (nrxr + 1);
    const int e = alx ? q : q - 4 * (nrxr + 1);
    wu[q] = bsw(e & 3, (double)(e / 4) / (double)(alx ? nrxr : nrzr));
  }
  __syncthreads();
  const int ldv = job.nvz + 2;
  const double *velv = job.velv + (size_t)map * (job.nvx + 2) * ldv;
  const int n = nrgx * nrgz;
  for (int node = blockIdx.x * blockDim.x + threadIdx.x; node < n; node += gridDim.x * blockDim.x) {
    const int st1 = node % nrgz + 1, st2 = node / nrgz + 1;
    int i = (st1 - 1) / nrzr + 1; if (i > job.nvz - 1) i = job.nvz - 1;
    const int k = st1 - nrzr * (i - 1);
    int j = (st2 - 1) / nrxr + 1; if (j > job.nvx - 1) j = job.nvx - 1;
    const int l = st2 - nrxr * (j - 1);
    const double *bu = wu + 4 * (l - 1), *bv = wv + 4 * (k - 1);
    double sum[4];
    for (int i1 = 1; i1 <= 4; ++i1) {
      sum[i1 - 1] = 0.0;
      for (int j1 = 1; j1 <= 4; ++j1)
        sum[i1 - 1] = sum[i1 - 1] + bu[j1 - 1] * velv[(size_t)(j - 2 + j1) * ldv + (i - 2 + i1)];
      sum[i1 - 1] = bv[i1 - 1] * sum[i1 - 1];
    }
    store_slowness(job.sref, (size_t)map * job.nref_map + node, 1.0 / (sum[0] + sum[1] + sum[2] + sum[3]),
                   job.precision);
  }
}

// bsplrefine (fm2dray_cartesian.f90:608-674): the cubic B-spline velocity of
// refined node (idm1, idm2) (1-based z, x) of the source box whose corner is
// refined node (origz, origx) of the whole grid; 0 outside the coarse box
// [vnl, vnr] x [vnt, vnb].
struct RefineBox {
  const double *velv;   // this map's padded vertex grid
  int ldv, origx, origz, nrxr, nrzr, vnl, vnr, vnt, vnb;
};
__device__ double refined_velocity(const Fm2dJob &job, const RefineBox &rb, int idm1, int idm2) {
  const int sgdl = job.sgdl;
  int st1 = idm1 + rb.origz - 1, st2 = idm2 + rb.origx - 1;
  int i = (st1 - 1) / rb.nrzr + 1; if (i > job.nvz - 1) i = job.nvz - 1;
  int k = st1 - rb.nrzr * (i - 1);
  int j = (st2 - 1) / rb.nrxr + 1; if (j > job.nvx - 1) j = job.nvx - 1;
  int l = st2 - rb.nrxr * (j - 1);
  int c1 = job.gdz * (i - 1) + (k - 1) / sgdl + 1;
  int c2 = job.gdx * (j - 1) + (l - 1) / sgdl + 1;
  if (c1 < rb.vnt || c1 > rb.vnb || c2 < rb.vnl || c2 > rb.vnr) return 0.0;
  double u = (double)(l - 1) / (double)rb.nrxr;
  double v = (double)(k - 1) / (double)rb.nrzr;
  double sum[4];
  for (int i1 = 1; i1 <= 4; ++i1) {
    sum[i1 - 1] = 0.0;
    for (int j1 = 1; j1 <= 4; ++j1)
      sum[i1 - 1] = sum[i1 - 1] + bsw(j1 - 1, u) * rb.velv[(size_t)(j - 2 + j1) * rb.ldv + (i - 2 + i1)];
    sum[i1 - 1] = bsw(i1 - 1, v) * sum[i1 - 1];
  }
  return sum[0] + sum[1] + sum[2] + sum[3];
}

// GetVelocity (src/likelihood_surf.F90:496-521): bilinear velocity of one
// map of the model grid (Fortran (nvz, nvx)) at (px, pz).
__device__ double get_velocity(const double *vel, int nx, int nz, double gox, double goz, double dx, double dz,
                               double px, double pz) {
  int ix = (int)floor((px - gox) / dx) + 1;
  int iy = (int)floor((pz - goz) / dz) + 1;
  if (ix < 1) ix = 1;
  if (iy < 1) iy = 1;
  if (ix >= nx) ix = nx - 1;
  if (iy >= nz) iy = nz - 1;
  const double dsx = px - (gox + (double)(ix - 1) * dx);
  const double dsy = pz - (goz + (double)(iy - 1) * dz);
  double qv = 0;
  for (int i = 1; i <= 2; ++i)
    for (int j = 1; j <= 2; ++j) {
      const double weight = (1.0 - fabs((double)(i - 1) * dx - dsx) / dx) *
                            (1.0 - fabs((double)(j - 1) * dz - dsy) / dz);
      qv = qv + weight * vel[(size_t)(ix + i - 2) * nz + (iy + j - 2)];
    }
  return qv;
}

// Per-solve geometry shared by the two kernels (modrays' source cell and
// refined box, fm2dray_cartesian.f90:283-330).
struct SolveGeom {
  int map, src;
  double x, z;
  int isx, isz, vnl, vnr, vnt, vnb;
  Grid2 gc;
};
__device__ __forceinline__ bool solve_geom(const Fm2dJob &job, int solve, SolveGeom &s) {
  s.map = job.solves[solve].x; s.src = job.solves[solve].y;
  const int nnx = (job.nvx - 1) * job.gdx + 1, nnz = (job.nvz - 1) * job.gdz + 1;
  s.gc = Grid2{nnx, nnz, nnz, job.goxd, job.gozd, job.dvxd / job.gdx, job.dvzd / job.gdz};
  s.x = job.scx[s.src]; s.z = job.scz[s.src];
  s.isx = (int)((s.x - s.gc.gox) / s.gc.dnx) + 1;
  s.isz = (int)((s.z - s.gc.goz) / s.gc.dnz) + 1;
  if (s.isx < 1 || s.isx > nnx || s.isz < 1 || s.isz > nnz) return false;
  if (s.isx == nnx) s.isx = s.isx - 1;
  if (s.isz == nnz) s.isz = s.isz - 1;
  s.vnl = max(s.isx - job.sgs, 1); s.vnr = min(s.isx + job.sgs, nnx);
  s.vnt = max(s.isz - job.sgs, 1); s.vnb = min(s.isz + job.sgs, nnz);
  return true;
}

// Fixed-point scale (precision 2): the largest time is below 3 x diagonal /
// slowest velocity; keep it under 2^31 units.
template <class TT>
__device__ __forceinline__ Fx time_scale(const Fm2dJob &job) {
  Fx fx{1.f, 1.f};
  if constexpr (std::is_same<TT, int>::value) {
    const float vmin = __int_as_float(*job.vmin_bits);
    const double ext = sqrt(((job.nvx - 1) * job.dvxd) * ((job.nvx - 1) * job.dvxd) +
                            ((job.nvz - 1) * job.dvzd) * ((job.nvz - 1) * job.dvzd));
    const double tmax = 3.0 * ext / (double)vmin;
    int shift = 30;
    while (shift > 4 && ldexp(tmax, shift) > 2.0e9) --shift;
    fx.scale = ldexpf(1.f, shift); fx.inv = ldexpf(1.f, -shift);
  }
  return fx;
}

template <class TT>
__device__ __forceinline__ WarpStateT<TT> warp_state(unsigned char *base, char *slot, int nmax, bool sglobal,
                                                     int nodes, int cap) {
  WarpStateT<TT> w;
  const SolveLayout lay = solve_layout(nodes, cap, sglobal);
  w.cap = cap;
  w.overflow = false;
  w.T = reinterpret_cast<TT *>(slot);
  w.S = sglobal ? reinterpret_cast<short *>(slot + slot_bytes(nmax, (int)sizeof(TT), false))
                : reinterpret_cast<short *>(base + lay.offS);
  w.H = reinterpret_cast<unsigned short *>(base + lay.offH);
  w.tab = reinterpret_cast<CaseTab *>(base + lay.offTab);
  w.ntr = 0;
  w.ld = 1;
  return w;
}

// Stage 1, source-grid refinement (asgr = 1): one warp per solve marches the
// refined source box (travel with urg = 1) and leaves the times and states
// of the box nodes that coincide with coarse nodes in the mapping scratch.
// The refined box has up to (2*sgs*sgdl+1)^2 nodes, more than the coarse grid
// usually has, so this stage runs with its own (smaller) warps per block.
// First pass: every solve with a heap of REFINED_HEAP_CAP entries, solves
// whose band outgrows it listed in job.ovf_list. Overflow pass (redo = 1): the
// listed solves again with a heap as large as the box.
template <class TT, int SPW>
__device__ __forceinline__ void refined_block(const Fm2dJob &job, int solve_bytes, int heap_cap, int redo, int blk) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int pair = threadIdx.x >> 6, t64 = threadIdx.x & 63, lane = t64 & 31;
  const int slot = SPW == 2 ? (lane >> 4) : 0;                          // this thread's solve in the pair
  const int sub = SPW == 2 ? ((t64 >> 5) << 4) + (lane & 15) : t64;   // thread index within the solve
  constexpr int NSUB = 64 / SPW;
  const bool leader = t64 < 32 && (lane & 15) == 0 && (SPW == 2 || lane == 0);
  const int bar1 = 1 + 2 * pair, bar2 = 2 + 2 * pair;
  int solve = (blk * (blockDim.x >> 6) + pair) * SPW + slot;
  if (redo) solve = solve < *job.ovf_count ? job.ovf_list[solve] : job.nsolve;
  else if (job.ref_list) solve = solve < *job.ref_count ? job.ref_list[solve] : job.nsolve;
  SolveGeom sg;
  const bool active = solve < job.nsolve && solve_geom(job, solve, sg);   // geometry errors: coarse stage
  if (!__any_sync(0xffffffffu, active)) return;   // the same for both warps of the pair
  unsigned char *base = smem + ((size_t)pair * SPW + slot) * solve_bytes;
  // the time-field slot of this solve's place in the grid (block, pair, slot)
  const size_t tslot = ((size_t)blockIdx.x * (blockDim.x >> 6) + pair) * SPW + slot;
  WarpStateT<TT> w = warp_state<TT>(
      base, static_cast<char *>(job.tws_ref) + tslot * slot_bytes(job.nref_max, (int)sizeof(TT), job.sglobal_ref),
      job.nref_max, job.sglobal_ref, job.nref_max, heap_cap);
  Mailbox<TT> *mb = reinterpret_cast<Mailbox<TT> *>(base + solve_bytes - MAILBOX_BYTES);
  const Fx fx = time_scale<TT>(job);
  const int sgdl = job.sgdl;
  const int vnl = sg.vnl, vnr = sg.vnr, vnt = sg.vnt, vnb = sg.vnb;
  const Grid2 &gc = sg.gc;
  const int nrnx = active ? (vnr - vnl) * sgdl + 1 : 0, nrnz = active ? (vnb - vnt) * sgdl + 1 : 0;
  Grid2 gr{nrnx, nrnz, nrnz, gc.gox + gc.dnx * (double)(vnl - 1), gc.goz + gc.dnz * (double)(vnt - 1),
           job.dvxd / (double)(job.gdx * sgdl), job.dvzd / (double)(job.gdz * sgdl)};
  Trace trace{job.trace_i, job.trace_t, job.trace_max / 2, 0};
  Trace *tr = (job.trace_i && active && solve == job.trace_solve && leader) ? &trace : nullptr;
  // the box's nodes in the map's refined slowness field (refine_slowness
  // kernel): refined node (iz, ix) of the box is node (iz + (vnt-1) sgdl,
  // ix + (vnl-1) sgdl) of the whole refined grid, and every node of the box
  // lies inside the box's coarse cells, where bsplrefine gives the same
  // velocity from either numbering
  const int ldv = job.nvz + 2;
  const RefineBox rb{job.velv + (size_t)(active ? sg.map : 0) * (job.nvx + 2) * ldv, ldv, (vnl - 1) * sgdl + 1,
                     (vnt - 1) * sgdl + 1, job.gdx * sgdl, job.gdz * sgdl, vnl, vnr, vnt, vnb};
  const int nrgz = (job.nvz - 1) * job.gdz * sgdl + 1;
  const SlowT<TT> *SLr = active ? reinterpret_cast<const SlowT<TT> *>(job.sref) + (size_t)sg.map * job.nref_map +
                                      (size_t)(vnl - 1) * sgdl * nrgz + (size_t)(vnt - 1) * sgdl
                                : nullptr;
  for (int q = sub; q < nrnx * nrnz; q += NSUB) w.S[q] = -1;
  w.ld = gr.ld;
  pair_sync(bar1);
  if (leader && active)
    init_source(w, gr, [&](int zz, int xx) { return refined_velocity(job, rb, zz, xx); }, sg.x, sg.z, fx);
  pair_sync(bar1);
  const int end = march(w, mb, active, SPW == 2 || lane < 16, gr, SLr, nrgz, job.fom, 1, vnl, vnr, vnt, vnb, fx,
                        bar1, bar2, tr);
  if (!active) return;
  if (end == 2) {
    if (leader) job.ovf_list[atomicAdd(job.ovf_count, 1)] = solve;
    return;
  }
  // the refined nodes that map onto coarse nodes (fm2dray_cartesian.f90:365-383)
  const int mx = (nrnx - 1) / sgdl + 1, mz = (nrnz - 1) / sgdl + 1;   // = vnr-vnl+1, vnb-vnt+1
  double *tmpT = job.map_tmp_t + (size_t)solve * job.map_tmp_max;
  short *tmpS = job.map_tmp_s + (size_t)solve * job.map_tmp_max;
  for (int q = sub; q < mx * mz; q += NSUB) {
    int a = q % mz, b = q / mz;
    int k = a * sgdl + 1, l = b * sgdl + 1;
    int r = lin(gr, k, l);
    tmpT[q] = bit_store(w.T[r]);
    tmpS[q] = w.S[r];
  }
  if (job.rays) {
    // the refined field and states for the ray tracer (far nodes hold
    // uninitialised memory in the reference; 0 here)
    double *rt = job.ref_t + (size_t)solve * job.nref_max;
    short *rs = job.ref_s + (size_t)solve * job.nref_max;
    for (int q = sub; q < nrnx * nrnz; q += NSUB) {
      const short st = w.S[q];
      rs[q] = st;
      rt[q] = st == -1 ? 0.0 : to_double(w.T[q], fx);
    }
  }
}

// A persistent grid: at most as many blocks as are resident at once (fewer
// with an SM share), each walking logical blocks blockIdx.x, blockIdx.x +
// gridDim.x, ... below nblk, with the time-field slots of its own place in
// the grid. Both warps of a pair meet at the pair's barrier before the next
// logical block reuses the pair's shared memory and slots.
template <class TT, int SPW>
__global__ void __launch_bounds__(64 * PAIRS_MAX)
fm2d_refined_kernel(Fm2dJob job, int solve_bytes, int heap_cap, int redo, int nblk) {
  const int bar1 = 1 + 2 * (threadIdx.x >> 6);
  for (int blk = blockIdx.x; blk < nblk; blk += gridDim.x) {
    if (blk != (int)blockIdx.x) { __syncwarp(); pair_sync(bar1); }
    refined_block<TT, SPW>(job, solve_bytes, heap_cap, redo, blk);
  }
}

// FLOOR of a ray coordinate. Where the travel-time gradient vanishes the
// reference's next point is NaN, and FLOOR(NaN) is -2^31 on the x86 targets
// the reference is built for, which the boundary clamp then moves to the
// lower grid edge; that is made explicit here.
__device__ __forceinline__ int floor_idx(double v) { return isnan(v) ? INT_MIN : (int)floor(v); }

// rpaths (fm2d/fm2dray_cartesian.f90:801-1455, without Frechet derivatives)
// followed by CalGroupTime (src/likelihood_surf.F90:455-494) and the ray
// length (T_RAY%length), one receiver per lane: steepest descent from the
// receiver on the final coarse field (shared memory) or, inside the refined
// box where the four corners of the current cell were accepted, on the
// refined field; the group delay sums each segment's length over the mean of
// the end points' velocities as the ray is traced. A ray that reaches the
// point limit counts as crazy (its delay and length stay 0, as the reference
// stores a one-point ray).
template <class TT>
__device__ void trace_rays(const Fm2dJob &job, const WarpStateT<TT> &w, const Fx &fx, const SolveGeom &sg, int solve,
                           int sub, int nsub) {
  const int map = sg.map, src = sg.src;
  const Grid2 &gc = sg.gc;
  const int nnx = gc.nnx, nnz = gc.nnz;
  const double gox = gc.gox, goz = gc.goz, dnx = gc.dnx, dnz = gc.dnz;
  const int asgr = job.asgr, sgdl = job.sgdl;
  int nnxr = 0, nnzr = 0;
  double goxr = 0, gozr = 0, dnxr = 1, dnzr = 1;
  const double *TR = nullptr;
  const short *SR = nullptr;
  if (asgr == 1) {
    nnxr = (sg.vnr - sg.vnl) * sgdl + 1; nnzr = (sg.vnb - sg.vnt) * sgdl + 1;
    goxr = gox + dnx * (double)(sg.vnl - 1); gozr = goz + dnz * (double)(sg.vnt - 1);
    dnxr = job.dvxd / (double)(job.gdx * sgdl); dnzr = job.dvzd / (double)(job.gdz * sgdl);
    TR = job.ref_t + (size_t)solve * job.nref_max;
    SR = job.ref_s + (size_t)solve * job.nref_max;
  }
  auto T = [&](int iz, int ix) { return to_double(w.T[(iz - 1) + nnz * (ix - 1)], fx); };
  auto tr = [&](int iz, int ix) { return TR[(size_t)(iz - 1) + (size_t)nnzr * (ix - 1)]; };
  auto srf = [&](int iz, int ix) { return SR[(size_t)(iz - 1) + (size_t)nnzr * (ix - 1)]; };
  const double scx = sg.x, scz = sg.z;
  const double *gv = job.gvel + (size_t)map * job.nvx * job.nvz;
  const int maxrp = nnx * nnz;
  int isx, isz;
  if (asgr == 1) { isx = floor_idx((scx - goxr) / dnxr) + 1; isz = floor_idx((scz - gozr) / dnzr) + 1; }
  else { isx = floor_idx((scx - gox) / dnx) + 1; isz = floor_idx((scz - goz) / dnz) + 1; }
  double dpl = dnx, rd1 = dnz;
  if (rd1 < dpl) dpl = rd1;
  dpl = 0.5 * dpl;
  const int *srs = job.srs + (size_t)(map % job.srs_nmaps) * job.nsrc * job.nrc + (size_t)src * job.nrc;
  const size_t o0 = ((size_t)map * job.nsrc + src) * job.nrc;
  for (int r = sub; r < job.nrc; r += nsub) {
    if (srs[r] == 0) continue;
    const double rcx = job.rcx[r], rcz = job.rcz[r];
    int ipx = floor_idx((rcx - gox) / dnx) + 1;
    int ipz = floor_idx((rcz - goz) / dnz) + 1;
    if (ipx < 1 || ipx >= nnx || ipz < 1 || ipz >= nnz) { atomicExch(job.status, MCT_ERR_OUTSIDE); continue; }
    // the delay and length accumulate over the ray's points as they are made
    double px = rcx, pz = rcz;
    double vhead = get_velocity(gv, job.nvx, job.nvz, job.goxd, job.gozd, job.dvxd, job.dvzd, px, pz);
    double gt = 0, len = 0;
    auto add_point = [&](double qx, double qz) {
      double dist = (qx - px) * (qx - px) + (qz - pz) * (qz - pz);
      dist = sqrt(dist);
      const double vtail = get_velocity(gv, job.nvx, job.nvz, job.goxd, job.gozd, job.dvxd, job.dvzd, qx, qz);
      gt = gt + dist * 2 / (vhead + vtail);
      len = len + dist;
      vhead = vtail;
      px = qx; pz = qz;
    };
    int sw = 0;
    double sred = (scx - rcx) * (scx - rcx);
    sred = sred + (scz - rcz) * (scz - rcz);
    sred = sqrt(sred);
    if (sred < 2.0 * dpl) { add_point(scx, scz); sw = 1; }
    int ipxr = 0, ipzr = 0, igref = 0;
    auto in_refined = [&](double qx, double qz) {
      ipxr = floor_idx((qx - goxr) / dnxr) + 1;
      ipzr = floor_idx((qz - gozr) / dnzr) + 1;
      int g = 1;
      if (ipxr < 1 || ipxr >= nnxr) g = 0;
      if (ipzr < 1 || ipzr >= nnzr) g = 0;
      if (g == 1) {
        if (srf(ipzr, ipxr) != 0 || srf(ipzr + 1, ipxr) != 0) g = 0;
        if (srf(ipzr, ipxr + 1) != 0 || srf(ipzr + 1, ipxr + 1) != 0) g = 0;
      }
      return g;
    };
    if (asgr == 1) igref = in_refined(rcx, rcz);
    if (sw == 0) {
      if (asgr == 1) {
        if (igref == 1 && ipxr == isx && ipzr == isz) { add_point(scx, scz); sw = 1; }
      } else {
        if (ipx == isx && ipz == isz) { add_point(scx, scz); sw = 1; }
      }
    }
    int crazy = 0;
    for (int j = 1; j <= maxrp; ++j) {
      if (sw == 1) break;
      double dtx, dtz;
      if (igref == 1) {
        if (ipxr == 1) dtx = (tr(ipzr, ipxr + 1) - tr(ipzr, ipxr)) / dnxr;
        else if (ipxr == nnxr) dtx = (tr(ipzr, ipxr) - tr(ipzr, ipxr - 1)) / dnxr;
        else dtx = (tr(ipzr, ipxr + 1) - tr(ipzr, ipxr - 1)) / (2.0 * dnxr);
        if (ipzr == 1) dtz = (tr(ipzr + 1, ipxr) - tr(ipzr, ipxr)) / dnzr;
        else if (ipzr == nnzr) dtz = (tr(ipzr, ipxr) - tr(ipzr - 1, ipxr)) / dnzr;
        else dtz = (tr(ipzr + 1, ipxr) - tr(ipzr - 1, ipxr)) / (2.0 * dnzr);
      } else {
        if (ipx == 1) dtx = (T(ipz, ipx + 1) - T(ipz, ipx)) / dnx;
        else if (ipx == nnx) dtx = (T(ipz, ipx) - T(ipz, ipx - 1)) / dnx;
        else dtx = (T(ipz, ipx + 1) - T(ipz, ipx - 1)) / (2.0 * dnx);
        // the reference tests the refined index here (ipzr == nnzr); without
        // refinement that is an unset local, and the intended coarse test
        // (ipz == nnz) is used
        if (ipz == 1) dtz = (T(ipz + 1, ipx) - T(ipz, ipx)) / dnz;
        else if (asgr == 1 ? ipzr == nnzr : ipz == nnz) dtz = (T(ipz, ipx) - T(ipz - 1, ipx)) / dnz;
        else dtz = (T(ipz + 1, ipx) - T(ipz - 1, ipx)) / (2.0 * dnz);
      }
      rd1 = sqrt(dtx * dtx + dtz * dtz);
      double nx = px - dpl * dtx / rd1;
      double nz = pz - dpl * dtz / rd1;
      if (asgr == 1) igref = in_refined(nx, nz);
      else igref = 0;
      ipx = floor_idx((nx - gox) / dnx) + 1;
      ipz = floor_idx((nz - goz) / dnz) + 1;
      sred = (scx - nx) * (scx - nx);
      sred = sred + (scz - nz) * (scz - nz);
      sred = sqrt(sred);
      if (sred < 2.0 * dpl) { add_point(nx, nz); add_point(scx, scz); sw = 1; break; }
      if (asgr == 1) {
        if (igref == 1 && ipxr == isx && ipzr == isz) { add_point(nx, nz); add_point(scx, scz); sw = 1; break; }
      } else {
        if (ipx == isx && ipz == isz) { add_point(nx, nz); add_point(scx, scz); sw = 1; break; }
      }
      if (ipx < 1) { nx = gox; ipx = 1; }
      if (ipx >= nnx) { nx = gox + (double)(nnx - 1) * dnx; ipx = nnx - 1; }
      if (ipz < 1) { nz = goz; ipz = 1; }
      if (ipz >= nnz) { nz = goz + (double)(nnz - 1) * dnz; ipz = nnz - 1; }
      if (j == maxrp - 1) { crazy = 1; break; }
      add_point(nx, nz);
    }
    if (crazy) { gt = 0; len = 0; atomicAdd(&job.crazy[map], 1); }
    job.gtime[o0 + r] = gt;
    job.raylen[o0 + r] = len;
  }
}

// Stage 2, the coarse grid: the refined box's times and states mapped in, the
// narrow band repaired and re-heaped, travel with urg = 2 (or, without
// refinement, the point source and travel with urg = 0); then the optional
// time field and srtimes.
template <class TT, int SPW>
__device__ __forceinline__ void coarse_block(const Fm2dJob &job, int solve_bytes, int blk) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int pair = threadIdx.x >> 6, t64 = threadIdx.x & 63, lane = t64 & 31;
  const int slot = SPW == 2 ? (lane >> 4) : 0;                          // this thread's solve in the pair
  const int sub = SPW == 2 ? ((t64 >> 5) << 4) + (lane & 15) : t64;   // thread index within the solve
  constexpr int NSUB = 64 / SPW;
  const bool leader = t64 < 32 && (lane & 15) == 0 && (SPW == 2 || lane == 0);
  const int bar1 = 1 + 2 * pair, bar2 = 2 + 2 * pair;
  const int solve = (blk * (blockDim.x >> 6) + pair) * SPW + slot;
  SolveGeom sg;
  bool active = solve < job.nsolve;
  if (active && !solve_geom(job, solve, sg)) {
    if (leader) atomicExch(job.status, MCT_ERR_OUTSIDE);
    active = false;
  }
  if (!__any_sync(0xffffffffu, active)) return;   // the same for both warps of the pair
  const Grid2 gc = sg.gc;
  const int nnx = active ? gc.nnx : 0, nnz = active ? gc.nnz : 0;
  unsigned char *base = smem + ((size_t)pair * SPW + slot) * solve_bytes;
  const size_t tslot = ((size_t)blockIdx.x * (blockDim.x >> 6) + pair) * SPW + slot;
  WarpStateT<TT> w = warp_state<TT>(
      base, static_cast<char *>(job.tws) + tslot * slot_bytes(job.nodes_max, (int)sizeof(TT), job.sglobal),
      job.nodes_max, job.sglobal, nnx * nnz, nnx * nnz);
  Mailbox<TT> *mb = reinterpret_cast<Mailbox<TT> *>(base + solve_bytes - MAILBOX_BYTES);
  const Fx fx = time_scale<TT>(job);
  const int map = active ? sg.map : 0, src = active ? sg.src : 0;
  const double x = sg.x, z = sg.z;
  const int sgdl = job.sgdl;
  const int vnl = sg.vnl, vnr = sg.vnr, vnt = sg.vnt, vnb = sg.vnb;
  const double *Vc = job.veln + (size_t)map * nnx * nnz;
  const SlowT<TT> *SLc = reinterpret_cast<const SlowT<TT> *>(job.slon) + (size_t)map * nnx * nnz;
  Trace trace{job.trace_i ? job.trace_i + 3 * (job.trace_max / 2) : nullptr,
              job.trace_t ? job.trace_t + job.trace_max / 2 : nullptr, job.trace_max / 2, 0};
  Trace *tr = (job.trace_i && active && solve == job.trace_solve && leader) ? &trace : nullptr;
  const bool marches = SPW == 2 || lane < 16;
  w.ld = active ? gc.ld : 1;
  for (int q = sub; q < nnx * nnz; q += NSUB) w.S[q] = -1;
  pair_sync(bar1);
  if (job.asgr == 1) {
    if (active) {
      const int nrnx = (vnr - vnl) * sgdl + 1, nrnz = (vnb - vnt) * sgdl + 1;
      const int mx = (nrnx - 1) / sgdl + 1, mz = (nrnz - 1) / sgdl + 1;
      const double *tmpT = job.map_tmp_t + (size_t)solve * job.map_tmp_max;
      const short *tmpS = job.map_tmp_s + (size_t)solve * job.map_tmp_max;
      for (int q = sub; q < mx * mz; q += NSUB) {
        int a = q % mz, b = q / mz;
        int c = lin(gc, vnt + a, vnl + b);
        short s = tmpS[q];
        w.S[c] = s;
        if (s >= 0) w.T[c] = bit_load<TT>(tmpT[q]);
      }
    }
    pair_sync(bar1);
    // narrow band repair (fm2dray_cartesian.f90:384-405); order-independent
    for (int q = sub; q < nnx * nnz; q += NSUB) {
      int l = q % nnz + 1, k = q / nnz + 1;
      if (w.S[q] == 0) {
        bool far = (l - 1 >= 1 && w.S[lin(gc, l - 1, k)] == -1) || (l + 1 <= nnz && w.S[lin(gc, l + 1, k)] == -1) ||
                   (k - 1 >= 1 && w.S[lin(gc, l, k - 1)] == -1) || (k + 1 <= nnx && w.S[lin(gc, l, k + 1)] == -1);
        if (far) w.S[q] = 1;
      }
    }
    pair_sync(bar1);
    // travel(urg=2): heap from all nodes marked close, i outer, j inner
    if (leader && active) {
      w.ntr = 0;
      for (int i = 1; i <= nnx; ++i)
        for (int j = 1; j <= nnz; ++j)
          if (w.S[lin(gc, j, i)] > 0) addtree(w, gc, j, i);
    }
    pair_sync(bar1);
    march(w, mb, active, marches, gc, SLc, nnz, job.fom, 2, vnl, vnr, vnt, vnb, fx, bar1, bar2, tr);
  } else {
    if (leader && active) init_source(w, gc, [&](int zz, int xx) { return Vc[lin(gc, zz, xx)]; }, x, z, fx);
    pair_sync(bar1);
    march(w, mb, active, marches, gc, SLc, nnz, job.fom, 0, vnl, vnr, vnt, vnb, fx, bar1, bar2, tr);
  }
  if (!active) return;
  // optional travel-time field
  if (job.tfield) {
    double *tf = job.tfield + ((size_t)map * job.nsrc + src) * nnx * nnz;
    for (int q = sub; q < nnx * nnz; q += NSUB) tf[q] = to_double(w.T[q], fx);
  }
  // srtimes (fm2dray_cartesian.f90:682-797), one receiver per lane
  const int *srs = job.srs + (size_t)(map % job.srs_nmaps) * job.nsrc * job.nrc + (size_t)src * job.nrc;
  double *tt = job.ttime + ((size_t)map * job.nsrc + src) * job.nrc;
  for (int r = sub; r < job.nrc; r += NSUB) {
    if (srs[r] == 0) continue;
    const double rx = job.rcx[r], rz = job.rcz[r];
    int irx = (int)floor((rx - gc.gox) / gc.dnx) + 1;
    int irz = (int)floor((rz - gc.goz) / gc.dnz) + 1;
    if (irx < 1 || irx > nnx || irz < 1 || irz > nnz) { atomicExch(job.status, MCT_ERR_OUTSIDE); continue; }
    if (irx == nnx) irx = irx - 1;
    if (irz == nnz) irz = irz - 1;
    int jsx = (int)floor((x - gc.gox) / gc.dnx) + 1;
    int jsz = (int)floor((z - gc.goz) / gc.dnz) + 1;
    double dpl = gc.dnx, rd1 = gc.dnz;
    if (rd1 < dpl) dpl = rd1;
    double sred = (x - rx) * (x - rx);
    sred = sred + (z - rz) * (z - rz);
    sred = sqrt(sred);
    int sw = 0;
    if (sred < dpl) sw = 1;
    if (jsx == irx && jsz == irz) sw = 1;
    double trr;
    if (sw == 1) {
      // source and receiver velocities (the source cell is not clamped,
      // as in the reference; callers keep sources off the max edges)
      int jx = min(jsx, nnx - 1), jz = min(jsz, nnz - 1);
      double vss[2][2];
      for (int k = 1; k <= 2; ++k)
        for (int l = 1; l <= 2; ++l) vss[k - 1][l - 1] = Vc[lin(gc, jz - 1 + l, jx - 1 + k)];
      double drx = (x - gc.gox) - (double)(jsx - 1) * gc.dnx;
      double drz = (z - gc.goz) - (double)(jsz - 1) * gc.dnz;
      double vels = bilinear(vss, drx, drz, gc.dnx, gc.dnz);
      for (int k = 1; k <= 2; ++k)
        for (int l = 1; l <= 2; ++l) vss[k - 1][l - 1] = Vc[lin(gc, irz - 1 + l, irx - 1 + k)];
      drx = (rx - gc.gox) - (double)(irx - 1) * gc.dnx;
      drz = (rz - gc.goz) - (double)(irz - 1) * gc.dnz;
      double velr = bilinear(vss, drx, drz, gc.dnx, gc.dnz);
      trr = 2.0 * sred / (vels + velr);
    } else {
      double drx = (rx - gc.gox) - (double)(irx - 1) * gc.dnx;
      double drz = (rz - gc.goz) - (double)(irz - 1) * gc.dnz;
      trr = 0.0;
      for (int k = 1; k <= 2; ++k)
        for (int l = 1; l <= 2; ++l) {
          double produ = (1.0 - fabs(((double)(l - 1) * gc.dnz - drz) / gc.dnz)) *
                         (1.0 - fabs(((double)(k - 1) * gc.dnx - drx) / gc.dnx));
          const double tv = to_double(w.T[lin(gc, irz - 1 + l, irx - 1 + k)], fx);
          trr = trr + tv * produ;
        }
    }
    tt[r] = trr;
  }
  if (job.rays) trace_rays(job, w, fx, sg, solve, sub, NSUB);
}

// The persistent grid of fm2d_refined_kernel.
template <class TT, int SPW>
__global__ void __launch_bounds__(64 * PAIRS_MAX)
fm2d_coarse_kernel(Fm2dJob job, int solve_bytes, int nblk) {
  const int bar1 = 1 + 2 * (threadIdx.x >> 6);
  for (int blk = blockIdx.x; blk < nblk; blk += gridDim.x) {
    if (blk != (int)blockIdx.x) { __syncwarp(); pair_sync(bar1); }
    coarse_block<TT, SPW>(job, solve_bytes, blk);
  }
}

}  // namespace

namespace {
// The refined stage's reuse test, one warp per solve: the solve's map and
// its committed map agree over the padded vertices the box's B-spline
// velocities read (the box's vertex cells and 3 vertices beyond, which
// covers the 4-vertex support of every refined node and the source); then
// the committed box mapping is copied in, else the solve joins the list
// that marches. The refined result depends on nothing else (the march
// stops at the box, its update and slowness read only the box).
__global__ void ref_reuse_kernel(Fm2dJob job) {
  const int lane = threadIdx.x & 31;
  const int q = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  if (q >= job.nsolve) return;
  SolveGeom sg;
  const bool geom = solve_geom(job, q, sg);
  const int cs = job.csolve[q];
  const int cm = geom ? job.cmap[sg.map] : -1;
  bool same = geom && cs >= 0 && cm >= 0;
  if (same) {
    const int ldv = job.nvz + 2;
    const int xl = max((sg.vnl - 1) / job.gdx + 1 - 3, 0), xr = min((sg.vnr - 1) / job.gdx + 1 + 3, job.nvx + 1);
    const int zl = max((sg.vnt - 1) / job.gdz + 1 - 3, 0), zr = min((sg.vnb - 1) / job.gdz + 1 + 3, job.nvz + 1);
    const double *a = job.velv + (size_t)sg.map * (job.nvx + 2) * ldv;
    const double *b = job.cvelv + (size_t)cm * (job.nvx + 2) * ldv;
    const int w = zr - zl + 1, n = (xr - xl + 1) * w;
    bool diff = false;
    for (int i = lane; i < n; i += 32) {
      const size_t o = (size_t)(xl + i / w) * ldv + zl + i % w;
      diff |= __double_as_longlong(a[o]) != __double_as_longlong(b[o]);
    }
    same = !__any_sync(0xffffffffu, diff);
  }
  if (same) {
    const double *ct = job.cref_t + (size_t)cs * job.map_tmp_max;
    const short *cs2 = job.cref_s + (size_t)cs * job.map_tmp_max;
    double *tt = job.map_tmp_t + (size_t)q * job.map_tmp_max;
    short *ts = job.map_tmp_s + (size_t)q * job.map_tmp_max;
    for (int i = lane; i < job.map_tmp_max; i += 32) { tt[i] = ct[i]; ts[i] = cs2[i]; }
  } else if (lane == 0) {
    job.ref_list[atomicAdd(job.ref_count, 1)] = q;
  }
}
}  // namespace

namespace {
// Warp pairs per block for kernel k with pair_bytes of shared memory per
// pair: the block size that keeps the most pairs resident per SM (shared
// memory, registers and the block limit all counted by the occupancy
// calculator). Remembered per (kernel, footprint).
template <class K>
int pairs_for(K k, int pair_bytes) {
  static std::mutex mu;
  static std::vector<std::pair<std::pair<const void *, int>, int>> memo;
  std::lock_guard<std::mutex> lk(mu);
  for (auto &m : memo)
    if (m.first.first == (const void *)k && m.first.second == pair_bytes) return m.second;
  int best = 0, best_pairs = 0;
  for (int ppb = 1; ppb <= PAIRS_MAX; ++ppb) {
    const size_t bytes = (size_t)ppb * pair_bytes;
    if (bytes > 227 * 1024) break;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, 64 * ppb, bytes) != cudaSuccess) continue;
    if (nb * ppb > best_pairs) { best_pairs = nb * ppb; best = ppb; }
  }
  memo.push_back({{(const void *)k, pair_bytes}, best});
  return best;
}
}  // namespace

namespace {
int g_ref_heap_cap = REFINED_HEAP_CAP;
}  // namespace

// Test hook (not part of the C ABI): the refined-stage heap capacity used by
// plans made after the call; cap < 4 restores the default. Small capacities
// force the overflow pass.
extern "C" int mct_debug_fm2d_heap_cap(int cap) {
  g_ref_heap_cap = cap < 4 ? REFINED_HEAP_CAP : cap;
  return MCT_OK;
}

namespace {
// Solves per warp pair of the refined and coarse stages. One solve per pair
// keeps five refined boxes resident per SM (two would share each FP64
// instruction but fit only four); the coarse stage's ten resident solves
// share their update warps in twos.
int g_spw_refined = 2, g_spw_coarse = 2;
}  // namespace

// Diagnostics (not part of the public header): solves per warp pair (1 or 2)
// of the refined and coarse stages; 0 keeps a setting. Returns the previous
// settings as refined * 10 + coarse.
extern "C" int mct_debug_fm2d_spw(int refined, int coarse) {
  const int old = g_spw_refined * 10 + g_spw_coarse;
  if (refined == 1 || refined == 2) g_spw_refined = refined;
  if (coarse == 1 || coarse == 2) g_spw_coarse = coarse;
  return old;
}

namespace {
__device__ __forceinline__ unsigned long long splitmix64(unsigned long long &x) {
  unsigned long long z = (x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Inputs of four kinds, by index mod 4: random positive normal numbers over
// the whole exponent range; products y * y and their neighbours within
// 3 ulps (exact and near-exact squares); products y * next(y), next to the
// squares of the midpoints between two doubles (the hardest rounding cases),
// and their neighbours; zeros, subnormals, infinities, NaNs and negative
// numbers.
__global__ void sqrt_check_kernel(unsigned long long count, unsigned long long seed, unsigned long long *out) {
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < count;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    unsigned long long st = seed ^ (i * 0xD1B54A32D192ED03ull);
    const unsigned long long r1 = splitmix64(st), r2 = splitmix64(st);
    unsigned long long bits;
    switch (i & 3) {
      case 0:
        bits = (r1 & 0xFFFFFFFFFFFFFull) | ((1 + r2 % 2046) << 52);
        break;
      case 1:
      case 2: {
        // y in [2^-500, 2^500)
        const unsigned long long yb = (r1 & 0xFFFFFFFFFFFFFull) | ((523 + r2 % 1000) << 52);
        const double y = __longlong_as_double((long long)yb);
        const double y2 = (i & 3) == 1 ? y : __longlong_as_double((long long)(yb + 1));
        bits = (unsigned long long)__double_as_longlong(__dmul_rn(y, y2));
        bits += (long long)((r2 >> 40) % 7) - 3;
        break;
      }
      default: {
        const unsigned k = (unsigned)(r2 % 8);
        if (k == 0) bits = 0;
        else if (k == 1) bits = 1ull << 63;
        else if (k <= 3) bits = r1 & 0xFFFFFFFFFFFFFull;                 // subnormal
        else if (k == 4) bits = 0x7FFull << 52;                          // +inf
        else if (k == 5) bits = (0x7FFull << 52) | (r1 & 0xFFFFFFFFFFFFFull) | 1;   // NaN
        else bits = (1ull << 63) | (r1 & 0x7FFFFFFFFFFFFFFFull);         // negative
        break;
      }
    }
    const double x = __longlong_as_double((long long)bits);
    const double a = exact_sqrt_rn(x), b = sqrt(x);
    const bool same = __double_as_longlong(a) == __double_as_longlong(b) || (isnan(a) && isnan(b));
    if (!same) {
      atomicAdd(&out[0], 1ull);
      atomicCAS(&out[2], 0ull, bits);
    }
  }
}
}  // namespace

// Diagnostics (not part of the public header): exact_sqrt_rn against the
// library's sqrt on count generated inputs (sqrt_check_kernel); out[0]
// receives the number of results whose bits differ, out[1] the count, out[2]
// the bits of one differing input (0 if none).
extern "C" int mct_debug_exact_sqrt_check(unsigned long long count, unsigned long long seed,
                                          unsigned long long *out) {
  unsigned long long *d = nullptr;
  MCT_CUDA_TRY(cudaMalloc(&d, 3 * sizeof(unsigned long long)));
  cudaError_t e = cudaMemset(d, 0, 3 * sizeof(unsigned long long));
  if (e == cudaSuccess) {
    sqrt_check_kernel<<<152 * 8, 256>>>(count, seed, d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(out, d, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  cudaFree(d);
  MCT_CUDA_TRY(e);
  out[1] = count;
  return MCT_OK;
}

int fm2d_plan(const Fm2dJob &job, Fm2dPlan *plan) {
  const int nnx = (job.nvx - 1) * job.gdx + 1, nnz = (job.nvz - 1) * job.gdz + 1;
  int nodes = nnx * nnz;
  int nref = 0, tmp = 0;
  if (job.asgr == 1) {
    int nr = 2 * job.sgs * job.sgdl + 1;
    nref = nr * nr;
    tmp = (2 * job.sgs + 1) * (2 * job.sgs + 1);
  }
  int nodes_max = nodes > nref ? nodes : nref;
  if (nodes_max > 32000) return MCT_ERR_ARG;   // int16 heap positions / node ids
  if (nnx > 256 || nnz > 256 || (job.asgr == 1 && 2 * job.sgs * job.sgdl + 1 > 256)) return MCT_ERR_ARG;
  plan->nodes_max = nodes_max;
  plan->nref_max = nref;
  plan->nref_map = 0;
  if (job.asgr == 1) {
    // the map's whole refined grid, and the refine kernel's weight tables
    const long nrx = (long)(job.nvx - 1) * job.gdx * job.sgdl + 1, nrz = (long)(job.nvz - 1) * job.gdz * job.sgdl + 1;
    const long tab = 8L * 4 * ((long)job.gdx * job.sgdl + 1 + (long)job.gdz * job.sgdl + 1);
    if (nrx * nrz > (1L << 30) || tab > 48 * 1024) return MCT_ERR_ARG;
    plan->nref_map = (int)(nrx * nrz);
  }
  plan->map_tmp_max = tmp;
  // node states stay in shared memory when 16 solves (the solve kernels'
  // register limit per SM) fit beside each other, else they join the times
  // in the global slot, so that shared memory does not cut the residency
  const int per_sm_target = 16, smem_sm = 228 * 1024;
  plan->sglobal = solve_layout(nodes, nodes, false).bytes * per_sm_target > smem_sm;
  plan->warp_bytes = solve_layout(nodes, nodes, plan->sglobal).bytes;
  plan->ref_heap_cap = nref < g_ref_heap_cap ? nref : g_ref_heap_cap;
  plan->sglobal_ref = nref > 0 && solve_layout(nref, plan->ref_heap_cap, false).bytes * per_sm_target > smem_sm;
  plan->ref_warp_bytes = nref > 0 ? solve_layout(nref, plan->ref_heap_cap, plan->sglobal_ref).bytes : 0;
  plan->ref_full_warp_bytes = nref > 0 ? solve_layout(nref, nref, plan->sglobal_ref).bytes : 0;
  if (plan->warp_bytes > 227 * 1024 || plan->ref_full_warp_bytes > 227 * 1024) return MCT_ERR_ARG;
  plan->tbytes = job.precision == 2 ? (int)sizeof(int) : (int)sizeof(double);
  // time-field slots: a bound on the solves resident at once, from the
  // shared memory per solve (228 KB per SM) and the threads per SM (2,048:
  // 32 warp pairs of at most two solves), times the device's SM count (a
  // 152-SM GB300 when no device is visible, for sizing without one)
  int sms = 152, dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                cudaSuccess) {
    cudaGetLastError();
    sms = 152;
  }
  auto per_sm = [](int bytes) { return bytes > 0 ? std::min(228 * 1024 / bytes, 32) : 0; };
  plan->tslots = sms * per_sm(plan->warp_bytes);
  plan->tslots_ref = nref > 0 ? sms * per_sm(plan->ref_warp_bytes) : 0;
  return MCT_OK;
}

size_t fm2d_tws_bytes(const Fm2dPlan &plan, long nsolve_max) {
  const long r = std::min<long>(plan.tslots_ref, nsolve_max + 32), c = std::min<long>(plan.tslots, nsolve_max + 32);
  const size_t ref = ((size_t)r * slot_bytes(plan.nref_max, plan.tbytes, plan.sglobal_ref) + 255) & ~size_t(255);
  return ref + (size_t)c * slot_bytes(plan.nodes_max, plan.tbytes, plan.sglobal);
}

void fm2d_bind_tws(Fm2dJob &job, const Fm2dPlan &plan, long nsolve_max, void *mem) {
  const long r = std::min<long>(plan.tslots_ref, nsolve_max + 32), c = std::min<long>(plan.tslots, nsolve_max + 32);
  const size_t ref = ((size_t)r * slot_bytes(plan.nref_max, plan.tbytes, plan.sglobal_ref) + 255) & ~size_t(255);
  job.tws_ref = mem;
  job.tslots_ref = plan.nref_max > 0 ? (int)r : 0;
  job.tws = static_cast<char *>(mem) + ref;
  job.tslots = (int)c;
  job.sglobal_ref = plan.sglobal_ref;
  job.sglobal = plan.sglobal;
}

namespace {
// Blocks to launch for nblk logical blocks of kernel k: the blocks resident
// at once on the device, or with a share in (0, 1) on share x the SM count
// (rounded, at least one), so that the launch leaves the other SMs to other
// streams' kernels for its whole duration; at most nblk.
template <class K>
int grid_for(K k, int nblk, int threads, size_t smem, double share, int *grid) {
  int dev = 0, sms = 0, occ = 0;
  MCT_CUDA_TRY(cudaGetDevice(&dev));
  MCT_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  MCT_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, threads, smem));
  const int nsm = share > 0.0 && share < 1.0 ? std::max(1, (int)(share * sms + 0.5)) : sms;
  const long cap = (long)nsm * std::max(occ, 1);
  *grid = cap < nblk ? (int)cap : nblk;
  return MCT_OK;
}

// A launch's blocks also stay within the job's time-field slots (a block
// uses the slots of its place in the grid).
template <class TT, int SPW>
int launch_refined(const Fm2dJob &job, int solve_bytes, int heap_cap, int redo, double share, cudaStream_t s) {
  auto kern = fm2d_refined_kernel<TT, SPW>;
  int rc = mct_smem_attr(kern, 227 * 1024);
  if (rc) return rc;
  const int ppb = pairs_for(kern, SPW * solve_bytes);
  if (ppb < 1) return MCT_ERR_ARG;
  const int per_block = ppb * SPW;
  const int nblk = (job.nsolve + per_block - 1) / per_block;
  const size_t smem = (size_t)per_block * solve_bytes;
  int grid = nblk;
  if ((rc = grid_for(kern, nblk, 64 * ppb, smem, share, &grid))) return rc;
  grid = std::min(grid, job.tslots_ref / per_block);
  if (grid < 1 || !job.tws_ref) return MCT_ERR_ARG;
  kern<<<grid, 64 * ppb, smem, s>>>(job, solve_bytes, heap_cap, redo, nblk);
  MCT_CUDA_TRY(cudaGetLastError());
  return MCT_OK;
}

template <class TT, int SPW>
int launch_coarse(const Fm2dJob &job, int solve_bytes, double share, cudaStream_t s) {
  auto kern = fm2d_coarse_kernel<TT, SPW>;
  int rc = mct_smem_attr(kern, 227 * 1024);
  if (rc) return rc;
  const int ppb = pairs_for(kern, SPW * solve_bytes);
  if (ppb < 1) return MCT_ERR_ARG;
  const int per_block = ppb * SPW;
  const int nblk = (job.nsolve + per_block - 1) / per_block;
  const size_t smem = (size_t)per_block * solve_bytes;
  int grid = nblk;
  if ((rc = grid_for(kern, nblk, 64 * ppb, smem, share, &grid))) return rc;
  grid = std::min(grid, job.tslots / per_block);
  if (grid < 1 || !job.tws) return MCT_ERR_ARG;
  kern<<<grid, 64 * ppb, smem, s>>>(job, solve_bytes, nblk);
  MCT_CUDA_TRY(cudaGetLastError());
  return MCT_OK;
}

template <class TT>
int launch_solves(const Fm2dJob &job, const Fm2dPlan &plan, cudaStream_t s) {
  int rc;
  const double sh = plan.sm_share;
  if (job.asgr == 1) {
    if (!job.ovf_list || !job.ovf_count) return MCT_ERR_ARG;
    MCT_CUDA_TRY(cudaMemsetAsync(job.ovf_count, 0, sizeof(int), s));
    if (job.ref_list) {
      MCT_CUDA_TRY(cudaMemsetAsync(job.ref_count, 0, sizeof(int), s));
      ref_reuse_kernel<<<(job.nsolve + 7) / 8, 256, 0, s>>>(job);
      MCT_CUDA_TRY(cudaGetLastError());
    }
    rc = g_spw_refined == 2 ? launch_refined<TT, 2>(job, plan.ref_warp_bytes, plan.ref_heap_cap, 0, sh, s)
                            : launch_refined<TT, 1>(job, plan.ref_warp_bytes, plan.ref_heap_cap, 0, sh, s);
    if (rc) return rc;
    if (plan.ref_heap_cap < job.nref_max) {
      // overflow pass: solves beyond the device-side count exit at once
      rc = launch_refined<TT, 1>(job, plan.ref_full_warp_bytes, job.nref_max, 1, sh, s);
      if (rc) return rc;
    }
  }
  return g_spw_coarse == 2 ? launch_coarse<TT, 2>(job, plan.warp_bytes, sh, s)
                           : launch_coarse<TT, 1>(job, plan.warp_bytes, sh, s);
}
}  // namespace

int launch_fm2d(const Fm2dJob &job, const Fm2dPlan &plan, cudaStream_t s) {
  if (job.precision == 2) {
    if (!job.vmin_bits) return MCT_ERR_ARG;
    set_int_kernel<<<1, 1, 0, s>>>(job.vmin_bits, 0x7f7fffff);   // FLT_MAX bits
    MCT_CUDA_TRY(cudaGetLastError());
  }
  gridder_kernel<<<job.nmaps, 256, 0, s>>>(job);
  MCT_CUDA_TRY(cudaGetLastError());
  if (job.nsolve == 0) return MCT_OK;
  if (job.asgr == 1) {
    const int nrxr = job.gdx * job.sgdl, nrzr = job.gdz * job.sgdl;
    const size_t tab = sizeof(double) * 4 * (size_t)(nrxr + 1 + nrzr + 1);
    const int bx = (int)std::min<long>((job.nref_map + 255) / 256, 64);
    refine_slowness_kernel<<<dim3(bx, job.nmaps), 256, tab, s>>>(job);
    MCT_CUDA_TRY(cudaGetLastError());
  }
  if (job.ref_list && (job.asgr != 1 || job.rays || job.precision == 2 || !job.ref_count || !job.cvelv ||
                        !job.cmap || !job.csolve || !job.cref_t || !job.cref_s))
    return MCT_ERR_ARG;
  if (job.precision == 2) return launch_solves<int>(job, plan, s);
  if (job.precision == 1) return launch_solves<float2>(job, plan, s);
  return launch_solves<double>(job, plan, s);
}
