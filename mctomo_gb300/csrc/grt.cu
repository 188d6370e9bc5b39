// Generalized reflection/transmission (GRT) fundamental-mode dispersion for
// layered columns with a low-velocity layer: the reference's single-mode
// surfmodes path for such columns (surfmodes/surfmodes.f90:39-108 routes
// them to RayleighModes / LoveModes, :185-303).
//
// One thread evaluates one column: the frequency loop of RayleighModes /
// LoveModes (each root starts from the previous frequency's), the
// fundamental-mode search of SearchRayleigh / SearchLove (FundaMode), the
// trial-velocity list of C_Interval / C_Interval_L, startl's truncation
// depth, the secular functions SecFunSurf (Rayleigh.f90:92-125) and
// SecFuns_L (Love.f90:118-132) and the root refinement bisecim
// (util.f90:90-167). The arithmetic is the reference's, term by term, in
// FP64 without fused multiply-add: complex products (ar*br - ai*bi,
// ar*bi + ai*br), complex quotients by Smith's method (gfortran's default
// complex division), exp(re)*(cos im, sin im), and sqrt of a real argument.
// The 4x4 matrices E^-1 E of EinvE (Rayleigh.f90:404-440) have six distinct
// entries in each factor; each product entry is formed from them with the
// factors' signs, the same products summed in the same order as the full
// matrix product.
//
// Memory: the trial-velocity list lives in a per-thread slot of global
// scratch sized for the reference's 20,000-entry arrays (a column that would
// need more gets ierr 1, where the reference's arrays would overflow); the
// grid is persistent (threads walk the columns), so the scratch is
// resident-threads x 160 KB. Per-column derived data (normalised shear
// moduli, sorted body-wave velocities) is written once per column to a
// column-major scratch.
#include "grt.cuh"
#include <algorithm>
#include <cmath>
#include <cfloat>
#include <cstdlib>

namespace {

struct cx { double re, im; };
__device__ __forceinline__ cx C(double r) { return {r, 0.0}; }
__device__ __forceinline__ cx add(cx a, cx b) { return {a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ cx sub(cx a, cx b) { return {a.re - b.re, a.im - b.im}; }
__device__ __forceinline__ cx neg(cx a) { return {-a.re, -a.im}; }
__device__ __forceinline__ cx mul(cx a, cx b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
__device__ __forceinline__ cx rmul(double r, cx a) { return {r * a.re, r * a.im}; }
__device__ __forceinline__ cx cdiv(cx a, cx b) {
  double tr, ti;
  if (fabs(b.re) < fabs(b.im)) {
    const double ratio = b.re / b.im, den = b.re * ratio + b.im;
    tr = (a.re * ratio + a.im) / den;
    ti = (a.im * ratio - a.re) / den;
  } else {
    const double ratio = b.im / b.re, den = b.im * ratio + b.re;
    tr = (a.im * ratio + a.re) / den;
    ti = (a.im - a.re * ratio) / den;
  }
  return {tr, ti};
}
__device__ __forceinline__ cx cexp_(cx z) {
  double s, c;
  if (fabs(z.im) > DBL_MIN) sincos(z.im, &s, &c);
  else { s = z.im; c = 1.0; }
  const double e = z.re == 0.0 ? 1.0 : exp(z.re);   // exp(+-0) = 1 exactly
  return {e * c, e * s};
}
__device__ __forceinline__ cx csqrt_real(double x) {
  return x >= 0.0 ? cx{sqrt(x), 0.0} : cx{0.0, sqrt(-x)};
}
// csq (GRT.f90:107-111)
__device__ __forceinline__ cx csq(double c, double vel) { const double t = c / vel; return csqrt_real(1.0 - t * t); }

constexpr double kPiS = (double)3.1415926f;   // the single-precision pi literals
constexpr double kPiD = 3.1415926535897932;   // m_GRT's pi
constexpr double kExpo = 46.0;
constexpr double kEpsGrt = 1e-10;
constexpr int kNccc = 20000;

struct Col {
  int nl, lvlast, nlvl1, ll;
  int stride;                  // column-major stride of the layer arrays
  const double *d, *vp, *vs;   // layer arrays of the column (element i at i*stride)
  const double *mu, *v;        // normalised moduli (stride), sorted velocities (stride, 2nl)
  double vs1, vsm, vsy;
  double w, tol, smin, dc;
  long long evals;
  __device__ double D(int i) const { return d[(size_t)i * stride]; }
  __device__ double VP(int i) const { return vp[(size_t)i * stride]; }
  __device__ double VS(int i) const { return vs[(size_t)i * stride]; }
  __device__ double MU(int i) const { return mu[(size_t)i * stride]; }
  __device__ double V(int i) const { return v[(size_t)i * stride]; }
};

// startl (Rayleigh.f90:53-90)
__device__ void startl(double c, Col &g) {
  int sl = g.nl;
  const double vk = g.w / c;
  double su = 0;
  for (int j = g.lvlast; j <= g.nl - 1; ++j) {
    const double b = g.VS(j - 1);
    if (c < b) {
      su = su + vk * csq(c, b).re * g.D(j - 1);
      if (su > kExpo) { sl = j; break; }
    } else {
      su = 0;
    }
  }
  g.ll = sl;
}

__device__ __forceinline__ cx decay(double d, double vk, cx q) { return cexp_(neg(rmul(d * vk, q))); }

// The distinct entries of EinvE's two factors (Rayleigh.f90:404-440): b44
// (E^-1 of the layer above, divided by 2(1 - xi)) and a44 (E of the layer
// below).
struct Ev {
  cx P[6];      // b44: P0 = 1/den, P1..P5 the other entries / den
  cx A[6];      // a44: 1, cs1, cp1, n1, n2, n3
};
// Entry (R, Q) of a44 alone
template <int R, int Q> __device__ __forceinline__ cx aent(const Ev &e) {
  constexpr int ai[4][4] = {{0, 1, 0, 1}, {2, 0, 2, 0}, {3, 4, 3, 4}, {4, 5, 4, 5}};
  constexpr int as[4][4] = {{1, 1, 1, 1}, {1, 1, -1, -1}, {1, 1, -1, -1}, {1, 1, 1, 1}};
  return as[R][Q] > 0 ? e.A[ai[R][Q]] : neg(e.A[ai[R][Q]]);
}

struct M2 { cx a, b, c, d; };   // [[a, b], [c, d]]
__device__ __forceinline__ M2 mm2(const M2 &x, const M2 &y) {
  M2 o;
  o.a = add(add(C(0.0), mul(x.a, y.a)), mul(x.b, y.c));
  o.b = add(add(C(0.0), mul(x.a, y.b)), mul(x.b, y.d));
  o.c = add(add(C(0.0), mul(x.c, y.a)), mul(x.d, y.c));
  o.d = add(add(C(0.0), mul(x.c, y.b)), mul(x.d, y.d));
  return o;
}
// inv2 (Rayleigh.f90:24-30)
__device__ __forceinline__ M2 inv2(const M2 &x) {
  const cx det = sub(mul(x.a, x.d), mul(x.c, x.b));
  return {cdiv(x.d, det), cdiv(neg(x.b), det), cdiv(neg(x.c), det), cdiv(x.a, det)};
}

// A layer's quantities at phase velocity c: the vertical slownesses cp, cs
// (csq of a real argument: real, or imaginary when c exceeds the velocity;
// zero when c equals it), xi = 1 - (c/vs)^2/2 and the normalised modulus.
struct Lay {
  cx cp, cs;
  double xi, am;
  bool cpi, csi, zero;           // cp / cs imaginary; either exactly zero
};
__device__ __forceinline__ Lay layer_at(const Col &g, int L, double c) {
  Lay q;
  q.am = g.MU(L);
  const double b = g.VS(L);
  q.cp = csq(c, g.VP(L)); q.cs = csq(c, b);
  const double t = c / b;
  q.xi = 1.0 - t * t / 2.0;
  q.cpi = q.cp.re == 0.0; q.csi = q.cs.re == 0.0;
  q.zero = (q.cp.re == 0.0 && q.cp.im == 0.0) || (q.cs.re == 0.0 && q.cs.im == 0.0);
  return q;
}
__device__ __forceinline__ double nz(const cx &v, bool imag) { return imag ? v.im : v.re; }

// E^-1 E of interface j from the layer above (u) and below (w), as EinvE
// (Rayleigh.f90:404-440) evaluates it. Every entry of both factors is exactly
// real or exactly imaginary (the other part an exact zero), so each product
// term is one multiplication of the nonzero parts, added to the real or the
// imaginary sum; the values are those of the full complex arithmetic. A
// layer whose slowness is exactly zero takes the general path.
struct E44 { cx e[4][4]; };
__device__ void einve_pair(const Lay &u, const Lay &w, E44 &E) {
  constexpr int bi[4][4] = {{0, 1, 2, 3}, {4, 0, 3, 5}, {0, 1, 2, 3}, {4, 0, 3, 5}};
  constexpr int bs[4][4] = {{1, 1, 1, 1}, {1, 1, 1, 1}, {1, -1, -1, 1}, {1, -1, -1, 1}};
  constexpr int ai[4][4] = {{0, 1, 0, 1}, {2, 0, 2, 0}, {3, 4, 3, 4}, {4, 5, 4, 5}};
  constexpr int as[4][4] = {{1, 1, 1, 1}, {1, 1, -1, -1}, {1, 1, -1, -1}, {1, 1, 1, 1}};
  if (u.zero || w.zero) {
    Ev e;
    e.A[0] = C(1.0); e.A[1] = w.cs; e.A[2] = w.cp;
    e.A[3] = neg(rmul(w.am, w.cp)); e.A[4] = neg(rmul(w.am, C(w.xi))); e.A[5] = neg(rmul(w.am, w.cs));
    const cx xi = C(u.xi);
    const cx den = rmul(2.0, sub(C(1.0), xi));
    e.P[0] = cdiv(C(1.0), den);
    e.P[1] = cdiv(neg(cdiv(xi, u.cp)), den);
    e.P[2] = cdiv(neg(cdiv(C(1.0), rmul(u.am, u.cp))), den);
    e.P[3] = cdiv(cdiv(C(1.0), C(u.am)), den);
    e.P[4] = cdiv(neg(cdiv(xi, u.cs)), den);
    e.P[5] = cdiv(neg(cdiv(C(1.0), rmul(u.am, u.cs))), den);
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        cx sm = C(0.0);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const cx pr = mul(e.P[bi[r][k]], e.A[ai[k][q]]);
          sm = (bs[r][k] * as[k][q] > 0) ? add(sm, pr) : sub(sm, pr);
        }
        E.e[r][q] = sm;
      }
    return;
  }
  // b44's distinct entries (the layer above), Smith's quotients by the real
  // 2(1 - xi) reduced to their nonzero parts
  const double D = 2.0 * (1.0 - u.xi);
  const double cpv = nz(u.cp, u.cpi), csv = nz(u.cs, u.csi);
  double Pv[6];
  bool Pi[6];
  Pv[0] = 1.0 / D; Pi[0] = false;
  Pv[3] = (1.0 / u.am) / D; Pi[3] = false;
  Pv[1] = u.cpi ? (u.xi / cpv) / D : (-(u.xi / cpv)) / D; Pi[1] = u.cpi;
  Pv[2] = u.cpi ? (1.0 / (u.am * cpv)) / D : (-(1.0 / (u.am * cpv))) / D; Pi[2] = u.cpi;
  Pv[4] = u.csi ? (u.xi / csv) / D : (-(u.xi / csv)) / D; Pi[4] = u.csi;
  Pv[5] = u.csi ? (1.0 / (u.am * csv)) / D : (-(1.0 / (u.am * csv))) / D; Pi[5] = u.csi;
  // a44's distinct entries (the layer below)
  const double wcp = nz(w.cp, w.cpi), wcs = nz(w.cs, w.csi);
  const double Av[6] = {1.0, wcs, wcp, -(w.am * wcp), -(w.am * w.xi), -(w.am * wcs)};
  const bool Ai[6] = {false, w.csi, w.cpi, w.cpi, false, w.csi};
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      double re = 0.0, im = 0.0;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const bool pim = Pi[bi[r][k]], aim = Ai[ai[k][q]];
        double pr = Pv[bi[r][k]] * Av[ai[k][q]];
        if (pim && aim) pr = -pr;                    // i * i
        const bool plus = bs[r][k] * as[k][q] > 0;
        if (pim != aim) im = plus ? im + pr : im - pr;
        else re = plus ? re + pr : re - pr;
      }
      E.e[r][q] = cx{re, im};
    }
}

// SecFunSurf (Rayleigh.f90:92-125) after propup (Rayleigh.f90:455-491). The
// layer below one interface is the layer above the previous one: its
// slownesses and its decay exp(-d vk [cp, cs]) carry over (the same values
// the reference recomputes).
__device__ double secfun_surf(Col &g, double c, double *imf) {
  g.evals++;
  const double vk = g.w / c;
  const int j2 = g.ll - 1;
  Lay w = layer_at(g, j2, c), u = layer_at(g, j2 - 1, c);
  E44 E;
  einve_pair(u, w, E);
  M2 a22 = inv2(M2{E.e[0][0], E.e[0][1], E.e[1][0], E.e[1][1]});
  cx la0 = decay(g.D(j2 - 1), vk, u.cp), la1 = decay(g.D(j2 - 1), vk, u.cs);
  a22.a = mul(a22.a, la0); a22.c = mul(a22.c, la0);
  a22.b = mul(a22.b, la1); a22.d = mul(a22.d, la1);
  M2 rdu = mm2(M2{E.e[2][0], E.e[2][1], E.e[3][0], E.e[3][1]}, a22);
  for (int j = j2 - 1; j >= 1; --j) {
    w = u;
    u = layer_at(g, j - 1, c);
    einve_pair(u, w, E);
    const cx lb0 = la0, lb1 = la1;                  // decay(D(j), vk, [cp, cs] of layer j)
    M2 b22{mul(rdu.a, lb0), mul(rdu.b, lb0), mul(rdu.c, lb1), mul(rdu.d, lb1)};
    M2 t = mm2(M2{E.e[0][2], E.e[0][3], E.e[1][2], E.e[1][3]}, b22);
    a22 = inv2(M2{add(E.e[0][0], t.a), add(E.e[0][1], t.b), add(E.e[1][0], t.c), add(E.e[1][1], t.d)});
    la0 = decay(g.D(j - 1), vk, u.cp); la1 = decay(g.D(j - 1), vk, u.cs);
    a22.a = mul(a22.a, la0); a22.c = mul(a22.c, la0);
    a22.b = mul(a22.b, la1); a22.d = mul(a22.d, la1);
    t = mm2(M2{E.e[2][2], E.e[2][3], E.e[3][2], E.e[3][3]}, b22);
    b22 = M2{add(E.e[2][0], t.a), add(E.e[2][1], t.b), add(E.e[3][0], t.c), add(E.e[3][1], t.d)};
    rdu = mm2(b22, a22);
  }
  // la now holds layer 1's decays; u is layer 1
  Ev top;
  top.A[0] = C(1.0); top.A[1] = u.cs; top.A[2] = u.cp;
  top.A[3] = neg(rmul(u.am, u.cp)); top.A[4] = neg(rmul(u.am, C(u.xi))); top.A[5] = neg(rmul(u.am, u.cs));
  M2 b22{mul(aent<2, 2>(top), la0), mul(aent<2, 3>(top), la1), mul(aent<3, 2>(top), la0),
         mul(aent<3, 3>(top), la1)};
  const M2 t = mm2(b22, rdu);
  const M2 a{add(aent<2, 0>(top), t.a), add(aent<2, 1>(top), t.b), add(aent<3, 0>(top), t.c),
             add(aent<3, 1>(top), t.d)};
  const cx dsp = sub(mul(a.a, a.d), mul(a.b, a.c));
  *imf = dsp.im;
  return dsp.re;
}

// SecFuns_L at lay = 1 (Love.f90:118-132): propdn_L (Love.f90:69-90) gives
// RudL(0), propup_L (Love.f90:92-116) RduL(1); EinvE_L (Love.f90:39-67)
__device__ double secfun_love(Col &g, double c, double *imf) {
  g.evals++;
  const double vk = g.w / c;
  cx rud0;
  {
    const double am = g.MU(0);
    const cx cs1 = csq(c, g.VS(0));
    const cx a22_22 = rmul(am, cs1), a22_21 = neg(a22_22);
    const cx la2 = decay(g.D(0), vk, cs1);
    rud0 = neg(cdiv(mul(a22_22, la2), a22_21));
  }
  // EinvE_L(j, c, 0) = b22 @ a22 with a22 = [[1, 1], [-m1 cs1, m1 cs1]] (the
  // layer below) and b22 = [[m0 cs0, -1], [m0 cs0, 1]] / (2 m0 cs0) (above);
  // the layer below one interface is the layer above the previous one, so
  // its slowness and decay carry over
  auto einve_l = [&](int j, const cx &cs0, const cx &cs1, M2 &E) {
    const double am1 = g.MU(j), am0 = g.MU(j - 1);
    const cx a12 = rmul(am1, cs1);
    const M2 a{C(1.0), C(1.0), neg(a12), a12};
    const cx b0 = rmul(am0, cs0);
    const cx den = rmul(2.0, b0);
    const cx h = cdiv(b0, den);
    const M2 b{h, cdiv(C(-1.0), den), h, cdiv(C(1.0), den)};
    E = mm2(b, a);
  };
  const int j2 = g.ll - 1;
  cx cs1 = csq(c, g.VS(j2)), cs0 = csq(c, g.VS(j2 - 1));
  M2 E;
  einve_l(j2, cs0, cs1, E);
  cx dec0 = decay(g.D(j2 - 1), vk, cs0);
  cx td = cdiv(dec0, E.a);
  cx rdu = mul(E.c, td);
  for (int j = j2 - 1; j >= 1; --j) {
    cs1 = cs0;
    cs0 = csq(c, g.VS(j - 1));
    einve_l(j, cs0, cs1, E);
    const cx r = mul(dec0, rdu);                    // decay(D(j), vk, cs of layer j)
    dec0 = decay(g.D(j - 1), vk, cs0);
    td = cdiv(dec0, add(E.a, mul(E.b, r)));
    rdu = mul(add(E.c, mul(E.d, r)), td);
  }
  const cx dsp = sub(C(1.0), mul(rud0, rdu));
  *imf = dsp.re;
  return dsp.im;
}

template <int W> __device__ __forceinline__ double secfun(Col &g, double c, double *imf) {
  return W == 1 ? secfun_surf(g, c, imf) : secfun_love(g, c, imf);
}

// N_cf (C_interval.f90:188-208) / N_cf_L (C_interval_L.f90:186-204)
template <int W> __device__ double n_cf(const Col &g, double c) {
  double s = 0;
  for (int i = 0; i < g.nl - 1; ++i) {
    double yr = 0;
    if (W == 1) { const double t = c / g.VP(i); yr = csqrt_real(t * t - 1.0).re; }
    double ys = 0;
    const double b = g.VS(i);
    if (b > 0.0) { const double t = c / b; ys = csqrt_real(t * t - 1.0).re; }
    s = s + ((2.0 * (yr + ys)) * g.D(i)) / c;
  }
  return g.w / (2.0 * (W == 1 ? kPiS : kPiD)) * s;
}

// In-place ascending Shell sort of x[0..n) (the reference's sort,
// util.f90:389-437, with the same increments)
__device__ void shell_sort(double *x, int n) {
  int inc = 1;
  do { inc = 3 * inc + 1; } while (inc <= n);
  do {
    inc /= 3;
    for (int i = inc; i < n; ++i) {
      const double v = x[i];
      int j = i;
      while (x[j - inc] > v) {
        x[j] = x[j - inc];
        j -= inc;
        if (j < inc) break;
      }
      x[j] = v;
    }
  } while (inc > 1);
}

// C_Interval (C_interval.f90:1-186) / C_Interval_L (C_interval_L.f90:1-184):
// the trial phase velocities, thinned and sorted, into buf (capacity cap + 1
// entries; the list starts at *start). Returns the count, or -1 where more
// than 20,000 entries (or more than cap) would be needed.
template <int W> __device__ int c_interval(const Col &g, double *buf, int cap, int *start, int *im1) {
  double *vv = buf + 1;                 // room to prepend vsm + tol
  const int lim = cap < kNccc ? cap : kNccc;
  int n = 0;
#define PUSH(x) do { if (n >= lim) return -1; vv[n++] = (x); } while (0)
  const double freq = g.w / (2.0 * (W == 1 ? kPiS : kPiD));
  const long long NN = llround(n_cf<W>(g, g.vsy) - n_cf<W>(g, g.vsm));
  const double v1 = g.V(0);
  if (freq < (double)0.12f || NN < 2) {
    const long long m = (NN + 1) * (W == 1 ? 1024 : 512);
    if (m > lim || m < 0) return -1;
    const double lo = W == 1 ? v1 - 0.1 : g.vsm - 0.01;
    const double span = W == 1 ? g.vsy - v1 + 0.1 : g.vsy - g.vsm + 0.01;
    for (long long i = 1; i <= m; ++i) vv[n++] = lo + (double)i * span / (double)m;
    for (int i = 1; i <= 100; ++i) PUSH(g.vsy * (1.0 - 0.008 * (double)i));
  } else {
    const double c1 = W == 1 ? v1 : g.vsm;
    PUSH(c1);
    double c2 = g.vsy, c0 = c2, dc = 0;
    long long NNc = NN;
    while (c0 > c1) {
      if (NNc > 0) dc = (c2 - c1) / (double)NNc;
      c0 = c2 - dc;
      for (int h = 0;; ++h) {
        const double dN = n_cf<W>(g, c2) - n_cf<W>(g, c0);
        if (dN < 0.5) { PUSH(c0); NNc--; c2 = c0; break; }
        if (h >= 1100) return -1;          // not finite: c0 == c2 after ~1,075 halvings
        c0 = (c2 + c0) / 2.0;
      }
    }
    int ij = 1;
    while (ij <= 2 * g.nl && g.V(ij - 1) <= g.vsy) ij++;
    for (int i = 1; i <= ij - 2; ++i) {
      const double c01 = g.V(i - 1);
      int ii = 0;
      for (int j = 1; j <= g.nl; ++j)
        if (fabs(g.VS(j - 1) - c01) < kEpsGrt || fabs(g.VP(j - 1) - c01) < kEpsGrt) ii = j;
      if (ii == 0) continue;
      const double hi = g.D(ii - 1);
      const double Ni = 2.0 * freq * hi / c01 + kEpsGrt;
      const long long nj = (long long)floor(Ni);
      for (long long j = 1; j <= nj; ++j) {
        const double r = (double)j / Ni;
        const double c00 = c01 / sqrt(1.0 - r * r);
        if (c00 <= g.vsy) PUSH(c00);
      }
    }
    shell_sort(vv, n);
    for (int rep = 0; rep < 2; ++rep) {
      const int m = n;
      for (int i = 0; i < m - 1; ++i) PUSH((vv[i] + vv[i + 1]) / 2.0);
    }
    for (int i = 1; i <= 100; ++i) PUSH(g.vsy - (double)i / 100.0 * 0.1);
  }
  for (int i = 1; i <= 10; ++i) PUSH(g.vsy - (double)(i * 10) * g.tol);
  PUSH(g.vsy - 3.0 * g.tol);
  PUSH(g.vs1 + 4.0 * g.tol);
  PUSH(g.vs1 - 4.0 * g.tol);
#undef PUSH
  shell_sort(vv, n);
  // no point at or below vsm: the list restarts at the first point above it,
  // preceded by vsm + tol
  int s = 0, e = n;
  for (int i = 0; i < n; ++i) {
    if (vv[i] > g.vsm) { s = i - 1; vv[s] = g.vsm + g.tol; break; }
  }
  // vv[-1] is buf[0]: a list whose first point is above vsm is prepended
  while (e - 1 >= s && vv[e - 1] >= g.vsy) e--;
  if (e - 1 < s) return -1;
  const double tol0 = 10.0 * g.tol;
  double prev = vv[s];
  int k = s + 1;
  for (int i = s + 1; i < e; ++i) {
    const double x = vv[i];
    if (x - prev < tol0) { prev = x; continue; }
    prev = x;
    vv[k++] = x;
  }
  const int cnt = k - s;
  int m1 = 0;
  for (int i = 0; i < cnt; ++i) {
    const double x = vv[s + i];
    if (W == 1 ? x >= g.vs1 : x > g.vs1) { m1 = i + 1; break; }
  }
  if (m1 == 0 && W == 1) m1 = cnt;
  *im1 = m1;
  *start = s + 1;                        // index into buf
  return cnt;
}

// CR0_Finder (SearchRayleigh.f90:898-933): Newton on the half-space Rayleigh
// function; the reference's loop is unbounded, 10,000 iterations here
__device__ double cr0_finder(double v1, double v2) {
  const double tol = 1e-7;
  double c = 0.8 * v1;
  for (int it = 0; it < 10000; ++it) {
    const double ps = 1.0 / v1, pp = 1.0 / v2, p = 1.0 / c;
    const double p2 = p * p, ps2 = ps * ps, pp2 = pp * pp;
    const double sps = sqrt(p2 - ps2), spp = sqrt(p2 - pp2);
    const double a = ps2 - 2.0 * p2;
    const double R = a * a - 4.0 * p2 * sps * spp;
    const double DR = p2 * (8.0 * p * (ps2 - 2.0 * p2) + 8.0 * p * sps * spp +
                            4.0 * (p2 * p) * (spp / sps + sps / spp));
    c = c - R / DR;
    if (v1 - c < tol || v2 - c < tol || c != c) break;
    if (fabs(R / DR) < tol) break;
  }
  return c;
}

// setup_grt (surfmodes.f90:320-450) for column c; returns 0, -1 for a layer
// count outside 2..nl_max, or -2 for a fluid layer (the Stoneley-mode path,
// not built)
__device__ int setup_col(const GrtJob &J, int c, Col &g) {
  const double eps = (double)1e-6f;
  const int nl = J.nl[c];
  if (nl < 2 || nl > J.nl_max) return -1;
  g.nl = nl; g.stride = J.ncol;
  g.d = J.thk + c; g.vp = J.vp + c; g.vs = J.vs + c; g.mu = J.mu + c; g.v = J.v + c;
  double *mu = J.mu + c, *v = J.v + c;
  const size_t S = (size_t)J.ncol;
  int n = 0;
  for (int i = 0; i < nl; ++i) {
    const double b = g.VS(i);
    if (!(fabs(b) > eps)) return -2;
    // insertion into the sorted list of vs and vp values
    for (int r = 0; r < 2; ++r) {
      const double x = r == 0 ? b : g.VP(i);
      int k = n;
      while (k > 0 && v[(size_t)(k - 1) * S] > x) { v[(size_t)k * S] = v[(size_t)(k - 1) * S]; --k; }
      v[(size_t)k * S] = x;
      ++n;
    }
  }
  int idx = 0;
  double mu0 = 0;
  for (int i = 0; i < nl; ++i) {
    const double b = g.VS(i);
    const double m = J.rho[(size_t)i * S + c] * (b * b);
    if (fabs(m) > eps) { idx++; mu0 += m; }
    mu[(size_t)i * S] = m;
  }
  mu0 = mu0 / idx;
  for (int i = 0; i < nl; ++i) mu[(size_t)i * S] = mu[(size_t)i * S] / mu0;
  double vsy = g.VS(0), vmin = g.VS(0);
  for (int i = 1; i < nl; ++i) { vsy = fmax(vsy, g.VS(i)); vmin = fmin(vmin, g.VS(i)); }
  g.vsy = vsy;
  g.vs1 = g.VS(0);
  g.vsm = J.modetype == 1 ? g.V(0) : vmin;
  int nlvl1 = 0, no_lvl = 0, last = 0;
  for (int i = 1; i < nl - 1; ++i) {
    if (g.VP(i) < g.VP(i + 1) && g.VP(i) < g.VP(i - 1)) {
      no_lvl++;
      last = i + 1;
      if (g.VS(i) < g.vs1) nlvl1++;
    }
  }
  g.nlvl1 = nlvl1;
  g.lvlast = no_lvl == 0 ? 1 : last;
  if (g.lvlast < 2) g.lvlast = 2;
  g.dc = J.dc;
  g.evals = 0;
  return 0;
}

// The fundamental-mode search of RayleighModes / LoveModes for one column as
// a resumable state machine: advance() runs the reference's control flow
// (SearchRayleigh's FundaMode, SearchRayleigh.f90:455-605; SearchLove's
// FundaMode, SearchLove.f90:204-270; bisecim, util.f90:90-167; the
// frequency loop and CalGroup, surfmodes.f90:185-318) up to the next
// secular-function evaluation or trial-velocity list it needs, and stops.
// The kernel then evaluates the pending requests of all the lanes of a warp
// together, so the expensive evaluation runs converged however far apart
// the columns' searches are. Each column sees exactly the sequence of
// evaluations of the sequential search. SearchLove's layer-velocity test
// reads a variable the single-mode path never sets and passes here.
enum : int {
  S_FREQ, S_DONE_SEARCH, S_COLUMN_DONE,
  R_BEGIN, R_WIN_FIRST, R_WIN_NEXT, R_WIN_GOT, R_WIN_BIS, R_WIN_CHECK,
  R_FB_BEGIN, R_FB_CI, R_FB_FIRST, R_FB_NEXT, R_FB_GOT, R_FB_BIS, R_END,
  L_BEGIN, L_CI, L_FIRST, L_NEXT, L_GOT, L_BIS, L_FB_BEGIN, L_FB_FIRST, L_FB_NEXT, L_FB_GOT, L_FB_BIS, L_END,
  B_ITER, B_GOT3, B_FINAL
};
enum : int { REQ_NONE = 0, REQ_EVAL = 1, REQ_CI = 2 };

struct Search {
  int s, ret, req;
  int sl;                      // run startl(rc) before the requested evaluation
  double rc;                   // requested phase velocity
  double f, imf;               // delivered secular-function value
  int index0, start, im1;      // delivered trial list
  int i, grp, e;               // frequency (1-based), group search, ierr
  double c0, cray, fr;
  double *ph, *gr;
  int j, nk, ip, iq, ierr;
  double cmn, step, k1, k2, f1, f2, c0l;
  double xa, xb, ya, yb, fa, xt1, xt2, x3, y3, imf3, dx, kt;
  int nc;
};

__device__ __forceinline__ void bis_begin(Search &S, double x1, double x2, double f1, double f2, int ret) {
  S.nc = 0; S.dx = fabs(x1 - x2); S.fa = f1;
  S.xa = x1; S.xb = x2; S.ya = f1; S.yb = f2;
  S.xt1 = (S.xa + S.xb) / 2.0; S.ret = ret; S.s = B_ITER;
}

#define REQUEST(c, next) do { S.rc = (c); S.sl = 0; S.req = REQ_EVAL; S.s = (next); return; } while (0)
// an evaluation at a scan point, which the reference precedes by startl at it
#define REQUEST_SL(c, next) do { S.rc = (c); S.sl = 1; S.req = REQ_EVAL; S.s = (next); return; } while (0)

template <int W>
__device__ void advance(Search &S, Col &g, const GrtJob &J, const double *buf) {
  const double dh = (double)0.005f;
  S.req = REQ_NONE;
  for (;;) {
    switch (S.s) {
    case S_FREQ:
      if (S.i > J.np) { S.s = S_COLUMN_DONE; return; }
      S.fr = J.freqs[S.i - 1];
      g.w = S.fr * 2.0 * kPiS;
      g.tol = J.tolmin + (double)(J.np + 1 - S.i) * (J.tolmax - J.tolmin) / (double)J.np;
      g.smin = J.smin_min + (double)(S.i - 1) * (J.smin_max - J.smin_min) / (double)J.np;
      S.grp = 0; S.cray = S.c0;
      S.s = W == 1 ? R_BEGIN : L_BEGIN;
      break;
    case S_DONE_SEARCH:
      if (S.e) { S.s = S_COLUMN_DONE; return; }
      if (!S.grp) {
        S.ph[S.i - 1] = S.cray; S.c0 = S.cray;
        if (J.phase_group == 1) {
          S.grp = 1; g.w = (S.fr + dh) * 2.0 * kPiS; S.cray = S.c0;
          S.s = W == 1 ? R_BEGIN : L_BEGIN;
          break;
        }
      } else {
        const double grp = (S.fr + dh) / S.cray - S.fr / S.ph[S.i - 1];
        S.gr[S.i - 1] = grp > 0 ? dh / grp : 0.0;
      }
      S.i++; S.s = S_FREQ;
      break;
    // ---- SearchRayleigh's FundaMode
    case R_BEGIN: {
      S.ierr = 1; S.iq = -1;
      double cmn; int nk;
      if (S.cray > 0.) { cmn = (double)0.90f * S.cray; nk = 10; }
      else { cmn = cr0_finder(g.vs1, g.VP(0)); cmn = cmn - 0.1; nk = 100; }
      const double cmx = g.vs1 - 4.0 * g.tol;
      if (cmx > cmn) {
        S.cmn = cmn; S.nk = nk; S.step = (cmx - cmn) / (double)nk;
        startl(cmn + S.step * (double)nk, g);
        S.j = 1; S.iq = 1; S.k2 = cmn + S.step * 1.0;
        REQUEST(S.k2, R_WIN_FIRST);
      }
      S.s = R_FB_BEGIN;
      break;
    }
    case R_WIN_FIRST: S.f2 = S.f; S.s = R_WIN_NEXT; break;
    case R_WIN_NEXT:
      S.k1 = S.k2; S.f1 = S.f2; S.j++;
      S.k2 = S.cmn + S.step * (double)S.j;
      REQUEST(S.k2, R_WIN_GOT);
    case R_WIN_GOT:
      S.f2 = S.f;
      if (S.f1 * S.f2 < 0.) { bis_begin(S, S.k1, S.k2, S.f1, S.f2, R_WIN_BIS); break; }
      S.s = R_WIN_CHECK;
      break;
    case R_WIN_BIS:
      if (S.iq == 0) { S.cray = S.kt; S.ierr = 0; S.s = R_END; break; }
      S.s = R_WIN_CHECK;
      break;
    case R_WIN_CHECK:
      S.s = S.j == S.nk ? R_FB_BEGIN : R_WIN_NEXT;
      break;
    case R_FB_BEGIN: S.req = REQ_CI; S.s = R_FB_CI; return;
    case R_FB_CI: {
      if (S.index0 < 0) { S.e = 2; S.s = S_DONE_SEARCH; break; }
      const double *ccc = buf + S.start - 1;
      int im2 = S.im1;
      if (g.nlvl1 == 0) {
        while (ccc[im2] < S.cray - 2.0 * g.dc) { im2++; if (im2 == S.index0) break; }
      }
      S.k2 = ccc[im2]; S.ip = im2 + 1;
      REQUEST_SL(S.k2, R_FB_FIRST);
    }
    case R_FB_FIRST: S.f2 = S.f; S.s = R_FB_NEXT; break;
    case R_FB_NEXT: {
      if (S.ip > S.index0) { S.s = R_END; break; }
      const double *ccc = buf + S.start - 1;
      S.k1 = S.k2; S.f1 = S.f2; S.k2 = ccc[S.ip]; S.iq = -1;
      REQUEST_SL(S.k2, R_FB_GOT);
    }
    case R_FB_GOT:
      S.f2 = S.f;
      if (S.f1 * S.f2 < 0.) { bis_begin(S, S.k1, S.k2, S.f1, S.f2, R_FB_BIS); break; }
      S.ip++; S.s = R_FB_NEXT;
      break;
    case R_FB_BIS:
      if (S.iq == 0) { S.cray = S.kt; S.ierr = 0; S.s = R_END; break; }
      S.ip++; S.s = R_FB_NEXT;
      break;
    case R_END: S.e = S.ierr; S.s = S_DONE_SEARCH; break;
    // ---- SearchLove's FundaMode
    case L_BEGIN: S.req = REQ_CI; S.s = L_CI; return;
    case L_CI: {
      if (S.index0 < 0) { S.e = 2; S.s = S_DONE_SEARCH; break; }
      S.ierr = 1; S.iq = -1; S.c0l = S.cray;
      const double *ccc = buf + S.start - 1;
      S.k2 = ccc[1]; S.ip = 2;
      REQUEST_SL(S.k2, L_FIRST);
    }
    case L_FIRST: S.f2 = S.f; S.s = L_NEXT; break;
    case L_NEXT: {
      if (S.ip > S.index0) { S.s = L_FB_BEGIN; break; }
      const double *ccc = buf + S.start - 1;
      S.k1 = S.k2; S.f1 = S.f2; S.k2 = ccc[S.ip]; S.iq = -1;
      REQUEST_SL(S.k2, L_GOT);
    }
    case L_GOT:
      S.f2 = S.f;
      if (S.f1 * S.f2 < 0.) { bis_begin(S, S.k1, S.k2, S.f1, S.f2, L_BIS); break; }
      S.ip++; S.s = L_NEXT;
      break;
    case L_BIS:
      if (S.iq == 0) { S.cray = S.kt; S.ierr = 0; S.s = L_END; break; }
      S.ip++; S.s = L_NEXT;
      break;
    case L_FB_BEGIN:
      if (S.ierr == 1 && isfinite(S.c0l)) {
        S.k2 = (double)1.1f * S.c0l;
        REQUEST_SL(S.k2, L_FB_FIRST);
      }
      S.s = L_END;
      break;
    case L_FB_FIRST: S.f2 = S.f; S.s = L_FB_NEXT; break;
    case L_FB_NEXT:
      S.k1 = S.k2 - g.dc;
      if (S.k1 < g.vsm) { S.s = L_END; break; }
      REQUEST_SL(S.k1, L_FB_GOT);
    case L_FB_GOT:
      S.f1 = S.f; S.iq = -1;
      if (S.f1 * S.f2 < 0.) { bis_begin(S, S.k1, S.k2, S.f1, S.f2, L_FB_BIS); break; }
      S.k2 = S.k1; S.f2 = S.f1; S.s = L_FB_NEXT;
      break;
    case L_FB_BIS:
      if (S.iq == 0) { S.cray = S.kt; S.ierr = 0; S.s = L_END; break; }
      S.k2 = S.k1; S.f2 = S.f1; S.s = L_FB_NEXT;
      break;
    case L_END:
      if (S.ierr == 1) S.cray = 0;
      S.e = S.ierr; S.s = S_DONE_SEARCH;
      break;
    // ---- bisecim
    case B_ITER:
      S.x3 = (S.xa + S.xb) / 2.0;
      REQUEST(S.x3, B_GOT3);
    case B_GOT3: {
      S.y3 = S.f; S.imf3 = S.imf;
      const double u1 = (S.xb - S.xa) / (S.yb - S.ya);
      const double u2 = (S.xb - S.x3) / (S.yb - S.y3);
      S.xt2 = S.xa - S.ya * (u1 - S.yb * ((u2 - u1) / (S.y3 - S.ya)));
      double dxt = fabs(S.xt2 - S.xt1);
      S.dx = S.dx / 2.0;
      if (S.dx < dxt) dxt = S.dx;
      if (dxt < g.tol) REQUEST(S.xt2, B_FINAL);
      S.xt1 = S.xt2;
      if (S.fa * S.y3 < 0) { S.xb = S.x3; S.yb = S.y3; }
      else { S.xa = S.x3; S.ya = S.y3; }
      S.nc++;
      if (S.nc >= 1000) { S.iq = -1; S.kt = 0.0; S.s = S.ret; break; }
      S.s = B_ITER;
      break;
    }
    case B_FINAL: {
      const double smin2 = g.smin * g.smin * 2.0;
      const double u1 = S.f, u2 = S.y3;
      if (u1 * u1 + S.imf * S.imf < smin2 || u2 * u2 + S.imf3 * S.imf3 < smin2) {
        S.iq = 0; S.kt = fabs(u1) < fabs(u2) ? S.xt2 : S.x3;
      } else {
        S.iq = -1; S.kt = 0.0;
      }
      S.s = S.ret;
      break;
    }
    default:
      S.s = S_COLUMN_DONE;
      return;
    }
  }
}
#undef REQUEST
#undef REQUEST_SL

// Persistent grid over the columns: a lane whose column is done takes the
// next one from the pool counter J.next; redo runs only the columns a
// previous pass left with ierr 2
// (trial list over that pass's room). Every round, each lane advances its
// search to its next request; lanes wanting a trial list build it, then all
// lanes wanting an evaluation evaluate together.
template <int W>
__global__ void __launch_bounds__(128, W == 1 ? 3 : 4) grt_kernel(GrtJob J, int cap, int redo) {
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  double *buf = J.scratch + (size_t)tid * (cap + 1);
  unsigned long long evals = 0;
  Search S;
  S.s = S_COLUMN_DONE; S.req = REQ_NONE; S.e = 0;
  Col g;
  g.evals = 0;
  int c = -1;
  bool active = true;
  for (;;) {
    while (active && S.req == REQ_NONE) {
      if (S.s == S_COLUMN_DONE) {
        if (c >= 0) {
          J.ierr[c] = S.e;
          if (!(S.e == 2 && !redo)) evals += g.evals;   // a column redone in the next pass counts there
          c = -1;
        }
        const unsigned q = atomicAdd(J.next, 1u);          // the next column of the pool
        if (q >= (unsigned)J.n) { active = false; break; }
        const int cc = J.cols ? J.cols[q] : (int)q;
        if (redo && J.ierr[cc] != 2) continue;
        c = cc;
        S.ph = J.phase + (size_t)c * J.np; S.gr = J.group + (size_t)c * J.np;
        for (int i = 0; i < J.np; ++i) { S.ph[i] = 0.0; S.gr[i] = 0.0; }
        g.evals = 0;
        S.e = setup_col(J, c, g);
        if (S.e) continue;                              // S.s is still S_COLUMN_DONE
        S.i = 1; S.c0 = 0.0; S.s = S_FREQ;
      }
      advance<W>(S, g, J, buf);
    }
    if (!__any_sync(0xffffffffu, active)) break;
    __syncwarp();                                       // the lanes take the requests together
    if (active && S.req == REQ_CI) {
      S.index0 = c_interval<W>(g, buf, cap, &S.start, &S.im1);
      S.req = REQ_NONE;
    }
    __syncwarp();
    if (active && S.req == REQ_EVAL) {
      if (S.sl) startl(S.rc, g);
      S.f = secfun<W>(g, S.rc, &S.imf);
      S.req = REQ_NONE;
    }
  }
  if (J.nevals && evals) atomicAdd(J.nevals, evals);
}

__global__ void grt_transpose_kernel(const double *src, double *dst, int ncol, int nl_max) {
  const size_t n = (size_t)ncol * nl_max;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    const size_t c = k % ncol, i = k / ncol;
    dst[k] = src[c * nl_max + i];
  }
}

}  // namespace

int grt_threads(int n, int pass, int modetype) {
  int dev = 0, sms = 152, occ = 2;
  if (cudaGetDevice(&dev) == cudaSuccess) {
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const cudaError_t e = modetype == 1 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, grt_kernel<1>, 128, 0)
                                        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, grt_kernel<0>, 128, 0);
    if (e != cudaSuccess || occ < 1) occ = 1;
  }
  const long want = (long)sms * (pass == 0 ? occ * 128 : 32);
  // columns per lane: one. Each lane's search is a chain of dependent FP64
  // work, so the kernel's rate grows with the lanes in flight; two per lane
  // balance a warp's lanes better only when the columns are several times
  // the resident lanes (Rayleigh curves of 27,049 columns: 51 s with two,
  // 61 s with one; of 6,700: four times slower with two).
  // MCT_GRT_COLS_PER_LANE overrides it for tuning.
  static const int per = [] {
    const char *e = getenv("MCT_GRT_COLS_PER_LANE");
    const int v = e ? atoi(e) : 1;
    return v >= 1 ? v : 1;
  }();
  const long byn = (n + per - 1) / per;
  long t = byn < want ? byn : want;
  t = (t + 127) / 128 * 128;
  return (int)(t > 0 ? t : 128);
}

size_t grt_scratch_doubles(int n, int modetype) {
  const size_t a = (size_t)grt_threads(n, 0, modetype) * (kGrtCap0 + 1);
  const size_t b = (size_t)grt_threads(n, 1, modetype) * (kGrtCap1 + 1);
  return a > b ? a : b;
}

int launch_grt(const GrtJob &J, const double *const rows[4], double *cols4, cudaStream_t s) {
  if (J.n <= 0) return MCT_OK;
  GrtJob K = J;
  const size_t lay = (size_t)J.ncol * J.nl_max;
  double *dst[4];
  for (int a = 0; a < 4; ++a) {
    dst[a] = cols4 + a * lay;
    grt_transpose_kernel<<<(int)std::min<size_t>((lay + 255) / 256, 4096), 256, 0, s>>>(rows[a], dst[a], J.ncol,
                                                                                       J.nl_max);
  }
  MCT_CUDA_TRY(cudaGetLastError());
  K.thk = dst[0]; K.vp = dst[1]; K.vs = dst[2]; K.rho = dst[3];
  for (int pass = 0; pass < 2; ++pass) {
    MCT_CUDA_TRY(cudaMemsetAsync(K.next, 0, sizeof(unsigned), s));
    const int threads = grt_threads(J.n, pass, J.modetype);
    if (J.modetype == 1) grt_kernel<1><<<threads / 128, 128, 0, s>>>(K, pass == 0 ? kGrtCap0 : kGrtCap1, pass);
    else grt_kernel<0><<<threads / 128, 128, 0, s>>>(K, pass == 0 ? kGrtCap0 : kGrtCap1, pass);
    MCT_CUDA_TRY(cudaGetLastError());
  }
  return MCT_OK;
}
