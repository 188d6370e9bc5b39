// Rayleigh/Love phase and group velocities of 1D layered columns: the GPU
// replacement of surfdisp96 / surfdisp_mmodes (surfmodes/surfdisp96.f:52-701)
// as routed by surfmodes (surfmodes/surfmodes.f90:39-183).
//
// One thread owns one column and walks its periods in order, because each
// period's root search starts from the previous period's root
// (surfdisp96.f:272-281); the batch supplies the parallelism (columns x
// chains). The period equation (dltar4 / dltar1, surfdisp96.f:1056-1217) is
// evaluated in FP64 with the reference's operation order (this file is built
// with -fmad=false, so no FMA contraction). The REAL*4 model, the REAL*4
// search increment and group-velocity formula, and the REAL*4 literal 0.01 in
// nevill are reproduced.
//
// precision == 1 runs the bracketing scan of getsol (surfdisp96.f:793-815),
// which is most of the work, with an FP32 period equation, then re-evaluates
// both ends of the bracket it found in FP64; only if their FP64 signs confirm
// it (start sign on the low side, opposite sign on the high side) does the
// FP64 Neville/bisection polish start from it, otherwise the scan is redone
// in FP64. The polished roots are therefore the FP64 algorithm's.
#include "mct_common.cuh"

namespace {

constexpr int NPMAX = 60;   // surfdisp96.f:58 NP

struct Col {
  const float *d, *a, *b, *rho;
  int mmax, llw;
};

template <class T> struct M;
template <> struct M<double> {
  static __device__ __forceinline__ double sin_(double x) { return sin(x); }
  static __device__ __forceinline__ double cos_(double x) { return cos(x); }
  static __device__ __forceinline__ double exp_(double x) { return exp(x); }
  static __device__ __forceinline__ double sqrt_(double x) { return sqrt(x); }
};
template <> struct M<float> {
  static __device__ __forceinline__ float sin_(float x) { return sinf(x); }
  static __device__ __forceinline__ float cos_(float x) { return cosf(x); }
  static __device__ __forceinline__ float exp_(float x) { return expf(x); }
  static __device__ __forceinline__ float sqrt_(float x) { return sqrtf(x); }
};

template <class T> struct VarOut { T w, cosp, a0, cpcq, cpy, cpz, cqw, cqx, xy, xz, wy, wz; };

// surfdisp96.f:1220-1337 var (the final rescale of cosq/y/z only touches
// locals that are not returned and is omitted)
template <class T>
__device__ __forceinline__ void var(T p, T q, T ra, T rb, T wvno, T xka, T xkb, T dpth, VarOut<T> &o) {
  T pex = 0, sex = 0, sinp = 0, w = 0, x = 0, cosp = 0, sinq = 0, y = 0, z = 0, cosq = 0, fac;
  if (wvno < xka) {
    sinp = M<T>::sin_(p); w = sinp / ra; x = -ra * sinp; cosp = M<T>::cos_(p);
  } else if (wvno == xka) {
    cosp = 1; w = dpth; x = 0;
  } else if (wvno > xka) {
    pex = p; fac = 0;
    if (p < 16) fac = M<T>::exp_(T(-2) * p);
    cosp = (T(1) + fac) * T(0.5); sinp = (T(1) - fac) * T(0.5);
    w = sinp / ra; x = ra * sinp;
  }
  if (wvno < xkb) {
    sinq = M<T>::sin_(q); y = sinq / rb; z = -rb * sinq; cosq = M<T>::cos_(q);
  } else if (wvno == xkb) {
    cosq = 1; y = dpth; z = 0;
  } else if (wvno > xkb) {
    sex = q; fac = 0;
    if (q < 16) fac = M<T>::exp_(T(-2) * q);
    cosq = (T(1) + fac) * T(0.5); sinq = (T(1) - fac) * T(0.5);
    y = sinq / rb; z = rb * sinq;
  }
  T exa = pex + sex;
  T a0 = 0;
  if (exa < 60) a0 = M<T>::exp_(-exa);
  o.w = w; o.cosp = cosp; o.a0 = a0;
  o.cpcq = cosp * cosq; o.cpy = cosp * y; o.cpz = cosp * z;
  o.cqw = cosq * w; o.cqx = cosq * x;
  o.xy = x * y; o.xz = x * z; o.wy = w * y; o.wz = w * z;
}

// surfdisp96.f:1119-1217 dltar4 with dnka (1370-1414) and normc (1341-1366)
// fused: the 5x5 Dunkin matrix is formed column by column and applied to the
// propagated 5-vector in the same summation order as the reference.
template <class T>
__device__ T dltar4(T wvno, T omga, const Col &m) {
  T omega = omga;
  if (omega < T(1.0e-4)) omega = T(1.0e-4);
  T wvno2 = wvno * wvno;
  int mm = m.mmax - 1;
  T xka = omega / (T)__ldg(&m.a[mm]);
  T xkb = omega / (T)__ldg(&m.b[mm]);
  T wvnop = wvno + xka, wvnom = fabs(wvno - xka);
  T ra = M<T>::sqrt_(wvnop * wvnom);
  wvnop = wvno + xkb; wvnom = fabs(wvno - xkb);
  T rb = M<T>::sqrt_(wvnop * wvnom);
  T t = (T)__ldg(&m.b[mm]) / omega;
  T gammk = T(2) * t * t;
  T gam = gammk * wvno2;
  T gamm1 = gam - T(1);
  T rho1 = (T)__ldg(&m.rho[mm]);
  T e[5];
  e[0] = rho1 * rho1 * (gamm1 * gamm1 - gam * gammk * ra * rb);
  e[1] = -rho1 * ra;
  e[2] = rho1 * (gamm1 - gammk * ra * rb);
  e[3] = rho1 * rb;
  e[4] = wvno2 - ra * rb;
  VarOut<T> v;
  for (int l = m.mmax - 2; l >= m.llw - 1; --l) {
    T al = (T)__ldg(&m.a[l]), bl = (T)__ldg(&m.b[l]);
    xka = omega / al;
    xkb = omega / bl;
    t = bl / omega;
    gammk = T(2) * t * t;
    gam = gammk * wvno2;
    wvnop = wvno + xka; wvnom = fabs(wvno - xka);
    ra = M<T>::sqrt_(wvnop * wvnom);
    wvnop = wvno + xkb; wvnom = fabs(wvno - xkb);
    rb = M<T>::sqrt_(wvnop * wvnom);
    T dpth = (T)__ldg(&m.d[l]);
    rho1 = (T)__ldg(&m.rho[l]);
    var<T>(ra * dpth, rb * dpth, ra, rb, wvno, xka, xkb, dpth, v);
    // dnka
    const T one = 1, two = 2;
    T gm1 = gam - one;
    T twgm1 = gam + gm1;
    T gmgmk = gam * gammk;
    T gmgm1 = gam * gm1;
    T gm1sq = gm1 * gm1;
    T rho2 = rho1 * rho1;
    T a0pq = v.a0 - v.cpcq;
    T ca[5][5];
    ca[0][0] = v.cpcq - two * gmgm1 * a0pq - gmgmk * v.xz - wvno2 * gm1sq * v.wy;
    ca[0][1] = (wvno2 * v.cpy - v.cqx) / rho1;
    ca[0][2] = -(twgm1 * a0pq + gammk * v.xz + wvno2 * gm1 * v.wy) / rho1;
    ca[0][3] = (v.cpz - wvno2 * v.cqw) / rho1;
    ca[0][4] = -(two * wvno2 * a0pq + v.xz + wvno2 * wvno2 * v.wy) / rho2;
    ca[1][0] = (gmgmk * v.cpz - gm1sq * v.cqw) * rho1;
    ca[1][1] = v.cpcq;
    ca[1][2] = gammk * v.cpz - gm1 * v.cqw;
    ca[1][3] = -v.wz;
    ca[1][4] = ca[0][3];
    ca[3][0] = (gm1sq * v.cpy - gmgmk * v.cqx) * rho1;
    ca[3][1] = -v.xy;
    ca[3][2] = gm1 * v.cpy - gammk * v.cqx;
    ca[3][3] = ca[1][1];
    ca[3][4] = ca[0][1];
    ca[4][0] = -(two * gmgmk * gm1sq * a0pq + gmgmk * gmgmk * v.xz + gm1sq * gm1sq * v.wy) * rho2;
    ca[4][1] = ca[3][0];
    ca[4][2] = -(gammk * gm1 * twgm1 * a0pq + gam * gammk * gammk * v.xz + gm1 * gm1sq * v.wy) * rho1;
    ca[4][3] = ca[1][0];
    ca[4][4] = ca[0][0];
    T tt = -two * wvno2;
    ca[2][0] = tt * ca[4][2];
    ca[2][1] = tt * ca[3][2];
    ca[2][2] = v.a0 + two * (v.cpcq - ca[0][0]);
    ca[2][3] = tt * ca[1][2];
    ca[2][4] = tt * ca[0][2];
    T ee[5];
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      T cr = 0;
#pragma unroll
      for (int j = 0; j < 5; ++j) cr = cr + e[j] * ca[j][i];
      ee[i] = cr;
    }
    T t1 = 0;
#pragma unroll
    for (int i = 0; i < 5; ++i) if (fabs(ee[i]) > t1) t1 = fabs(ee[i]);
    if (t1 < T(1.0e-40)) t1 = 1;
#pragma unroll
    for (int i = 0; i < 5; ++i) e[i] = ee[i] / t1;
  }
  if (m.llw != 1) {
    xka = omega / (T)__ldg(&m.a[0]);
    wvnop = wvno + xka; wvnom = fabs(wvno - xka);
    ra = M<T>::sqrt_(wvnop * wvnom);
    T dpth = (T)__ldg(&m.d[0]);
    rho1 = (T)__ldg(&m.rho[0]);
    const T znul = T(1.0e-05);
    var<T>(ra * dpth, znul, ra, znul, wvno, xka, znul, dpth, v);
    T w0 = -rho1 * v.w;
    return v.cosp * e[0] + w0 * e[1];
  }
  return e[0];
}

// surfdisp96.f:1056-1115 dltar1 (Love)
template <class T>
__device__ T dltar1(T wvno, T omega, const Col &m) {
  int mm = m.mmax - 1;
  T beta1 = (T)__ldg(&m.b[mm]);
  T rho1 = (T)__ldg(&m.rho[mm]);
  T xkb = omega / beta1;
  T wvnop = wvno + xkb, wvnom = fabs(wvno - xkb);
  T rb = M<T>::sqrt_(wvnop * wvnom);
  T e1 = rho1 * rb;
  T e2 = T(1) / (beta1 * beta1);
  for (int l = m.mmax - 2; l >= m.llw - 1; --l) {
    beta1 = (T)__ldg(&m.b[l]);
    rho1 = (T)__ldg(&m.rho[l]);
    T xmu = rho1 * beta1 * beta1;
    xkb = omega / beta1;
    wvnop = wvno + xkb; wvnom = fabs(wvno - xkb);
    rb = M<T>::sqrt_(wvnop * wvnom);
    T dl = (T)__ldg(&m.d[l]);
    T q = dl * rb;
    T sinq, y, z, cosq;
    if (wvno < xkb) {
      sinq = M<T>::sin_(q); y = sinq / rb; z = -rb * sinq; cosq = M<T>::cos_(q);
    } else if (wvno == xkb) {
      cosq = 1; y = dl; z = 0;
    } else {
      T fac = 0;
      if (q < 16) fac = M<T>::exp_(T(-2) * q);
      cosq = (T(1) + fac) * T(0.5); sinq = (T(1) - fac) * T(0.5);
      y = sinq / rb; z = rb * sinq;
    }
    T e10 = e1 * cosq + e2 * xmu * z;
    T e20 = e1 * y / xmu + e2 * cosq;
    T xnor = fabs(e10), ynor = fabs(e20);
    if (ynor > xnor) xnor = ynor;
    if (xnor < T(1.0e-40)) xnor = 1;
    e1 = e10 / xnor;
    e2 = e20 / xnor;
  }
  return e1;
}

struct Ctx {
  Col m;
  unsigned long long n64, n32;
};

__device__ __forceinline__ double dltar64(double wvno, double omega, int ifunc, Ctx &cx) {
  cx.n64++;
  return ifunc == 1 ? dltar1<double>(wvno, omega, cx.m) : dltar4<double>(wvno, omega, cx.m);
}
__device__ __forceinline__ float dltar32(double wvno, double omega, int ifunc, Ctx &cx) {
  cx.n32++;
  float w = (float)wvno, o = (float)omega;
  return ifunc == 1 ? dltar1<float>(w, o, cx.m) : dltar4<float>(w, o, cx.m);
}

__device__ __forceinline__ double fsign1(double x) { return signbit(x) ? -1.0 : 1.0; }
__device__ __forceinline__ float fsign1f(float x) { return signbit(x) ? -1.f : 1.f; }

__device__ __forceinline__ void half(double c1, double c2, double &c3, double &del3, double omega,
                                     int ifunc, Ctx &cx) {
  c3 = 0.5 * (c1 + c2);
  del3 = dltar64(omega / c3, omega, ifunc, cx);
}

// surfdisp96.f:903-1020 nevill
__device__ double nevill(double t, double c1, double c2, double del1, double del2, int ifunc, Ctx &cx) {
  const double twopi = 2.0 * 3.141592653589793;
  double x[11], y[11];
  double omega = twopi / t;
  double c3, del3;
  half(c1, c2, c3, del3, omega, ifunc, cx);
  int nev = 1, nctrl = 1, m = 1;
  for (;;) {
    nctrl = nctrl + 1;
    if (nctrl >= 100) break;
    if (c3 < fmin(c1, c2) || c3 > fmax(c1, c2)) {
      nev = 0;
      half(c1, c2, c3, del3, omega, ifunc, cx);
    }
    double s13 = del1 - del3;
    double s32 = del3 - del2;
    if (fsign1(del3) * fsign1(del1) < 0.0) { c2 = c3; del2 = del3; }
    else { c1 = c3; del1 = del3; }
    if (fabs(c1 - c2) <= 1.e-6 * c1) break;
    if (fsign1(s13) != fsign1(s32)) nev = 0;
    double ss1 = fabs(del1), s1 = (double)0.01f * ss1;
    double ss2 = fabs(del2), s2 = (double)0.01f * ss2;
    if (s1 > ss2 || s2 > ss1 || nev == 0) {
      half(c1, c2, c3, del3, omega, ifunc, cx);
      nev = 1; m = 1;
    } else {
      if (nev == 2) { x[m] = c3; y[m] = del3; }
      else { x[0] = c1; y[0] = del1; x[1] = c2; y[1] = del2; m = 1; }
      bool fallback = false;
      for (int kk = 1; kk <= m; ++kk) {
        int j = m - kk + 1;
        double denom = y[m] - y[j - 1];
        if (fabs(denom) < 1.0e-10 * fabs(y[m])) { fallback = true; break; }
        x[j - 1] = (-y[j - 1] * x[j] + y[m] * x[j - 1]) / denom;
      }
      if (!fallback) {
        c3 = x[0];
        del3 = dltar64(omega / c3, omega, ifunc, cx);
        nev = 2;
        m = m + 1;
        if (m > 10) m = 10;
      } else {
        half(c1, c2, c3, del3, omega, ifunc, cx);
        nev = 1; m = 1;
      }
    }
  }
  return c3;
}

// Scans step dc from at most (betmx - cm)/dc + a margin; a NaN trial
// velocity (which the reference would step forever) ends the scan as a
// failure after this many steps.
constexpr int kMaxScan = 1 << 20;

// The reference's sequential bracketing scan in FP64 (surfdisp96.f:793-815).
// Returns 1 with c1/c2/del1/del2 set on a bracket, -1 on failure.
__device__ __forceinline__ int scan64(double t1, double &c1, double &del1, double &c2, double &del2,
                                      int idir, double clow, double dc, double cm, float betmx,
                                      int ifunc, Ctx &cx) {
  const double twopi = 2.0 * 3.141592653589793;
  for (int it = 0; it < kMaxScan; ++it) {
    if (idir > 0) c2 = c1 + dc; else c2 = c1 - dc;
    if (c2 <= clow) { idir = +1; c1 = clow; continue; }
    double omega = twopi / t1;
    del2 = dltar64(omega / c2, omega, ifunc, cx);
    if (fsign1(del1) != fsign1(del2)) return 1;
    c1 = c2; del1 = del2;
    if (c1 < cm) return -1;
    if (c1 >= ((double)betmx + dc)) return -1;
  }
  return -1;
}

// surfdisp96.f:734-827 getsol
__device__ void getsol(double t1, double &c1, double clow, double dc, double cm, float betmx,
                       int &iret, int ifunc, int ifirst, double &del1st, int precision, Ctx &cx) {
  const double twopi = 2.0 * 3.141592653589793;
  double omega = twopi / t1;
  double del1 = dltar64(omega / c1, omega, ifunc, cx);
  if (ifirst == 1) del1st = del1;
  double plmn = fsign1(del1st) * fsign1(del1);
  int idir = (ifirst == 1 || plmn >= 0.0) ? +1 : -1;
  double c2 = 0, del2 = 0;
  int r = 0;
  if (precision == 1 && idir > 0) {
    // FP32 scan along the same c sequence, FP64 confirmation of the bracket.
    double ca = c1, cb;
    float fa = dltar32(omega / c1, omega, ifunc, cx);
    float s0 = fsign1f(fa);
    bool found = false, fail = false;
    for (int it = 0;; ++it) {
      if (it >= kMaxScan) { fail = true; break; }
      cb = ca + dc;
      if (cb <= clow) { found = false; break; }  // cannot happen going up; fall back
      float fb = dltar32(omega / cb, omega, ifunc, cx);
      if (fsign1f(fb) != s0) { found = true; break; }
      ca = cb;
      if (ca < cm || ca >= ((double)betmx + dc)) { fail = true; break; }
    }
    if (found) {
      double da = (ca == c1) ? del1 : dltar64(omega / ca, omega, ifunc, cx);
      double db = dltar64(omega / cb, omega, ifunc, cx);
      if (fsign1(da) == fsign1(del1) && fsign1(db) != fsign1(del1)) {
        c1 = ca; del1 = da; c2 = cb; del2 = db; r = 1;
      }
    } else if (fail) {
      // confirm the failure in FP64 at the failing point's predecessor chain
      r = 0;
    }
  }
  if (r == 0) r = scan64(t1, c1, del1, c2, del2, idir, clow, dc, cm, betmx, ifunc, cx);
  if (r < 0) { iret = -1; return; }
  c1 = nevill(t1, c1, c2, del1, del2, ifunc, cx);
  if (c1 > (double)betmx || !isfinite(c1)) { iret = -1; return; }
  iret = 1;
}

// surfdisp96.f:711-732 gtsolh, REAL*4
__device__ float gtsolh(float a, float b) {
  float c = 0.95f * b;
  for (int i = 0; i < 5; ++i) {
    float gamma = b / a;
    float kappa = c / b;
    float k2 = kappa * kappa;
    float gk = gamma * kappa;
    float gk2 = gk * gk;
    float fac1 = sqrtf(1.0f - gk2);
    float fac2 = sqrtf(1.0f - k2);
    float tk = 2.0f - k2;
    float fr = tk * tk - 4.0f * fac1 * fac2;
    float frp = -(4.0f * (2.0f - k2) * kappa) + 4.0f * fac2 * gamma * gamma * kappa / fac1 +
                4.0f * fac1 * kappa / fac2;
    frp = frp / b;
    c = c - fr / frp;
  }
  return c;
}

// One warp-sized block per COLS_PER_WARP columns. The active columns of a
// batch are the leading ones, so small blocks spread them over all SMs (and
// their FP64 pipes) instead of packing them onto a few.
#ifndef DISP_COLS_PER_WARP
#define DISP_COLS_PER_WARP 32
#endif
constexpr int COLS_PER_WARP = DISP_COLS_PER_WARP;

__global__ void __launch_bounds__(32) surfdisp_kernel(DispJob job) {
  if ((int)threadIdx.x >= COLS_PER_WARP) return;
  const int col = blockIdx.x * COLS_PER_WARP + threadIdx.x;
  if (col >= job.ncol) return;
  if (job.ncol_dev && col >= *job.ncol_dev) return;
  const int nl = job.nl[col];
  const int kmax = job.np, mode = job.mode, igr = job.igr;
  const bool mm_ = job.multimode != 0;
  double *cp = job.cp + (size_t)col * mode * kmax;
  double *cg = job.cg + (size_t)col * mode * kmax;
  for (int i = 0; i < kmax * mode; ++i) { cp[i] = mm_ ? 0.0 : 100.0; cg[i] = mm_ ? 0.0 : 100.0; }
  if (nl < 1 || nl > job.nl_max || kmax > NPMAX) { job.ierr[col] = 1; return; }
  Ctx cx;
  size_t off = (size_t)col * job.nl_max;
  cx.m.d = job.thk + off; cx.m.a = job.vp + off; cx.m.b = job.vs + off; cx.m.rho = job.rho + off;
  cx.m.mmax = nl;
  cx.m.llw = (__ldg(&cx.m.b[0]) <= 0.0f) ? 2 : 1;
  cx.n64 = cx.n32 = 0;
  int ierr = 0;
  const float sone0 = 1.500f, ddc0 = (float)job.dphase, h0 = 0.005f;
  const double one = 1.0e-2;
  int jmn = 1, jsol = 1;
  float betmx = -1.e20f, betmn = 1.e20f;
  for (int i = 0; i < nl; ++i) {
    float bi = __ldg(&cx.m.b[i]), ai = __ldg(&cx.m.a[i]);
    if (bi > 0.01f && bi < betmn) { betmn = bi; jmn = i + 1; jsol = 1; }
    else if (bi <= 0.01f && ai < betmn) { betmn = ai; jmn = i + 1; jsol = 0; }
    if (bi > betmx) betmx = bi;
  }
  const int ifunc = job.iwave;   // 1 Love, 2 Rayleigh
  double del1st = 0.0;
  double c[NPMAX], cb[NPMAX];
  {
    float sone = sone0, h = h0;
    double onea = (double)sone;
    float cc1 = (jsol == 0) ? betmn : gtsolh(__ldg(&cx.m.a[jmn - 1]), __ldg(&cx.m.b[jmn - 1]));
    cc1 = 0.95f * cc1;
    cc1 = 0.90f * cc1;
    double cc = (double)cc1;
    double dc = fabs((double)ddc0);
    double c1 = cc, cm = cc, clow = cc;
    for (int i = 0; i < kmax; ++i) { cb[i] = 0.0; c[i] = 0.0; }
    int ift = 999;
    for (int iq = 1; iq <= mode; ++iq) {
      int kfail = -1;
      for (int k = 1; k <= kmax; ++k) {
        if (k >= ift) { kfail = k; break; }
        double t1 = job.periods[k - 1];
        float t1a, t1b = 0.0f;
        if (igr > 0) {
          t1a = (float)(t1 / (double)(1.0f + h));
          t1b = (float)(t1 / (double)(1.0f - h));
          t1 = (double)t1a;
        } else {
          t1a = (float)t1;
        }
        int ifirst;
        if (k == 1 && iq == 1) { c1 = cc; clow = cc; ifirst = 1; }
        else if (k == 1 && iq > 1) { c1 = c[0] + one * dc; clow = c1; ifirst = 1; }
        else if (k > 1 && iq > 1) {
          ifirst = 0; clow = c[k - 1] + one * dc; c1 = c[k - 2];
          if (c1 < clow) c1 = clow;
        } else {
          ifirst = 0;
          if (mm_) {
            c1 = c[k - 2] - onea * dc;
          } else {
            c1 = cc;
            for (int previd = k - 1; previd >= 1; --previd)
              if (c[previd - 1] > 0) { c1 = c[previd - 1] - onea * dc; break; }
          }
          clow = cm;
        }
        int iret;
        getsol(t1, c1, clow, dc, cm, betmx, iret, ifunc, ifirst, del1st, job.precision, cx);
        if (iret == -1) { kfail = k; break; }
        c[k - 1] = c1;
        if (igr > 0) {
          t1 = (double)t1b;
          ifirst = 0;
          clow = cb[k - 1] + one * dc;
          c1 = c1 - onea * dc;
          getsol(t1, c1, clow, dc, cm, betmx, iret, ifunc, ifirst, del1st, job.precision, cx);
          if (iret == -1) { c1 = c[k - 1]; ierr = 1; }
          cb[k - 1] = c1;
        } else {
          c1 = 0.0;
        }
        float cc0 = (float)c[k - 1];
        float ccg = (float)c1;
        size_t o = mm_ ? (size_t)(iq - 1) * kmax + (k - 1) : (size_t)(k - 1);
        if (igr == 0) {
          cp[o] = cc0;
        } else {
          float gvel = (1.0f / t1a - 1.0f / t1b) / (1.0f / (t1a * cc0) - 1.0f / (t1b * ccg));
          cg[o] = gvel;
          cp[o] = cc0;
          if (!mm_ && (gvel < 0 || c[k - 1] == 0)) ierr = 1;
        }
      }
      if (kfail > 0) {
        ift = kfail;
        for (int i = kfail; i <= kmax; ++i) cg[mm_ ? (size_t)(iq - 1) * kmax + (i - 1) : (size_t)(i - 1)] = 0.0;
        ierr = 1;
      }
    }
  }
  job.ierr[col] = ierr;
  if (job.ndltar) {
    atomicAdd(&job.ndltar[0], cx.n64);
    atomicAdd(&job.ndltar[1], cx.n32);
  }
}

}  // namespace

int launch_surfdisp(const DispJob &job, cudaStream_t s) {
  if (job.ncol < 0 || job.np < 1 || job.np > NPMAX || job.mode < 1) return MCT_ERR_ARG;
  if (job.iwave != 1 && job.iwave != 2) return MCT_ERR_ARG;
  if (job.ncol == 0) return MCT_OK;
  const int blocks = (job.ncol + COLS_PER_WARP - 1) / COLS_PER_WARP;
  surfdisp_kernel<<<blocks, 32, 0, s>>>(job);
  MCT_CUDA_TRY(cudaGetLastError());
  return MCT_OK;
}
