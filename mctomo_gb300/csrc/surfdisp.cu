// Rayleigh/Love phase and group velocities of 1D layered columns: the GPU
// replacement of surfdisp96 / surfdisp_mmodes (surfmodes/surfdisp96.f:52-701)
// as routed by surfmodes (surfmodes/surfmodes.f90:39-183).
//
// One thread owns one column and walks its periods in order, because each
// period's root search starts from the previous period's root
// (surfdisp96.f:272-281); the batch supplies the parallelism (columns x
// chains). Each column's search is a resumable state machine that stops at
// every evaluation of the period equation it needs, and the warp evaluates
// the pending points of all its columns together, so the lanes of a warp
// stay converged on the expensive evaluation whatever step of the search
// each column has reached. The period equation (dltar4 / dltar1, surfdisp96.f:1056-1217) is
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

__device__ __forceinline__ double dltar64(double wvno, double omega, int ifunc, const Col &m) {
  return ifunc == 1 ? dltar1<double>(wvno, omega, m) : dltar4<double>(wvno, omega, m);
}
__device__ __forceinline__ float dltar32(double wvno, double omega, int ifunc, const Col &m) {
  float w = (float)wvno, o = (float)omega;
  return ifunc == 1 ? dltar1<float>(w, o, m) : dltar4<float>(w, o, m);
}

__device__ __forceinline__ double fsign1(double x) { return signbit(x) ? -1.0 : 1.0; }
__device__ __forceinline__ float fsign1f(float x) { return signbit(x) ? -1.f : 1.f; }

// A bracketing scan moves by dc between clow >= cm and betmx + dc, at most
// once down and once up, so it ends within scan_limit steps; a scan that
// does not (a NaN trial velocity, which the reference would step forever)
// ends as a failure there.
__device__ __forceinline__ int scan_limit(double betmx, double cm, double dc) {
  const double n = (betmx + dc - cm) / dc;
  return (n >= 0.0 && n < 1.0e8) ? 2 * (int)n + 16 : 16;
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

// ---------------------------------------------------------------------------
// One column's root searches as a resumable state machine.
//
// The reference walks, per column, modes x periods x (phase root, group
// root), each root a bracketing scan (getsol, surfdisp96.f:734-827) and a
// Neville / bisection polish (nevill, :903-1020), every step one evaluation
// of the period equation. Written as straight-line code, the 32 columns of
// a warp drift into different steps and the (FP64) evaluations run with few
// lanes active. Here each lane's search is a state machine that stops at
// every evaluation it needs; the warp loop then evaluates all lanes' pending
// points together (one FP32 and one FP64 pass) and resumes each lane with
// its value. The sequence of trial velocities and evaluations of every
// column is the reference's, so the roots are unchanged.
// ---------------------------------------------------------------------------
enum : int {
  S_PERIOD, S_G_BEGIN, S_G_BEGIN_RES, S_S32_FIRST_RES, S_S32_STEP, S_S32_RES, S_S32_END, S_CONF_A_RES, S_CONF_B,
  S_CONF_B_RES, S_S64_INIT, S_S64_STEP, S_S64_RES, S_G_FAIL, S_NEV_BEGIN, S_NEV_INIT_RES, S_NEV_LOOP,
  S_NEV_HALF1_RES, S_NEV_BODY, S_NEV_HALF2_RES, S_NEV_STEP_RES, S_NEV_END, S_G_DONE, S_AFTER_PHASE,
  S_AFTER_GROUP, S_OUTPUT, S_MODE_END, S_DONE
};

struct Search {
  // column constants
  int kmax, mode, igr, mm, precision;
  double dc, cc, cm;
  float betmx, h;
  const double *periods;
  double *cp, *cg;
  // column state (surfdisp96 / surfdisp_mmodes main loops)
  int iq, k, ift, kfail, ierr, pass, st;
  int max_scan;   // scan_limit of the column
  double c[NPMAX], cb[NPMAX];
  double del1st;
  float t1a, t1b;
  // getsol
  double t1, omega, c1, clow, del1, c2, del2, ca, cbv, da;
  int ifirst, idir, it, found, iret;
  float s0;
  // nevill
  double nc1, nc2, nd1, nd2, c3, del3;
  double x[11], y[11];
  int nev, nctrl, m;
  // the pending evaluation: trial velocity and whether the FP32 equation
  double req;
  int req32;
  // Values of the scan's next trial velocities, evaluated ahead by idle
  // lanes: pfc[i] / pfv[i] for i in [pf_i, pf_n), FP32 values if pf32. A
  // scan step takes the next entry only if its trial velocity is exactly
  // the one the step computes; any real request empties the buffer.
  double pfc[32], pfv[32];
  int pf_n, pf_i, pf32;
  unsigned long long used64, used32;   // values ahead that the search used

  __device__ void request(double cval, int fp32, int resume) {
    req = cval; req32 = fp32; st = resume; pf_n = 0; pf_i = 0;
  }
  __device__ bool prefetched(double cval, int fp32, double &v) {
    if (pf_i < pf_n && pf32 == fp32 && pfc[pf_i] == cval) {
      v = pfv[pf_i++];
      if (fp32) ++used32; else ++used64;
      return true;
    }
    return false;
  }
  // The trial velocity `ahead` steps after the pending request `c` of a
  // scan, if no sign change and no stop comes first: the FP32 scan steps
  // up by dc; the FP64 scan steps along idir and turns up at clow
  // (S_S32_STEP / S_S64_STEP below).
  __device__ static double scan_ahead(double c, int fp32, int idir, double clow, double dc, int ahead) {
    for (int j = 0; j < ahead; ++j) {
      if (fp32) { c = c + dc; continue; }
      double c2 = idir > 0 ? c + dc : c - dc;
      if (c2 <= clow) { idir = +1; c2 = clow + dc; }
      c = c2;
    }
    return c;
  }

  // Runs until the search needs an evaluation (returns false, request set)
  // or the column is finished (returns true). v64 / v32 hold the value of
  // the evaluation requested last.
  __device__ bool advance(double v64, float v32) {
    const double one = 1.0e-2, onea = 1.5;    // REAL*4 sone = 1.500 (exact)
    const double twopi = 2.0 * 3.141592653589793;
    for (;;) {
      switch (st) {
        case S_PERIOD: {
          if (k > kmax) { st = S_MODE_END; break; }
          if (k >= ift) { kfail = k; st = S_MODE_END; break; }
          double tt = periods[k - 1];
          if (igr > 0) {
            t1a = (float)(tt / (double)(1.0f + h));
            t1b = (float)(tt / (double)(1.0f - h));
            tt = (double)t1a;
          } else {
            t1a = (float)tt;
          }
          t1 = tt;
          if (k == 1 && iq == 1) { c1 = cc; clow = cc; ifirst = 1; }
          else if (k == 1 && iq > 1) { c1 = c[0] + one * dc; clow = c1; ifirst = 1; }
          else if (k > 1 && iq > 1) {
            ifirst = 0; clow = c[k - 1] + one * dc; c1 = c[k - 2];
            if (c1 < clow) c1 = clow;
          } else {
            ifirst = 0;
            if (mm) {
              c1 = c[k - 2] - onea * dc;
            } else {
              c1 = cc;
              for (int previd = k - 1; previd >= 1; --previd)
                if (c[previd - 1] > 0) { c1 = c[previd - 1] - onea * dc; break; }
            }
            clow = cm;
          }
          pass = 0;
          st = S_G_BEGIN;
          break;
        }
        // ---- getsol (surfdisp96.f:734-827)
        case S_G_BEGIN:
          omega = twopi / t1;
          request(c1, 0, S_G_BEGIN_RES);
          return false;
        case S_G_BEGIN_RES: {
          del1 = v64;
          if (ifirst == 1) del1st = del1;
          const double plmn = fsign1(del1st) * fsign1(del1);
          idir = (ifirst == 1 || plmn >= 0.0) ? +1 : -1;
          c2 = 0; del2 = 0;
          if (precision == 1 && idir > 0) {
            // FP32 scan along the same c sequence, FP64 confirmation
            ca = c1;
            request(c1, 1, S_S32_FIRST_RES);
            return false;
          }
          st = S_S64_INIT;
          break;
        }
        case S_S32_FIRST_RES:
          s0 = fsign1f(v32); found = 0; it = 0;
          st = S_S32_STEP;
          break;
        case S_S32_STEP:
          if (it >= max_scan) { found = 0; st = S_S32_END; break; }
          cbv = ca + dc;
          if (cbv <= clow) { found = 0; st = S_S32_END; break; }   // cannot happen going up
          {
            double pv;
            if (prefetched(cbv, 1, pv)) { v32 = (float)pv; st = S_S32_RES; break; }
          }
          request(cbv, 1, S_S32_RES);
          return false;
        case S_S32_RES:
          if (fsign1f(v32) != s0) { found = 1; st = S_S32_END; break; }
          ca = cbv;
          if (ca < cm || ca >= ((double)betmx + dc)) { found = 0; st = S_S32_END; break; }
          ++it;
          st = S_S32_STEP;
          break;
        case S_S32_END:
          if (!found) { st = S_S64_INIT; break; }
          if (ca == c1) { da = del1; st = S_CONF_B; break; }
          request(ca, 0, S_CONF_A_RES);
          return false;
        case S_CONF_A_RES:
          da = v64;
          st = S_CONF_B;
          break;
        case S_CONF_B:
          request(cbv, 0, S_CONF_B_RES);
          return false;
        case S_CONF_B_RES:
          if (fsign1(da) == fsign1(del1) && fsign1(v64) != fsign1(del1)) {
            c1 = ca; del1 = da; c2 = cbv; del2 = v64;
            st = S_NEV_BEGIN;
          } else {
            st = S_S64_INIT;
          }
          break;
        // ---- the FP64 bracketing scan (surfdisp96.f:793-815)
        case S_S64_INIT:
          it = 0;
          st = S_S64_STEP;
          break;
        case S_S64_STEP:
          if (it >= max_scan) { st = S_G_FAIL; break; }
          c2 = idir > 0 ? c1 + dc : c1 - dc;
          if (c2 <= clow) { idir = +1; c1 = clow; ++it; break; }
          if (prefetched(c2, 0, v64)) { st = S_S64_RES; break; }
          request(c2, 0, S_S64_RES);
          return false;
        case S_S64_RES:
          del2 = v64;
          if (fsign1(del1) != fsign1(del2)) { st = S_NEV_BEGIN; break; }
          c1 = c2; del1 = del2;
          if (c1 < cm || c1 >= ((double)betmx + dc)) { st = S_G_FAIL; break; }
          ++it;
          st = S_S64_STEP;
          break;
        case S_G_FAIL:
          iret = -1;
          st = S_G_DONE;
          break;
        // ---- nevill (surfdisp96.f:903-1020); nc1/nc2/nd1/nd2 are its copies
        case S_NEV_BEGIN:
          nc1 = c1; nc2 = c2; nd1 = del1; nd2 = del2;
          c3 = 0.5 * (nc1 + nc2);
          request(c3, 0, S_NEV_INIT_RES);
          return false;
        case S_NEV_INIT_RES:
          del3 = v64; nev = 1; nctrl = 1; m = 1;
          st = S_NEV_LOOP;
          break;
        case S_NEV_LOOP:
          nctrl = nctrl + 1;
          if (nctrl >= 100) { st = S_NEV_END; break; }
          if (c3 < fmin(nc1, nc2) || c3 > fmax(nc1, nc2)) {
            nev = 0;
            c3 = 0.5 * (nc1 + nc2);
            request(c3, 0, S_NEV_HALF1_RES);
            return false;
          }
          st = S_NEV_BODY;
          break;
        case S_NEV_HALF1_RES:
          del3 = v64;
          st = S_NEV_BODY;
          break;
        case S_NEV_BODY: {
          const double s13 = nd1 - del3;
          const double s32 = del3 - nd2;
          if (fsign1(del3) * fsign1(nd1) < 0.0) { nc2 = c3; nd2 = del3; }
          else { nc1 = c3; nd1 = del3; }
          if (fabs(nc1 - nc2) <= 1.e-6 * nc1) { st = S_NEV_END; break; }
          if (fsign1(s13) != fsign1(s32)) nev = 0;
          const double ss1 = fabs(nd1), s1 = (double)0.01f * ss1;
          const double ss2 = fabs(nd2), s2 = (double)0.01f * ss2;
          bool bisect = s1 > ss2 || s2 > ss1 || nev == 0;
          if (!bisect) {
            if (nev == 2) { x[m] = c3; y[m] = del3; }
            else { x[0] = nc1; y[0] = nd1; x[1] = nc2; y[1] = nd2; m = 1; }
            for (int kk = 1; kk <= m; ++kk) {
              const int j = m - kk + 1;
              const double denom = y[m] - y[j - 1];
              if (fabs(denom) < 1.0e-10 * fabs(y[m])) { bisect = true; break; }
              x[j - 1] = (-y[j - 1] * x[j] + y[m] * x[j - 1]) / denom;
            }
          }
          if (bisect) {
            c3 = 0.5 * (nc1 + nc2);
            request(c3, 0, S_NEV_HALF2_RES);
          } else {
            c3 = x[0];
            request(c3, 0, S_NEV_STEP_RES);
          }
          return false;
        }
        case S_NEV_HALF2_RES:
          del3 = v64; nev = 1; m = 1;
          st = S_NEV_LOOP;
          break;
        case S_NEV_STEP_RES:
          del3 = v64; nev = 2; m = m + 1;
          if (m > 10) m = 10;
          st = S_NEV_LOOP;
          break;
        case S_NEV_END:
          c1 = c3;
          iret = (c1 > (double)betmx || !isfinite(c1)) ? -1 : 1;
          st = S_G_DONE;
          break;
        // ---- the period loop around the two root searches (surfdisp96.f:283-320)
        case S_G_DONE:
          if (pass == 0) {
            if (iret == -1) { kfail = k; st = S_MODE_END; break; }
            c[k - 1] = c1;
            if (igr > 0) {
              t1 = (double)t1b;
              ifirst = 0;
              clow = cb[k - 1] + one * dc;
              c1 = c1 - onea * dc;
              pass = 1;
              st = S_G_BEGIN;
            } else {
              c1 = 0.0;
              st = S_OUTPUT;
            }
          } else {
            if (iret == -1) { c1 = c[k - 1]; ierr = 1; }
            cb[k - 1] = c1;
            st = S_OUTPUT;
          }
          break;
        case S_OUTPUT: {
          const float cc0 = (float)c[k - 1];
          const float ccg = (float)c1;
          const size_t o = mm ? (size_t)(iq - 1) * kmax + (k - 1) : (size_t)(k - 1);
          if (igr == 0) {
            cp[o] = cc0;
          } else {
            const float gvel = (1.0f / t1a - 1.0f / t1b) / (1.0f / (t1a * cc0) - 1.0f / (t1b * ccg));
            cg[o] = gvel;
            cp[o] = cc0;
            if (!mm && (gvel < 0 || c[k - 1] == 0)) ierr = 1;
          }
          ++k;
          st = S_PERIOD;
          break;
        }
        case S_MODE_END:
          if (kfail > 0) {
            ift = kfail;
            for (int i = kfail; i <= kmax; ++i) cg[mm ? (size_t)(iq - 1) * kmax + (i - 1) : (size_t)(i - 1)] = 0.0;
            ierr = 1;
          }
          if (++iq > mode) { st = S_DONE; return true; }
          k = 1; kfail = -1;
          st = S_PERIOD;
          break;
        default:   // S_DONE
          return true;
      }
    }
  }
};

// One warp-sized block per COLS_PER_WARP columns. The active columns of a
// batch are the leading ones, so small blocks spread them over all SMs (and
// their FP64 pipes) instead of packing them onto a few.
#ifndef DISP_COLS_PER_WARP
#define DISP_COLS_PER_WARP 32
#endif
constexpr int COLS_PER_WARP = DISP_COLS_PER_WARP;

// Warp-loop limit: a column needs at most mode x periods x 2 root searches,
// each at most one evaluation to start, a scan of max_scan steps, two
// confirmations and a polish of 100 evaluations; every pending evaluation is
// served within two passes of the warp loop. Past twice the largest column
// bound of the warp the remaining columns report ierr = 1.
__device__ __forceinline__ long long column_eval_bound(int mode, int kmax, int max_scan) {
  return (long long)mode * kmax * 2 * (2LL * max_scan + 110);
}
// Idle lanes evaluate ahead only for FP64 scans that have already taken
// this many steps: most scans find their bracket within a few steps, and
// evaluations past the bracket would take FP64 issue slots from other
// warps. FP32 scans get help from their first step.
constexpr int kAheadAfter = 4;

__device__ __forceinline__ int nth_lane(unsigned mask, int n) {
  for (int i = 0; i < n; ++i) mask &= mask - 1;
  return __ffs(mask) - 1;
}

__device__ __forceinline__ const float *shfl_ptr(const float *p, int src) {
  return reinterpret_cast<const float *>(
      __shfl_sync(0xffffffffu, reinterpret_cast<unsigned long long>(p), src));
}

// The columns in order of decreasing layer count (a counting sort; the
// order within one count is arbitrary): the lanes of a warp then run the
// layer loop of the period equation the same number of times, and the
// longest columns start first. The results of a column do not depend on
// where it runs.
constexpr int kOrderThreads = 1024;

__global__ void __launch_bounds__(kOrderThreads) disp_order_kernel(int ncol, const int *ncol_dev, const int *nl,
                                                                   int nl_max, int *order) {
  __shared__ int bin_base[256];
  const int n = ncol_dev ? min(ncol, *ncol_dev) : ncol;
  const int nbins = nl_max + 2;   // bin 0: nl = nl_max ... bin nl_max - 1: nl = 1; last: out-of-range nl
  for (int i = threadIdx.x; i < nbins; i += blockDim.x) bin_base[i] = 0;
  __syncthreads();
  auto bin_of = [&](int c) {
    const int v = nl[c];
    return (v >= 1 && v <= nl_max) ? nl_max - v : nbins - 1;
  };
  const unsigned lanes_lt = (1u << (threadIdx.x & 31)) - 1;
  for (int c0 = 0; c0 < n; c0 += blockDim.x) {
    const int c = c0 + threadIdx.x;
    const unsigned act = __ballot_sync(0xffffffffu, c < n);
    if (c < n) {
      const int b = bin_of(c);
      const unsigned peers = __match_any_sync(act, b);
      if ((peers & lanes_lt) == 0) atomicAdd(&bin_base[b], __popc(peers));
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int i = 0; i < nbins; ++i) { const int k = bin_base[i]; bin_base[i] = run; run += k; }
  }
  __syncthreads();
  for (int c0 = 0; c0 < n; c0 += blockDim.x) {
    const int c = c0 + threadIdx.x;
    const unsigned act = __ballot_sync(0xffffffffu, c < n);
    if (c < n) {
      const int b = bin_of(c);
      const unsigned peers = __match_any_sync(act, b);
      const int leader = __ffs(peers) - 1;
      int base = 0;
      if ((threadIdx.x & 31) == leader) base = atomicAdd(&bin_base[b], __popc(peers));
      base = __shfl_sync(peers, base, leader);
      order[base + __popc(peers & lanes_lt)] = c;
    }
  }
}

__global__ void __launch_bounds__(32) surfdisp_kernel(DispJob job, int share) {
  constexpr unsigned kFull = 0xffffffffu;
  const int lane = threadIdx.x;
  const int idx = blockIdx.x * COLS_PER_WARP + lane;
  bool valid = lane < COLS_PER_WARP && idx < job.ncol && (!job.ncol_dev || idx < *job.ncol_dev);
  const int col = (valid && job.order) ? job.order[idx] : idx;
  const int kmax = job.np, mode = job.mode;
  const bool mm_ = job.multimode != 0;
  Col cm{};
  unsigned long long n64 = 0, n32 = 0;
  Search S;
  S.st = S_DONE; S.req = 0.0; S.req32 = 0; S.omega = 0.0; S.dc = 0.0; S.clow = 0.0; S.idir = 1; S.it = 0;
  S.pf_n = S.pf_i = 0; S.pf32 = 0; S.used64 = S.used32 = 0;
  if (valid) {
    const int nl = job.nl[col];
    double *cp = job.cp + (size_t)col * mode * kmax;
    double *cg = job.cg + (size_t)col * mode * kmax;
    for (int i = 0; i < kmax * mode; ++i) { cp[i] = mm_ ? 0.0 : 100.0; cg[i] = mm_ ? 0.0 : 100.0; }
    if (nl < 1 || nl > job.nl_max || kmax > NPMAX) {
      job.ierr[col] = 1;
      valid = false;
    } else {
      const size_t off = (size_t)col * job.nl_max;
      cm.d = job.thk + off; cm.a = job.vp + off; cm.b = job.vs + off; cm.rho = job.rho + off;
      cm.mmax = nl;
      cm.llw = (__ldg(&cm.b[0]) <= 0.0f) ? 2 : 1;
      int jmn = 1, jsol = 1;
      float betmx = -1.e20f, betmn = 1.e20f;
      for (int i = 0; i < nl; ++i) {
        const float bi = __ldg(&cm.b[i]), ai = __ldg(&cm.a[i]);
        if (bi > 0.01f && bi < betmn) { betmn = bi; jmn = i + 1; jsol = 1; }
        else if (bi <= 0.01f && ai < betmn) { betmn = ai; jmn = i + 1; jsol = 0; }
        if (bi > betmx) betmx = bi;
      }
      float cc1 = (jsol == 0) ? betmn : gtsolh(__ldg(&cm.a[jmn - 1]), __ldg(&cm.b[jmn - 1]));
      cc1 = 0.95f * cc1;
      cc1 = 0.90f * cc1;
      S.kmax = kmax; S.mode = mode; S.igr = job.igr; S.mm = mm_; S.precision = job.precision;
      S.dc = fabs((double)(float)job.dphase);
      S.cc = (double)cc1; S.cm = S.cc;
      S.betmx = betmx; S.h = 0.005f;
      S.periods = job.periods; S.cp = cp; S.cg = cg;
      S.iq = 1; S.k = 1; S.ift = 999; S.kfail = -1; S.ierr = 0;
      S.max_scan = scan_limit((double)betmx, S.cm, S.dc);
      S.del1st = 0.0; S.t1b = 0.0f;
      for (int i = 0; i < kmax; ++i) { S.cb[i] = 0.0; S.c[i] = 0.0; }
      S.st = S_PERIOD;
    }
  }
  const int ifunc = job.iwave;   // 1 Love, 2 Rayleigh
  // Every lane advances its search to its next evaluation point. A pass
  // then evaluates either all pending FP32 requests or, when there are
  // none, all pending FP64 requests, so FP64 passes (the FP64 pipe works
  // per warp instruction, whatever the active lanes) run with every
  // unfinished column of the warp. Lanes not served by a pass evaluate
  // ahead for the long scans of the others: idle lane r (in lane order)
  // takes scan r mod nO (nO scans) and evaluates its trial velocity
  // 1 + r / nO steps ahead, with that column's model; the scans then
  // collect their values ahead in step order.
  bool done = !valid, pending = false;
  double v64 = 0.0;
  float v32 = 0.0f;
  long long steps = 0;
  long long max_steps = valid ? 2 * column_eval_bound(mode, kmax, S.max_scan) + 16 : 0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) max_steps = max(max_steps, __shfl_xor_sync(kFull, max_steps, o));
  while (__any_sync(kFull, !done)) {
    if (++steps > max_steps) {
      if (!done) S.ierr = 1;
      break;
    }
    if (!done && !pending) { done = S.advance(v64, v32); pending = !done; }
    const bool pass32 = __any_sync(kFull, pending && S.req32);
    const bool serve = pending && (S.req32 != 0) == pass32;
    const bool ext = share && serve && (S.st == S_S64_RES || S.st == S_S32_RES) && (pass32 || S.it >= kAheadAfter);
    const unsigned O = __ballot_sync(kFull, ext);
    const unsigned I = __ballot_sync(kFull, !serve);
    const int nO = __popc(O), nI = __popc(I);
    const bool sharing = nO > 0 && nI > 0;
    int src = lane, ahead = 0;
    if (sharing && !serve) {
      const int r = __popc(I & ((1u << lane) - 1));
      src = nth_lane(O, r % nO);
      ahead = 1 + r / nO;
    }
    bool eval = serve;
    double ec = S.req, eom = S.omega;
    Col em = cm;
    if (sharing) {
      ec = __shfl_sync(kFull, S.req, src);
      eom = __shfl_sync(kFull, S.omega, src);
      const double edc = __shfl_sync(kFull, S.dc, src), eclow = __shfl_sync(kFull, S.clow, src);
      const int eidir = __shfl_sync(kFull, S.idir, src);
      em.d = shfl_ptr(cm.d, src); em.a = shfl_ptr(cm.a, src); em.b = shfl_ptr(cm.b, src);
      em.rho = shfl_ptr(cm.rho, src);
      em.mmax = __shfl_sync(kFull, cm.mmax, src); em.llw = __shfl_sync(kFull, cm.llw, src);
      if (ahead > 0) {
        eval = true;
        ec = Search::scan_ahead(ec, pass32, eidir, eclow, edc, ahead);
      }
    }
    double ev = 0.0;
    if (eval) {
      if (pass32) ev = (double)dltar32(eom / ec, eom, ifunc, em);
      else ev = dltar64(eom / ec, eom, ifunc, em);
    }
    if (serve) {
      if (pass32) { v32 = (float)ev; ++n32; } else { v64 = ev; ++n64; }
      pending = false;
    }
    if (sharing) {
      // scan o's j-th value ahead is on idle lane of rank o + j * nO
      const int oi = __popc(O & ((1u << lane) - 1));
      const int maxj = (nI + nO - 1) / nO;
      if (ext) { S.pf_n = 0; S.pf_i = 0; S.pf32 = pass32; }
      for (int j = 0; j < maxj; ++j) {
        const int r = oi + j * nO;
        const bool mine = ext && r < nI;
        const int hl = mine ? nth_lane(I, r) : lane;
        const double hc = __shfl_sync(kFull, ec, hl), hv = __shfl_sync(kFull, ev, hl);
        if (mine) { S.pfc[j] = hc; S.pfv[j] = hv; S.pf_n = j + 1; }
      }
    }
  }
  if (valid) job.ierr[col] = S.ierr;
  // evaluations the searches used (values evaluated ahead and not reached
  // are not counted), so the FP64 count of precision 0 is the reference's
  n64 += S.used64; n32 += S.used32;
  if (job.ndltar && (n64 | n32)) {
    atomicAdd(&job.ndltar[0], n64);
    atomicAdd(&job.ndltar[1], n32);
  }
}

}  // namespace

static int g_disp_share = 1;
static int g_disp_order = 1;

// Diagnostics (not part of the public header): bit 0 lets idle lanes
// evaluate ahead for long scans, bit 1 runs the columns in order of layer
// count (both on by default); returns the previous value. The roots are the
// same either way.
extern "C" int mct_debug_disp_share(int v) {
  const int old = g_disp_share | (g_disp_order << 1);
  if (v >= 0 && v <= 3) { g_disp_share = v & 1; g_disp_order = (v >> 1) & 1; }
  return old;
}

int launch_surfdisp(const DispJob &job, cudaStream_t s) {
  if (job.ncol < 0 || job.np < 1 || job.np > NPMAX || job.mode < 1) return MCT_ERR_ARG;
  if (job.iwave != 1 && job.iwave != 2) return MCT_ERR_ARG;
  if (job.ncol == 0) return MCT_OK;
  DispJob j = job;
  if (j.order && g_disp_order && j.nl_max >= 1 && j.nl_max + 2 <= 256) {
    disp_order_kernel<<<1, kOrderThreads, 0, s>>>(j.ncol, j.ncol_dev, j.nl, j.nl_max, j.order);
    MCT_CUDA_TRY(cudaGetLastError());
  } else {
    j.order = nullptr;
  }
  const int blocks = (j.ncol + COLS_PER_WARP - 1) / COLS_PER_WARP;
  surfdisp_kernel<<<blocks, 32, 0, s>>>(j, g_disp_share);
  MCT_CUDA_TRY(cudaGetLastError());
  return MCT_OK;
}
