// ORACLE (test infrastructure only): CPU restatement of Herrmann's surfdisp96
// dispersion code as shipped in the MCTomo reference, used as the parity
// checker for the GPU dispersion kernel. Never linked into the product.
//
// Parity status: unpinned by reference execution (the reference is Fortran 77
// and no Fortran compiler exists on this image). Pinned instead by analytic
// known answers in tests/ (Rayleigh half-space root, Love layer-over-half-space
// dispersion relation) and by line-by-line restatement.
//
// Follows surfmodes/surfdisp96.f. Fortran 77 implicit typing is reproduced:
// names starting a-h,o-z without declarations are REAL*4 in surfdisp96 and
// gtsolh, DOUBLE PRECISION in nevill/half/dltar*/var/normc/dnka.
// Build with -ffp-contract=off so no FMA contraction changes rounding.
#include <cmath>
#include <cstring>
#include "oracle.h"

namespace {

const int NL = 200;

struct Model {
  float d[NL], a[NL], b[NL], rho[NL];
  int mmax, llw;
};

inline double fsign1(double x) { return std::signbit(x) ? -1.0 : 1.0; }

// surfdisp96.f:1341-1366 normc. The exponent it returns (dlog of the scale)
// is dead in dltar4 (overwritten by var before any use), so it is not formed.
inline void normc(double ee[5]) {
  double t1 = 0.0;
  for (int i = 0; i < 5; ++i)
    if (std::fabs(ee[i]) > t1) t1 = std::fabs(ee[i]);
  if (t1 < 1.0e-40) t1 = 1.0;
  for (int i = 0; i < 5; ++i) ee[i] = ee[i] / t1;
}

struct VarOut {
  double w, cosp, a0, cpcq, cpy, cpz, cqw, cqx, xy, xz, wy, wz;
};

// surfdisp96.f:1220-1337 var. The trailing rescale of cosq/y/z by exp(qmp)
// only touches locals that are never returned, so it is omitted.
inline void var(double p, double q, double ra, double rb, double wvno,
                double xka, double xkb, double dpth, VarOut &o) {
  double pex = 0.0, sex = 0.0, sinp = 0, w = 0, x = 0, cosp = 0;
  double sinq = 0, y = 0, z = 0, cosq = 0, fac;
  if (wvno < xka) {
    sinp = std::sin(p); w = sinp / ra; x = -ra * sinp; cosp = std::cos(p);
  } else if (wvno == xka) {
    cosp = 1.0; w = dpth; x = 0.0;
  } else if (wvno > xka) {
    pex = p; fac = 0.0;
    if (p < 16) fac = std::exp(-2.0 * p);
    cosp = (1.0 + fac) * 0.5; sinp = (1.0 - fac) * 0.5;
    w = sinp / ra; x = ra * sinp;
  }
  if (wvno < xkb) {
    sinq = std::sin(q); y = sinq / rb; z = -rb * sinq; cosq = std::cos(q);
  } else if (wvno == xkb) {
    cosq = 1.0; y = dpth; z = 0.0;
  } else if (wvno > xkb) {
    sex = q; fac = 0.0;
    if (q < 16) fac = std::exp(-2.0 * q);
    cosq = (1.0 + fac) * 0.5; sinq = (1.0 - fac) * 0.5;
    y = sinq / rb; z = rb * sinq;
  }
  double exa = pex + sex;
  double a0 = 0.0;
  if (exa < 60.0) a0 = std::exp(-exa);
  o.w = w; o.cosp = cosp; o.a0 = a0;
  o.cpcq = cosp * cosq; o.cpy = cosp * y; o.cpz = cosp * z;
  o.cqw = cosq * w; o.cqx = cosq * x;
  o.xy = x * y; o.xz = x * z; o.wy = w * y; o.wz = w * z;
}

// surfdisp96.f:1370-1414 dnka (ca stored [row][col] with Fortran 1-based map).
inline void dnka(double ca[5][5], double wvno2, double gam, double gammk,
                 double rho, const VarOut &v) {
  const double one = 1.0, two = 2.0;
  double gamm1 = gam - one;
  double twgm1 = gam + gamm1;
  double gmgmk = gam * gammk;
  double gmgm1 = gam * gamm1;
  double gm1sq = gamm1 * gamm1;
  double rho2 = rho * rho;
  double a0pq = v.a0 - v.cpcq;
  ca[0][0] = v.cpcq - two * gmgm1 * a0pq - gmgmk * v.xz - wvno2 * gm1sq * v.wy;
  ca[0][1] = (wvno2 * v.cpy - v.cqx) / rho;
  ca[0][2] = -(twgm1 * a0pq + gammk * v.xz + wvno2 * gamm1 * v.wy) / rho;
  ca[0][3] = (v.cpz - wvno2 * v.cqw) / rho;
  ca[0][4] = -(two * wvno2 * a0pq + v.xz + wvno2 * wvno2 * v.wy) / rho2;
  ca[1][0] = (gmgmk * v.cpz - gm1sq * v.cqw) * rho;
  ca[1][1] = v.cpcq;
  ca[1][2] = gammk * v.cpz - gamm1 * v.cqw;
  ca[1][3] = -v.wz;
  ca[1][4] = ca[0][3];
  ca[3][0] = (gm1sq * v.cpy - gmgmk * v.cqx) * rho;
  ca[3][1] = -v.xy;
  ca[3][2] = gamm1 * v.cpy - gammk * v.cqx;
  ca[3][3] = ca[1][1];
  ca[3][4] = ca[0][1];
  ca[4][0] = -(two * gmgmk * gm1sq * a0pq + gmgmk * gmgmk * v.xz +
               gm1sq * gm1sq * v.wy) * rho2;
  ca[4][1] = ca[3][0];
  ca[4][2] = -(gammk * gamm1 * twgm1 * a0pq + gam * gammk * gammk * v.xz +
               gamm1 * gm1sq * v.wy) * rho;
  ca[4][3] = ca[1][0];
  ca[4][4] = ca[0][0];
  double t = -two * wvno2;
  ca[2][0] = t * ca[4][2];
  ca[2][1] = t * ca[3][2];
  ca[2][2] = v.a0 + two * (v.cpcq - ca[0][0]);
  ca[2][3] = t * ca[1][2];
  ca[2][4] = t * ca[0][2];
}

// surfdisp96.f:1119-1217 dltar4 (Rayleigh / P-SV period equation).
double dltar4(double wvno, double omga, const Model &m) {
  double omega = omga;
  if (omega < 1.0e-4) omega = 1.0e-4;
  double wvno2 = wvno * wvno;
  int mm = m.mmax - 1;
  double xka = omega / (double)m.a[mm];
  double xkb = omega / (double)m.b[mm];
  double wvnop = wvno + xka, wvnom = std::fabs(wvno - xka);
  double ra = std::sqrt(wvnop * wvnom);
  wvnop = wvno + xkb; wvnom = std::fabs(wvno - xkb);
  double rb = std::sqrt(wvnop * wvnom);
  double t = (double)m.b[mm] / omega;
  double gammk = 2.0 * t * t;
  double gam = gammk * wvno2;
  double gamm1 = gam - 1.0;
  double rho1 = (double)m.rho[mm];
  double e[5], ee[5], ca[5][5];
  e[0] = rho1 * rho1 * (gamm1 * gamm1 - gam * gammk * ra * rb);
  e[1] = -rho1 * ra;
  e[2] = rho1 * (gamm1 - gammk * ra * rb);
  e[3] = rho1 * rb;
  e[4] = wvno2 - ra * rb;
  VarOut v;
  for (int l = m.mmax - 2; l >= m.llw - 1; --l) {
    xka = omega / (double)m.a[l];
    xkb = omega / (double)m.b[l];
    t = (double)m.b[l] / omega;
    gammk = 2.0 * t * t;
    gam = gammk * wvno2;
    wvnop = wvno + xka; wvnom = std::fabs(wvno - xka);
    ra = std::sqrt(wvnop * wvnom);
    wvnop = wvno + xkb; wvnom = std::fabs(wvno - xkb);
    rb = std::sqrt(wvnop * wvnom);
    double dpth = (double)m.d[l];
    rho1 = (double)m.rho[l];
    double p = ra * dpth, q = rb * dpth;
    var(p, q, ra, rb, wvno, xka, xkb, dpth, v);
    dnka(ca, wvno2, gam, gammk, rho1, v);
    for (int i = 0; i < 5; ++i) {
      double cr = 0.0;
      for (int j = 0; j < 5; ++j) cr = cr + e[j] * ca[j][i];
      ee[i] = cr;
    }
    normc(ee);
    for (int i = 0; i < 5; ++i) e[i] = ee[i];
  }
  if (m.llw != 1) {
    // water layer on top
    xka = omega / (double)m.a[0];
    wvnop = wvno + xka; wvnom = std::fabs(wvno - xka);
    ra = std::sqrt(wvnop * wvnom);
    double dpth = (double)m.d[0];
    rho1 = (double)m.rho[0];
    double p = ra * dpth;
    const double znul = 1.0e-05;
    var(p, znul, ra, znul, wvno, xka, znul, dpth, v);
    double w0 = -rho1 * v.w;
    return v.cosp * e[0] + w0 * e[1];
  }
  return e[0];
}

// surfdisp96.f:1056-1115 dltar1 (Love / SH period equation).
double dltar1(double wvno, double omega, const Model &m) {
  int mm = m.mmax - 1;
  double beta1 = (double)m.b[mm];
  double rho1 = (double)m.rho[mm];
  double xkb = omega / beta1;
  double wvnop = wvno + xkb, wvnom = std::fabs(wvno - xkb);
  double rb = std::sqrt(wvnop * wvnom);
  double e1 = rho1 * rb;
  double e2 = 1.0 / (beta1 * beta1);
  for (int l = m.mmax - 2; l >= m.llw - 1; --l) {
    beta1 = (double)m.b[l];
    rho1 = (double)m.rho[l];
    double xmu = rho1 * beta1 * beta1;
    xkb = omega / beta1;
    wvnop = wvno + xkb; wvnom = std::fabs(wvno - xkb);
    rb = std::sqrt(wvnop * wvnom);
    double q = (double)m.d[l] * rb;
    double sinq, y, z, cosq;
    if (wvno < xkb) {
      sinq = std::sin(q); y = sinq / rb; z = -rb * sinq; cosq = std::cos(q);
    } else if (wvno == xkb) {
      cosq = 1.0; y = (double)m.d[l]; z = 0.0;
    } else {
      double fac = 0.0;
      if (q < 16) fac = std::exp(-2.0 * q);
      cosq = (1.0 + fac) * 0.5; sinq = (1.0 - fac) * 0.5;
      y = sinq / rb; z = rb * sinq;
    }
    double e10 = e1 * cosq + e2 * xmu * z;
    double e20 = e1 * y / xmu + e2 * cosq;
    double xnor = std::fabs(e10), ynor = std::fabs(e20);
    if (ynor > xnor) xnor = ynor;
    if (xnor < 1.0e-40) xnor = 1.0;
    e1 = e10 / xnor;
    e2 = e20 / xnor;
  }
  return e1;
}

struct Ctx {
  const Model *m;
  long long ndltar;  // number of period-equation evaluations (work counter)
};

inline double dltar(double wvno, double omega, int kk, Ctx &cx) {
  cx.ndltar++;
  return kk == 1 ? dltar1(wvno, omega, *cx.m) : dltar4(wvno, omega, *cx.m);
}

// surfdisp96.f:1022-1032 half
inline void half(double c1, double c2, double &c3, double &del3, double omega,
                 int ifunc, Ctx &cx) {
  c3 = 0.5 * (c1 + c2);
  double wvno = omega / c3;
  del3 = dltar(wvno, omega, ifunc, cx);
}

// surfdisp96.f:903-1020 nevill. 0.01 is a REAL*4 literal in the source.
double nevill(double t, double c1, double c2, double del1, double del2,
              int ifunc, Ctx &cx) {
  const double twopi = 2.0 * 3.141592653589793;
  double x[20], y[20];
  double omega = twopi / t;
  double c3, del3;
  half(c1, c2, c3, del3, omega, ifunc, cx);
  int nev = 1, nctrl = 1, m = 1;
  for (;;) {
    nctrl = nctrl + 1;
    if (nctrl >= 100) break;
    if (c3 < std::fmin(c1, c2) || c3 > std::fmax(c1, c2)) {
      nev = 0;
      half(c1, c2, c3, del3, omega, ifunc, cx);
    }
    double s13 = del1 - del3;
    double s32 = del3 - del2;
    if (fsign1(del3) * fsign1(del1) < 0.0) {
      c2 = c3; del2 = del3;
    } else {
      c1 = c3; del1 = del3;
    }
    if (std::fabs(c1 - c2) <= 1.e-6 * c1) break;
    if (fsign1(s13) != fsign1(s32)) nev = 0;
    double ss1 = std::fabs(del1);
    double s1 = (double)0.01f * ss1;
    double ss2 = std::fabs(del2);
    double s2 = (double)0.01f * ss2;
    if (s1 > ss2 || s2 > ss1 || nev == 0) {
      half(c1, c2, c3, del3, omega, ifunc, cx);
      nev = 1; m = 1;
    } else {
      if (nev == 2) {
        x[m] = c3; y[m] = del3;   // x(m+1), y(m+1)
      } else {
        x[0] = c1; y[0] = del1; x[1] = c2; y[1] = del2; m = 1;
      }
      bool fallback = false;
      for (int kk = 1; kk <= m; ++kk) {
        int j = m - kk + 1;                     // 1-based
        double denom = y[m] - y[j - 1];         // y(m+1) - y(j)
        if (std::fabs(denom) < 1.0e-10 * std::fabs(y[m])) { fallback = true; break; }
        x[j - 1] = (-y[j - 1] * x[j] + y[m] * x[j - 1]) / denom;
      }
      if (!fallback) {
        c3 = x[0];
        double wvno = omega / c3;
        del3 = dltar(wvno, omega, ifunc, cx);
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

// surfdisp96.f:734-827 getsol. del1st is SAVEd per thread in the reference;
// it is per-column state here (each column starts with ifirst=1).
void getsol(double t1, double &c1, double clow, double dc, double cm,
            float betmx, int &iret, int ifunc, int ifirst, double &del1st,
            Ctx &cx) {
  const double twopi = 2.0 * 3.141592653589793;
  double omega = twopi / t1;
  double wvno = omega / c1;
  double del1 = dltar(wvno, omega, ifunc, cx);
  if (ifirst == 1) del1st = del1;
  double plmn = fsign1(del1st) * fsign1(del1);
  int idir;
  if (ifirst == 1) idir = +1;
  else if (plmn >= 0.0) idir = +1;
  else idir = -1;
  double c2, del2;
  for (;;) {
    if (idir > 0) c2 = c1 + dc; else c2 = c1 - dc;
    if (c2 <= clow) { idir = +1; c1 = clow; continue; }
    omega = twopi / t1;
    wvno = omega / c2;
    del2 = dltar(wvno, omega, ifunc, cx);
    if (fsign1(del1) != fsign1(del2)) break;
    c1 = c2; del1 = del2;
    if (c1 < cm) { iret = -1; return; }
    if (c1 >= ((double)betmx + dc)) { iret = -1; return; }
  }
  double cn = nevill(t1, c1, c2, del1, del2, ifunc, cx);
  c1 = cn;
  if (c1 > (double)betmx) { iret = -1; return; }
  iret = 1;
}

// surfdisp96.f:711-732 gtsolh, all REAL*4.
float gtsolh(float a, float b) {
  float c = 0.95f * b;
  for (int i = 0; i < 5; ++i) {
    float gamma = b / a;
    float kappa = c / b;
    float k2 = kappa * kappa;
    float gk = gamma * kappa;
    float gk2 = gk * gk;
    float fac1 = std::sqrt(1.0f - gk2);
    float fac2 = std::sqrt(1.0f - k2);
    float tk = 2.0f - k2;
    float fr = tk * tk - 4.0f * fac1 * fac2;
    float frp = -(4.0f * (2.0f - k2) * kappa) +
                4.0f * fac2 * gamma * gamma * kappa / fac1 +
                4.0f * fac1 * kappa / fac2;
    frp = frp / b;
    c = c - fr / frp;
  }
  return c;
}

}  // namespace

// Shared driver for surfdisp96.f:52-382 (multimode=0) and
// surfdisp_mmodes (surfdisp96.f:385-701, multimode=1).
// cp/cg are (kmax, mode) column-major when multimode, (kmax) otherwise.
static int surfdisp_core(const float *thkm, const float *vpm, const float *vsm,
                         const float *rhom, int nlayer, int iwave, int mode,
                         int igr, int kmax, const double *t, double dphase,
                         double *cp, double *cg, int multimode,
                         long long *ndltar) {
  if (nlayer < 1 || nlayer > NL || kmax < 1 || kmax > 60 || mode < 1) return -1;
  Model m;
  int ierr = 0;
  for (int i = 0; i < kmax * (multimode ? mode : 1); ++i) {
    cp[i] = multimode ? 0.0 : 100.0;
    cg[i] = multimode ? 0.0 : 100.0;
  }
  m.mmax = nlayer;
  for (int i = 0; i < nlayer; ++i) {
    m.b[i] = vsm[i]; m.a[i] = vpm[i]; m.d[i] = thkm[i]; m.rho[i] = rhom[i];
  }
  int idispl = 0, idispr = 0;
  if (iwave == 1) { idispl = kmax; idispr = 0; }
  else if (iwave == 2) { idispl = 0; idispr = kmax; }
  int iverb[2] = {0, 0};
  const float sone0 = 1.500f;
  const float ddc0 = (float)dphase;
  const float h0 = 0.005f;
  m.llw = 1;
  if (m.b[0] <= 0.0f) m.llw = 2;
  const double one = 1.0e-2;
  int jmn = 1, jsol = 1;
  float betmx = -1.e20f, betmn = 1.e20f;
  for (int i = 0; i < m.mmax; ++i) {
    if (m.b[i] > 0.01f && m.b[i] < betmn) { betmn = m.b[i]; jmn = i + 1; jsol = 1; }
    else if (m.b[i] <= 0.01f && m.a[i] < betmn) { betmn = m.a[i]; jmn = i + 1; jsol = 0; }
    if (m.b[i] > betmx) betmx = m.b[i];
  }
  Ctx cx{&m, 0};
  double del1st = 0.0;
  double c[60], cb[60];
  for (int ifunc = 1; ifunc <= 2; ++ifunc) {
    if (ifunc == 1 && idispl <= 0) continue;
    if (ifunc == 2 && idispr <= 0) continue;
    float ddc = ddc0, sone = sone0, h = h0;
    if (sone < 0.01f) sone = 2.0f;
    double onea = (double)sone;
    float cc1;
    if (jsol == 0) cc1 = betmn;
    else cc1 = gtsolh(m.a[jmn - 1], m.b[jmn - 1]);
    cc1 = 0.95f * cc1;
    cc1 = 0.90f * cc1;
    double cc = (double)cc1;
    double dc = std::fabs((double)ddc);
    double c1 = cc, cm = cc, clow;
    for (int i = 0; i < kmax; ++i) { cb[i] = 0.0; c[i] = 0.0; }
    int ift = 999;
    for (int iq = 1; iq <= mode; ++iq) {
      const int is = 1, ie = kmax;
      int kfail = -1;
      for (int k = is; k <= ie; ++k) {
        if (k >= ift) { kfail = k; break; }
        double t1 = t[k - 1];
        float t1a, t1b = 0.0f;
        if (igr > 0) {
          t1a = (float)(t1 / (double)(1.0f + h));
          t1b = (float)(t1 / (double)(1.0f - h));
          t1 = (double)t1a;
        } else {
          t1a = (float)t1;
        }
        int ifirst;
        if (k == is && iq == 1) { c1 = cc; clow = cc; ifirst = 1; }
        else if (k == is && iq > 1) { c1 = c[is - 1] + one * dc; clow = c1; ifirst = 1; }
        else if (k > is && iq > 1) {
          ifirst = 0; clow = c[k - 1] + one * dc; c1 = c[k - 2];
          if (c1 < clow) c1 = clow;
        } else {
          ifirst = 0;
          if (multimode) {
            c1 = c[k - 2] - onea * dc;
          } else {
            c1 = cc;
            for (int previd = k - 1; previd >= 1; --previd)
              if (c[previd - 1] > 0) { c1 = c[previd - 1] - onea * dc; break; }
          }
          clow = cm;
        }
        int iret;
        getsol(t1, c1, clow, dc, cm, betmx, iret, ifunc, ifirst, del1st, cx);
        if (iret == -1) { kfail = k; break; }
        c[k - 1] = c1;
        if (igr > 0) {
          t1 = (double)t1b;
          ifirst = 0;
          clow = cb[k - 1] + one * dc;
          c1 = c1 - onea * dc;
          getsol(t1, c1, clow, dc, cm, betmx, iret, ifunc, ifirst, del1st, cx);
          if (iret == -1) { c1 = c[k - 1]; ierr = 1; }
          cb[k - 1] = c1;
        } else {
          c1 = 0.0;
        }
        float cc0 = (float)c[k - 1];
        float ccg = (float)c1;
        double *cpk = multimode ? &cp[(iq - 1) * kmax + (k - 1)] : &cp[k - 1];
        double *cgk = multimode ? &cg[(iq - 1) * kmax + (k - 1)] : &cg[k - 1];
        if (igr == 0) {
          *cpk = cc0;
        } else {
          float gvel = (1.0f / t1a - 1.0f / t1b) /
                       (1.0f / (t1a * cc0) - 1.0f / (t1b * ccg));
          *cgk = gvel;
          *cpk = cc0;
          if (!multimode && (gvel < 0 || c[k - 1] == 0)) ierr = 1;
        }
      }
      if (kfail > 0) {
        // label 1700 / 1750
        if (iq <= 1 && iverb[ifunc - 1] == 0) { iverb[ifunc - 1] = 1; ierr = 1; }
        ift = kfail;
        for (int i = kfail; i <= ie; ++i) {
          if (multimode) cg[(iq - 1) * kmax + (i - 1)] = 0.0;
          else cg[i - 1] = 0.0;
        }
        ierr = 1;
      }
    }
  }
  if (ndltar) *ndltar += cx.ndltar;
  return ierr;
}

extern "C" {

int orc_surfdisp96(const float *thkm, const float *vpm, const float *vsm,
                   const float *rhom, int nlayer, int iwave, int mode, int igr,
                   int kmax, const double *t, double dphase, double *cp,
                   double *cg, long long *ndltar) {
  return surfdisp_core(thkm, vpm, vsm, rhom, nlayer, iwave, mode, igr, kmax, t,
                       dphase, cp, cg, 0, ndltar);
}

int orc_surfdisp_mmodes(const float *thkm, const float *vpm, const float *vsm,
                        const float *rhom, int nlayer, int iwave, int mode,
                        int igr, int kmax, const double *t, double dphase,
                        double *cp, double *cg, long long *ndltar) {
  return surfdisp_core(thkm, vpm, vsm, rhom, nlayer, iwave, mode, igr, kmax, t,
                       dphase, cp, cg, 1, ndltar);
}

double orc_dltar(double wvno, double omega, int ifunc, const float *thkm,
                 const float *vpm, const float *vsm, const float *rhom,
                 int nlayer) {
  Model m;
  m.mmax = nlayer;
  for (int i = 0; i < nlayer; ++i) {
    m.b[i] = vsm[i]; m.a[i] = vpm[i]; m.d[i] = thkm[i]; m.rho[i] = rhom[i];
  }
  m.llw = (m.b[0] <= 0.0f) ? 2 : 1;
  return ifunc == 1 ? dltar1(wvno, omega, m) : dltar4(wvno, omega, m);
}

float orc_gtsolh(float a, float b) { return gtsolh(a, b); }

// surfmodes/surfmodes.f90:39-108 surfmodes for one column: casts the FP64
// layer model to REAL*4, routes to surfdisp96 when the column has no
// low-velocity layer (setup_grt, surfmodes.f90:320-450, nlvls1 == 0).
// Columns that need the generalized R/T solver return -2 (not restated).
// phase/group: (np). modetype: 1 Rayleigh, 0 Love.
int orc_surfmodes(const double *thick, const double *vp, const double *vs,
                  const double *rho, int nl, const double *freqs, int np,
                  int modetype, int phase_group, double dc, double *phase,
                  double *group, long long *ndltar) {
  if (orc_count_lvl(vp, vs, nl, modetype) > 0) return -2;
  float t4[NL], a4[NL], b4[NL], r4[NL];
  double per[60];
  if (nl > NL || np > 60) return -1;
  for (int i = 0; i < nl; ++i) {
    t4[i] = (float)thick[i]; a4[i] = (float)vp[i];
    b4[i] = (float)vs[i]; r4[i] = (float)rho[i];
  }
  for (int i = 0; i < np; ++i) per[i] = 1.0 / freqs[i];
  return surfdisp_core(t4, a4, b4, r4, nl, modetype == 1 ? 2 : 1, 1,
                       phase_group, np, per, dc, phase, group, 0, ndltar);
}

// setup_grt (surfmodes.f90:320-450): count of low-velocity layers that
// sends a column to the generalized R/T solver (nlvls1) for a column with
// no water layer: interior local P-velocity minima whose Vs is below the top
// layer's Vs (Love: below the top solid layer's Vs).
int orc_count_lvl(const double *vp, const double *vs, int nl, int modetype) {
  const double eps = (double)1e-6f;
  int ifs = 0;
  for (int i = 0; i < nl; ++i)
    if (!(std::fabs(vs[i]) > eps)) ifs++;
  double vs1 = (modetype == 1) ? (ifs > 0 ? vp[0] : vs[0]) : vs[ifs];
  int n = 0;
  if (ifs > 0 && modetype == 1) {
    // surfmodes.f90:387 counter (kept for water-over-solid Rayleigh columns)
    double vss1 = vs[ifs];
    for (int i = 1; i < nl - 1; ++i)
      if (i + 1 > ifs && vs[i] < vss1) n++;
    return n;
  }
  for (int i = 1; i < nl - 1; ++i) {
    if (vp[i] < vp[i + 1] && vp[i] < vp[i - 1]) {
      if (ifs == 0) {
        if (vs[i] < vs1) n++;
      } else if (modetype == 1) {
        if (vp[i] < vs1) n++;
      } else {
        if (vs[i] > 0.) { if (vs[i] < vs1) n++; }
      }
    }
  }
  return n;
}

}  // extern "C"
