// Oracle (test infrastructure only): CPU restatement of the reference's
// generalized reflection/transmission (GRT) fundamental-mode dispersion for
// layered columns with a low-velocity layer, the single-mode surfmodes path:
//   setup_grt                     surfmodes/surfmodes.f90:320-450
//   RayleighModes / LoveModes     surfmodes/surfmodes.f90:185-303 (allmodes 0)
//   CalGroup                      surfmodes/surfmodes.f90:305-318
//   SearchRayleigh FundaMode      surfmodes/SearchRayleigh.f90:1-80,455-605
//   CR0_Finder                    surfmodes/SearchRayleigh.f90:898-933
//   SearchLove FundaMode          surfmodes/SearchLove.f90:1-60,181-270
//   C_Interval / N_cf             surfmodes/C_interval.f90:1-208
//   C_Interval_L / N_cf_L         surfmodes/C_interval_L.f90:1-204
//   startl, SecFunSurf, EinvE, propup   surfmodes/Rayleigh.f90:53-125,323-351,404-491
//   SecFuns_L, EinvE_L, propdn_L, propup_L  surfmodes/Love.f90:39-132
//   bisecim                       surfmodes/util.f90:90-167
// Only columns without fluid layers (every vs > 0) are restated; the
// Stoneley-mode path of fluid-topped columns is not.
//
// Arithmetic follows the Fortran expressions term by term in FP64 (compiled
// with -ffp-contract=off): complex products as (ar*br - ai*bi, ar*bi + ai*br),
// real x complex as a scaling of both parts, complex quotients by Smith's
// method (the range-reduced division gfortran emits under its default
// complex rules), complex exp as exp(re) * (cos im, sin im), and the square
// root of a real argument x as (sqrt x, 0) or (0, sqrt -x). Single-precision
// literals of the source keep their single-precision values ((double)0.9f
// and so on).
//
// Two points where the reference's behaviour is undefined are pinned here:
// the trial-velocity arrays hold 20,000 entries in the reference and a
// column that would need more gets ierr 2; and SearchLove's FundaMode tests
// a host variable c that the single-mode path never sets, which this
// restatement treats as a test that passes.
#include <cmath>
#include <cstdint>
#include <vector>
#include <algorithm>

namespace {

struct cx { double re, im; };
inline cx C(double r) { return {r, 0.0}; }
inline cx add(cx a, cx b) { return {a.re + b.re, a.im + b.im}; }
inline cx sub(cx a, cx b) { return {a.re - b.re, a.im - b.im}; }
inline cx neg(cx a) { return {-a.re, -a.im}; }
inline cx mul(cx a, cx b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
inline cx rmul(double r, cx a) { return {r * a.re, r * a.im}; }
inline cx div(cx a, cx b) {
  double tr, ti;
  if (std::fabs(b.re) < std::fabs(b.im)) {
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
inline cx cexp_(cx z) {
  double s, c;
  if (std::fabs(z.im) > 2.2250738585072014e-308) { s = std::sin(z.im); c = std::cos(z.im); }
  else { s = z.im; c = 1.0; }
  const double e = std::exp(z.re);
  return {e * c, e * s};
}
inline cx csqrt_real(double x) { return x >= 0.0 ? cx{std::sqrt(x), 0.0} : cx{0.0, std::sqrt(-x)}; }
// csq (GRT.f90:107-111)
inline cx csq(double c, double vel) { const double t = c / vel; return csqrt_real(1.0 - t * t); }

const double PI_S = (double)3.1415926f;      // the single-precision pi literals
const double PI_D = 3.1415926535897932;      // m_GRT's pi
const double EXPO = 46.0;
const double EPS_GRT = 1e-10;                // m_GRT eps
const int NCCC = 20000;
thread_local long long g_evals = 0;            // secular-function evaluations

struct Grt {
  int nl = 0, ifs = 0, ilastvs = 0, nlvl1 = 0, nlvls1 = 0, no_lvl = 0, lvlast = 0, ll = 0;
  std::vector<double> d, vp, vs, rho, v, mu;
  double mu0 = 0, vsy = 0, vs1 = 0, vsm = 0;
  double w = 0, tol = 1e-5, smin = 1e-4, dc = 1e-4, dc2 = 1e-4, dcm = 1e-4;
};

// setup_grt (surfmodes.f90:320-450) for columns without fluid layers
int setup(Grt &g, const double *thk, const double *vp, const double *vs, const double *rho, int nl,
          int modetype) {
  const double eps = (double)1e-6f;          // m_surfmodes eps
  g.nl = nl;
  g.d.assign(thk, thk + nl); g.vp.assign(vp, vp + nl); g.vs.assign(vs, vs + nl); g.rho.assign(rho, rho + nl);
  g.v.clear();
  for (int i = 0; i < nl; ++i) {
    if (!(std::fabs(vs[i]) > eps)) return -2;  // fluid layer: the Stoneley path
    g.v.push_back(vs[i]);
    if (i == nl - 1) g.ilastvs = (int)g.v.size();
    g.v.push_back(vp[i]);
  }
  std::sort(g.v.begin(), g.v.end());
  g.mu.resize(nl);
  int idx = 0;
  double mu0 = 0;
  for (int i = 0; i < nl; ++i) {
    const double m = rho[i] * (vs[i] * vs[i]);
    if (std::fabs(m) > eps) { idx++; mu0 += m; }
    g.mu[i] = m;
  }
  mu0 = mu0 / idx;
  for (int i = 0; i < nl; ++i) g.mu[i] = g.mu[i] / mu0;
  g.mu0 = mu0;
  g.vsy = *std::max_element(g.vs.begin(), g.vs.end());
  g.vs1 = vs[0];
  if (modetype == 1) g.vsm = g.v[0];
  else g.vsm = *std::min_element(g.vs.begin(), g.vs.end());
  int last = 0;
  for (int i = 1; i < nl - 1; ++i) {         // Fortran i = 2 .. nl-1
    if (vp[i] < vp[i + 1] && vp[i] < vp[i - 1]) {
      g.no_lvl++;
      last = i + 1;
      if (vs[i] < g.vs1) g.nlvl1++;
    }
  }
  g.nlvls1 = g.nlvl1;
  g.lvlast = g.no_lvl == 0 ? 1 : last;
  g.lvlast = std::max(2, g.lvlast);
  return 0;
}

// startl (Rayleigh.f90:53-90): ll, the layer below which the evanescent
// field has decayed by e^-46 (1-based)
void startl(double c, Grt &g) {
  int sl = g.nl;
  const double vk = g.w / c;
  double su = 0;
  for (int j = g.lvlast; j <= g.nl - 1; ++j) {
    if (c < g.vs[j - 1]) {
      su = su + vk * csq(c, g.vs[j - 1]).re * g.d[j - 1];
      if (su > EXPO) { sl = j; break; }
    } else {
      su = 0;
    }
  }
  g.ll = sl;
}

typedef cx M4[4][4];
typedef cx M2[2][2];

// EinvE (Rayleigh.f90:404-440); j the interface (1-based), iq 0: E^-1 of the
// layer above times E of the layer below; iq 1: E of the layer below alone.
// cp/cs[k] receive the vertical slownesses of the layer above (0) / below (1).
void einve(const Grt &g, int j, double c, int iq, M4 out, cx cp[2], cx cs[2]) {
  M4 a44, b44;
  for (int k = 1; k >= iq; --k) {
    const int L = j + k - 1;                 // 0-based layer
    const double ap = g.vp[L], as = g.vs[L], am = g.mu[L];
    cp[k] = csq(c, ap); cs[k] = csq(c, as);
    const double t = c / as;
    const cx xi = C(1.0 - t * t / 2.0);
    if (k == 1) {
      const cx col0[4] = {C(1.0), cp[1], neg(rmul(am, cp[1])), neg(rmul(am, xi))};
      const cx col1[4] = {cs[1], C(1.0), neg(rmul(am, xi)), neg(rmul(am, cs[1]))};
      for (int r = 0; r < 4; ++r) { a44[r][0] = col0[r]; a44[r][1] = col1[r]; a44[r][2] = col0[r]; a44[r][3] = col1[r]; }
      a44[1][2] = neg(a44[1][2]); a44[1][3] = neg(a44[1][3]);
      a44[2][2] = neg(a44[2][2]); a44[2][3] = neg(a44[2][3]);
    } else {
      const cx row0[4] = {C(1.0), neg(div(xi, cp[0])), neg(div(C(1.0), rmul(am, cp[0]))), div(C(1.0), C(am))};
      const cx row1[4] = {neg(div(xi, cs[0])), C(1.0), div(C(1.0), C(am)), neg(div(C(1.0), rmul(am, cs[0])))};
      for (int cI = 0; cI < 4; ++cI) { b44[0][cI] = row0[cI]; b44[1][cI] = row1[cI]; b44[2][cI] = row0[cI]; b44[3][cI] = row1[cI]; }
      b44[2][1] = neg(b44[2][1]); b44[2][2] = neg(b44[2][2]);
      b44[3][1] = neg(b44[3][1]); b44[3][2] = neg(b44[3][2]);
      const cx den = rmul(2.0, sub(C(1.0), xi));
      for (int r = 0; r < 4; ++r) for (int q = 0; q < 4; ++q) b44[r][q] = div(b44[r][q], den);
    }
  }
  if (iq == 0) {
    for (int r = 0; r < 4; ++r)
      for (int q = 0; q < 4; ++q) {
        cx s = C(0.0);
        for (int k = 0; k < 4; ++k) s = add(s, mul(b44[r][k], a44[k][q]));
        out[r][q] = s;
      }
  } else {
    for (int r = 0; r < 4; ++r) for (int q = 0; q < 4; ++q) out[r][q] = a44[r][q];
  }
}

void mm2(const M2 a, const M2 b, M2 o) {
  for (int r = 0; r < 2; ++r)
    for (int q = 0; q < 2; ++q) {
      cx s = C(0.0);
      for (int k = 0; k < 2; ++k) s = add(s, mul(a[r][k], b[k][q]));
      o[r][q] = s;
    }
}
// inv2 (Rayleigh.f90:24-30)
void inv2(const M2 a, M2 o) {
  const cx det = sub(mul(a[0][0], a[1][1]), mul(a[1][0], a[0][1]));
  o[0][0] = div(a[1][1], det); o[1][0] = div(neg(a[1][0]), det);
  o[0][1] = div(neg(a[0][1]), det); o[1][1] = div(a[0][0], det);
}
inline cx decay(const Grt &g, int layer1, double vk, cx q) {
  // exp(-d(layer)*vk*q), the Fortran -((d*vk)*q)
  return cexp_(neg(rmul(g.d[layer1 - 1] * vk, q)));
}

// propup (Rayleigh.f90:455-491) from interface j2 up to interface 1; returns
// Rdu at interface 1 and the decays of layer 1 (la)
void propup(const Grt &g, double c, int j2, M2 rdu, cx la[2]) {
  const double vk = g.w / c;
  M4 E; cx cp[2], cs[2];
  einve(g, j2, c, 0, E, cp, cs);
  M2 a22, t, b22;
  M2 e11 = {{E[0][0], E[0][1]}, {E[1][0], E[1][1]}};
  inv2(e11, a22);
  la[0] = decay(g, j2, vk, cp[0]); la[1] = decay(g, j2, vk, cs[0]);
  for (int k = 0; k < 2; ++k) for (int r = 0; r < 2; ++r) a22[r][k] = mul(a22[r][k], la[k]);
  M2 e21 = {{E[2][0], E[2][1]}, {E[3][0], E[3][1]}};
  mm2(e21, a22, rdu);
  for (int j = j2 - 1; j >= 1; --j) {
    einve(g, j, c, 0, E, cp, cs);
    for (int r = 0; r < 2; ++r) for (int q = 0; q < 2; ++q) b22[r][q] = rdu[r][q];
    la[0] = decay(g, j + 1, vk, cp[1]); la[1] = decay(g, j + 1, vk, cs[1]);
    for (int k = 0; k < 2; ++k) for (int q = 0; q < 2; ++q) b22[k][q] = mul(b22[k][q], la[k]);
    M2 e12 = {{E[0][2], E[0][3]}, {E[1][2], E[1][3]}};
    M2 e22 = {{E[2][2], E[2][3]}, {E[3][2], E[3][3]}};
    M2 e11j = {{E[0][0], E[0][1]}, {E[1][0], E[1][1]}};
    M2 e21j = {{E[2][0], E[2][1]}, {E[3][0], E[3][1]}};
    mm2(e12, b22, t);
    M2 s;
    for (int r = 0; r < 2; ++r) for (int q = 0; q < 2; ++q) s[r][q] = add(e11j[r][q], t[r][q]);
    inv2(s, a22);
    la[0] = decay(g, j, vk, cp[0]); la[1] = decay(g, j, vk, cs[0]);
    for (int k = 0; k < 2; ++k) for (int r = 0; r < 2; ++r) a22[r][k] = mul(a22[r][k], la[k]);
    mm2(e22, b22, t);
    for (int r = 0; r < 2; ++r) for (int q = 0; q < 2; ++q) b22[r][q] = add(e21j[r][q], t[r][q]);
    mm2(b22, a22, rdu);
  }
}

// SecFunSurf (Rayleigh.f90:92-125): real part of the free-surface secular
// determinant; imf its imaginary part
double secfun_surf(const Grt &g, double c, double *imf) {
  g_evals++;
  M2 rdu; cx la[2];
  propup(g, c, g.ll - 1, rdu, la);
  M4 a44; cx cp[2], cs[2];
  einve(g, 0, c, 1, a44, cp, cs);
  M2 b22 = {{a44[2][2], a44[2][3]}, {a44[3][2], a44[3][3]}};
  for (int k = 0; k < 2; ++k) for (int r = 0; r < 2; ++r) b22[r][k] = mul(b22[r][k], la[k]);
  M2 t, a22;
  mm2(b22, rdu, t);
  for (int r = 0; r < 2; ++r) for (int q = 0; q < 2; ++q) a22[r][q] = add(a44[2 + r][q], t[r][q]);
  const cx dsp = sub(mul(a22[0][0], a22[1][1]), mul(a22[0][1], a22[1][0]));
  *imf = dsp.im;
  return dsp.re;
}

// EinvE_L (Love.f90:39-67)
void einve_l(const Grt &g, int j, double c, int iq, M2 out, cx cs[2]) {
  M2 a22, b22;
  for (int k = 1; k >= iq; --k) {
    const int L = j + k - 1;
    const double as = g.vs[L], am = g.mu[L];
    cs[k] = csq(c, as);
    if (k == 1) {
      a22[0][1] = C(1.0); a22[1][1] = rmul(am, cs[1]);
      a22[0][0] = C(1.0); a22[1][0] = neg(a22[1][1]);
    } else {
      b22[0][0] = rmul(am, cs[0]); b22[1][0] = rmul(am, cs[0]);
      b22[0][1] = C(-1.0); b22[1][1] = C(1.0);
      const cx den = rmul(2.0, b22[0][0]);
      for (int r = 0; r < 2; ++r) for (int q = 0; q < 2; ++q) b22[r][q] = div(b22[r][q], den);
    }
  }
  if (iq == 0) mm2(b22, a22, out);
  else for (int r = 0; r < 2; ++r) for (int q = 0; q < 2; ++q) out[r][q] = a22[r][q];
}

// SecFuns_L (Love.f90:118-132) at lay = 1: propdn_L (Love.f90:69-90) gives
// RudL(0), propup_L (Love.f90:92-116) RduL(1)
double secfun_love(const Grt &g, double c, double *imf) {
  g_evals++;
  const double vk = g.w / c;
  M2 a22; cx cs[2];
  einve_l(g, 0, c, 1, a22, cs);
  const cx la2 = decay(g, 1, vk, cs[1]);
  const cx rud0 = neg(div(mul(a22[1][1], la2), a22[1][0]));
  const int j2 = g.ll - 1;
  einve_l(g, j2, c, 0, a22, cs);
  cx td = div(decay(g, j2, vk, cs[0]), a22[0][0]);
  cx rdu = mul(a22[1][0], td);
  for (int j = j2 - 1; j >= 1; --j) {
    einve_l(g, j, c, 0, a22, cs);
    const cx r = mul(decay(g, j + 1, vk, cs[1]), rdu);
    td = div(decay(g, j, vk, cs[0]), add(a22[0][0], mul(a22[0][1], r)));
    rdu = mul(add(a22[1][0], mul(a22[1][1], r)), td);
  }
  const cx dsp = sub(C(1.0), mul(rud0, rdu));
  *imf = dsp.re;
  return dsp.im;
}

typedef double (*SecFn)(const Grt &, double, double *);

// bisecim (util.f90:90-167)
double bisecim(SecFn f, const Grt &g, double x1, double x2, double f1, double f2, int *iq) {
  const double smin2 = g.smin * g.smin * 2.0;
  int nc = 0;
  double dx = std::fabs(x1 - x2);
  const double fa = f1;
  double x[3] = {x1, x2, 0}, y[3] = {fa, f2, 0};
  double xt1 = (x[0] + x[1]) / 2.0, imf = 0, imf2 = 0;
  for (;;) {
    x[2] = (x[0] + x[1]) / 2.0;
    y[2] = f(g, x[2], &imf);
    double u1 = (x[1] - x[0]) / (y[1] - y[0]);
    double u2 = (x[1] - x[2]) / (y[1] - y[2]);
    const double xt2 = x[0] - y[0] * (u1 - y[1] * ((u2 - u1) / (y[2] - y[0])));
    double dxt = std::fabs(xt2 - xt1);
    dx = dx / 2.0;
    if (dx < dxt) dxt = dx;
    if (dxt < g.tol) {
      u1 = f(g, xt2, &imf2);
      u2 = y[2];
      if (u1 * u1 + imf2 * imf2 < smin2 || u2 * u2 + imf * imf < smin2) {
        *iq = 0;
        return std::fabs(u1) < std::fabs(u2) ? xt2 : x[2];
      }
      *iq = -1;
      return 0.0;
    }
    xt1 = xt2;
    if (fa * y[2] < 0) { x[1] = x[2]; y[1] = y[2]; }
    else { x[0] = x[2]; y[0] = y[2]; }
    nc++;
    if (nc >= 1000) { *iq = -1; return 0.0; }
  }
}

// N_cf (C_interval.f90:188-208) and N_cf_L (C_interval_L.f90:186-204)
double n_cf(const Grt &g, double c, bool love) {
  double s = 0;
  for (int i = 0; i < g.nl - 1; ++i) {
    double yr = 0;
    if (!love) { const double t = c / g.vp[i]; yr = csqrt_real(t * t - 1.0).re; }
    double ys = 0;
    if (g.vs[i] > 0.0) { const double t = c / g.vs[i]; ys = csqrt_real(t * t - 1.0).re; }
    s = s + ((2.0 * (yr + ys)) * g.d[i]) / c;
  }
  return g.w / (2.0 * (love ? PI_D : PI_S)) * s;
}

// C_Interval (C_interval.f90:1-186) / C_Interval_L: the sorted, thinned
// trial phase velocities ccc and (Rayleigh) im1, the first >= vs1 (1-based).
// Returns -1 where the reference's 20,000-entry arrays would overflow.
int c_interval(const Grt &g, bool love, std::vector<double> &ccc, int *im1) {
  std::vector<double> vvv;
  vvv.reserve(4096);
  auto push = [&](double x) { vvv.push_back(x); return (int)vvv.size() <= NCCC; };
  const double freq = g.w / (2.0 * (love ? PI_D : PI_S));
  const long NN = std::lround(n_cf(g, g.vsy, love) - n_cf(g, g.vsm, love));
  if (freq < (double)0.12f || NN < 2) {
    const long n = (NN + 1) * (love ? 512 : 1024);
    if (n > NCCC || n < 0) return -1;
    const double lo = love ? g.vsm - 0.01 : g.v[0] - 0.1;
    for (long i = 1; i <= n; ++i) vvv.push_back(lo + (double)i * (g.vsy - (love ? g.vsm : g.v[0]) + (love ? 0.01 : 0.1)) / (double)n);
    for (int i = 1; i <= 100; ++i) if (!push(g.vsy * (1.0 - 0.008 * (double)i))) return -1;
  } else {
    const double c1 = love ? g.vsm : g.v[0];
    vvv.push_back(c1);
    double c2 = g.vsy, c0 = c2, dc = 0;
    long NNc = NN;
    while (c0 > c1) {
      if (NNc > 0) dc = (c2 - c1) / (double)NNc;
      c0 = c2 - dc;
      for (int h = 0;; ++h) {
        const double dN = n_cf(g, c2, love) - n_cf(g, c0, love);
        if (h >= 1100 && !(dN < 0.5)) return -1;
        if (dN < 0.5) {
          if (!push(c0)) return -1;
          NNc--;
          c2 = c0;
          break;
        }
        c0 = (c2 + c0) / 2.0;
      }
    }
    int ij = 1;
    while (ij <= (int)g.v.size() && g.v[ij - 1] <= g.vsy) ij++;
    for (int i = 1; i <= ij - 2; ++i) {
      const double c01 = g.v[i - 1];
      int ii = 0;
      for (int j = 1; j <= g.nl; ++j)
        if (std::fabs(g.vs[j - 1] - c01) < EPS_GRT || std::fabs(g.vp[j - 1] - c01) < EPS_GRT) ii = j;
      if (ii == 0) continue;
      const double hi = g.d[ii - 1];
      const double Ni = 2.0 * freq * hi / c01 + EPS_GRT;
      const long nj = (long)std::floor(Ni);
      for (long j = 1; j <= nj; ++j) {
        const double r = (double)j / Ni;
        const double c00 = c01 / std::sqrt(1.0 - r * r);
        if (c00 <= g.vsy && !push(c00)) return -1;
      }
    }
    std::sort(vvv.begin(), vvv.end());
    for (int rep = 0; rep < 2; ++rep) {
      const int n = (int)vvv.size();
      for (int i = 0; i < n - 1; ++i) if (!push((vvv[i] + vvv[i + 1]) / 2.0)) return -1;
    }
    for (int i = 1; i <= 100; ++i) if (!push(g.vsy - (double)i / 100.0 * 0.1)) return -1;
  }
  for (int i = 1; i <= 10; ++i) if (!push(g.vsy - (double)(i * 10) * g.tol)) return -1;
  if (!push(g.vsy - 3.0 * g.tol)) return -1;
  if (!push(g.vs1 + 4.0 * g.tol)) return -1;
  if (!push(g.vs1 - 4.0 * g.tol)) return -1;
  std::sort(vvv.begin(), vvv.end());
  // no points at or below vsm (the first becomes vsm + tol)
  for (size_t i = 0; i < vvv.size(); ++i) {
    if (vvv[i] > g.vsm) {
      std::vector<double> t;
      t.push_back(g.vsm + g.tol);
      t.insert(t.end(), vvv.begin() + i, vvv.end());
      vvv.swap(t);
      break;
    }
  }
  int ii = (int)vvv.size();
  while (ii >= 1 && vvv[ii - 1] >= g.vsy) ii--;
  ccc.clear();
  if (ii < 1) return -1;
  const double tol0 = 10.0 * g.tol;
  ccc.push_back(vvv[0]);
  for (int i = 2; i <= ii; ++i) {
    if (vvv[i - 1] - vvv[i - 2] < tol0) continue;
    ccc.push_back(vvv[i - 1]);
  }
  int m = 0;
  for (size_t i = 0; i < ccc.size(); ++i)
    if (love ? ccc[i] > g.vs1 : ccc[i] >= g.vs1) { m = (int)i + 1; break; }
  if (m == 0 && !love) m = (int)ccc.size();
  *im1 = m;
  return 0;
}

// CR0_Finder (SearchRayleigh.f90:898-933): Newton on the half-space
// Rayleigh function; the reference's loop has no iteration bound, 10,000 here
double cr0_finder(double v1, double v2) {
  const double tol = 1e-7;
  double c = 0.8 * v1;
  for (int it = 0; it < 10000; ++it) {
    const double ps = 1.0 / v1, pp = 1.0 / v2, p = 1.0 / c;
    const double p2 = p * p, ps2 = ps * ps, pp2 = pp * pp;
    const double sps = std::sqrt(p2 - ps2), spp = std::sqrt(p2 - pp2);
    const double a = ps2 - 2.0 * p2;
    const double R = a * a - 4.0 * p2 * sps * spp;
    const double DR = p2 * (8.0 * p * (ps2 - 2.0 * p2) + 8.0 * p * sps * spp +
                            4.0 * (p2 * p) * (spp / sps + sps / spp));
    c = c - R / DR;
    if (v1 - c < tol || v2 - c < tol || c != c) break;
    if (std::fabs(R / DR) < tol) break;
  }
  return c;
}

// SearchRayleigh's FundaMode for columns without fluid layers
// (SearchRayleigh.f90:455-605); returns ierr, the root in *cray
int funda_rayleigh(Grt &g, double *cray) {
  int ierr = 1, iq = -1;
  double cmn;
  int nk;
  if (*cray > 0.) { cmn = (double)0.90f * *cray; nk = 10; }
  else { cmn = cr0_finder(g.vs1, g.vp[0]); cmn = cmn - 0.1; nk = 100; }
  const double cmx = g.vs1 - 4.0 * g.tol;
  double imf;
  if (cmx > cmn) {
    double kk[100];
    for (int i = 1; i <= nk; ++i) kk[i - 1] = cmn + (cmx - cmn) / (double)nk * (double)i;
    startl(kk[nk - 1], g);
    int j = 1;
    iq = 1;
    double k2 = kk[0], f2 = secfun_surf(g, k2, &imf);
    for (;;) {
      const double k1 = k2, f1 = f2;
      j++;
      k2 = kk[j - 1];
      f2 = secfun_surf(g, k2, &imf);
      if (f1 * f2 < 0.) {
        const double kt = bisecim(secfun_surf, g, k1, k2, f1, f2, &iq);
        if (iq == 0) { *cray = kt; ierr = 0; break; }
      }
      if (j == nk) break;
    }
  }
  if (iq != 0) {
    std::vector<double> ccc;
    int im1 = 0;
    if (c_interval(g, false, ccc, &im1)) return 2;
    const int index0 = (int)ccc.size();
    int im2 = im1;
    if (g.nlvl1 == 0) {
      while (ccc[im2 - 1] < *cray - 2.0 * g.dc) { im2++; if (im2 == index0) break; }
    }
    double k2 = ccc[im2 - 1];
    startl(k2, g);
    double f2 = secfun_surf(g, k2, &imf);
    for (int ip = im2 + 1; ip <= index0; ++ip) {
      const double k1 = k2, f1 = f2;
      k2 = ccc[ip - 1];
      startl(k2, g);
      f2 = secfun_surf(g, k2, &imf);
      iq = -1;
      if (f1 * f2 < 0.) {
        const double kt = bisecim(secfun_surf, g, k1, k2, f1, f2, &iq);
        if (iq == 0) { *cray = kt; ierr = 0; break; }
      }
    }
  }
  return ierr;
}

// SearchLove's FundaMode (SearchLove.f90:204-270)
int funda_love(Grt &g, double *cray) {
  std::vector<double> ccc;
  int im1 = 0;
  if (c_interval(g, true, ccc, &im1)) return 2;
  const int index0 = (int)ccc.size();
  int ierr = 1, iq = -1;
  const double c0 = *cray;
  double imf;
  double k2 = ccc[0];
  startl(k2, g);
  double f2 = secfun_love(g, k2, &imf);
  for (int ip = 2; ip <= index0; ++ip) {
    const double k1 = k2, f1 = f2;
    k2 = ccc[ip - 1];
    startl(k2, g);
    f2 = secfun_love(g, k2, &imf);
    iq = -1;
    if (f1 * f2 < 0.) {
      const double kt = bisecim(secfun_love, g, k1, k2, f1, f2, &iq);
      if (iq == 0) { *cray = kt; ierr = 0; break; }
    }
  }
  if (ierr == 1 && std::isfinite(c0)) {
    k2 = (double)1.1f * c0;
    startl(k2, g);
    f2 = secfun_love(g, k2, &imf);
    for (;;) {
      const double k1 = k2 - g.dc;
      if (k1 < g.vsm) break;
      startl(k1, g);
      const double f1 = secfun_love(g, k1, &imf);
      iq = -1;
      if (f1 * f2 < 0.) {
        const double kt = bisecim(secfun_love, g, k1, k2, f1, f2, &iq);
        if (iq == 0) { *cray = kt; ierr = 0; break; }
      }
      k2 = k1;
      f2 = f1;
    }
  }
  if (ierr == 1) *cray = 0;
  return ierr;
}

}  // namespace

extern "C" {

// setup_grt's count of low-velocity layers slower than the top layer
// (nlvls1 for columns without fluid layers): the surfmodes routing test.
int orc_grt_nlvls1(int nl, const double *thk, const double *vp, const double *vs, const double *rho,
                   int modetype) {
  Grt g;
  if (setup(g, thk, vp, vs, rho, nl, modetype)) return -2;
  return g.nlvls1;
}

// The secular function the searches bracket (SecFunSurf's real part for
// Rayleigh, SecFuns_L's imaginary part for Love) at phase velocity c and
// frequency freq, with startl's truncation for c; *imf the other part.
double orc_grt_secfun(int nl, const double *thk, const double *vp, const double *vs, const double *rho,
                      int modetype, double freq, double c, double *imf) {
  Grt g;
  if (setup(g, thk, vp, vs, rho, nl, modetype)) return 0.0;
  g.w = freq * 2.0 * PI_S;
  startl(c, g);
  double im = 0;
  const double f = modetype == 1 ? secfun_surf(g, c, &im) : secfun_love(g, c, &im);
  if (imf) *imf = im;
  return f;
}

// RayleighModes (modetype 1) / LoveModes (modetype 0), fundamental mode, for
// one column: phase[np] and, with phase_group 1, group[np] (entries after a
// failed frequency keep 0); nevals (optional) receives the number of
// secular-function evaluations. Returns ierr: 0, 1 (no root), 2 (more than
// 20,000 trial velocities) or -2 (a fluid layer).
int orc_grt_modes(int nl, const double *thk, const double *vp, const double *vs, const double *rho, int np,
                  const double *freqs, int modetype, int phase_group, double tolmin, double tolmax,
                  double smin_min, double smin_max, double dc, double dcm, double dc2, double *phase,
                  double *group, long long *nevals) {
  Grt g;
  if (setup(g, thk, vp, vs, rho, nl, modetype)) return -2;
  g.dc = dc; g.dc2 = dc2; g.dcm = dcm;
  for (int i = 0; i < np; ++i) { phase[i] = 0; group[i] = 0; }
  const double dh = (double)0.005f;
  double c0 = 0;
  g_evals = 0;
  struct Count { long long *p; ~Count() { if (p) *p = g_evals; } } count{nevals};
  for (int i = 1; i <= np; ++i) {
    g.w = freqs[i - 1] * 2.0 * PI_S;
    g.tol = tolmin + (double)(np + 1 - i) * (tolmax - tolmin) / (double)np;
    g.smin = smin_min + (double)(i - 1) * (smin_max - smin_min) / (double)np;
    double cray = c0;
    int e = modetype == 1 ? funda_rayleigh(g, &cray) : funda_love(g, &cray);
    if (e) return e;
    phase[i - 1] = cray;
    c0 = cray;
    if (phase_group == 1) {
      const double freq0 = freqs[i - 1] + dh;
      g.w = freq0 * 2.0 * PI_S;
      double cp0 = c0;
      e = modetype == 1 ? funda_rayleigh(g, &cp0) : funda_love(g, &cp0);
      if (e) return e;
      double grp = (freqs[i - 1] + dh) / cp0 - freqs[i - 1] / phase[i - 1];
      grp = grp > 0 ? dh / grp : 0.0;
      group[i - 1] = grp;
    }
  }
  return 0;
}

}  // extern "C"
