// ORACLE (test infrastructure only): CPU restatement of Rawlinson's fm2d fast
// marching code in Cartesian form as shipped with MCTomo
// (fm2d/fm2dray_cartesian.f90 modrays/gridder/bsplrefine/srtimes and
// fm2d/fm2d_ttime.f90 travel/fouds1/fouds2/addtree/downtree/updtree/bilinear).
// Used as the parity checker for the GPU 2D eikonal kernel. Never linked into
// the product.
//
// Parity status: unpinned by reference execution (Fortran, no compiler on this
// image); pinned by homogeneous-medium known answers and line-by-line
// restatement. Arithmetic order follows the Fortran expressions; build with
// -ffp-contract=off.
//
// Ray path tracing (rpaths, fm2dray_cartesian.f90:801-1455) is not restated
// here: it only runs for group-velocity data (uar == 0).
#include <climits>
#include <cmath>
#include <vector>
#include <cstdlib>
#include "oracle.h"

namespace {

int g_trace_src = -1, g_trace_n = 0, g_trace_max = 0, g_cur_src = -1;
int *g_trace_i = nullptr;
double *g_trace_t = nullptr;

struct FM2D {
  // grid of nodes currently being marched (coarse or refined)
  int nnx, nnz;
  double gox, goz, dnx, dnz;
  int fom;
  // refined-box bounds (1-based, coarse node units)
  int vnl, vnr, vnt, vnb;
  int ld;                   // leading dimension (rows) of veln/ttn/nsts
  std::vector<double> veln, ttn;
  std::vector<int> nsts;
  std::vector<int> btgx, btgz;  // heap backpointers (1-based slots)
  int ntr;

  double &V(int iz, int ix) { return veln[(size_t)(ix - 1) * ld + (iz - 1)]; }
  double &T(int iz, int ix) { return ttn[(size_t)(ix - 1) * ld + (iz - 1)]; }
  int &S(int iz, int ix) { return nsts[(size_t)(ix - 1) * ld + (iz - 1)]; }

  // fm2d_ttime.f90:527-566 addtree
  void addtree(int iz, int ix) {
    ntr = ntr + 1;
    if ((size_t)ntr >= btgx.size()) { btgx.resize(ntr * 2 + 8); btgz.resize(ntr * 2 + 8); }
    S(iz, ix) = ntr;
    btgx[ntr] = ix; btgz[ntr] = iz;
    int tpc = ntr, tpp = tpc / 2;
    while (tpp > 0) {
      if (T(iz, ix) < T(btgz[tpp], btgx[tpp])) {
        S(iz, ix) = tpp;
        S(btgz[tpp], btgx[tpp]) = tpc;
        std::swap(btgx[tpc], btgx[tpp]); std::swap(btgz[tpc], btgz[tpp]);
        tpc = tpp; tpp = tpc / 2;
      } else {
        tpp = 0;
      }
    }
  }

  // fm2d_ttime.f90:576-640 downtree
  void downtree() {
    if (ntr == 1) { ntr = ntr - 1; return; }
    S(btgz[ntr], btgx[ntr]) = 1;
    btgx[1] = btgx[ntr]; btgz[1] = btgz[ntr];
    ntr = ntr - 1;
    int tpp = 1, tpc = 2 * tpp;
    while (tpc < ntr) {
      double rd1 = T(btgz[tpc], btgx[tpc]);
      double rd2 = T(btgz[tpc + 1], btgx[tpc + 1]);
      if (rd1 > rd2) tpc = tpc + 1;
      rd1 = T(btgz[tpc], btgx[tpc]);
      rd2 = T(btgz[tpp], btgx[tpp]);
      if (rd1 < rd2) {
        S(btgz[tpp], btgx[tpp]) = tpc;
        S(btgz[tpc], btgx[tpc]) = tpp;
        std::swap(btgx[tpc], btgx[tpp]); std::swap(btgz[tpc], btgz[tpp]);
        tpp = tpc; tpc = 2 * tpp;
      } else {
        tpc = ntr + 1;
      }
    }
    if (tpc == ntr) {
      double rd1 = T(btgz[tpc], btgx[tpc]);
      double rd2 = T(btgz[tpp], btgx[tpp]);
      if (rd1 < rd2) {
        S(btgz[tpp], btgx[tpp]) = tpc;
        S(btgz[tpc], btgx[tpc]) = tpp;
        std::swap(btgx[tpc], btgx[tpp]); std::swap(btgz[tpc], btgz[tpp]);
      }
    }
  }

  // fm2d_ttime.f90:650-672 updtree
  void updtree(int iz, int ix) {
    int tpc = S(iz, ix), tpp = tpc / 2;
    while (tpp > 0) {
      if (T(iz, ix) < T(btgz[tpp], btgx[tpp])) {
        S(iz, ix) = tpp;
        S(btgz[tpp], btgx[tpp]) = tpc;
        std::swap(btgx[tpc], btgx[tpp]); std::swap(btgz[tpc], btgz[tpp]);
        tpc = tpp; tpp = tpc / 2;
      } else {
        tpp = 0;
      }
    }
  }

  // fm2d_ttime.f90:248-332 fouds1 (first-order upwind)
  void fouds1(int iz, int ix) {
    int tsw1 = 0;
    double travm = 0.0;
    double slown = 1.0 / V(iz, ix);
    for (int j = ix - 1; j <= ix + 1; j += 2) {
      for (int k = iz - 1; k <= iz + 1; k += 2) {
        if (j >= 1 && j <= nnx && k >= 1 && k <= nnz) {
          int swsol = 0;
          double a = 0, b = 0, c = 0, tref = 0;
          if (S(iz, j) == 0) {
            swsol = 1;
            if (S(k, ix) == 0) {
              double u = dnx, v = dnz;
              double em = T(k, ix) - T(iz, j);
              a = u * u + v * v;
              b = -(2.0 * (u * u) * em);
              c = (u * u) * (em * em - (v * v) * (slown * slown));
              tref = T(iz, j);
            } else {
              a = 1.0; b = 0.0;
              c = -((slown * slown) * (dnx * dnx));
              tref = T(iz, j);
            }
          } else if (S(k, ix) == 0) {
            swsol = 1;
            a = 1.0; b = 0.0;
            double sd = slown * dnz;
            c = -(sd * sd);
            tref = T(k, ix);
          }
          if (swsol == 1) {
            double rd1 = b * b - 4.0 * a * c;
            if (rd1 < 0.0) rd1 = 0.0;
            double tdsh = (-b + std::sqrt(rd1)) / (2.0 * a);
            double trav = tref + tdsh;
            if (tsw1 == 1) travm = std::fmin(trav, travm);
            else { travm = trav; tsw1 = 1; }
          }
        }
      }
    }
    T(iz, ix) = travm;
  }

  // fm2d_ttime.f90:342-518 fouds2 (mixed-order upwind)
  void fouds2(int iz, int ix) {
    int tsw1 = 0;
    double travm = 0.0;
    double slown = 1.0 / V(iz, ix);
    for (int j = ix - 1; j <= ix + 1; j += 2) {
      if (!(j >= 1 && j <= nnx)) continue;
      int swj = -1, j2;
      if (j == ix - 1) {
        j2 = j - 1;
        if (j2 >= 1) { if (S(iz, j2) == 0) swj = 0; }
      } else {
        j2 = j + 1;
        if (j2 <= nnx) { if (S(iz, j2) == 0) swj = 0; }
      }
      if (S(iz, j) == 0 && swj == 0) {
        swj = -1;
        if (T(iz, j) > T(iz, j2)) swj = 0;
      } else {
        swj = -1;
      }
      for (int k = iz - 1; k <= iz + 1; k += 2) {
        if (!(k >= 1 && k <= nnz)) continue;
        int swk = -1, k2;
        if (k == iz - 1) {
          k2 = k - 1;
          if (k2 >= 1) { if (S(k2, ix) == 0) swk = 0; }
        } else {
          k2 = k + 1;
          if (k2 <= nnz) { if (S(k2, ix) == 0) swk = 0; }
        }
        if (S(k, ix) == 0 && swk == 0) {
          swk = -1;
          if (T(k, ix) > T(k2, ix)) swk = 0;
        } else {
          swk = -1;
        }
        int swsol = 0;
        double a = 0, b = 0, c = 0, tref = 0, tdiv = 1.0;
        if (swj == 0) {
          swsol = 1;
          if (swk == 0) {
            double u = 2.0 * dnx, v = 2.0 * dnz;
            double em = 4.0 * T(iz, j) - T(iz, j2) - 4.0 * T(k, ix);
            em = em + T(k2, ix);
            a = v * v + u * u;
            b = 2.0 * em * (u * u);
            c = (u * u) * (em * em - (slown * slown) * (v * v));
            tref = 4.0 * T(iz, j) - T(iz, j2);
            tdiv = 3.0;
          } else if (S(k, ix) == 0) {
            double u = dnz, v = 2.0 * dnx;
            double em = 3.0 * T(k, ix) - 4.0 * T(iz, j) + T(iz, j2);
            a = v * v + 9.0 * (u * u);
            b = 6.0 * em * (u * u);
            c = (u * u) * (em * em - (slown * slown) * (v * v));
            tref = T(k, ix);
            tdiv = 1.0;
          } else {
            double u = 2.0 * dnx;
            a = 1.0; b = 0.0;
            c = -((u * u) * (slown * slown));
            tref = 4.0 * T(iz, j) - T(iz, j2);
            tdiv = 3.0;
          }
        } else if (S(iz, j) == 0) {
          swsol = 1;
          if (swk == 0) {
            double u = dnx, v = 2.0 * dnz;
            double em = 3.0 * T(iz, j) - 4.0 * T(k, ix) + T(k2, ix);
            a = v * v + 9.0 * (u * u);
            b = 6.0 * em * (u * u);
            c = (u * u) * (em * em - (v * v) * (slown * slown));
            tref = T(iz, j);
            tdiv = 1.0;
          } else if (S(k, ix) == 0) {
            double u = dnx, v = dnz;
            double em = T(k, ix) - T(iz, j);
            a = u * u + v * v;
            b = -(2.0 * (u * u) * em);
            c = (u * u) * (em * em - (v * v) * (slown * slown));
            tref = T(iz, j);
            tdiv = 1.0;
          } else {
            a = 1.0; b = 0.0;
            c = -((slown * slown) * (dnx * dnx));
            tref = T(iz, j);
            tdiv = 1.0;
          }
        } else {
          if (swk == 0) {
            swsol = 1;
            double u = 2.0 * dnz;
            a = 1.0; b = 0.0;
            c = -((u * u) * (slown * slown));
            tref = 4.0 * T(k, ix) - T(k2, ix);
            tdiv = 3.0;
          } else if (S(k, ix) == 0) {
            swsol = 1;
            a = 1.0; b = 0.0;
            c = -((slown * slown) * (dnz * dnz));
            tref = T(k, ix);
            tdiv = 1.0;
          }
        }
        if (swsol == 1) {
          double rd1 = b * b - 4.0 * a * c;
          if (rd1 < 0.0) rd1 = 0.0;
          double tdsh = (-b + std::sqrt(rd1)) / (2.0 * a);
          double trav = (tref + tdsh) / tdiv;
          if (tsw1 == 1) travm = std::fmin(trav, travm);
          else { travm = trav; tsw1 = 1; }
        }
      }
    }
    T(iz, ix) = travm;
  }

  void fouds(int iz, int ix) { if (fom == 0) fouds1(iz, ix); else fouds2(iz, ix); }

  // fm2d_ttime.f90:682-711 bilinear
  double bilinear(const double nv[2][2], double dsx, double dsz) {
    double biv = 0.0;
    for (int i = 1; i <= 2; ++i)
      for (int j = 1; j <= 2; ++j) {
        double produ = (1.0 - std::fabs(((double)(i - 1) * dnx - dsx) / dnx)) *
                       (1.0 - std::fabs(((double)(j - 1) * dnz - dsz) / dnz));
        biv = biv + nv[i - 1][j - 1] * produ;
      }
    return biv;
  }

  // fm2d_ttime.f90:41-238 travel. Returns -1 if the source is outside.
  int travel(double scx, double scz, int urg) {
    int isx = (int)((scx - gox) / dnx) + 1;
    int isz = (int)((scz - goz) / dnz) + 1;
    if (isx < 1 || isx > nnx || isz < 1 || isz > nnz) return -1;
    if (isx == nnx) isx = isx - 1;
    if (isz == nnz) isz = isz - 1;
    if (urg != 2) std::fill(nsts.begin(), nsts.end(), -1);
    ntr = 0;
    if (urg == 2) {
      for (int i = 1; i <= nnx; ++i)
        for (int j = 1; j <= nnz; ++j)
          if (S(j, i) > 0) addtree(j, i);
    } else {
      std::fill(nsts.begin(), nsts.end(), -1);
      double vss[2][2];
      for (int i = 1; i <= 2; ++i)
        for (int j = 1; j <= 2; ++j) vss[i - 1][j - 1] = V(isz - 1 + j, isx - 1 + i);
      double dsx = (scx - gox) - (double)(isx - 1) * dnx;
      double dsz = (scz - goz) - (double)(isz - 1) * dnz;
      double vsrc = bilinear(vss, dsx, dsz);
      for (int i = 1; i <= 2; ++i)
        for (int j = 1; j <= 2; ++j) {
          double ex = dsx - (double)(i - 1) * dnx;
          double ez = dsz - (double)(j - 1) * dnz;
          double ds = std::sqrt(ex * ex + ez * ez);
          T(isz - 1 + j, isx - 1 + i) = 2.0 * ds / (vss[i - 1][j - 1] + vsrc);
          addtree(isz - 1 + j, isx - 1 + i);
        }
    }
    while (ntr > 0) {
      if (urg == 1) {
        int ix = btgx[1], iz = btgz[1];
        int swrg = 0;
        if (ix == 1) { if (vnl != 1) swrg = 1; }
        // vnr/vnb are coarse node indices compared with the refined grid
        // size, exactly as the reference's module variables are at this point
        if (ix == nnx) { if (vnr != nnx) swrg = 1; }
        if (iz == 1) { if (vnt != 1) swrg = 1; }
        if (iz == nnz) { if (vnb != nnz) swrg = 1; }
        if (swrg == 1) { S(iz, ix) = 0; break; }
      }
      int ix = btgx[1], iz = btgz[1];
      if (g_cur_src == g_trace_src && g_trace_n < g_trace_max) {
        g_trace_i[3 * g_trace_n] = urg; g_trace_i[3 * g_trace_n + 1] = (iz - 1) + nnz * (ix - 1);
        g_trace_i[3 * g_trace_n + 2] = ntr; g_trace_t[g_trace_n] = T(iz, ix); g_trace_n++;
      }
      S(iz, ix) = 0;
      downtree();
      for (int i = ix - 1; i <= ix + 1; i += 2) {
        if (i >= 1 && i <= nnx) {
          if (S(iz, i) == -1) { fouds(iz, i); addtree(iz, i); }
          else if (S(iz, i) > 0) { fouds(iz, i); updtree(iz, i); }
        }
      }
      for (int i = iz - 1; i <= iz + 1; i += 2) {
        if (i >= 1 && i <= nnz) {
          if (S(i, ix) == -1) { fouds(i, ix); addtree(i, ix); }
          else if (S(i, ix) > 0) { fouds(i, ix); updtree(i, ix); }
        }
      }
    }
    return 0;
  }

};

}  // namespace

namespace {

// ---- ray paths and group times ---------------------------------------------

// Rectangular grid description shared by the ray tracer and GetVelocity.
struct G2 { int nx, nz; double gox, goz, dx, dz; };

// GetVelocity (src/likelihood_surf.F90:496-521): bilinear velocity of the
// model grid vel (column-major (nz, nx), i.e. vel(iy, ix)) at point p.
double get_velocity(const double *vel, const G2 &g, double px, double pz) {
  int ix = (int)std::floor((px - g.gox) / g.dx) + 1;
  int iy = (int)std::floor((pz - g.goz) / g.dz) + 1;
  if (ix < 1) ix = 1;
  if (iy < 1) iy = 1;
  if (ix >= g.nx) ix = g.nx - 1;
  if (iy >= g.nz) iy = g.nz - 1;
  double dsx = px - (g.gox + (double)(ix - 1) * g.dx);
  double dsy = pz - (g.goz + (double)(iy - 1) * g.dz);
  double qv = 0;
  for (int i = 1; i <= 2; ++i)
    for (int j = 1; j <= 2; ++j) {
      double weight = (1.0 - std::fabs((double)(i - 1) * g.dx - dsx) / g.dx) *
                      (1.0 - std::fabs((double)(j - 1) * g.dz - dsy) / g.dz);
      qv = qv + weight * vel[(size_t)(ix + i - 2) * g.nz + (iy + j - 2)];
    }
  return qv;
}

// CalGroupTime (src/likelihood_surf.F90:455-494) for one ray, and the ray's
// length (T_RAY%length, fm2d/fm2dray_cartesian.f90:51-65).
void group_time(const std::vector<double> &rx, const std::vector<double> &rz, const double *vel, const G2 &g,
                double *time, double *length) {
  *time = 0; *length = 0;
  const size_t n = rx.size();
  if (n < 2) return;
  double vhead = get_velocity(vel, g, rx[0], rz[0]);
  for (size_t k = 1; k < n; ++k) {
    double dist = (rx[k] - rx[k - 1]) * (rx[k] - rx[k - 1]) + (rz[k] - rz[k - 1]) * (rz[k] - rz[k - 1]);
    dist = std::sqrt(dist);
    double vtail = get_velocity(vel, g, rx[k], rz[k]);
    *time = *time + dist * 2 / (vhead + vtail);
    *length = *length + dist;
    vhead = vtail;
  }
}

// FLOOR of a ray coordinate. Where the travel-time gradient vanishes the
// reference's next point is NaN, and FLOOR(NaN) is -2^31 on the x86 targets
// the reference is built for, which the boundary clamp then moves to the
// lower grid edge; that is made explicit here.
int floor_idx(double v) { return std::isnan(v) ? INT_MIN : (int)std::floor(v); }

// rpaths (fm2d/fm2dray_cartesian.f90:801-1455) without Frechet derivatives,
// one receiver: steepest descent on the final coarse field ttn (nnz, nnx),
// or on the refined-box field ttnr / states nstsr where the ray is inside the
// box and the four corners of its cell are accepted. Returns 1 for a ray
// that reached the point limit (the reference's crazy ray).
int trace_ray(double rcx, double rcz, double scx, double scz, const G2 &c, const double *ttn, int asgr,
              const G2 &r, const double *ttnr, const int *nstsr, std::vector<double> &rx, std::vector<double> &rz) {
  auto T = [&](int iz, int ix) { return ttn[(size_t)(ix - 1) * c.nz + (iz - 1)]; };
  auto TR = [&](int iz, int ix) { return ttnr[(size_t)(ix - 1) * r.nz + (iz - 1)]; };
  auto SR = [&](int iz, int ix) { return nstsr[(size_t)(ix - 1) * r.nz + (iz - 1)]; };
  const int nnx = c.nx, nnz = c.nz, nnxr = r.nx, nnzr = r.nz;
  const double gox = c.gox, goz = c.goz, dnx = c.dx, dnz = c.dz;
  const double goxr = r.gox, gozr = r.goz, dnxr = r.dx, dnzr = r.dz;
  const int maxrp = nnx * nnz;
  int isx, isz;
  if (asgr == 1) { isx = floor_idx((scx - goxr) / dnxr) + 1; isz = floor_idx((scz - gozr) / dnzr) + 1; }
  else { isx = floor_idx((scx - gox) / dnx) + 1; isz = floor_idx((scz - goz) / dnz) + 1; }
  double dpl = dnx, rd1 = dnz;
  if (rd1 < dpl) dpl = rd1;
  dpl = 0.5 * dpl;
  rx.assign(1, rcx); rz.assign(1, rcz);
  int ipx = floor_idx((rcx - gox) / dnx) + 1;
  int ipz = floor_idx((rcz - goz) / dnz) + 1;
  int sw = 0;
  if (ipx < 1 || ipx >= nnx) sw = 1;
  if (ipz < 1 || ipz >= nnz) sw = 1;
  if (sw == 1) return -1;   // the reference stops the program
  if (ipx == nnx) ipx = ipx - 1;
  if (ipz == nnz) ipz = ipz - 1;
  int nrp = 1;
  double sred = (scx - rx[0]) * (scx - rx[0]);
  sred = sred + (scz - rz[0]) * (scz - rz[0]);
  sred = std::sqrt(sred);
  if (sred < 2.0 * dpl) { rx.push_back(scx); rz.push_back(scz); nrp = 2; sw = 1; }
  int ipxr = 0, ipzr = 0, igref = 0;
  auto in_refined = [&](double px, double pz) {
    ipxr = floor_idx((px - goxr) / dnxr) + 1;
    ipzr = floor_idx((pz - gozr) / dnzr) + 1;
    int g = 1;
    if (ipxr < 1 || ipxr >= nnxr) g = 0;
    if (ipzr < 1 || ipzr >= nnzr) g = 0;
    if (g == 1) {
      if (SR(ipzr, ipxr) != 0 || SR(ipzr + 1, ipxr) != 0) g = 0;
      if (SR(ipzr, ipxr + 1) != 0 || SR(ipzr + 1, ipxr + 1) != 0) g = 0;
    }
    return g;
  };
  if (asgr == 1) igref = in_refined(rcx, rcz);
  if (sw == 0) {
    if (asgr == 1) {
      if (igref == 1 && ipxr == isx && ipzr == isz) { rx.push_back(scx); rz.push_back(scz); nrp = 2; sw = 1; }
    } else {
      if (ipx == isx && ipz == isz) { rx.push_back(scx); rz.push_back(scz); nrp = 2; sw = 1; }
    }
  }
  int crazy = 0;
  for (int j = 1; j <= maxrp; ++j) {
    if (sw == 1) break;
    double dtx, dtz;
    const double px = rx[(size_t)j - 1], pz = rz[(size_t)j - 1];
    if (igref == 1) {
      if (ipxr == 1) dtx = (TR(ipzr, ipxr + 1) - TR(ipzr, ipxr)) / dnxr;
      else if (ipxr == nnxr) dtx = (TR(ipzr, ipxr) - TR(ipzr, ipxr - 1)) / dnxr;
      else dtx = (TR(ipzr, ipxr + 1) - TR(ipzr, ipxr - 1)) / (2.0 * dnxr);
      if (ipzr == 1) dtz = (TR(ipzr + 1, ipxr) - TR(ipzr, ipxr)) / dnzr;
      else if (ipzr == nnzr) dtz = (TR(ipzr, ipxr) - TR(ipzr - 1, ipxr)) / dnzr;
      else dtz = (TR(ipzr + 1, ipxr) - TR(ipzr - 1, ipxr)) / (2.0 * dnzr);
    } else {
      if (ipx == 1) dtx = (T(ipz, ipx + 1) - T(ipz, ipx)) / dnx;
      else if (ipx == nnx) dtx = (T(ipz, ipx) - T(ipz, ipx - 1)) / dnx;
      else dtx = (T(ipz, ipx + 1) - T(ipz, ipx - 1)) / (2.0 * dnx);
      // the reference tests the refined index here (ipzr == nnzr); without
      // refinement those are undefined (an unset local), and the coarse
      // index test the code intends (ipz == nnz) is used
      if (ipz == 1) dtz = (T(ipz + 1, ipx) - T(ipz, ipx)) / dnz;
      else if (asgr == 1 ? ipzr == nnzr : ipz == nnz) dtz = (T(ipz, ipx) - T(ipz - 1, ipx)) / dnz;
      else dtz = (T(ipz + 1, ipx) - T(ipz - 1, ipx)) / (2.0 * dnz);
    }
    rd1 = std::sqrt(dtx * dtx + dtz * dtz);
    double nx = px - dpl * dtx / rd1;
    double nz = pz - dpl * dtz / rd1;
    rx.push_back(nx); rz.push_back(nz);
    if (asgr == 1) {
      igref = in_refined(nx, nz);
      ipx = floor_idx((nx - gox) / dnx) + 1;
      ipz = floor_idx((nz - goz) / dnz) + 1;
    } else {
      ipx = floor_idx((nx - gox) / dnx) + 1;
      ipz = floor_idx((nz - goz) / dnz) + 1;
      igref = 0;
    }
    sred = (scx - nx) * (scx - nx);
    sred = sred + (scz - nz) * (scz - nz);
    sred = std::sqrt(sred);
    sw = 0;
    if (sred < 2.0 * dpl) { rx.push_back(scx); rz.push_back(scz); nrp = j + 2; sw = 1; break; }
    if (asgr == 1) {
      if (igref == 1 && ipxr == isx && ipzr == isz) { rx.push_back(scx); rz.push_back(scz); nrp = j + 2; sw = 1; break; }
    } else {
      if (ipx == isx && ipz == isz) { rx.push_back(scx); rz.push_back(scz); nrp = j + 2; sw = 1; break; }
    }
    if (ipx < 1) { rx.back() = gox; ipx = 1; }
    if (ipx >= nnx) { rx.back() = gox + (double)(nnx - 1) * dnx; ipx = nnx - 1; }
    if (ipz < 1) { rz.back() = goz; ipz = 1; }
    if (ipz >= nnz) { rz.back() = goz + (double)(nnz - 1) * dnz; ipz = nnz - 1; }
    if (j == maxrp - 1 && sw == 0) { crazy = 1; sw = 1; break; }
  }
  rx.resize((size_t)nrp); rz.resize((size_t)nrp);
  return crazy;
}

// What modrays returns with uar = 0 besides the phase times: per path the
// group time along its ray (CalGroupTime on gvel, the model grid
// (nvz, nvx)), the ray length, and the number of crazy rays.
struct RayOut {
  const double *gvel;
  double *gtime, *raylen;
  int crazy;
};

}  // namespace

extern "C" {

// Test hook: record the marching order (stage, node, heap size, time) of one
// source of the next orc_modrays call.
int orc_fm2d_trace(int src, int *idx, double *t, int max) {
  g_trace_src = src; g_trace_i = idx; g_trace_t = t; g_trace_max = max; g_trace_n = 0;
  return 0;
}
int orc_fm2d_trace_count(void) { return g_trace_n; }

// modrays (fm2dray_cartesian.f90:67-480) for uar=1 (no ray paths).
// velvin: (nvz+2, nvx+2) column-major padded vertex grid. srs: (nrc*nsrc)
// path-exists flags, source-major (pn = (i-1)*nrc + j). ttime: (nrc, nsrc)
// column-major, written only where srs==1. tfield (optional, may be NULL):
// (nnz, nnx, nsrc) final coarse travel-time fields.
// Returns 0, or -1 for a source/receiver outside the grid (the reference
// stops the program there).
}  // extern "C"

namespace {
int modrays_impl(int nsrc, const double *scx, const double *scz, int nrc,
                 const double *rcx, const double *rcz, const int *srs, int nvx,
                 int nvz, double goxd, double gozd, double dvxd, double dvzd,
                 const double *velvin, int gdx, int gdz, int asgr, int sgdl,
                 int sgs, int fom, double *ttime, double *tfield, RayOut *ro) {
  // gridder (fm2dray_cartesian.f90:491-600)
  int ldv = nvz + 2;
  auto velv = [&](int i, int j) { return velvin[(size_t)j * ldv + i]; };  // velv(i,j), i=0..nvz+1
  int nnx = (nvx - 1) * gdx + 1, nnz = (nvz - 1) * gdz + 1;
  double dvx = dvxd, dvz = dvzd, gox = goxd, goz = gozd;
  double dnx = dvx / gdx, dnz = dvz / gdz;
  std::vector<double> velc((size_t)nnx * nnz);
  {
    std::vector<double> ui((gdx + 1) * 4), vi((gdz + 1) * 4);
    for (int i = 1; i <= gdx + 1; ++i) {
      double u = gdx; u = (double)(i - 1) / u;
      double om = 1.0 - u;
      ui[(i - 1) * 4 + 0] = om * om * om / 6.0;
      ui[(i - 1) * 4 + 1] = (4.0 - 6.0 * (u * u) + 3.0 * (u * u * u)) / 6.0;
      ui[(i - 1) * 4 + 2] = (1.0 + 3.0 * u + 3.0 * (u * u) - 3.0 * (u * u * u)) / 6.0;
      ui[(i - 1) * 4 + 3] = (u * u * u) / 6.0;
    }
    for (int i = 1; i <= gdz + 1; ++i) {
      double u = gdz; u = (double)(i - 1) / u;
      double om = 1.0 - u;
      vi[(i - 1) * 4 + 0] = om * om * om / 6.0;
      vi[(i - 1) * 4 + 1] = (4.0 - 6.0 * (u * u) + 3.0 * (u * u * u)) / 6.0;
      vi[(i - 1) * 4 + 2] = (1.0 + 3.0 * u + 3.0 * (u * u) - 3.0 * (u * u * u)) / 6.0;
      vi[(i - 1) * 4 + 3] = (u * u * u) / 6.0;
    }
    for (int i = 1; i <= nvz - 1; ++i) {
      int conz = (i == nvz - 1) ? gdz + 1 : gdz;
      for (int j = 1; j <= nvx - 1; ++j) {
        int conx = (j == nvx - 1) ? gdx + 1 : gdx;
        for (int l = 1; l <= conz; ++l) {
          int stz = gdz * (i - 1) + l;
          for (int m = 1; m <= conx; ++m) {
            int stx = gdx * (j - 1) + m;
            double sumi = 0.0;
            for (int i1 = 1; i1 <= 4; ++i1) {
              double sumj = 0.0;
              for (int j1 = 1; j1 <= 4; ++j1)
                sumj = sumj + ui[(m - 1) * 4 + j1 - 1] * velv(i - 2 + i1, j - 2 + j1);
              sumi = sumi + vi[(l - 1) * 4 + i1 - 1] * sumj;
            }
            velc[(size_t)(stx - 1) * nnz + (stz - 1)] = sumi;
          }
        }
      }
    }
  }

  FM2D f;
  f.fom = fom;
  int nrx_max = 2 * sgs * sgdl + 1;
  int ld = std::max(nnz, nrx_max), cols = std::max(nnx, nrx_max);
  f.ld = ld;
  f.veln.assign((size_t)ld * cols, 0.0);
  f.ttn.assign((size_t)ld * cols, 0.0);
  f.nsts.assign((size_t)ld * cols, -1);
  f.btgx.resize(ld * cols + 8); f.btgz.resize(ld * cols + 8);
  auto load_coarse = [&]() {
    f.nnx = nnx; f.nnz = nnz; f.gox = gox; f.goz = goz; f.dnx = dnx; f.dnz = dnz;
    for (int i = 1; i <= nnx; ++i)
      for (int k = 1; k <= nnz; ++k) f.V(k, i) = velc[(size_t)(i - 1) * nnz + (k - 1)];
  };
  load_coarse();

  std::vector<double> ttnr;
  std::vector<int> nstsr;
  G2 rgeom{0, 0, 0, 0, 1, 1};
  if (ro) ro->crazy = 0;
  for (int i = 1; i <= nsrc; ++i) {
    int any = 0;
    for (int j = 0; j < nrc; ++j) any += srs[(size_t)(i - 1) * nrc + j];
    if (any == 0 && i != 1) continue;
    double x = scx[i - 1], z = scz[i - 1];
    g_cur_src = i - 1;
    int isx = (int)((x - gox) / dnx) + 1;
    int isz = (int)((z - goz) / dnz) + 1;
    if (isx < 1 || isx > nnx || isz < 1 || isz > nnz) return -1;
    if (isx == nnx) isx = isx - 1;
    if (isz == nnz) isz = isz - 1;
    f.vnl = std::max(isx - sgs, 1); f.vnr = std::min(isx + sgs, nnx);
    f.vnt = std::max(isz - sgs, 1); f.vnb = std::min(isz + sgs, nnz);
    if (asgr == 1) {
      // refined source grid (fm2dray_cartesian.f90:292-415)
      int nrnx = (f.vnr - f.vnl) * sgdl + 1, nrnz = (f.vnb - f.vnt) * sgdl + 1;
      double drnx = dvx / (double)(gdx * sgdl), drnz = dvz / (double)(gdz * sgdl);
      double gorx = gox + dnx * (double)(f.vnl - 1), gorz = goz + dnz * (double)(f.vnt - 1);
      f.nnx = nrnx; f.nnz = nrnz; f.dnx = drnx; f.dnz = drnz; f.gox = gorx; f.goz = gorz;
      // bsplrefine (fm2dray_cartesian.f90:608-674)
      {
        int nrxr = gdx * sgdl, nrzr = gdz * sgdl;
        std::vector<double> ui((nrxr + 1) * (nrzr + 1) * 4), vi((nrxr + 1) * (nrzr + 1) * 4);
        auto UI = [&](int j, int ii, int q) -> double & { return ui[((size_t)(ii - 1) * (nrxr + 1) + (j - 1)) * 4 + q - 1]; };
        auto VI = [&](int j, int ii, int q) -> double & { return vi[((size_t)(ii - 1) * (nrxr + 1) + (j - 1)) * 4 + q - 1]; };
        for (int ii = 1; ii <= nrzr + 1; ++ii) {
          double v = nrzr; v = (double)(ii - 1) / v;
          for (int j = 1; j <= nrxr + 1; ++j) {
            double u = nrxr; u = (double)(j - 1) / u;
            double om = 1.0 - u, ov = 1.0 - v;
            UI(j, ii, 1) = om * om * om / 6.0;
            UI(j, ii, 2) = (4.0 - 6.0 * (u * u) + 3.0 * (u * u * u)) / 6.0;
            UI(j, ii, 3) = (1.0 + 3.0 * u + 3.0 * (u * u) - 3.0 * (u * u * u)) / 6.0;
            UI(j, ii, 4) = (u * u * u) / 6.0;
            VI(j, ii, 1) = ov * ov * ov / 6.0;
            VI(j, ii, 2) = (4.0 - 6.0 * (v * v) + 3.0 * (v * v * v)) / 6.0;
            VI(j, ii, 3) = (1.0 + 3.0 * v + 3.0 * (v * v) - 3.0 * (v * v * v)) / 6.0;
            VI(j, ii, 4) = (v * v * v) / 6.0;
          }
        }
        int origx = (f.vnl - 1) * sgdl + 1, origz = (f.vnt - 1) * sgdl + 1;
        for (int ii = 1; ii <= nvz - 1; ++ii) {
          int conz = (ii == nvz - 1) ? nrzr + 1 : nrzr;
          for (int j = 1; j <= nvx - 1; ++j) {
            int conx = (j == nvx - 1) ? nrxr + 1 : nrxr;
            for (int k = 1; k <= conz; ++k) {
              int st1 = gdz * (ii - 1) + (k - 1) / sgdl + 1;
              if (st1 < f.vnt || st1 > f.vnb) continue;
              st1 = nrzr * (ii - 1) + k;
              for (int l = 1; l <= conx; ++l) {
                int st2 = gdx * (j - 1) + (l - 1) / sgdl + 1;
                if (st2 < f.vnl || st2 > f.vnr) continue;
                st2 = nrxr * (j - 1) + l;
                double sum[4];
                for (int i1 = 1; i1 <= 4; ++i1) {
                  sum[i1 - 1] = 0.0;
                  for (int j1 = 1; j1 <= 4; ++j1)
                    sum[i1 - 1] = sum[i1 - 1] + UI(l, k, j1) * velv(ii - 2 + i1, j - 2 + j1);
                  sum[i1 - 1] = VI(l, k, i1) * sum[i1 - 1];
                }
                int idm1 = st1 - origz + 1, idm2 = st2 - origx + 1;
                if (idm1 < 1 || idm1 > f.nnz) continue;
                if (idm2 < 1 || idm2 > f.nnx) continue;
                f.V(idm1, idm2) = sum[0] + sum[1] + sum[2] + sum[3];
              }
            }
          }
        }
      }
      if (f.travel(x, z, 1) != 0) return -1;
      // map refined grid onto coarse grid
      ttnr.assign((size_t)nrnz * nrnx, 0.0);
      nstsr.assign((size_t)nrnz * nrnx, -1);
      rgeom = G2{nrnx, nrnz, gorx, gorz, drnx, drnz};
      for (int l = 1; l <= nrnx; ++l)
        for (int k = 1; k <= nrnz; ++k) {
          // far nodes hold uninitialised memory in the reference; 0 here
          nstsr[(size_t)(l - 1) * nrnz + k - 1] = f.S(k, l);
          ttnr[(size_t)(l - 1) * nrnz + k - 1] = f.S(k, l) == -1 ? 0.0 : f.T(k, l);
        }
      std::fill(f.nsts.begin(), f.nsts.end(), -1);
      for (int k = 1; k <= nrnz; k += sgdl) {
        int idm1 = f.vnt + (k - 1) / sgdl;
        for (int l = 1; l <= nrnx; l += sgdl) {
          int idm2 = f.vnl + (l - 1) / sgdl;
          f.S(idm1, idm2) = nstsr[(size_t)(l - 1) * nrnz + k - 1];
          if (f.S(idm1, idm2) >= 0) f.T(idm1, idm2) = ttnr[(size_t)(l - 1) * nrnz + k - 1];
        }
      }
      load_coarse();
      // narrow band repair
      for (int k = 1; k <= nnx; ++k)
        for (int l = 1; l <= nnz; ++l)
          if (f.S(l, k) == 0) {
            if (l - 1 >= 1) { if (f.S(l - 1, k) == -1) f.S(l, k) = 1; }
            if (l + 1 <= nnz) { if (f.S(l + 1, k) == -1) f.S(l, k) = 1; }
            if (k - 1 >= 1) { if (f.S(l, k - 1) == -1) f.S(l, k) = 1; }
            if (k + 1 <= nnx) { if (f.S(l, k + 1) == -1) f.S(l, k) = 1; }
          }
      if (f.travel(x, z, 2) != 0) return -1;
    } else {
      if (f.travel(x, z, 0) != 0) return -1;
    }
    if (tfield) {
      for (int ix = 1; ix <= nnx; ++ix)
        for (int iz = 1; iz <= nnz; ++iz)
          tfield[(size_t)(i - 1) * nnx * nnz + (size_t)(ix - 1) * nnz + iz - 1] = f.T(iz, ix);
    }
    // srtimes (fm2dray_cartesian.f90:682-797)
    for (int r = 1; r <= nrc; ++r) {
      if (srs[(size_t)(i - 1) * nrc + r - 1] == 0) continue;
      int irx = (int)std::floor((rcx[r - 1] - gox) / dnx) + 1;
      int irz = (int)std::floor((rcz[r - 1] - goz) / dnz) + 1;
      int sw = 0;
      if (irx < 1 || irx > nnx || irz < 1 || irz > nnz) return -1;
      if (irx == nnx) irx = irx - 1;
      if (irz == nnz) irz = irz - 1;
      int jsx = (int)std::floor((x - gox) / dnx) + 1;
      int jsz = (int)std::floor((z - goz) / dnz) + 1;
      double dpl = dnx, rd1 = dnz;
      if (rd1 < dpl) dpl = rd1;
      double sred = (x - rcx[r - 1]) * (x - rcx[r - 1]);
      sred = sred + (z - rcz[r - 1]) * (z - rcz[r - 1]);
      sred = std::sqrt(sred);
      if (sred < dpl) sw = 1;
      if (jsx == irx && jsz == irz) sw = 1;
      double trr;
      if (sw == 1) {
        double vss[2][2];
        for (int k = 1; k <= 2; ++k)
          for (int l = 1; l <= 2; ++l) vss[k - 1][l - 1] = f.V(jsz - 1 + l, jsx - 1 + k);
        double drx = (x - gox) - (double)(jsx - 1) * dnx;
        double drz = (z - goz) - (double)(jsz - 1) * dnz;
        double vels = f.bilinear(vss, drx, drz);
        for (int k = 1; k <= 2; ++k)
          for (int l = 1; l <= 2; ++l) vss[k - 1][l - 1] = f.V(irz - 1 + l, irx - 1 + k);
        drx = (rcx[r - 1] - gox) - (double)(irx - 1) * dnx;
        drz = (rcz[r - 1] - goz) - (double)(irz - 1) * dnz;
        double velr = f.bilinear(vss, drx, drz);
        trr = 2.0 * sred / (vels + velr);
      } else {
        double drx = (rcx[r - 1] - gox) - (double)(irx - 1) * dnx;
        double drz = (rcz[r - 1] - goz) - (double)(irz - 1) * dnz;
        trr = 0.0;
        for (int k = 1; k <= 2; ++k)
          for (int l = 1; l <= 2; ++l) {
            double produ = (1.0 - std::fabs(((double)(l - 1) * dnz - drz) / dnz)) *
                           (1.0 - std::fabs(((double)(k - 1) * dnx - drx) / dnx));
            trr = trr + f.T(irz - 1 + l, irx - 1 + k) * produ;
          }
      }
      ttime[(size_t)(i - 1) * nrc + r - 1] = trr;
    }
    if (ro) {
      // rpaths (modrays calls it after srtimes when uar = 0)
      std::vector<double> ttc((size_t)nnx * nnz);
      for (int ix = 1; ix <= nnx; ++ix)
        for (int iz = 1; iz <= nnz; ++iz) ttc[(size_t)(ix - 1) * nnz + iz - 1] = f.T(iz, ix);
      const G2 cg{nnx, nnz, gox, goz, dnx, dnz};
      const G2 mg{nvx, nvz, goxd, gozd, dvxd, dvzd};
      std::vector<double> rx, rz;
      for (int r = 1; r <= nrc; ++r) {
        if (srs[(size_t)(i - 1) * nrc + r - 1] == 0) continue;
        int cz = trace_ray(rcx[r - 1], rcz[r - 1], x, z, cg, ttc.data(), asgr, rgeom, ttnr.data(), nstsr.data(),
                           rx, rz);
        if (cz < 0) return -1;
        ro->crazy += cz;
        double gt, len;
        group_time(rx, rz, ro->gvel, mg, &gt, &len);
        ro->gtime[(size_t)(i - 1) * nrc + r - 1] = gt;
        ro->raylen[(size_t)(i - 1) * nrc + r - 1] = len;
      }
    }
  }
  return 0;
}
}  // namespace

extern "C" {

int orc_modrays(int nsrc, const double *scx, const double *scz, int nrc,
                const double *rcx, const double *rcz, const int *srs, int nvx,
                int nvz, double goxd, double gozd, double dvxd, double dvzd,
                const double *velvin, int gdx, int gdz, int asgr, int sgdl,
                int sgs, int fom, double snb, double *ttime, double *tfield) {
  (void)snb;  // narrow-band capacity only; heap here grows as needed
  return modrays_impl(nsrc, scx, scz, nrc, rcx, rcz, srs, nvx, nvz, goxd, gozd, dvxd, dvzd, velvin, gdx, gdz,
                      asgr, sgdl, sgs, fom, ttime, tfield, nullptr);
}

// modrays with uar = 0 followed by CalGroupTime: ttime as orc_modrays (phase
// times); gvel the model-grid velocity for the group delay ((nvz, nvx)
// column-major); gtime / raylen (nrc, nsrc) the group time and length of
// each path's ray; *crazy the number of rays that hit the point limit.
int orc_modrays_group(int nsrc, const double *scx, const double *scz, int nrc,
                      const double *rcx, const double *rcz, const int *srs, int nvx,
                      int nvz, double goxd, double gozd, double dvxd, double dvzd,
                      const double *velvin, int gdx, int gdz, int asgr, int sgdl,
                      int sgs, int fom, const double *gvel, double *ttime, double *gtime,
                      double *raylen, int *crazy) {
  RayOut ro{gvel, gtime, raylen, 0};
  int rc = modrays_impl(nsrc, scx, scz, nrc, rcx, rcz, srs, nvx, nvz, goxd, gozd, dvxd, dvzd, velvin, gdx, gdz,
                        asgr, sgdl, sgs, fom, ttime, nullptr, &ro);
  *crazy = ro.crazy;
  return rc;
}

// setup_straightRays + CalGroupTime (src/likelihood_surf.F90:412-494) for one
// period: straight rays from each source to each receiver with points every
// min(dx, dy)/2, group delay on vel (model grid (ny, nx) column-major).
// dist (nrev, nsrc) always receives the source-receiver distance; time only
// where raystat == 1 (0 elsewhere). Returns -1 if a ray point leaves the grid
// (the reference's fatal 'Straight ray out of area').
int orc_straight_group(int nsrc, const double *src, int nrev, const double *rev, const int *raystat, int nx,
                       int ny, double xmin, double ymin, double dx, double dy, const double *vel, double *time,
                       double *dist) {
  const G2 g{nx, ny, xmin, ymin, dx, dy};
  const double xmax = xmin + (double)(nx - 1) * dx, ymax = ymin + (double)(ny - 1) * dy;
  const double dl = std::min(dx, dy) / 2;
  std::vector<double> rx, rz;
  for (int j = 1; j <= nsrc; ++j)
    for (int k = 1; k <= nrev; ++k) {
      const int n = k + (j - 1) * nrev;
      const double ddx = rev[2 * (k - 1)] - src[2 * (j - 1)];
      const double ddy = rev[2 * (k - 1) + 1] - src[2 * (j - 1) + 1];
      const double ds = std::sqrt(ddx * ddx + ddy * ddy);
      dist[n - 1] = ds;
      time[n - 1] = 0;
      if (raystat[n - 1] != 1) continue;
      const int npts = (int)std::floor(ds / dl) + 1;
      rx.assign((size_t)npts, 0.0); rz.assign((size_t)npts, 0.0);
      for (int l = 1; l <= npts - 1; ++l) {
        rx[(size_t)l - 1] = src[2 * (j - 1)] + (double)(l - 1) * dl * ddx / ds;
        rz[(size_t)l - 1] = src[2 * (j - 1) + 1] + (double)(l - 1) * dl * ddy / ds;
        if (rx[(size_t)l - 1] < xmin || rx[(size_t)l - 1] > xmax || rz[(size_t)l - 1] < ymin ||
            rz[(size_t)l - 1] > ymax)
          return -1;
      }
      rx[(size_t)npts - 1] = rev[2 * (k - 1)];
      rz[(size_t)npts - 1] = rev[2 * (k - 1) + 1];
      double t, len;
      group_time(rx, rz, vel, g, &t, &len);
      time[n - 1] = t;
    }
  return 0;
}

}  // extern "C"
