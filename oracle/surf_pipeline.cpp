// ORACLE (test infrastructure only): the reference's surface-wave likelihood
// path composed from the restatements in this directory, as the sampler runs
// it for one proposal: kdtree_to_grid (src/mcmc_loc2.f90:2002-2082), the
// material laws (src/likelihood.f90:75-76), check_model, convert_to_layer,
// surfmodes -> surfdisp96 per column, padded phase maps, modrays per period
// and the misfit (src/likelihood_surf.F90:110-410). OpenMP over columns and
// over periods follows the reference's parallel loops
// (likelihood_surf.F90:197-206,295-334). It is the parity checker for the
// batched GPU pipeline and the timed CPU baseline. Never linked into the
// product.
#include <cmath>
#include <cfloat>
#include <vector>
#include <cstring>
#include "oracle.h"

extern "C" {

// grid: nx,ny,nz (int), dbl: xmin,ymin,zmin,dx,dy,dz,scaling,water_depth.
// iset: raylov, gridx, gridy, sgref, sgdic, sgext, order, sigdep, law.
// points/params: [n][3]. freqs[np]; src/rev [nsrc][2]/[nrev][2];
// raystat/ttime/sigma: [np][nsrc*nrev]. n0/n1[np].
// col_mask (optional, [nx*ny]): columns to recompute; the others take their
// phase velocities from pvel_io. pvel_io ([np][nx][ny]) always receives the
// proposal's phase maps. phase_time (optional): [np][nsrc][nrev].
// out[4] = like, misfit, unweighted misfit, status (bit 1 check_model, bit 2
// dispersion failure).
// phase_group 1: group velocities (surfdisp96 with igr = 1), travel times
// along the rays of the phase field (modrays uar = 0 + CalGroupTime,
// likelihood_surf.F90:286-345), srdist = ray length, gvel_io ([np][nx][ny])
// as pvel_io for the group maps; a crazy ray sets status bit 4. straight 1:
// straight rays (setup_straightRays + CalGroupTime on the group maps, or the
// phase maps for phase_group 0, likelihood_surf.F90:233-242), srdist = the
// source-receiver distance; no fast marching. srdist_out (optional):
// [np][nsrc][nrev].
int orc_surf_likelihood_ex(const int *gi, const double *gd, const int *iset, double dphase,
                           double rho_value, int n, const double *points, const double *params,
                           int np, const double *freqs, int nsrc, const double *src, int nrev,
                           const double *rev, const int *raystat, const double *ttime,
                           const double *sigma, int nrays, const double *n0, const double *n1,
                           const int *col_mask, int phase_group, int straight, double *pvel_io,
                           double *gvel_io, double *phase_time, double *srdist_out, double *out) {
  const int nx = gi[0], ny = gi[1], nz = gi[2];
  const double xmin = gd[0], ymin = gd[1], zmin = gd[2], dx = gd[3], dy = gd[4], dz = gd[5];
  const double scaling = gd[6], water = gd[7];
  const int raylov = iset[0], gridx = iset[1], gridy = iset[2], sgref = iset[3], sgdic = iset[4];
  const int sgext = iset[5], order = iset[6], sigdep = iset[7], law = iset[8];
  const size_t nodes = (size_t)nx * ny * nz, ncol = (size_t)nx * ny;
  const int npairs = nsrc * nrev;
  // material laws per nucleus
  std::vector<double> par((size_t)n * 3);
  for (int i = 0; i < n; ++i) {
    double vs = params[3 * i + 1], vp, rho;
    if (law == 0) { vp = params[3 * i]; rho = params[3 * i + 2]; }
    else { vp = orc_vs2vp(vs); rho = law == 1 ? orc_vp2rho(vp) : rho_value; }
    par[3 * i] = vp; par[3 * i + 1] = vs; par[3 * i + 2] = rho;
  }
  std::vector<int> sid(nodes);
  std::vector<double> vp(nodes), vs(nodes), rho(nodes);
  orc_kdtree_to_grid(3, n, points, par.data(), nx, ny, nz, xmin, ymin, zmin, dx, dy, dz, 1, nx, 1, ny, 1,
                     nz, sid.data(), vp.data(), vs.data(), rho.data());
  int status = 0;
  if (orc_check_model(vs.data(), nz, ny, nx)) status |= 1;
  std::vector<double> per(np);
  for (int p = 0; p < np; ++p) per[p] = 1.0 / freqs[p];
  int bad = 0;
#pragma omp parallel for schedule(dynamic, 4) reduction(| : bad)
  for (long col = 0; col < (long)ncol; ++col) {
    if (col_mask && !col_mask[col]) continue;
    const size_t o = (size_t)col * nz;
    double a[256], b[256], r[256], t[256];
    int nl = orc_convert_to_layer(vp.data() + o, vs.data() + o, rho.data() + o, nz, dz, scaling, water, a, b,
                                  r, t);
    float t4[256], a4[256], b4[256], r4[256];
    for (int i = 0; i < nl; ++i) { t4[i] = (float)t[i]; a4[i] = (float)a[i]; b4[i] = (float)b[i]; r4[i] = (float)r[i]; }
    double cp[60], cg[60];
    int ierr = orc_surfdisp96(t4, a4, b4, r4, nl, raylov == 1 ? 2 : 1, 1, phase_group, np, per.data(), dphase,
                              cp, cg, nullptr);
    if (ierr) bad = 1;
    for (int p = 0; p < np; ++p) pvel_io[(size_t)p * ncol + col] = cp[p];
    if (phase_group)
      for (int p = 0; p < np; ++p) gvel_io[(size_t)p * ncol + col] = cg[p];
  }
  if (bad) status |= 2;
  // padded maps and modrays per period
  std::vector<double> pt((size_t)np * npairs, 0.0), srd((size_t)np * npairs, 0.0);
  const int nvx = nx + 2, nvz = ny + 2;
  std::vector<double> sx(nsrc), sz(nsrc), rx(nrev), rz(nrev);
  for (int i = 0; i < nsrc; ++i) { sx[i] = src[2 * i]; sz[i] = src[2 * i + 1]; }
  for (int i = 0; i < nrev; ++i) { rx[i] = rev[2 * i]; rz[i] = rev[2 * i + 1]; }
  int fmerr = 0, crazy = 0;
  if (straight) {
    for (int p = 0; p < np; ++p) {
      const double *vel = (phase_group ? gvel_io : pvel_io) + (size_t)p * ncol;
      if (orc_straight_group(nsrc, src, nrev, rev, raystat + (size_t)p * npairs, nx, ny, xmin, ymin, dx, dy, vel,
                             pt.data() + (size_t)p * npairs, srd.data() + (size_t)p * npairs))
        fmerr = 1;
    }
  }
#pragma omp parallel for schedule(dynamic, 1) reduction(| : fmerr) reduction(+ : crazy)
  for (int p = 0; p < (straight ? 0 : np); ++p) {
    std::vector<double> velv((size_t)nvx * nvz);
    for (int ii = 0; ii < nvx; ++ii)
      for (int jj = 0; jj < nvz; ++jj) {
        int j = std::min(std::max(jj, 1), ny) - 1, i = std::min(std::max(ii, 1), nx) - 1;
        velv[(size_t)ii * nvz + jj] = pvel_io[(size_t)p * ncol + (size_t)i * ny + j];
      }
    std::vector<int> srs(npairs);
    for (int q = 0; q < npairs; ++q) srs[q] = raystat[(size_t)p * npairs + q] == 1;
    int rc;
    if (phase_group) {
      std::vector<double> tph(npairs);
      int cz = 0;
      rc = orc_modrays_group(nsrc, sx.data(), sz.data(), nrev, rx.data(), rz.data(), srs.data(), nx, ny, xmin,
                             ymin, dx, dy, velv.data(), gridx, gridy, sgref, sgdic, sgext, order,
                             gvel_io + (size_t)p * ncol, tph.data(), pt.data() + (size_t)p * npairs,
                             srd.data() + (size_t)p * npairs, &cz);
      crazy += cz;
    } else {
      rc = orc_modrays(nsrc, sx.data(), sz.data(), nrev, rx.data(), rz.data(), srs.data(), nx, ny, xmin, ymin,
                       dx, dy, velv.data(), gridx, gridy, sgref, sgdic, sgext, order, 0.5,
                       pt.data() + (size_t)p * npairs, nullptr);
      for (int q = 0; q < npairs; ++q) srd[(size_t)p * npairs + q] = pt[(size_t)p * npairs + q];
    }
    if (rc) fmerr = 1;
  }
  if (fmerr) return -1;
  if (crazy) status |= 4;
  if (srdist_out) std::memcpy(srdist_out, srd.data(), sizeof(double) * srd.size());
  if (phase_time) std::memcpy(phase_time, pt.data(), sizeof(double) * pt.size());
  // misfit with sigma = n0*srdist + n1, srdist = phaseTime (phaseGroup = 0)
  std::vector<double> dtt((size_t)np * npairs * 3), sig((size_t)np * npairs);
  std::vector<int> rs((size_t)np * npairs * 2, 0);
  for (int p = 0; p < np; ++p)
    for (int q = 0; q < npairs; ++q) {
      dtt[(size_t)p * npairs * 3 + q] = ttime[(size_t)p * npairs + q];
      dtt[(size_t)p * npairs * 3 + npairs + q] = sigma ? sigma[(size_t)p * npairs + q] : 1.0;
      rs[(size_t)p * npairs * 2 + q] = raystat[(size_t)p * npairs + q];
    }
  double o3[3];
  int st = orc_surf_misfit(nsrc, nrev, np, pt.data(), dtt.data(), rs.data(), srd.data(), sigdep, n0, n1, nrays,
                           sig.data(), o3);
  if (st) status |= 8;
  out[0] = status ? DBL_MAX : o3[0];
  out[1] = o3[1]; out[2] = o3[2]; out[3] = status;
  return 0;
}

int orc_surf_likelihood(const int *gi, const double *gd, const int *iset, double dphase,
                        double rho_value, int n, const double *points, const double *params,
                        int np, const double *freqs, int nsrc, const double *src, int nrev,
                        const double *rev, const int *raystat, const double *ttime,
                        const double *sigma, int nrays, const double *n0, const double *n1,
                        const int *col_mask, double *pvel_io, double *phase_time, double *out) {
  return orc_surf_likelihood_ex(gi, gd, iset, dphase, rho_value, n, points, params, np, freqs, nsrc, src, nrev,
                                rev, raystat, ttime, sigma, nrays, n0, n1, col_mask, 0, 0, pvel_io, nullptr,
                                phase_time, nullptr, out);
}

}  // extern "C"
