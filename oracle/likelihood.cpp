// ORACLE (test infrastructure only): CPU restatement of the reference's
// model checks, column layering and misfit / log-likelihood reductions, used
// as the parity checker for the GPU reduction and layering kernels. Never
// linked into the product.
//
// Parity status: unpinned by reference execution (Fortran); these are short
// sums restated line by line from:
//   check_model       src/likelihood_surf.F90:631-646
//   convert_to_layer  src/likelihood_surf.F90:523-629
//   surf_likelihood   src/likelihood_surf.F90:354-404 (after the forward)
//   surf_noise_likelihood src/likelihood_surf.F90:56-99
//   body_likelihood   src/likelihood_body.F90:176-195,284-333
//   body_noise_likelihood src/likelihood_body.F90:38-80
//   2D body_likelihood mcmc2d/likelihood_dd.F90:455-529 (datatypes 0, 1)
//   2D body_noise_likelihood mcmc2d/likelihood_dd.F90:32-106
//   vs2vp / vp2rho    src/utils.f90:90-135
#include <cmath>
#include <vector>
#include "oracle.h"

namespace {
const double PI2 = (double)6.283185f;  // REAL*8 parameter set from a REAL*4 literal
const double EPS2D = (double)0.000000001f;  // utils/utils.f90:58, a REAL*4 literal

// INTEGER = REAL*8 as the x86 build does it: truncation, -2^31 out of range
int fortran_int(double x) {
  if (!(x > -2147483649.0 && x < 2147483648.0)) return -2147483647 - 1;
  return (int)x;
}
}

extern "C" {

// Returns 1 when some column has a deeper node slower than its top node.
int orc_check_model(const double *vs, int nz, int ny, int nx) {
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j < ny; ++j) {
      const double *col = vs + ((size_t)i * ny + j) * nz;
      for (int k = 1; k < nz; ++k)
        if (col[k] < col[0]) return 1;
    }
  return 0;
}

// One column (vp, vs, rho of length nz) to a layer stack. Returns nlayers.
// thick already divided by scaling (water depth unscaled), no vbnd.
int orc_convert_to_layer(const double *vp, const double *vs, const double *rho,
                         int nz, double dz, double scaling, double water_depth,
                         double *alpha, double *beta, double *rho_k,
                         double *thick) {
  const double EPS = 1.0E-10;
  int nl;
  if (water_depth > EPS) {
    nl = 1; alpha[0] = (double)1.5f; beta[0] = 0; rho_k[0] = 1; thick[0] = water_depth;
  } else {
    nl = 0;
  }
  double last_vp = vp[0], last_vs = vs[0], last_rho = rho[0];
  int last_k = 1;
  for (int k = 2; k <= nz; ++k) {
    if (std::fabs(vs[k - 1] - last_vs) > EPS) {
      nl = nl + 1;
      alpha[nl - 1] = last_vp; beta[nl - 1] = last_vs; rho_k[nl - 1] = last_rho;
      thick[nl - 1] = (double)(k - last_k) * dz;
      last_vp = vp[k - 1]; last_vs = vs[k - 1]; last_rho = rho[k - 1];
      last_k = k;
    }
  }
  nl = nl + 1;
  if (last_k != nz) {
    alpha[nl - 1] = vp[nz - 1]; beta[nl - 1] = vs[nz - 1]; rho_k[nl - 1] = rho[nz - 1];
    thick[nl - 1] = (double)(nz - last_k) * dz;
    thick[nl - 1] = 0;
  } else {
    alpha[nl - 1] = vp[nz - 1]; beta[nl - 1] = vs[nz - 1]; rho_k[nl - 1] = rho[nz - 1];
    thick[nl - 1] = 0;
  }
  for (int i = 0; i < nl; ++i) thick[i] = thick[i] / scaling;
  if (water_depth > 0) thick[0] = water_depth;
  return nl;
}

// Surface-wave misfit (src/likelihood_surf.F90:356-404; with sigdep != 0 and
// srdist = phase_time it is also surf_noise_likelihood, :56-99, whose sigma
// of unused paths is reset to 1 the same way).
// phase_time: (nrev, nsrc, np); dat_ttime: (npairs, 3, np)
// with column 1 the observed time and column 2 the data sigma; raystat:
// (npairs, 2, np); srdist (npairs, np). sigdep != 0: sigma = n0*srdist + n1.
// sigma_out (npairs, np) receives the final sigma. out[0..2] = like, misfit,
// unweighted misfit. Returns -1 if a used sigma is below 1e-10.
int orc_surf_misfit(int nsrc, int nrev, int np, const double *phase_time,
                    const double *dat_ttime, const int *raystat,
                    const double *srdist, int sigdep, const double *n0,
                    const double *n1, int nrays, double *sigma_out,
                    double *out) {
  const double EPS = 1.0E-10;
  const int npairs = nsrc * nrev;
  for (int i = 0; i < np; ++i) {
    for (int r = 0; r < npairs; ++r) {
      double s;
      if (sigdep != 0) {
        s = (raystat[(size_t)i * npairs * 2 + r] == 1)
                ? n0[i] * srdist[(size_t)i * npairs + r] + n1[i] : 1.0;
      } else {
        s = dat_ttime[(size_t)i * npairs * 3 + npairs + r];
      }
      sigma_out[(size_t)i * npairs + r] = s;
    }
  }
  double like = 0, misfit = 0, umisfit = 0;
  int status = 0;
  for (int i = 0; i < np; ++i) {
    int nrr = 0;
    for (int j = 0; j < nsrc; ++j)
      for (int k = 0; k < nrev; ++k) {
        nrr = nrr + 1;
        size_t si = (size_t)i * npairs + nrr - 1;
        if (raystat[(size_t)i * npairs * 2 + nrr - 1] == 1) {
          if (sigma_out[si] < EPS) status = -1;
          double r = phase_time[((size_t)i * nsrc + j) * nrev + k] -
                     dat_ttime[(size_t)i * npairs * 3 + nrr - 1];
          like = like + (r * r) / (2 * (sigma_out[si] * sigma_out[si]));
          misfit = misfit + (r * r) / (sigma_out[si] * sigma_out[si]);
          umisfit = umisfit + r * r;
        } else {
          sigma_out[si] = 1.0;
        }
      }
  }
  double slog = 0;
  for (int i = 0; i < np; ++i)
    for (int r = 0; r < npairs; ++r) slog = slog + std::log(sigma_out[(size_t)i * npairs + r]);
  like = like + slog + (double)((float)nrays / 2.0f) * std::log(PI2);
  out[0] = like; out[1] = misfit; out[2] = umisfit;
  return status;
}

// Location-step read-out (src/likelihood_body.F90:104-111): phase_time(k, j,
// p) = Interpolate3d (:976-1005, point2idx :1038-1054) of field (p, k) at
// event j, fields [np][nrev][nx][ny][nz] (z fastest), events [nsrc][4],
// times [np][nsrc][nrev]; OpenMP over phases and stations.
int orc_location_times(int nx, int ny, int nz, double xmin, double ymin, double zmin, double dx, double dy,
                       double dz, double scaling, int np, int nsrc, int nrev, const double *fields,
                       const double *events, double *times) {
  const size_t nn = (size_t)nx * ny * nz;
#pragma omp parallel for collapse(2) schedule(static)
  for (int p = 0; p < np; ++p)
    for (int k = 0; k < nrev; ++k) {
      const double *f = fields + ((size_t)p * nrev + k) * nn;
      for (int j = 0; j < nsrc; ++j) {
        const double *pt = events + 4 * (size_t)j;
        int ix = (int)std::floor((pt[0] - xmin) / dx) + 1;
        int iy = (int)std::floor((pt[1] - ymin) / dy) + 1;
        int iz = (int)std::floor((pt[2] - zmin / scaling) / (dz / scaling)) + 1;
        if (ix < 1) ix = 1;
        if (iy < 1) iy = 1;
        if (iz < 1) iz = 1;
        if (ix >= nx) ix = nx - 1;
        if (iy >= ny) iy = ny - 1;
        if (iz >= nz) iz = nz - 1;
        const double dsx = pt[0] - (xmin + (ix - 1) * dx);
        const double dsy = pt[1] - (ymin + (iy - 1) * dy);
        const double dsz = pt[2] - (zmin + (iz - 1) * dz) / scaling;
        double qv = 0;
        for (int i = 1; i <= 2; ++i)
          for (int jj = 1; jj <= 2; ++jj)
            for (int kk = 1; kk <= 2; ++kk) {
              const double w = (1.0 - std::fabs((i - 1) * dx - dsx) / dx) * (1.0 - std::fabs((jj - 1) * dy - dsy) / dy) *
                               (1.0 - std::fabs((kk - 1) * dz / scaling - dsz) / (dz / scaling));
              qv = qv + w * f[((size_t)(ix + i - 2) * ny + (iy + jj - 2)) * nz + (iz + kk - 2)];
            }
        times[((size_t)p * nsrc + j) * nrev + k] = qv;
      }
    }
  return 0;
}

// Body-wave misfit (src/likelihood_body.F90:284-333; with sigdep != 0 and
// srdist = phase_time also body_noise_likelihood, :38-80): residual adds the
// event origin time t0[j] (locations(4,j)).
int orc_body_misfit(int nsrc, int nrev, int np, const double *phase_time,
                    const double *t0, const double *dat_ttime,
                    const int *raystat, const double *srdist, int sigdep,
                    const double *n0, const double *n1, int nrays,
                    double *sigma_out, double *out) {
  const double EPS = 2.2250738585072014e-308 * 10;  // tiny(0d0)*10
  const int npairs = nsrc * nrev;
  for (int i = 0; i < np; ++i)
    for (int r = 0; r < npairs; ++r) {
      double s = (sigdep != 0) ? n0[i] * srdist[(size_t)i * npairs + r] + n1[i]
                               : dat_ttime[(size_t)i * npairs * 3 + npairs + r];
      sigma_out[(size_t)i * npairs + r] = s;
    }
  double like = 0, misfit = 0, umisfit = 0;
  int status = 0;
  for (int i = 0; i < np; ++i) {
    int nrr = 0;
    for (int j = 0; j < nsrc; ++j)
      for (int k = 0; k < nrev; ++k) {
        nrr = nrr + 1;
        size_t si = (size_t)i * npairs + nrr - 1;
        if (raystat[(size_t)i * npairs * 2 + nrr - 1] == 1) {
          if (sigma_out[si] < EPS) status = -1;
          double r = phase_time[((size_t)i * nsrc + j) * nrev + k] + t0[j] -
                     dat_ttime[(size_t)i * npairs * 3 + nrr - 1];
          like = like + (r * r) / (2 * (sigma_out[si] * sigma_out[si]));
          misfit = misfit + (r * r) / (sigma_out[si] * sigma_out[si]);
          umisfit = umisfit + r * r;
        } else {
          sigma_out[si] = 1.0;
        }
      }
  }
  double slog = 0;
  for (int i = 0; i < np; ++i)
    for (int r = 0; r < npairs; ++r) slog = slog + std::log(sigma_out[(size_t)i * npairs + r]);
  like = like + slog + (double)((float)nrays / 2.0f) * std::log(PI2);
  out[0] = like; out[1] = misfit; out[2] = umisfit;
  return status;
}

// src/utils.f90:98-135 vs2vp_3d / vp2rho_3d: vp = vs*1.730, rho = 1.74*vp**0.25
// (both constants are REAL*4 literals widened to double).
// 2D body_likelihood after modrays (mcmc2d/likelihood_dd.F90:455-529).
// phase_time [nsrc][nrev] = phaseTime(k,j,1); dat_ttime, dat_sigma,
// raystat per pair nrr = k + (j-1)*nrev; dtime, dcc (nrev, ndd)
// column-major = dat%dtime(:,:,1), dat%dcc(:,:,1); n0, n1 [2] = snoise0/1
// (travel times, differential times). out = like, misfit, unweighted.
// Returns 8 where the reference raises 'The noise level is 0!'.
int orc_tt2d_misfit(int nsrc, int nrev, const double *phase_time, const double *dat_ttime, const double *dat_sigma,
                    const int *raystat, int sigdep, int datatype, const double *dtime, const double *dcc, int ndtime,
                    const double *n0, const double *n1, int nrays, double *out) {
  const int npairs = nsrc * nrev;
  std::vector<double> sigma(npairs);
  for (int q = 0; q < npairs; ++q) sigma[q] = sigdep != 0 ? n0[0] * phase_time[q] + n1[0] : dat_sigma[q];
  const int ndd = nsrc * (nsrc - 1) / 2;
  std::vector<double> dtm, dsig;
  if (datatype == 1) {
    dtm.resize((size_t)ndd * nrev); dsig.resize((size_t)ndd * nrev);
    int dd = 0;
    for (int i = 0; i < nsrc; ++i)
      for (int j = i + 1; j < nsrc; ++j, ++dd)
        for (int k = 0; k < nrev; ++k) {
          dtm[(size_t)dd * nrev + k] = phase_time[(size_t)j * nrev + k] - phase_time[(size_t)i * nrev + k];
          dsig[(size_t)dd * nrev + k] = n0[1] * (1 - dcc[(size_t)dd * nrev + k]) + n1[1];
        }
  }
  int status = 0;
  double like = 0, misfit = 0, umis = 0;
  int nrr = 0;
  for (int j = 0; j < nsrc; ++j)
    for (int k = 0; k < nrev; ++k, ++nrr) {
      if (raystat[nrr] == 1) {
        if (sigma[nrr] == 0) status = 8;
        const double r = phase_time[(size_t)j * nrev + k] - dat_ttime[nrr];
        like = like + (r * r) / (2 * (sigma[nrr] * sigma[nrr]));
        misfit = misfit + (r * r) / (sigma[nrr] * sigma[nrr]);
        umis = umis + r * r;
      } else {
        sigma[nrr] = 1.0;
      }
    }
  double slog = 0;
  for (int q = 0; q < npairs; ++q) slog = slog + std::log(sigma[q]);
  like = like + slog + (double)((float)nrays / 2.0f) * std::log(PI2);
  if (datatype == 1) {
    double sumdsigma = 0;
    int dd = 0;
    for (int i = 0; i < nsrc; ++i)
      for (int j = i + 1; j < nsrc; ++j, ++dd)
        for (int k = 0; k < nrev; ++k) {
          // dat%dtime(ddindex,k,1): indices swapped, column-major element
          if (std::fabs(dtime[(size_t)dd + (size_t)k * nrev]) > EPS2D) {
            const double r = dtm[(size_t)dd * nrev + k] - dtime[(size_t)dd * nrev + k];
            const double s2 = dsig[(size_t)dd * nrev + k];
            like = like + (r * r) / (2 * (s2 * s2));
            misfit = misfit + (r * r) / (s2 * s2);
            umis = umis + r * r;
            sumdsigma = sumdsigma + std::log(s2);
          }
        }
    like = like + sumdsigma + (double)((float)ndtime / 2.0f) * std::log(PI2);
  }
  out[0] = like; out[1] = misfit; out[2] = umis;
  return status;
}

// 2D body_noise_likelihood (mcmc2d/likelihood_dd.F90:32-106) on given
// times: sigma = n0 * srdist + n1; the differential sigma log-sum is an
// INTEGER there. out = like, misfit (the unweighted misfit is untouched).
int orc_tt2d_noise(int nsrc, int nrev, const double *phase_time, const double *dat_ttime, const int *raystat,
                   const double *srdist, int datatype, const double *dtime, const double *dcc, int ndtime,
                   const double *n0, const double *n1, int nrays, double *out) {
  const int npairs = nsrc * nrev;
  std::vector<double> sigma(npairs);
  for (int q = 0; q < npairs; ++q) sigma[q] = n0[0] * srdist[q] + n1[0];
  int status = 0;
  double like = 0, misfit = 0;
  int nrr = 0;
  for (int j = 0; j < nsrc; ++j)
    for (int k = 0; k < nrev; ++k, ++nrr) {
      if (raystat[nrr] == 1) {
        if (sigma[nrr] == 0) status = 8;
        const double r = phase_time[(size_t)j * nrev + k] - dat_ttime[nrr];
        like = like + (r * r) / (2 * (sigma[nrr] * sigma[nrr]));
        misfit = misfit + (r * r) / (sigma[nrr] * sigma[nrr]);
      } else {
        sigma[nrr] = 1.0;
      }
    }
  for (int q = 0; q < npairs; ++q)
    if (sigma[q] < EPS2D) status = 8;
  double slog = 0;
  for (int q = 0; q < npairs; ++q) slog = slog + std::log(sigma[q]);
  like = like + slog + (double)((float)nrays / 2.0f) * std::log(PI2);
  if (datatype == 1) {
    int sumdsigma = 0;
    int dd = 0;
    for (int i = 0; i < nsrc; ++i)
      for (int j = i + 1; j < nsrc; ++j, ++dd)
        for (int k = 0; k < nrev; ++k) {
          if (std::fabs(dtime[(size_t)dd + (size_t)k * nrev]) > EPS2D) {
            const double dtm = phase_time[(size_t)j * nrev + k] - phase_time[(size_t)i * nrev + k];
            const double s2 = n0[1] * (1 - dcc[(size_t)dd * nrev + k]) + n1[1];
            const double r = dtm - dtime[(size_t)dd * nrev + k];
            like = like + (r * r) / (2 * (s2 * s2));
            misfit = misfit + (r * r) / (s2 * s2);
            sumdsigma = fortran_int((double)sumdsigma + std::log(s2));
          }
        }
    like = like + (double)sumdsigma + (double)((float)ndtime / 2.0f) * std::log(PI2);
  }
  out[0] = like; out[1] = misfit;
  return status;
}

double orc_vs2vp(double vs) { return vs * (double)1.730f; }
double orc_vp2rho(double vp) { return (double)1.74f * std::pow(vp, 0.25); }

}  // extern "C"
