// Host side of the reversible-jump sampler: the reference's random number
// stream (src/mt19937.f90) and its Metropolis-Hastings proposal steps and
// acceptance test (src/mcmc_loc2.f90), so that a C or Fortran host can drive
// the GPU likelihood with the reference's own sequence of random draws and
// moves. Host code only (no kernels).
//
// MT19937 (M. Matsumoto and T. Nishimura, "Mersenne Twister: a
// 623-dimensionally equidistributed uniform pseudo-random number generator",
// ACM TOMACS 8(1), 1998) seeded by init_genrand's recursion
// (src/mt19937.f90:96-115), with the reference's real conversion
// grnd = u / (2^32 - 1) of the 32-bit output u (:117-172), unirand = grnd
// (:224-236) and gasdev, the polar Box-Muller method on two grnd draws
// (:200-222). Each generator counts its draws as RTI%randcount does.
#include "mct_common.cuh"
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <new>
#include <utility>

struct mct_rng {
  unsigned mt[624];
  int mti;
  long long count;   // draws so far (RTI%randcount)
};

namespace {

constexpr int kN = 624, kM = 397;
constexpr unsigned kMatrixA = 0x9908B0DFu, kUpper = 0x80000000u, kLower = 0x7FFFFFFFu;

void init_genrand(mct_rng *r, unsigned seed) {
  r->mt[0] = seed;
  for (int i = 1; i < kN; ++i) {
    const unsigned prev = r->mt[i - 1];
    r->mt[i] = 1812433253u * (prev ^ (prev >> 30)) + (unsigned)i;
  }
  r->mti = kN;
}

unsigned next_u32(mct_rng *r) {
  if (r->mti >= kN) {
    for (int k = 0; k < kN; ++k) {
      const unsigned y = (r->mt[k] & kUpper) | (r->mt[(k + 1) % kN] & kLower);
      r->mt[k] = r->mt[(k + kM) % kN] ^ (y >> 1) ^ ((y & 1u) ? kMatrixA : 0u);
    }
    r->mti = 0;
  }
  unsigned y = r->mt[r->mti++];
  y ^= y >> 11;
  y ^= (y << 7) & 0x9D2C5680u;
  y ^= (y << 15) & 0xEFC60000u;
  y ^= y >> 18;
  return y;
}

// grnd: the unsigned 32-bit output over 2^32 - 1, in double
double grnd(mct_rng *r) { return (double)next_u32(r) / (4294967296.0 - 1.0); }

}  // namespace

extern "C" {

int mct_rng_create(unsigned seed, mct_rng **out) {
  if (!out) return MCT_ERR_ARG;
  mct_rng *r = new (std::nothrow) mct_rng;
  if (!r) return MCT_ERR_NOMEM;
  init_genrand(r, seed);
  r->count = 0;
  *out = r;
  return MCT_OK;
}

void mct_rng_destroy(mct_rng *r) { delete r; }

int mct_rng_seed(mct_rng *r, unsigned seed) {
  if (!r) return MCT_ERR_ARG;
  init_genrand(r, seed);
  r->count = 0;
  return MCT_OK;
}

double mct_rng_unirand(mct_rng *r) {
  const double v = grnd(r);
  ++r->count;
  return v;
}

double mct_rng_gasdev(mct_rng *r) {
  for (;;) {
    const double v1 = 2 * grnd(r) - 1;
    ++r->count;
    const double v2 = 2 * grnd(r) - 1;
    ++r->count;
    const double rr = v1 * v1 + v2 * v2;
    if (rr >= 1 || rr == 0) continue;
    const double fac = std::sqrt(-2 * std::log(rr) / rr);
    return v2 * fac;
  }
}

unsigned mct_rng_u32(mct_rng *r) {
  ++r->count;
  return next_u32(r);
}

long long mct_rng_count(const mct_rng *r) { return r ? r->count : -1; }

}  // extern "C"

// ---------------------------------------------------------------------------
// Proposal steps of the reference's MCMC loop (src/mcmc_loc2.f90:72-687).
// The Voronoi model is held as RTI%points / RTI%parameters are; the CGAL
// triangulation the reference keeps beside them only serves to find the cell
// containing a point (cgal_delaunay_locate) and the box of grid nodes to
// recompute. Here the cell containing a point is its nearest nucleus (the
// first in index order on an exact tie), and the likelihood finds the
// changed grid columns itself.
// ---------------------------------------------------------------------------
namespace {

// REAL*4 literals of the reference, widened to REAL*8 as its expressions do
const double kPii = (double)3.1415926f;      // mcmc_loc2.f90:49 PII
const double kPoisson = (double)1.730f;      // utils.f90:95 vs2vp
const double kRho0 = (double)2.35f, kRho1 = (double)0.036f;   // utils.f90:120 vp2rho (crust)
const double kVpVs = (double)1.1f;           // the vp >= 1.1 vs test

double vs2vp(double vs) { return vs * kPoisson; }
double vp2rho(double vp) { return kRho0 + kRho1 * ((vp - 3) * (vp - 3)); }

// Fortran CEILING of a non-negative double, as an index (1-based); 0 -> 1
int pick_index(double u, long long n) {
  int i = (int)std::ceil(u * (double)n);
  return i == 0 ? 1 : i;
}

int nearest_cell(const mct_mcmc_state *st, double x, double y, double z) {
  int best = 0;
  double bd = 0;
  for (int i = 0; i < st->ncells; ++i) {
    const double *p = st->points + 3 * (size_t)i;
    const double dx = p[0] - x, dy = p[1] - y, dz = p[2] - z;
    const double d = dx * dx + dy * dy + dz * dz;
    if (i == 0 || d < bd) { bd = d; best = i; }
  }
  return best;
}

// proposeType2 (mcmc_loc2.f90:1384-1432) and proposeSigmaType (:1499-1519);
// the joint datatype's choice between the two noise types draws from the
// Fortran intrinsic random_number, which is not the chain's stream and is
// not reproducible, so it is taken from the chain's stream here.
int propose_type(const mct_mcmc_set *set, double propose, int iter, mct_rng *r) {
  auto sigma_type = [&]() {
    if (set->datatype == 0 || set->datatype == 1) return 5;
    if (set->datatype == 2) return 6;
    return mct_rng_unirand(r) < 0.1 ? 5 : 6;
  };
  if (iter % 2 == 0) {
    if (propose < (double)0.333f) return 1;
    if (propose < (double)0.666f) return 2;
    return 3;
  }
  if (set->sigdep != 0 && set->locate != 0) {
    if (propose < (double)0.300f) return 4;
    if (propose < (double)0.8f) return 7;
    return sigma_type();
  }
  if (set->sigdep != 0) return propose < (double)0.800f ? 4 : sigma_type();
  if (set->locate != 0) return propose < (double)0.500f ? 4 : 7;
  return 4;
}

bool in_prior(const mct_mcmc_set *set, double vp, double vs) {
  return !(vs < set->vsmin || vs > set->vsmax || vp < set->vpmin || vp > set->vpmax || vp < kVpVs * vs);
}

// cell_birth (mcmc_loc2.f90:1521-1613)
bool cell_birth(const mct_mcmc_set *set, mct_rng *r, mct_mcmc_state *st, double *prob) {
  *prob = 0;
  if (st->ncells == set->ncell_max) return false;
  const double x = set->xmin + mct_rng_unirand(r) * (set->xmax - set->xmin);
  const double y = set->ymin + mct_rng_unirand(r) * (set->ymax - set->ymin);
  const double z = set->zmin + mct_rng_unirand(r) * (set->zmax - set->zmin);
  double vp, vs, rho;
  if (set->kernel == 0) {
    const double *pm = st->parameters + 3 * (size_t)nearest_cell(st, x, y, z);
    vs = pm[1] + mct_rng_gasdev(r) * set->sigma_vs2;
    vp = pm[0] + mct_rng_gasdev(r) * set->sigma_vp2;
    rho = vp2rho(vp);
    const double gp = std::log(set->sigma_vp2 * std::sqrt(2 * kPii)) +
                      (vp - pm[0]) * (vp - pm[0]) / (2 * (set->sigma_vp2 * set->sigma_vp2));
    const double gs = std::log(set->sigma_vs2 * std::sqrt(2 * kPii)) +
                      (vs - pm[1]) * (vs - pm[1]) / (2 * (set->sigma_vs2 * set->sigma_vs2));
    *prob = set->datatype == 0 ? gp : (set->datatype == 2 ? gs : gp + gs);
  } else {
    vs = set->vsmin + mct_rng_unirand(r) * (set->vsmax - set->vsmin);
    vp = set->vpmin + mct_rng_unirand(r) * (set->vpmax - set->vpmin);
    if (set->datatype == 2) vp = vs2vp(vs);
    rho = vp2rho(vp);
  }
  if (!in_prior(set, vp, vs)) { *prob = 0; return false; }
  double *p = st->points + 3 * (size_t)st->ncells, *q = st->parameters + 3 * (size_t)st->ncells;
  p[0] = x; p[1] = y; p[2] = z;
  q[0] = vp; q[1] = vs; q[2] = rho;
  st->ncells += 1;
  return true;
}

// cell_death (mcmc_loc2.f90:1615-1683)
bool cell_death(const mct_mcmc_set *set, mct_rng *r, mct_mcmc_state *st, int *iremove, double *prob) {
  *prob = 0;
  if (st->ncells == set->ncell_min) return false;
  const int ir = pick_index(mct_rng_unirand(r), st->ncells);
  *iremove = ir;
  const double pt[3] = {st->points[3 * (size_t)(ir - 1)], st->points[3 * (size_t)(ir - 1) + 1],
                        st->points[3 * (size_t)(ir - 1) + 2]};
  const double pm1[3] = {st->parameters[3 * (size_t)(ir - 1)], st->parameters[3 * (size_t)(ir - 1) + 1],
                         st->parameters[3 * (size_t)(ir - 1) + 2]};
  for (int i = ir; i < st->ncells; ++i)
    for (int k = 0; k < 3; ++k) {
      st->points[3 * (size_t)(i - 1) + k] = st->points[3 * (size_t)i + k];
      st->parameters[3 * (size_t)(i - 1) + k] = st->parameters[3 * (size_t)i + k];
    }
  st->ncells -= 1;
  if (set->kernel == 0) {
    const double *pm2 = st->parameters + 3 * (size_t)nearest_cell(st, pt[0], pt[1], pt[2]);
    const double gp = std::log(1 / (set->sigma_vp2 * std::sqrt(2 * kPii))) -
                      (pm2[0] - pm1[0]) * (pm2[0] - pm1[0]) / (2 * (set->sigma_vp2 * set->sigma_vp2));
    const double gs = std::log(1 / (set->sigma_vs2 * std::sqrt(2 * kPii))) -
                      (pm2[1] - pm1[1]) * (pm2[1] - pm1[1]) / (2 * (set->sigma_vs2 * set->sigma_vs2));
    *prob = set->datatype == 0 ? gp : (set->datatype == 2 ? gs : gp + gs);
  }
  return true;
}

// cell_move (mcmc_loc2.f90:1685-1765): one coordinate moves; nuclei in the
// deeper half of the grid use pd2 (both draws are taken there, as the
// reference's code does)
bool cell_move(const mct_mcmc_set *set, mct_rng *r, mct_mcmc_state *st, int *imove) {
  const int im = pick_index(mct_rng_unirand(r), st->ncells);
  *imove = im;
  double *p = st->points + 3 * (size_t)(im - 1);
  double dst[3] = {p[0], p[1], p[2]};
  const double propose = mct_rng_unirand(r);
  const bool deep = p[2] > (set->zmin + set->zmax) / 2;
  const int axis = propose < (double)0.333f ? 0 : (propose < (double)0.666f ? 1 : 2);
  const double ext = axis == 0 ? set->xmax - set->xmin : (axis == 1 ? set->ymax - set->ymin : set->zmax - set->zmin);
  dst[axis] = p[axis] + mct_rng_gasdev(r) * set->pd * ext / 100;
  if (deep) dst[axis] = p[axis] + mct_rng_gasdev(r) * set->pd2 * ext / 100;
  if (dst[0] < set->xmin || dst[0] > set->xmax || dst[1] < set->ymin || dst[1] > set->ymax || dst[2] < set->zmin ||
      dst[2] > set->zmax)
    return false;
  p[0] = dst[0]; p[1] = dst[1]; p[2] = dst[2];
  return true;
}

// vel_change (mcmc_loc2.f90:1767-1835). The reference's one-line IF guards
// only the vs redraw for deep nuclei; the vp redraw with sigma_vp2 that
// follows it runs always, so three or four draws are taken.
bool vel_change(const mct_mcmc_set *set, mct_rng *r, mct_mcmc_state *st, int *ivalue) {
  const int iv = pick_index(mct_rng_unirand(r), st->ncells);
  *ivalue = iv;
  double *q = st->parameters + 3 * (size_t)(iv - 1);
  const bool deep = st->points[3 * (size_t)(iv - 1) + 2] > (set->zmin + set->zmax) / 2;
  double vs = q[1] + mct_rng_gasdev(r) * set->sigma_vs;
  double vp = q[0] + mct_rng_gasdev(r) * set->sigma_vp;
  if (deep) vs = q[1] + mct_rng_gasdev(r) * set->sigma_vs2;
  vp = q[0] + mct_rng_gasdev(r) * set->sigma_vp2;
  if (set->datatype == 2) vp = vs2vp(vs);
  const double rho = vp2rho(vp);
  if (vs < set->vsmin || vs > set->vsmax || vp < set->vpmin || vp > set->vpmax || vp < vs * kVpVs) return false;
  q[0] = vp; q[1] = vs; q[2] = rho;
  return true;
}

// bsigma_change / ssigma_change (mcmc_loc2.f90:1837-1903)
bool sigma_change(mct_rng *r, int np, double *n0, double *n1, double sig0, double sig1, double n0min, double n0max,
                  double n1min, double n1max, int *iperiod) {
  if (np < 1) return false;
  const int ip = pick_index(mct_rng_unirand(r), np);
  *iperiod = ip;
  if (mct_rng_unirand(r) < 0.5) n0[ip - 1] = n0[ip - 1] + mct_rng_gasdev(r) * sig0;
  else n1[ip - 1] = n1[ip - 1] + mct_rng_gasdev(r) * sig1;
  return !(n0[ip - 1] < n0min || n0[ip - 1] > n0max || n1[ip - 1] < n1min || n1[ip - 1] > n1max);
}

}  // namespace

extern "C" {

int mct_mcmc_propose(const mct_mcmc_set *set, mct_rng *rng, int iter, int redo, mct_mcmc_state *st,
                     mct_mcmc_step *step) {
  if (!set || !rng || !st || !step || !st->points || !st->parameters || st->ncells < 1 ||
      st->ncells > set->ncell_max)
    return MCT_ERR_ARG;
  // a new proposal draws the acceptance number and the type; a redo (the
  // previous proposal gave an invalid model) keeps both
  // (mcmc_loc2.f90:200-205)
  if (!redo) {
    step->random = mct_rng_unirand(rng);
    const double propose = mct_rng_unirand(rng);
    step->ptype = propose_type(set, propose, iter, rng);
  }
  step->index = 0;
  step->prob = 0;
  bool ok = false;
  switch (step->ptype) {
    case 1: ok = cell_birth(set, rng, st, &step->prob); step->index = st->ncells; break;
    case 2: ok = cell_death(set, rng, st, &step->index, &step->prob); break;
    case 3: ok = cell_move(set, rng, st, &step->index); break;
    case 4: ok = vel_change(set, rng, st, &step->index); break;
    case 5:
      ok = sigma_change(rng, st->nbnoise, st->bnoise0, st->bnoise1, set->sigma_bn0, set->sigma_bn1, set->bn0_min,
                        set->bn0_max, set->bn1_min, set->bn1_max, &step->index);
      break;
    case 6:
      ok = sigma_change(rng, st->nsnoise, st->snoise0, st->snoise1, set->sigma_sn0, set->sigma_sn1, set->sn0_min,
                        set->sn0_max, set->sn1_min, set->sn1_max, &step->index);
      break;
    default:
      // 7: source relocation (loc_change) is not restated
      mct_set_error("mct_mcmc_propose", "proposal type 7 (source relocation) is not supported", __FILE__, __LINE__);
      return MCT_ERR_UNSUPPORTED;
  }
  step->valid = ok ? 1 : 0;
  return MCT_OK;
}

int mct_mcmc_accept(const mct_mcmc_set *set, const mct_mcmc_step *step, double like_new, double like_old) {
  if (!set || !step) return MCT_ERR_ARG;
  // the acceptance ratios of mcmc_loc2.f90:241-246 (birth), :289-294
  // (death) and the rest (-like + like_copy)
  double a = -like_new + like_old;
  if (set->kernel == 0 && step->ptype == 1) a = step->prob - std::log(set->vsmax - set->vsmin) - like_new + like_old;
  if (set->kernel == 0 && step->ptype == 2) a = step->prob + std::log(set->vsmax - set->vsmin) - like_new + like_old;
  const double alpha = std::fmin(std::log(1.0), a);
  return std::log(step->random) < alpha ? 1 : 0;
}

int mct_mcmc_accept_tempered(const mct_mcmc_set *set, const mct_mcmc_step *step, double like_new, double like_old,
                             double temperature) {
  if (!set || !step || !(temperature > 0)) return MCT_ERR_ARG;
  // mcmc_pt's ratios (mcmc_loc2.f90:881-886 birth, :933-938 death, the rest
  // e.g. :979-981): the likelihood ratio divided by the chain's temperature
  const double t = (-like_new + like_old) / temperature;
  double a = t;
  if (set->kernel == 0 && step->ptype == 1) a = step->prob - std::log(set->vsmax - set->vsmin) + t;
  if (set->kernel == 0 && step->ptype == 2) a = step->prob + std::log(set->vsmax - set->vsmin) + t;
  const double alpha = std::fmin(std::log(1.0), a);
  return std::log(step->random) < alpha ? 1 : 0;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Parallel tempering of mcmc_pt (src/mcmc_loc2.f90:1222-1275): every
// tempering_step iterations after tempering_start, the first chain's
// process picks two chains (choose_t1 :2148-2169, choose_t2 :2171-2236) and
// offers them a swap of temperatures (do_tempering :2240-2280), drawing
// from its own random stream. The chains' temperatures are the ladder
// values0 (number_of_1s ones, then the temperature file's values,
// initialise.f90:128-134 and run_time_info.f90:186-192) permuted by the
// accepted swaps.
// ---------------------------------------------------------------------------
namespace {
// mcmc_loc2.f90:51, a REAL*4 literal widened to REAL*8
const double kEps = (double)1e-8f;

bool in_chains(const mct_pt *pt, int c) { return c >= 1 && c <= pt->nchains; }

// MINLOC(ABS(indices - t2_index), 1): the first chain holding that ladder position
int chain_of_index(const mct_pt *pt, int index) {
  int best = 1, bd = -1;
  for (int c = 1; c <= pt->nchains; ++c) {
    const int d = std::abs(pt->indices[c - 1] - index);
    if (bd < 0 || d < bd) { bd = d; best = c; }
  }
  return best;
}
}  // namespace

extern "C" {

int mct_pt_init(mct_pt *pt) {
  if (!pt || pt->nchains < 2 || !pt->values0 || !pt->values || !pt->indices || pt->number_of_1s < 1 ||
      pt->number_of_1s >= pt->nchains || pt->jump_type < 0 || pt->jump_type > 2)
    return MCT_ERR_ARG;
  for (int c = 0; c < pt->nchains; ++c) {
    if (!(pt->values0[c] > 0)) return MCT_ERR_ARG;
    pt->values[c] = pt->values0[c];
    pt->indices[c] = c + 1;
  }
  pt->accepted = 0;
  pt->total = 0;
  return MCT_OK;
}

int mct_pt_choose(mct_pt *pt, mct_rng *rng, int *t1_chain, int *t2_chain) {
  if (!pt || !rng || !t1_chain || !t2_chain || pt->nchains < 2) return MCT_ERR_ARG;
  const int n = pt->nchains, n1 = pt->number_of_1s;
  // choose_t1
  int t1 = 0;
  while (!in_chains(pt, t1)) t1 = pick_index(mct_rng_unirand(rng), n);
  const double t1v = pt->values[t1 - 1];
  const int t1i = pt->indices[t1 - 1];
  // choose_t2
  int t2 = 0;
  double t2v = 0;
  int t2i = 0;
  if (pt->jump_type == 0) {
    // a random chain of another temperature (the loop's first test is
    // decided by t2 = 0 alone); the reference loops for ever when every
    // chain has t1's temperature, here the draws are bounded
    long long tries = 0;
    do {
      if (++tries > (1LL << 24)) return MCT_ERR_INTERNAL;
      t2 = pick_index(mct_rng_unirand(rng), n);
      t2v = pt->values[t2 - 1];
      t2i = pt->indices[t2 - 1];
    } while (!in_chains(pt, t2) || std::fabs(t1v - t2v) < kEps);
  } else {
    int k;   // 1-based ladder position of the second temperature
    if (std::fabs(t1v - 1.0) < kEps) {
      k = n1 + 1;
    } else if (std::fabs(t1v - pt->values0[n - 1]) < kEps) {
      k = n - 1;
    } else if (pt->jump_type == 1) {
      k = t1i + (mct_rng_unirand(rng) < 0.5 ? -1 : 1);
    } else {
      // MINLOC(ABS(values0 - t1v), 1, MASK = ABS(values0 - t1v) > eps)
      k = 0;
      double bd = 0;
      for (int q = 1; q <= n; ++q) {
        const double d = std::fabs(pt->values0[q - 1] - t1v);
        if (!(d > kEps)) continue;
        if (k == 0 || d < bd) { bd = d; k = q; }
      }
      if (k == 1) k = pick_index(mct_rng_unirand(rng), n1);
    }
    if (k < 1 || k > n) return MCT_ERR_INTERNAL;
    t2i = k;   // temperature_indices0(k) = k
    t2 = chain_of_index(pt, t2i);
  }
  *t1_chain = t1;
  *t2_chain = t2;
  return MCT_OK;
}

int mct_pt_swap(mct_pt *pt, mct_rng *rng, int t1_chain, int t2_chain, double like_t1, double like_t2) {
  if (!pt || !rng || !in_chains(pt, t1_chain) || !in_chains(pt, t2_chain)) return MCT_ERR_ARG;
  const double t1v = pt->values[t1_chain - 1], t2v = pt->values[t2_chain - 1];
  // do_tempering: alpha_swap = min(0, -L1/T2 + L2/T2 - L2/T1 + L1/T1)
  const double a = -(like_t1 / t2v) + like_t2 / t2v - like_t2 / t1v + like_t1 / t1v;
  const double alpha = std::fmin(0.0, a);
  const double u = mct_rng_unirand(rng);
  int swapped = 0;
  if (std::log(u) <= alpha) {
    std::swap(pt->values[t1_chain - 1], pt->values[t2_chain - 1]);
    std::swap(pt->indices[t1_chain - 1], pt->indices[t2_chain - 1]);
    ++pt->accepted;
    swapped = 1;
  }
  ++pt->total;
  return swapped;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// The sample stream (samples_*.out and run_time_sample_*.dat): T_SAMPLE
// (src/run_time_info.f90:62-76) filled as the MCMC loop fills it
// (src/mcmc_loc2.f90:253-263, 305-315, 345-355, 425-436, 487-497, and
// :578-582 for every iteration) and written with stream access field by
// field, unpadded (write_samples, run_time_info.f90:306-340; the reference's
// plot/plot_point_values.m:46-56 reads the same layout).
// ---------------------------------------------------------------------------
namespace {
size_t sample_bytes(int dim) { return 4 + 1 + 4 + 8 + 3 * 8 + (size_t)dim * 8 + 3 * 8 + 2 * 8; }
}  // namespace

extern "C" {

int mct_mcmc_record(const mct_mcmc_state *st, const mct_mcmc_step *step, int accepted, double like, double misfit,
                    double unweighted_misfit, mct_sample *sm) {
  if (!st || !step || !sm) return MCT_ERR_ARG;
  *sm = mct_sample{};   // init_sample: zeros
  sm->step = step->ptype;
  const bool acc = accepted && step->valid;
  if (acc) {
    sm->accepted = 1;
    const int i = step->index - 1;
    switch (step->ptype) {
      case 1:   // birth: the new cell's nucleus and values
      case 3:   // move: the moved nucleus (vindex), no values
        if (i < 0 || i >= st->ncells) return MCT_ERR_ARG;
        sm->vindex = step->ptype == 1 ? 0 : step->index;
        for (int k = 0; k < 3; ++k) sm->coord[k] = st->points[3 * (size_t)i + k];
        if (step->ptype == 1)
          for (int k = 0; k < 3; ++k) sm->values[k] = st->parameters[3 * (size_t)i + k];
        break;
      case 2:   // death: the removed cell's index
        sm->vindex = step->index;
        break;
      case 4:   // value change: the cell's new values
        if (i < 0 || i >= st->ncells) return MCT_ERR_ARG;
        sm->vindex = step->index;
        for (int k = 0; k < 3; ++k) sm->values[k] = st->parameters[3 * (size_t)i + k];
        break;
      case 5:   // body-wave noise of period index
      case 6: { // surface-wave noise
        const int n = step->ptype == 5 ? st->nbnoise : st->nsnoise;
        const double *a = step->ptype == 5 ? st->bnoise0 : st->snoise0, *b = step->ptype == 5 ? st->bnoise1 : st->snoise1;
        if (i < 0 || i >= n || !a || !b) return MCT_ERR_ARG;
        sm->vindex = step->index;
        sm->noise0 = a[i];
        sm->noise1 = b[i];
        break;
      }
      default:
        return MCT_ERR_ARG;
    }
  }
  // every iteration: the chain's current state (mcmc_loc2.f90:578-582)
  sm->ncells = st->ncells;
  sm->like = like;
  sm->misfit = misfit;
  sm->unweighted_misfit = unweighted_misfit;
  return MCT_OK;
}

int mct_samples_write(const char *filename, int dim, const mct_sample *samples, int n) {
  if (!filename || (dim != 2 && dim != 3) || n < 0 || (n > 0 && !samples)) return MCT_ERR_ARG;
  if (n == 0) return MCT_OK;
  FILE *f = std::fopen(filename, "ab");   // appended, created when absent
  if (!f) { mct_set_error("mct_samples_write", "cannot open the file", __FILE__, __LINE__); return MCT_ERR_ARG; }
  std::vector<unsigned char> buf(sample_bytes(dim) * (size_t)n);
  unsigned char *p = buf.data();
  auto put = [&](const void *v, size_t b) { std::memcpy(p, v, b); p += b; };
  for (int r = 0; r < n; ++r) {
    const mct_sample &s = samples[r];
    const int32_t step = s.step, vindex = s.vindex;
    const unsigned char acc = s.accepted ? 1 : 0;
    const int64_t ncells = s.ncells;
    put(&step, 4); put(&acc, 1); put(&vindex, 4); put(&ncells, 8);
    put(&s.misfit, 8); put(&s.unweighted_misfit, 8); put(&s.like, 8);
    put(s.coord, 8 * (size_t)dim); put(s.values, 24); put(&s.noise0, 8); put(&s.noise1, 8);
  }
  const size_t w = std::fwrite(buf.data(), 1, buf.size(), f);
  const int cl = std::fclose(f);
  if (w != buf.size() || cl != 0) {
    mct_set_error("mct_samples_write", "short write", __FILE__, __LINE__);
    return MCT_ERR_INTERNAL;
  }
  return MCT_OK;
}

int mct_samples_read(const char *filename, int dim, mct_sample *samples, int n) {
  if (!filename || (dim != 2 && dim != 3) || n < 0 || (n > 0 && !samples)) return MCT_ERR_ARG;
  FILE *f = std::fopen(filename, "rb");
  if (!f) { mct_set_error("mct_samples_read", "cannot open the file", __FILE__, __LINE__); return MCT_ERR_ARG; }
  const size_t rb = sample_bytes(dim);
  std::vector<unsigned char> buf(rb);
  int got = 0;
  while (got < n && std::fread(buf.data(), 1, rb, f) == rb) {
    const unsigned char *p = buf.data();
    auto take = [&](void *v, size_t b) { std::memcpy(v, p, b); p += b; };
    mct_sample &s = samples[got];
    s = mct_sample{};
    int32_t step, vindex; unsigned char acc; int64_t ncells;
    take(&step, 4); take(&acc, 1); take(&vindex, 4); take(&ncells, 8);
    take(&s.misfit, 8); take(&s.unweighted_misfit, 8); take(&s.like, 8);
    take(s.coord, 8 * (size_t)dim); take(s.values, 24); take(&s.noise0, 8); take(&s.noise1, 8);
    s.step = step; s.accepted = acc != 0; s.vindex = vindex; s.ncells = ncells;
    ++got;
  }
  std::fclose(f);
  return got;
}

}  // extern "C"
