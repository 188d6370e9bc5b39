// fm2d job description shared by the fm2d kernels and the C ABI.
#pragma once
#include <cuda_runtime.h>

struct Fm2dJob {
  int nmaps;                 // velocity maps (e.g. chains x periods)
  int nvx, nvz;              // B-spline vertex grid
  double goxd, gozd, dvxd, dvzd;
  int gdx, gdz, asgr, sgdl, sgs, fom;
  int precision;             // 0 FP64 as the reference, 1 double-float (FP32 pairs), 2 FP32 on fixed-point times
  int *vmin_bits;            // scratch (precision 2): smallest vertex velocity, float bits
  const double *velv;        // [nmaps][nvx+2][nvz+2] padded vertex grids (Fortran (nvz+2,nvx+2))
  double *veln;              // [nmaps][nnx][nnz] scratch: B-spline node velocities
  double *slon;              // [nmaps][nnx][nnz] scratch: their slownesses (1 / veln)
  double *sref;              // [nmaps][nref_map] scratch: slowness of every node of the map's refined grid
  double *map_tmp_t;         // [nsolve][map_tmp_max] scratch
  short *map_tmp_s;          // [nsolve][map_tmp_max] scratch
  int *ovf_list;             // [nsolve] scratch: solves whose refined-box heap overflowed
  int *ovf_count;            // [1] scratch: their number
  // ray paths and group delays (modrays with uar = 0, then CalGroupTime)
  int rays;                  // 1: trace a ray for every path
  const double *gvel;        // [nmaps][nvx][nvz] velocity for the delay along the ray (model grid)
  double *gtime, *raylen;    // [nmaps][nsrc][nrc] group time and ray length
  int *crazy;                // [nmaps] rays that reached the point limit
  double *ref_t;             // [nsolve][nref_max] scratch: refined-box times after the refined march
  short *ref_s;              // [nsolve][nref_max] scratch: their states
  int nsrc, nrc;
  const double *scx, *scz, *rcx, *rcz;
  const int *srs;            // [srs_nmaps][nsrc][nrc] path flags
  int srs_nmaps;             // map m uses srs set (m % srs_nmaps)
  int nsolve;
  const int2 *solves;        // [nsolve] (map, 0-based source)
  double *ttime;             // [nmaps][nsrc][nrc]
  double *tfield;            // optional [nmaps][nsrc][nnx][nnz]
  int *status;
  // optional pop trace of one solve (debugging): [stage, node, ntr] ints and times
  int trace_solve; int *trace_i; double *trace_t; int trace_max;
  // from fm2d_plan
  int nodes_max, nref_max, map_tmp_max, nref_map;
  // time fields of the solves in flight (fm2d_bind_tws): [tslots_ref] slots
  // of nref_max and [tslots] slots of nodes_max nodes, each the times
  // (the precision's time type: int for precision 2, 8 bytes otherwise)
  // and, with sglobal(_ref), the node states (int16); a block's solves use
  // the slots of its place in the grid
  void *tws_ref, *tws;
  int tslots_ref, tslots;
  int sglobal_ref, sglobal;
  // optional reuse of committed refined-box results (asgr = 1, no rays,
  // precision 0 or 1): a solve whose map equals its committed map over the
  // refined box and the B-spline's reach gets the committed box mapping
  // instead of a march. cmap [nmaps]: the committed map (index into cvelv)
  // of each map, -1 for none; csolve [nsolve]: the committed solve (index
  // into cref_t / cref_s) of each solve, -1 for none; ref_list [nsolve] and
  // ref_count [1]: scratch, the solves that march
  const double *cvelv;       // [ncommitted maps][nvx+2][nvz+2]
  const int *cmap, *csolve;
  const double *cref_t;      // [ncommitted solves][map_tmp_max]
  const short *cref_s;
  int *ref_list, *ref_count;
};

struct Fm2dPlan {
  int nodes_max, nref_max, map_tmp_max;
  int nref_map;              // nodes of a map's whole refined grid (asgr = 1)
  int warp_bytes;            // shared memory per solve, coarse-grid stage
  int ref_heap_cap;          // heap entries of the refined source-box stage (asgr = 1)
  int ref_warp_bytes;        // shared memory per solve of that stage
  int ref_full_warp_bytes;   // the same with a heap as large as the box (overflow pass)
  int tbytes;                // bytes of one time value
  int tslots, tslots_ref;    // the most solves resident at once per stage
  int sglobal, sglobal_ref;  // node states in the global slots (shared memory would cut the residency)
  // launch policy, not set by fm2d_plan: the share of the device's SMs the
  // solve kernels may hold at once (0 or >= 1: all)
  double sm_share = 0.0;
};

int fm2d_plan(const Fm2dJob &job, Fm2dPlan *plan);
// Device memory of the time-field slots for at most nsolve_max solves per
// launch, and the binding of such a block (256-byte aligned) to a job.
size_t fm2d_tws_bytes(const Fm2dPlan &plan, long nsolve_max);
void fm2d_bind_tws(Fm2dJob &job, const Fm2dPlan &plan, long nsolve_max, void *mem);
int launch_fm2d(const Fm2dJob &job, const Fm2dPlan &plan, cudaStream_t s);
