// sweep_args.cuh -- argument block of the fused mixed-precision sweep kernel.
#pragma once
#include "letkf_common.cuh"

namespace letkf {

struct SweepScaleParams {
  double dx, dy, dlon_zero, dlat_zero, sigma_obs, sigma_obsv, sigma_obs_rain, sigma_obsv_rain, base_obsv_rain,
      sigma_obs_radar, sigma_obs_radar_noref, sigma_obsz_radar, radar_ref_thres_dbz, sigma_obs_tc, sigma_obsv_tc;
};

struct SweepArgs {
  int n, nv, npts, nlon, nlat, nobs;
  const int* G;           // nobsgrd [(nlon+1)*nlat]
  const float4* obsF;     // [nobs] ri, rj, vertical coordinate, 1/sigma_h^2
  const float4* obsA;     // [nobs] 1/sigma_v^2, 1/err^2, dep, var_local weight
  const int* obsMeta;     // [nobs] bit0 height vertical, bit1 rejected by var_local
  const double *ori, *orj, *olev, *odat;  // FP64 records for the exact re-test
  const int* ocls;
  SweepScaleParams P;
  const float* ens_obs;   // [nobs][n]
  const int* order;       // [npts]
  const double *pri, *prj, *prlev, *prz;
  const double* plogr;    // [npts] log(rlev)
  const float* xb;        // [nv][npts][n]
  int xb_bulk;            // rows of xb may be fetched with TMA bulk copies (16-byte rows and base)
  float* xa;
  double* infl;           // [npts] in/out
  int* nobsl_out;         // [npts] or NULL
  int* sweeps_out;        // [npts] or NULL
  int* status;            // [npts]
  int* counter;
  double minfl;
  int max_sweeps;   // Jacobi sweeps (fallback eigensolver)
  int max_ns_iter;  // Newton-Schulz iterations
  int use_ns;       // 1: Newton-Schulz inverse square root, 0: Jacobi eigensolver
  int nwork;            // entries of `order` to process (npts is the row stride of xb / xa)
  const int* npts_dev;  // if set, the number of entries of `order` to process (device scalar)
  int* defer_list;      // tensor-core sweep: points handed to the Jacobi pass
  int* defer_count;
  int* err_flag;        // set when a bounded wait gave up
  int tc_ns_max;        // tensor-core Newton-Schulz iterations before the FP32 polish
  int tc_ns_scaled;     // spectrum-scaled tensor-core steps (1) or plain ones (0)
  float tc_ns_tol;      // tensor-core phase ends once ||ZY - I||_F^2 < tc_ns_tol
  float polish_tol;     // FP32 polish: last step once ||Z A Z / s - I||_F^2 < polish_tol
  int tc_polish;        // the anchored polish step on the tensor cores (1) or in FP32 (0)
  int tc_scale_bound;   // scale s from min(||A||_F, Gershgorin), every step scaled (1); power iteration (0)
  float polish_probe;   // FP32 polish skipped where the anchored probe residual is below this (0: always polished)
  float ns_cond_max;    // Newton-Schulz only while the spectrum bound s / c is below this (0: no bound); a
                        // larger bound, or an iteration that does not converge, sends the point to the Jacobi pass
  int* defer_total;     // points handed to the Jacobi pass in this run (the deferred pass adds its count)
  // selection probe: for points with probe_slot[pt] >= 0 the search also
  // writes what it accepted, in emitted order (sorted observation index and
  // FP32 rloc), to probe_idx / probe_rloc[slot * probe_cap + i] for
  // i < probe_cap, and the accepted count to probe_count[slot]
  const int* probe_slot;  // [npts] or NULL (no probe)
  int probe_cap;
  int* probe_idx;
  float* probe_rloc;
  int* probe_count;
  // list mode: the local observations of order position q are given as
  // entries list_offs[q] .. list_offs[q+1] - 1 (sorted observation index and
  // FP64 rloc, in the order they enter letkf_core) instead of being searched
  const int64_t* list_offs;  // [nwork + 1] or NULL (search)
  const int* qmap;           // if set, work item q analyses order position qmap[q] (the deferred pass of list mode)
  const int* list_idx;
  const double* list_rloc;
  // column cache of the search (sweep_search.cuh SwCache): CTA b keeps the
  // horizontal survivors of its current column in col_ent[2 b col_cap ...]
  // (b < col_slots); a CTA takes col_unit consecutive order positions at a
  // time, so the levels of a column (consecutive in the order) meet in one CTA
  int4* col_ent;  // NULL: no cache
  int col_cap;
  int col_slots;
  int col_unit;  // >= 1
  // failure injection: > 0 makes the tensor-core sweep wait, before its first
  // point, on a barrier that nothing arrives at, giving up after this many
  // polls (LETKF_ERR_TIMEOUT through err_flag); 0 in normal runs
  uint32_t fault_wait_polls;
};

}  // namespace letkf
