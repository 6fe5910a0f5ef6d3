/*
 * letkf_gpu.h -- C ABI of the GB300 LETKF analysis library (libletkf_gpu.so).
 *
 * Plain pointers and sizes only.  All matrices keep the reference's Fortran
 * conventions: trans(ne,ne) is column-major, trans(k,m) being the weight of
 * background member k in analysis member m (common/common_letkf.f90:43-47).
 *
 * Every call returns a letkf status code (LETKF_OK == 0).  The library never
 * falls back to the CPU: without a usable CUDA device every entry point that
 * computes returns LETKF_ERR_NOGPU.
 */
#ifndef LETKF_GPU_H
#define LETKF_GPU_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define LETKF_OK 0
#define LETKF_ERR_ARG 1      /* bad argument (ne < 2, nobsl < 0, nobsl > nobs, NULL array) */
#define LETKF_ERR_EIG 2      /* common/common_mtx.f90:61-64,75-78: rs ierr /= 0 or all eigenvalues <= 0 (STOP 2) */
#define LETKF_ERR_CUDA 3     /* a CUDA runtime call failed */
#define LETKF_ERR_CAPACITY 4 /* size beyond this build's limits (ne > LETKF_MAX_NE, local obs overflow) */
#define LETKF_ERR_NOGPU 5    /* no CUDA device */
#define LETKF_ERR_TIMEOUT 6  /* a bounded device wait gave up */

#define LETKF_MAX_NE 128     /* largest ensemble size of the on-chip kernels */

/* ------------------------------------------------------------------------
 * Library information
 * ---------------------------------------------------------------------- */
const char* letkf_version(void);
const char* letkf_status_string(int status);
/* number of kernel launches issued by this library since load (all threads) */
int64_t letkf_launch_count(void);
int letkf_device_sync(void);

/* ------------------------------------------------------------------------
 * Per-point drop-in.  Replaces SUBROUTINE letkf_core(ne,nobs,nobsl,hdxb,
 * rdiag,rloc,dep,parm_infl,trans,transm,pao,rdiag_wloc,minfl) of
 * common/common_letkf.f90:50.  Host arrays, Fortran layout: hdxb(nobs,ne)
 * with leading dimension nobs, only rows 1..nobsl used.  transm and pao may
 * be NULL (absent optional arguments).  rdiag_wloc is 0/1 (absent = 0).
 * minfl <= 0 means absent (the reference only acts on minfl > 0).
 * Runs the FP64 plain form on the current CUDA device and blocks until done.
 * ---------------------------------------------------------------------- */
int letkf_core_c(int ne, int nobs, int nobsl, const double* hdxb, const double* rdiag,
                 const double* rloc, const double* dep, double* parm_infl, double* trans,
                 double* transm, double* pao, int rdiag_wloc, double minfl);

/* ------------------------------------------------------------------------
 * Batched cores on DEVICE buffers (one letkf_core per point).
 *   offs[npts+1]      int64, point p owns local obs rows offs[p]..offs[p+1]-1
 *   rows[nrows][ne]   obs-space perturbations hdxb, row-major (member fastest)
 *   rdiag, rloc, dep  [nrows]
 *   parm_infl[npts]   in/out
 *   trans[npts][ne*ne] column-major per point; transm[npts][ne], pao[npts][ne*ne]
 *                     may be NULL (absent)
 *   status[npts]      per-point status (LETKF_OK / LETKF_ERR_EIG)
 * The call is asynchronous on `stream` (a cudaStream_t, NULL = default).
 * Replaces the per-point loop of das_letkf (e.g. speedy/letkf/letkf_tools.f90:
 * 151-201) around common/common_letkf.f90:50.
 * ---------------------------------------------------------------------- */
int letkf_core_batch_f64(int ne, int npts, const int64_t* offs, const double* rows,
                         const double* rdiag, const double* rloc, const double* dep,
                         double* parm_infl, double* trans, double* transm, double* pao,
                         int rdiag_wloc, double minfl, int* status, void* stream);

/* Mixed-precision batched core: FP32 rows/weights, FP32 Gram and eigensolver
 * with an FP64 refinement of the transform; outputs FP32 trans/transm and
 * FP64 inflation.  Same layout and semantics as letkf_core_batch_f64. */
int letkf_core_batch_mixed(int ne, int npts, const int64_t* offs, const float* rows,
                           const float* rdiag, const float* rloc, const float* dep,
                           double* parm_infl, float* trans, float* transm, int rdiag_wloc,
                           double minfl, int* status, void* stream);

/* ------------------------------------------------------------------------
 * Ensemble update on DEVICE buffers (speedy/letkf/letkf_tools.f90:164-170;
 * scale/letkf/letkf_tools.f90:237-251 with beta = 1):
 *   xa(p,m,v) = mean(p,v) + sum_k xb'(p,k,v) * (trans_p(k,m) + transm_p(k))
 * xb[nv][npts][ne] full background members (member fastest); the mean is
 * formed in FP64 with the sequential member sum of
 * speedy/common/common_speedy.f90:335-370.  transm may be NULL.
 * ---------------------------------------------------------------------- */
int letkf_update_f64(int ne, int npts, int nv, const double* xb, const double* trans,
                     const double* transm, double* xa, void* stream);

/* ------------------------------------------------------------------------
 * Local observation search on DEVICE buffers.  Each search writes, per grid
 * point, the selected observations in the reference's order:
 *   count pass:  nobsl[npts]
 *   fill pass:   idx[offs[p]..], rloc[..], rdiag[..] with offs = exclusive
 *                scan of nobsl (computed by the caller or letkf_exclusive_scan)
 * ---------------------------------------------------------------------- */
/* SCALE Cartesian search (scale/letkf/letkf_tools.f90:853-1178 with
 * obs_choose, scale/letkf/letkf_obs.f90:1054-1119), one subdomain, no
 * MAX_NOBS_PER_GRID limit.  Observation arrays are the bucket-sorted ones.
 * cls: 0 default (log p vertical), 1 ps, 2 rain, 3 radar ref, 4 radar vr,
 * 5 radar prh, 6 tc.  var_local_row[nvarloc] may be NULL (nvar <= 0).
 * params[16]: dx, dy, dlon_zero, dlat_zero, sigma_obs, sigma_obsv,
 * sigma_obs_rain, sigma_obsv_rain, base_obsv_rain, sigma_obs_radar,
 * sigma_obs_radar_noref, sigma_obsz_radar, radar_ref_thres_dbz, sigma_obs_tc,
 * sigma_obsv_tc, (unused). */
int letkf_search_scale(int nlon, int nlat, const int* nobsgrd /* [(nlon+1)*nlat] */, int nobs,
                       const double* ori, const double* orj, const double* olev, const double* odat,
                       const double* oerr, const int* ocls, const int* ovarloc, int npts,
                       const double* pri, const double* prj, const double* prlev, const double* prz,
                       const double* var_local_row, const double* params, const int64_t* offs,
                       int* nobsl, int* idx, double* rloc, double* rdiag, void* stream);

/* SPEEDY lat/lon search (speedy/letkf/letkf_tools.f90:272-603).  nobsgrd is
 * [nlon*nlat] (i fastest); obselm holds the SPEEDY element ids.
 * params[5]: dist_zero, dist_zerov, dlat_zero, sigma_obs, sigma_obsv.
 * var_local_row[7]: u, v, t, q, rh, ps, rain. */
int letkf_search_speedy(int nlon, int nlat, const double* lon, const double* lat,
                        const int* nobsgrd, int nobs, const double* obselm, const double* obslon,
                        const double* obslat, const double* obslev, const double* obsdat,
                        const double* obserr, int npts, const double* plon, const double* plat,
                        const double* pdlon_zero, const int* pilev, const double* plogpfm,
                        const double* var_local_row, const double* params, const int64_t* offs,
                        int* nobsl, int* idx, double* rloc, double* rdiag, void* stream);

/* exclusive scan of n int32 counts into int64 offsets[n+1] (device) */
int letkf_exclusive_scan(int n, const int* counts, int64_t* offs, void* stream);

/* gather packed local rows: rows_out[r][ne] = ens[idx[r]][ne] (double or
 * float via elem_bytes 8/4), dep_out[r] = dep[idx[r]] */
int letkf_gather_rows(int ne, int64_t nrows, const int* idx, const void* ens, const void* dep,
                      int elem_bytes, void* rows_out, void* dep_out, void* stream);

#ifdef __cplusplus
}
#endif
#endif
