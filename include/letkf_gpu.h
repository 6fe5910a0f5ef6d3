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
#define LETKF_ERR_CAPACITY 4 /* size beyond the library's limits (ne > LETKF_MAX_NE, local obs overflow) */
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

/* Mixed-precision batched core: FP32 rows/weights and Gram; the transform by
 * spectrum-scaled Newton-Schulz (W = sqrt((k-1)/s) (A/s)^(-1/2)) where
 * mtx_eigen's truncation cannot act (c > 0, tr(G) < 1e6 c), else by the
 * parallel Jacobi eigensolver with the reference's truncation; outputs FP32
 * trans/transm and FP64 inflation.  Same layout and semantics as
 * letkf_core_batch_f64. */
int letkf_core_batch_mixed(int ne, int npts, const int64_t* offs, const float* rows,
                           const float* rdiag, const float* rloc, const float* dep,
                           double* parm_infl, float* trans, float* transm, int rdiag_wloc,
                           double minfl, int* status, void* stream);

/* Large-ensemble core (ne up to LETKF_LARGEK_MAX_NE): same arguments, layout and
 * semantics as letkf_core_batch_mixed, for ensembles whose ne x ne matrices
 * live in HBM.  Gram and the Newton-Schulz products of A^(-1/2) run on the
 * tensor cores with three-term TF32 splits; W = sqrt((ne-1)/s) Z, wbar = Pa
 * Ywᵀ dep.  Points with c <= 0 or tr(G) >= 1e6 c (where mtx_eigen's
 * truncation could act) get status LETKF_ERR_CAPACITY and an identity
 * transform; a transform that does not converge gets LETKF_ERR_EIG. */
#define LETKF_LARGEK_MAX_NE 1024
int letkf_core_batch_largek(int ne, int npts, const int64_t* offs, const float* rows,
                            const float* rdiag, const float* rloc, const float* dep,
                            double* parm_infl, float* trans, float* transm, int rdiag_wloc,
                            double minfl, int* status, void* stream);

/* The large-ensemble core over the index lists of a local search, without
 * packed copies of the rows: point p's local observations are idx[offs[p]]
 * .. idx[offs[p+1]-1] (the search's output), their rows are ens_obs[idx[l]]
 * ([nobs][ne]: FP32, or BF16 when ens_bf16) and their departures
 * dep_obs[idx[l]]; rdiag, rloc are per list entry.  Otherwise as
 * letkf_core_batch_largek.  With BF16 rows the Gram's operands are exact
 * BF16 values weighted in FP32. */
int letkf_core_batch_largek_indexed(int ne, int npts, const int64_t* offs, const int* idx, const void* ens_obs,
                                    int ens_bf16, const float* dep_obs, const float* rdiag, const float* rloc,
                                    double* parm_infl, float* trans, float* transm, int rdiag_wloc, double minfl,
                                    int* status, void* stream);

/* Ensemble update with BF16 storage (ne <= 512, nv <= 8): each member is
 * xmean [nv][npts] (FP32) plus its perturbation xpert [nv][npts][ne] (BF16);
 * the analysis is written the same way: amean = mean + xb' transm (FP64
 * sums) and apert = xb' trans (FP32 products, rounded to BF16), with xb' the
 * stored perturbations minus their mean.  The mean stays FP32 because BF16
 * values (8-bit mantissa) cannot hold a field's mean to a small fraction of
 * its spread. */
int letkf_update_bf16(int ne, int npts, int nv, const float* xmean, const void* xpert, const float* trans,
                      const float* transm, float* amean, void* apert, void* stream);

/* FP32 ensemble update for any ne <= 512: xb, xa [nv][npts][ne] float32,
 * trans [npts][ne*ne] column-major, transm [npts][ne] or NULL; FP32 products,
 * FP64 mean and mean increment (nv <= 8). */
int letkf_update_mixed(int ne, int npts, int nv, const float* xb, const float* trans,
                       const float* transm, float* xa, void* stream);

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

/* Relaxed update of the SCALE driver (scale/letkf/letkf_tools.f90:215-268),
 * per point p and variable v:
 *   mode 1 RTPP  W' = (1 - alpha) W + alpha I                  (:1224-1237)
 *   mode 2 RTPS  W' = infl W, infl = alpha sqrt(var_g / (var_a (ne-1)))
 *                - alpha + 1 with var_g = xb'.xb', var_a = xb' Pa xb'  (:1240-1268)
 *   T = (W' + transm 1^T) beta + (1 - beta) I;  beta == 0: xa = mean + xb'
 *   q_sprd_max > 0: the relative spread of variable q_var is clipped to it.
 * beta[nv][npts] may be NULL (1); pao is required for RTPS; rtps_infl[nv][npts]
 * may be NULL (1 where beta == 0, which skips the relaxation).  Mode 0 with
 * beta = 1 equals letkf_update_f64 bit for bit. */
typedef struct letkf_relax_desc {
  int mode;              /* 0 none, 1 RTPP, 2 RTPS */
  double alpha;          /* RELAX_ALPHA or RELAX_ALPHA_SPREAD */
  const double* beta;    /* device [nv][npts] or NULL */
  int q_var;             /* variable index of the spread clip, -1 none */
  double q_sprd_max;     /* Q_SPRD_MAX, <= 0 off */
} letkf_relax_desc;
int letkf_update_relax_f64(int ne, int npts, int nv, const double* xb, const double* trans,
                           const double* transm, const double* pao, const letkf_relax_desc* relax,
                           double* xa, double* rtps_infl, void* stream);

/* relax_beta (scale/letkf/letkf_tools.f90:1182-1220) for every point and
 * variable: 0 for variables q_lo..q_hi where rlev < q_update_top, the
 * boundary-buffer ramp min(dist_bdy, 1) (clipped at 0) when
 * boundary_buffer_width > 0, else 1.  beta[nv][npts] on the device. */
int letkf_relax_beta(int npts, int nv, const double* ri, const double* rj, const double* rlev,
                     int q_lo, int q_hi, double q_update_top, double boundary_buffer_width,
                     double dx, double dy, int nlong, int nlatg, int ihalo, int jhalo,
                     double* beta, void* stream);

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

/* SCALE search with the MAX_NOBS_PER_GRID limit (scale/letkf/letkf_tools.f90:
 * 853-1178 with MAX_NOBS_PER_GRID > 0; allocation :901-906, selection
 * :1063-1128, emission :1141-1156).  Same arguments as letkf_search_scale plus
 * each observation's element uid ouid[nobs] (1..nid, the reference's
 * uid_obs(elm)) and type otyp[nobs] (1..nobtype), nid and the limit M
 * (1..LETKF_MAX_NOBS_PER_GRID_LIMIT).  Per (uid, type) group the M accepted
 * observations of smallest rdiag = err^2 / rloc are kept (ties: the earlier
 * candidate), and the list is emitted grouped by type, then uid, each group
 * in the reference's slot order.  Count pass (idx == NULL) and fill pass as
 * for letkf_search_scale; each pass allocates stream-ordered scratch for the
 * unlimited lists and returns once its results are on the device. */
#define LETKF_MAX_NOBS_PER_GRID_LIMIT 256
int letkf_search_scale_limited(int nlon, int nlat, const int* nobsgrd, int nobs, const double* ori,
                               const double* orj, const double* olev, const double* odat, const double* oerr,
                               const int* ocls, const int* ovarloc, const int* ouid, const int* otyp, int nid,
                               int max_nobs_per_grid, int npts, const double* pri, const double* prj,
                               const double* prlev, const double* prz, const double* var_local_row,
                               const double* params, const int64_t* offs, int* nobsl, int* idx, double* rloc,
                               double* rdiag, void* stream);

/* GFS lat/lon search (gfs/letkf/letkf_tools.f90:686-955): the SPEEDY box walk
 * over the same bucket-sorted observations with the GFS tests:
 * dlat_zero = max(dist_zero, dist_zero_rain) / pi / re * 180 and
 * dlon_zero = dlat_zero / cos(lat pi / 180) per point; vertical distance
 * |ln obsdat - ln p| for ps, |ln base_obsv_rain - ln p| against dist_zerov_rain
 * for rain (19999), 0 for TC obs (>= 99991), |ln obslev - ln p| otherwise;
 * horizontal cut-off dist_zero_rain for rain; rloc = exp(-0.5 ((d/sigma_h)^2 +
 * (dlev/sigma_obsv)^2)) (sigma_h = sigma_obs_rain for rain) times the
 * variable localisation; rdiag = err^2.  prlev[npts] is the point's pressure
 * (pfull; the reference's rlev).  var_local_row[6] (u/v, t/tv, q/rh, ps, rain,
 * tc) or NULL for nvar = 0 (no variable localisation, as the EFSO and
 * obs-space calls use); with it, element codes outside the GFS list are not
 * selected.  params[8]: dist_zero, dist_zerov, dist_zero_rain,
 * dist_zerov_rain, sigma_obs, sigma_obsv, sigma_obs_rain, base_obsv_rain.
 * idx is the sorted observation index (the reference's oindex). */
int letkf_search_gfs(int nlon, int nlat, const double* lon, const double* lat, const int* nobsgrd, int nobs,
                     const double* obselm, const double* obslon, const double* obslat, const double* obslev,
                     const double* obsdat, const double* obserr, int npts, const double* plon, const double* plat,
                     const double* prlev, const double* var_local_row, const double* params, const int64_t* offs,
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

/* SPEEDY / GFS observation bucket sort on DEVICE buffers (speedy/letkf/
 * letkf_obs.f90:243-313): observations are ordered by latitude band j
 * (lat(j) <= y < lat(j+1), j = 1..nlat-1), then longitude cell i (lon(i) <=
 * x < lon(i+1), the last cell up to 360), input order inside a cell.  qc
 * [nobs] may be NULL; with it only qc == 1 observations are kept (the
 * selection of set_letkf_obs).  perm[nobs] receives the input index of each
 * kept observation in sorted order, *nsorted (host) their count, and
 * nobsgrd[nlat * nlon] (i fastest) the cumulative counts through each cell
 * (row nlat 0, as the reference leaves it).  Observations outside every
 * band or cell are dropped.  Returns when the results are on the device. */
int letkf_sort_obs_latlon(int nlon, int nlat, const double* lon, const double* lat, int nobs,
                          const double* olon, const double* olat, const int* qc, int* perm, int* nsorted,
                          int* nobsgrd, void* stream);

/* Observation-space perturbations and departures on DEVICE buffers
 * (speedy/letkf/letkf_obs.f90:157-174; lorenz96/letkf/letkf.f90:196-212):
 * mean = sum_m hx[n][m] / ne (member order, FP64), hdxf[n][m] = hx[n][m] - mean,
 * dep[n] = y[n] - mean; with gross_error > 0, |dep| > gross_error * err[n]
 * sets qc_out[n] = 0.  Observations with qc_in[n] != 1 are skipped (hdxf = hx,
 * dep = 0, qc_out = 0).  qc_in, qc_out and err (when gross_error <= 0) may be
 * NULL.  hx and hdxf are [nobs][ne]; ne <= 512. */
int letkf_obs_departure(int ne, int nobs, const double* hx, const double* y, const double* err,
                        double gross_error, const int* qc_in, double* hdxf, double* dep, int* qc_out,
                        void* stream);

/* ------------------------------------------------------------------------
 * Obs-space clients of the core (GFS driver), DEVICE buffers.
 * Analysis ensemble at n observation locations (gfs/letkf/letkf_tools.f90:
 * 466-497): trans[n][ne*ne] the merged transforms (T + wbar 1^T, column-
 * major) from a core run at the observation locations, ybar = obsdat -
 * obsdep, hdxf [n][ne] the observations' own perturbations; relax_alpha != 0
 * applies weight_RTPP (:959-970); mode[n] (NULL: all 0) is 0 update, 1 no
 * update (q above the update level: anal = ybar + hdxf), 2 update and clip
 * the relative spread to q_sprd_max.  anal [n][ne], anal_mean [n] (may be NULL). */
int letkf_obs_analysis(int ne, int n, const double* trans, const double* ybar, const double* hdxf,
                       double relax_alpha, const int* mode, double q_sprd_max, double* anal,
                       double* anal_mean, void* stream);

/* Ensemble forecast sensitivity to observations (EFSO, gfs/letkf/letkf_tools.f90:
 * 547-679) over npts grid points with their local lists offs/idx/rdiag/rloc
 * (a search's output): work1(t,m) = sum_v [term[v] == t] fcst(v,p,m) fcer(v,p),
 * djdy(n,t) = sum over the points that select n of sum_m work1(t,m)
 * hdxa(n,m) / rdiag * rloc, obsense(n,t) = djdy(n,t) obsdep(n).  fcst
 * [nv][npts][ne] (C^1/2 X^f_t), fcer [nv][npts] (C^1/2 (e^f_t + e^g_t) /
 * 2(K-1)), hdxa [nobs][ne] (Y^a_0), djdy and obsense [nobs][nterm].  term[nv]
 * is a HOST array (term index or -1); nv <= 16, nterm <= 8.  djdy is
 * accumulated with atomics (sum order differs from the serial loop by rounding). */
int letkf_efso(int ne, int npts, int nv, int nterm, const int* term, const int64_t* offs,
               const int* idx, const double* rdiag, const double* rloc, int nobs, const double* hdxa,
               const double* fcst, const double* fcer, const double* obsdep, double* djdy,
               double* obsense, void* stream);

/* SPEEDY observation operator H(x) for every member, replacing the obsope
 * program (speedy/letkf/obsope.f90:53-104) run once per member:
 * phys2ijk (speedy/common/common_obs_speedy.f90:137-206) against the member's
 * p_full = ps sig(k), the driver's range rules (CEILING(rk) > nlev rejected;
 * below the lowest level u/v use rk = 1.00001, others are rejected; ps with
 * odat < -100 rejected) and Trans_XtoY (:29-80: itpl_3d of u/v/t/q, itpl_2d
 * of ps/rain, calc_rh at the eight corners for RH).  Element codes are the
 * NINT of the reference's elm (2819 u, 2820 v, 3073 t, 3330 q, 3331 rh,
 * 14593 ps, 9999 rain); an unknown code gives hx = 0 with qc 1, like the
 * driver's zero-initialised ohx.  A non-positive level of a non-ps
 * observation is rejected (its log is undefined).
 * Fields (device, FP64): v3d(i,j,k,n) of member m at
 * v3d[m*v3d_mem_stride + (n*nlev + k)*v3d_rec_stride + j*nlon + i] (n = 0 u,
 * 1 v, 2 t, 3 q; 0-based), v2d(i,j,n) at v2d[m*v2d_mem_stride +
 * n*v2d_rec_stride + j*nlon + i] (n = 0 ps, 1 rain).  A grd file per member
 * is rec stride nlat*nlon, member stride (4 nlev + 2) nlat nlon.  lat[nlat]
 * (degrees, searched in order like the reference), sig[nlev] on the device.
 * Observations (device): elem[nobs] int, rlon/rlat/rlev/odat[nobs].
 * Outputs: hx[nobs][ne] (0 where rejected), qc_member[nobs][ne] (may be
 * NULL) and qc[nobs] = min over members (may be NULL), as set_letkf_obs
 * combines the members (speedy/letkf/letkf_obs.f90:157-158).
 * nlat >= 2, nlev >= 2. */
int letkf_speedy_obsope(int nlon, int nlat, int nlev, int ne, const double* lat, const double* sig,
                        const double* v3d, int64_t v3d_mem_stride, int64_t v3d_rec_stride,
                        const double* v2d, int64_t v2d_mem_stride, int64_t v2d_rec_stride, int nobs,
                        const int* elem, const double* rlon, const double* rlat, const double* rlev,
                        const double* odat, double* hx, int* qc_member, int* qc, void* stream);

/* SCALE observation operator H(x) for conventional observations, every
 * member (scale/obs/obsope_tools.f90:340-380, the OBS_IN_FORMAT 1 path):
 * phys2ijk (scale/common/common_obs_scale.f90:969-1075) then Trans_XtoY
 * (:262-334) for u 2819, v 2820, t 3073, tv 3074, q 3330, rh 3331 and ps
 * 14593 (prsadj to the observation height, :583-599).  Fields (device, FP64),
 * each member's local domain with halos, k fastest as the reference's
 * v3dg(nlevh, nlonh, nlath, nv3dd): v3d element (k, i, j, n) of member m at
 * v3d[m*v3d_mem_stride + n*v3d_var_stride + (j*nlonh + i)*nlevh + k] (0-based;
 * n = 0 u, 1 v, 2 t, 3 q, 4 rh, 5 full pressure p; nlevh = nlev + 2*khalo),
 * v2d (i, j, n) at v2d[m*v2d_mem_stride + n*v2d_var_stride + j*nlonh + i]
 * (n = 0 ps, 1 t2m, 2 q2m, 3 topo).  khalo >= 2 (KHALO).  Observations
 * (device): elem[nobs], ri / rj (1-based grid coordinates of the halo domain,
 * as obsope's ri / rj), rlev (Pa; the height in m for surface elements >
 * 9999), rotc[nobs][2] (the map projection's rotation coefficients at the
 * observation, MPRJ_rotcoef of SCALE-RM; NULL: (1, 0)); stggrd 1: u / v on
 * the staggered grid; ps_adjust_thres: PS_ADJUST_THRES (100 m by default).
 * Outputs: hx[nobs][ne] (0 where phys2ijk rejects, -9.99e33 with qc 90 for
 * another element), qc_member[nobs][ne] (may be NULL), qc[nobs] = the maximum
 * over members (obsope_tools.f90:602-608; may be NULL); qc codes 0 good, 10
 * ps height adjustment beyond the threshold, 20 too high, 21 too low, 22
 * outside the domain, 90 other element.  An interpolation stencil keeps its
 * upper index in [2, n] (the reference's value wherever its stencil stays in
 * its arrays; the staggered u / v at ri - 0.5 < 1 extrapolate from the edge
 * columns, where the reference reads outside its array). */
int letkf_scale_obsope(int nlonh, int nlath, int nlev, int khalo, int ne, const double* v3d,
                       int64_t v3d_mem_stride, int64_t v3d_var_stride, const double* v2d, int64_t v2d_mem_stride,
                       int64_t v2d_var_stride, int nobs, const int* elem, const double* ri, const double* rj,
                       const double* rlev, const double* rotc, int stggrd, double ps_adjust_thres, double* hx,
                       int* qc_member, int* qc, void* stream);

/* SPEEDY grid-file records (speedy/common/common_speedy.f90:163-287): a file
 * is nrec records of nij = nlon*nlat REAL(4) (u levels, v, t, q, ps, rain),
 * big-endian as the reference's -byteswapio build writes them.  raw holds ne
 * members' files back to back on the device (member m at m*nrec*nij floats,
 * 4-byte aligned).  Decode: records r0..r0+nr-1 of every member -> out
 * element (m, r, ij) at out[m*out_mem_stride + r*out_rec_stride + ij] (FP64
 * when out_f64, else FP32), byte-swapping when byteswap; this is
 * read_grd4 + the REAL(4) -> r_size widening of read_ens_mpi
 * (speedy/common/common_mpi_speedy.f90:354-382).  Encode: the reverse, FP64
 * rounded to nearest REAL(4) (write_ens_mpi, :386-414). */
int letkf_grd_decode(int64_t nij, int nrec, int ne, const void* raw, int byteswap, int r0, int nr, int out_f64,
                     void* out, int64_t out_mem_stride, int64_t out_rec_stride, void* stream);
int letkf_grd_encode(int64_t nij, int nrec, int ne, const void* in, int in_f64, int64_t in_mem_stride,
                     int64_t in_rec_stride, int r0, int nr, int byteswap, void* raw, void* stream);

/* Ensemble mean and spread per (record, point) (ensmean_grd,
 * speedy/common/common_speedy.f90:335-370; spread of write_ensmspr_mpi,
 * speedy/common/common_mpi_speedy.f90:461-515): x(m, r, ij) at
 * x[m*mem_stride + r*rec_stride + ij]; mean and sprd [nrec][nij] (either may
 * be NULL), sums in member order, sprd = sqrt(sum (x - mean)^2 / (ne - 1)). */
int letkf_ens_mean_spread(int64_t nij, int nrec, int ne, const double* x, int64_t mem_stride, int64_t rec_stride,
                          double* mean, double* sprd, void* stream);

/* Lorenz-96 selection (lorenz96/letkf/letkf.f90:220-254).  obs_cell[ny] is
 * the 1-based grid index of each observation (first maximum of its row of H,
 * see letkf_l96_obs_cell); pix[npts] are 1-based grid indices.  An
 * observation is kept when its cyclic distance d < xlocal * 2 sqrt(10/3) and
 * rloc = exp(-0.5 (d/xlocal)^2) * exp(-0.5 (tdif/tlocal)^2) >= 1e-4
 * (tdif = 0 when tlocal < 0); lists are in observation-index order and
 * rdiag = obserr^2.  rdiag may be NULL. */
int letkf_search_l96(int nx, int ny, const int* obs_cell, int npts, const int* pix, double xlocal,
                     double tdif, double tlocal, double obserr, const int64_t* offs, int* nobsl,
                     int* idx, double* rloc, double* rdiag, void* stream);

/* 4D-LETKF selection of the Lorenz-96 driver (lorenz96/letkf/letkf.f90:
 * 217-254, nwindow > 1): for analysis slot `slot` (0-based nn - 1) the
 * observations of every slot n = 0..nslot-1 in slot order, each slot's in
 * observation order, with tdif = |slot - n| (0 when tlocal < 0) in
 * rloc = exp(-0.5 (d/xlocal)^2) exp(-0.5 (tdif/tlocal)^2) and the 1e-4 drop.
 * obs_cell[nslot][ny] (1-based grid index per slot); idx is the row n*ny + i
 * of the slot-stacked observation arrays.  Count pass (idx NULL) then fill
 * pass as letkf_search_l96.  nslot = 1, slot = 0 equals letkf_search_l96 with
 * tdif = 0. */
int letkf_search_l96_4d(int nx, int nslot, int ny, const int* obs_cell, int npts, const int* pix, int slot,
                        double xlocal, double tlocal, double obserr, const int64_t* offs, int* nobsl, int* idx,
                        double* rloc, double* rdiag, void* stream);

/* Lorenz-96 selection with the driver's localisation mode switch msw_local
 * (lorenz96/letkf/letkf.f90:18-27,217-254), replacing its selection loop for
 * every mode: 0 = fixed (as letkf_search_l96_4d); 1 = adaptive, rloc =
 * wa^sa * wb^sb from com_correl (common/common.f90:111-128) between the
 * observation's perturbations hdxf[row][ne] and the point's first-guess
 * perturbations (xf[ix-1][ne] minus the sequential member mean): wb = |cor over
 * all members|, wa = 1 - |cor(members 1..ceil(ne/2)) - cor(the rest)| / 2;
 * 2 = the adaptive weight times both fixed factors.  Every candidate within
 * xmaxloc is weighted and dropped below 1e-4.  hdxf holds the slot-stacked
 * rows n*ny + i; xf is the analysis slot's first guess [nx][ne] (row-major).
 * Means, variances and covariances are sequential FP64 sums, each operation
 * rounded on its own.  Other msw_local values: LETKF_ERR_ARG. */
int letkf_search_l96_adaptive(int nx, int nslot, int ny, const int* obs_cell, int npts, const int* pix, int slot,
                              double xlocal, double tlocal, double obserr, int msw_local, double sa, double sb,
                              int ne, const double* hdxf, const double* xf, const int64_t* offs, int* nobsl,
                              int* idx, double* rloc, double* rdiag, void* stream);

/* Grid index of each observation of the Lorenz-96 driver: the first maximum
 * of row i of h (ny x nx, column-major, on the device), 1-based
 * (lorenz96/letkf/letkf.f90:226-228). */
int letkf_l96_obs_cell(int nx, int ny, const double* h, int* cell, void* stream);

/* ------------------------------------------------------------------------
 * Analysis sweep with the ensemble resident on the device.  Replaces the
 * das_letkf grid loop of the SCALE-style drivers (scale/letkf/letkf_tools.f90:
 * 38-476: obs_local + letkf_core(..., transm=, rdiag_wloc=.true., minfl=) +
 * the ensemble update with beta = 1) and the MPI scatter / gather around it
 * (scale/common/common_mpi_scale.f90): one handle owns the points, the
 * bucket-sorted observations (scale/letkf/letkf_obs.f90:735-830, sorted on
 * the device), the background and analysis ensembles and the inflation field.
 * Calls on one handle are serialised by the caller; distinct handles are
 * independent.
 * ---------------------------------------------------------------------- */
#define LETKF_PREC_F64 0   /* FP64 plain form */
#define LETKF_PREC_MIXED 1 /* FP32 ensemble, fused mixed-precision sweep */

#define LETKF_OPT_GRID_CAP 1   /* cap on the persistent grid (0 = #SM x occupancy) */
#define LETKF_OPT_MAX_SWEEPS 2 /* Jacobi sweep limit of the mixed form (default 12) */
#define LETKF_OPT_EIGENSOLVER 3 /* transform of the mixed form: */
#define LETKF_EIG_NEWTON_SCHULZ 0 /*   W = sqrt((k-1)) A^(-1/2) by Newton-Schulz (default) */
#define LETKF_EIG_JACOBI 1        /*   eigen-decomposition by parallel Jacobi */
#define LETKF_OPT_TENSOR_CORES 4  /* 1 (default): Gram and Newton-Schulz on tcgen05 for ne <= 128 (ne <= 64: four
                                     CTAs per SM; 64 < ne <= 128: one CTA of 256 threads per SM); 0: the FP32 SIMT
                                     sweep */
#define LETKF_OPT_TC_NS_ITERS 5   /* tensor-core Newton-Schulz iterations before the FP32 ones (default 14) */
#define LETKF_OPT_TC_NS_SCALING 6 /* 1 (default): spectrum-scaled tensor-core Newton-Schulz steps; 0: plain */
#define LETKF_OPT_TC_NS_TOL 7     /* v: the tensor-core phase ends once ||ZY - I||_F^2 < 10^-v (1..7, default 3) */
#define LETKF_OPT_POLISH_TOL 8    /* v: the FP32 polish takes its last step once ||Z A Z / s - I||_F^2 < 10^-v (4..12, default 7) */
#define LETKF_OPT_GRAPH 9         /* 1 (default): the mixed-form run is a CUDA graph, replayed while arguments stay the same */
#define LETKF_OPT_TC_POLISH 10    /* 1: the anchored polish step of the tensor-core sweep on the tensor cores; 0 (default): FP32 */
#define LETKF_OPT_TC_SCALE_BOUND 11 /* 1 (default): tensor-core scale s = min(||A||_F, Gershgorin), every step scaled; 0: power iteration */
#define LETKF_OPT_POLISH_PROBE 12  /* tensor-core sweep, v > 0 (default 9): a point skips the FP32 polish when
                                      ||Z (A/s) Z p - p||^2 < 10^-v ||p||^2 for a fixed pseudo-random p (three matvecs
                                      against the exact A); 0: every point polished */
#define LETKF_OPT_NS_COND 13       /* v > 0 (default 5): Newton-Schulz only where the spectrum bound s / c < 10^v, other
                                      points go to the Jacobi pass; 0: no bound.  Either way a point whose transform is
                                      not certified (no convergence, a large anchored residual) goes to the Jacobi pass */
#define LETKF_OPT_MAX_NOBS_PER_GRID 14 /* M > 0: MAX_NOBS_PER_GRID selection (scale/letkf/letkf_tools.f90:1041-1156)
                                      with the groups of letkf_sweep_set_obs_groups; the run then searches each piece
                                      of the processing order first (letkf_search_scale_limited) and analyses it from
                                      the lists (no CUDA graph); 0 (default): no limit */
#define LETKF_OPT_GRID_SHARE 16    /* v >= 1: each persistent sweep launch takes 1/v of the CTAs its kernel can keep
                                      resident (the server's slots share the SMs this way); replaces a grid cap */
#define LETKF_OPT_COLUMN_UNIT 17   /* where the points come in columns (equal ri, rj; the levels of a grid column), a
                                      tensor-core CTA (ne <= 128) takes v consecutive order positions at a time and keeps
                                      the search's horizontal candidates of its column for the next levels, which apply
                                      only the vertical test (same lists, order and weights); v >= 1, or -1 (default):
                                      the mean column length of the points; 0: off */
#define LETKF_OPT_FAULT_WAIT 15    /* failure injection, v > 0: the next mixed-form runs on the tensor-core sweep
                                      wait on a barrier that nothing arrives at and give up after v polls, so the
                                      run reports LETKF_ERR_TIMEOUT and analyses nothing; 0 (default): off */

typedef struct letkf_sweep_desc {
  int ne;           /* ensemble size (MEMBER) */
  int nv;           /* variables updated with each point's weights (1..8) */
  int nlon, nlat;   /* observation bucket grid (grid-index space, 1-based cells) */
  int npts;         /* analysed grid points */
  int precision;    /* LETKF_PREC_F64 or LETKF_PREC_MIXED */
  double params[16];/* SCALE search parameters in the order of letkf_search_scale */
  double minfl;     /* INFL_MUL_MIN; <= 0 absent */
} letkf_sweep_desc;

typedef struct letkf_sweep_s* letkf_sweep_t;

int letkf_sweep_create(letkf_sweep_t* h, const letkf_sweep_desc* desc);
int letkf_sweep_destroy(letkf_sweep_t h);
/* grid points (host arrays [npts]): ri, rj grid coordinates, rlev pressure,
 * rz height (may be NULL); tile > 0 orders processing in tile x tile columns */
int letkf_sweep_set_points(letkf_sweep_t h, const double* ri, const double* rj, const double* rlev,
                           const double* rz, int tile);
/* observations (host, unsorted, QC-passed): grid coordinates, level, value,
 * error, departure, class (see letkf_search_scale), var_local column and row
 * (NULL: no variable localisation) and the obs-space perturbations
 * hdxf[nobs][ne] (float32 when hdxf_f32, else float64) */
int letkf_sweep_set_obs(letkf_sweep_t h, int nobs, const double* ri, const double* rj, const double* lev,
                        const double* dat, const double* err, const double* dep, const int* cls,
                        const int* varloc, const double* var_local_row, int nvarloc, const void* hdxf,
                        int hdxf_f32);
/* background members xb[nv][npts][ne] (float64 for LETKF_PREC_F64, float32
 * for LETKF_PREC_MIXED); host or device pointer.  A device source is copied
 * after the work queued on the legacy default stream (and on the streams that
 * synchronise with it) has finished, so data written there need no extra
 * synchronisation; data written on a non-blocking stream must be complete. */
int letkf_sweep_set_background(letkf_sweep_t h, const void* xb, int on_device);
int letkf_sweep_set_inflation(letkf_sweep_t h, const double* infl, int on_device);
int letkf_sweep_set_option(letkf_sweep_t h, int option, int value);
/* analyse every point; asynchronous on `stream` (NULL: the handle's stream) */
int letkf_sweep_run(letkf_sweep_t h, void* stream);
/* One analysis from host buffers with the copies overlapped: the processing
 * order is cut into nchunks pieces; the background rows a piece reads go in
 * on a copy stream while earlier pieces are analysed on `stream`, and analysis
 * rows go out on a second copy stream once every point below them is done.
 * xb and xa are host arrays [nv][npts][ne] as in letkf_sweep_set_background /
 * letkf_sweep_get_analysis; the result equals those two calls around
 * letkf_sweep_run bit for bit.  Returns when xa holds the analysis.
 * Page-locked host buffers let the copies run beside the analysis.  The
 * plain form and nchunks = 1 run the three calls in sequence; the points
 * must be set (LETKF_ERR_ARG otherwise). */
int letkf_sweep_run_host(letkf_sweep_t h, const void* xb, void* xa, int nchunks, void* stream);
/* Autotuner of the mixed form: times every kernel / eigensolver variant the
 * handle can run (tensor-core sweep with spectrum-scaled or plain
 * Newton-Schulz steps when ne <= 64; SIMT sweep with Newton-Schulz or
 * parallel Jacobi) on the first `sample_points` points of the processing
 * order, with the points, observations and background already set, and
 * keeps the fastest.  The inflation field is restored afterwards; the
 * analysis buffer is overwritten.  choice[4] (may be NULL) receives
 * {tensor cores, Newton-Schulz (0: Jacobi), scaled steps, microseconds per
 * 1000 points of the winner}.  The plain form has nothing to tune. */
int letkf_sweep_autotune(letkf_sweep_t h, int sample_points, int* choice);
int letkf_sweep_get_analysis(letkf_sweep_t h, void* xa, int on_device);
/* points the last mixed-form run handed from the Newton-Schulz transform to the
 * Jacobi pass (spectrum bound beyond the option, or a transform that did not
 * certify); waits for the handle's stream.  0 for the plain form. */
int letkf_sweep_deferred(letkf_sweep_t h, int* count);
/* per-point updated inflation, local obs count, status and Jacobi sweeps (any may be NULL) */
int letkf_sweep_get_diagnostics(letkf_sweep_t h, double* infl, int* nobsl, int* status, int* sweeps);
/* the device-side nobsgrd table [(nlon+1)*nlat] after set_obs */
int letkf_sweep_sorted_obs(letkf_sweep_t h, int* nobsgrd);
/* device pointers of the resident buffers (for callers that stage data themselves) */
int letkf_sweep_device_buffers(letkf_sweep_t h, void** xb, void** xa, double** infl, int** nobsl);
/* Observation groups of the MAX_NOBS_PER_GRID limit, after set_obs (input
 * order, host arrays [nobs]): element uid 1..nid and type 1..ntyp (the
 * reference's uid_obs(elm) and obs%typ). */
int letkf_sweep_set_obs_groups(letkf_sweep_t h, const int* uid, const int* typ, int nid, int ntyp);
/* Selection probe (checks the fused search of the mixed-form sweeps): for
 * the npts_probe grid points points[] (host, point indices) the next runs
 * also record what their search accepted, in the order it enters the Gram:
 * up to cap entries per point.  npts_probe = 0 switches the probe off.  The
 * probe adds stores only; the analysis is unchanged. */
int letkf_sweep_set_probe(letkf_sweep_t h, int npts_probe, const int* points, int cap);
/* after a run: count[npts_probe] accepted observations per probed point (may
 * exceed cap), obs[npts_probe * cap] their indices in the observation input
 * order of letkf_sweep_set_obs, rloc[npts_probe * cap] the FP32 localisation
 * weights (either array may be NULL); host arrays */
int letkf_sweep_get_probe(letkf_sweep_t h, int* count, int* obs, float* rloc);
/* upper bound of the device bytes a handle with this descriptor and nobs
 * observations holds, including the staging of set_obs and run */
int letkf_sweep_footprint(const letkf_sweep_desc* desc, int nobs, size_t* bytes);

/* ------------------------------------------------------------------------
 * Serving: analysis jobs for domains of different sizes and ensemble sizes,
 * submitted as they arrive and run with continuous batching on one device.
 * No counterpart in the reference (its drivers analyse one domain per run).
 *   - nslots jobs are on the device at once, each on its own stream with
 *     1/nslots of the SMs for the sweep kernels, so a job that arrives while
 *     others run starts as soon as a slot and memory are free and overlaps
 *     with them;
 *   - admission is by device footprint (letkf_sweep_footprint and the L96
 *     equivalent) against hbm_budget, in arrival order;
 *   - jobs with the same domain key >= 0 reuse that domain's device state
 *     (points, observations and ensemble buffers stay resident between jobs);
 *     idle resident domains are released oldest first when memory is needed;
 *   - host buffers of a job must stay valid until the job is finished.
 * ---------------------------------------------------------------------- */
#define LETKF_PENDING 7            /* a job that has not finished */
#define LETKF_JOB_SCALE_SWEEP 0    /* regional sweep (letkf_sweep_* semantics) */
#define LETKF_JOB_L96 1            /* Lorenz-96 ring (letkf_search_l96 + core + update) */

typedef struct letkf_server_desc {
  int device;         /* CUDA device ordinal */
  int nslots;         /* jobs on the device at once, 1..16 */
  size_t hbm_budget;  /* device bytes for jobs and resident domains; 0: 80% of free memory */
} letkf_server_desc;

typedef struct letkf_job_desc {
  int kind;           /* LETKF_JOB_SCALE_SWEEP or LETKF_JOB_L96 */
  int64_t domain;     /* resident-domain key (>= 0), or -1: release the device state after the job */
  int precision;      /* LETKF_PREC_F64 or LETKF_PREC_MIXED */
  int ne, nv;
  /* grid points: SCALE sweep (nlon x nlat bucket grid, npts points) or the
   * L96 ring (npts = nx, nv = 1; pri/prj/prlev unused) */
  int nlon, nlat, npts;
  const double *pri, *prj, *prlev;
  double params[16];  /* SCALE search parameters (letkf_search_scale order) */
  double minfl;
  /* observations: SCALE records (unsorted), or for L96 obs_cell[nobs] */
  int nobs;
  const double *ori, *orj, *olev, *odat, *oerr;
  const int* ocls;
  const int* obs_cell;
  double xlocal, obserr, msw_infl; /* L96 localisation, obs error, fixed inflation (> 0) */
  const double* dep;  /* [nobs] departures */
  const void* hdxf;   /* [nobs][ne]: float32 (SCALE, MIXED) else float64 */
  /* ensemble [nv][npts][ne]: float32 (SCALE, MIXED) else float64; in / out */
  const void* xb;
  void* xa;
  double* infl;       /* [npts] adaptive inflation in / out, may be NULL (1.0) */
} letkf_job_desc;

typedef struct letkf_job_result {
  int status;         /* LETKF_OK, LETKF_PENDING or an error */
  double t_submit, t_start, t_done;  /* seconds since the server started */
  size_t device_bytes;               /* footprint charged to the job */
} letkf_job_result;

typedef struct letkf_server_stats {
  int64_t submitted, completed, failed;
  double p50_latency_s, p99_latency_s;  /* submit -> done, completed jobs */
  double points_per_s;                  /* grid points of completed jobs / (last done - first submit) */
  size_t peak_bytes;                    /* largest charged footprint in use at once */
  int resident_domains;
} letkf_server_stats;

typedef struct letkf_server_s* letkf_server_t;

int letkf_server_create(letkf_server_t* server, const letkf_server_desc* desc);
/* copies the descriptor (not the arrays) and queues the job; *job_id >= 0 */
int letkf_server_submit(letkf_server_t server, const letkf_job_desc* job, int64_t* job_id);
/* waits up to timeout_s (< 0: no limit) for the job; LETKF_PENDING on timeout.
 * Once it has returned a finished job's result the job's record is released:
 * a later wait on that id returns LETKF_ERR_ARG. */
int letkf_server_wait(letkf_server_t server, int64_t job_id, double timeout_s, letkf_job_result* result);
int letkf_server_stats_get(letkf_server_t server, letkf_server_stats* stats);
/* finishes every queued job, then releases the device state */
int letkf_server_destroy(letkf_server_t server);

/* exclusive scan of n int32 counts into int64 offsets[n+1] (device) */
int letkf_exclusive_scan(int n, const int* counts, int64_t* offs, void* stream);

/* Allocation-free exclusive scan.  No counterpart in the reference: it exists
 * for callers that must not allocate device memory (a Fortran driver whose
 * device memory comes from its own pool, code under a fixed memory budget).
 * Same result as letkf_exclusive_scan, but its scratch is a 128 KiB device
 * array inside the library instead of an allocation.
 *   - n <= LETKF_SCAN_STATIC_MAX_N, else LETKF_ERR_CAPACITY;
 *   - the first call on a device looks up that array's device address, so
 *     make it before any stream capture; the address is kept for the life of
 *     the process and is not valid after cudaDeviceReset of that device;
 *   - every call shares the array: calls that overlap on the GPU (other
 *     streams, other threads) race, so serialise them. */
#define LETKF_SCAN_STATIC_MAX_N (16 * 1024 * 1024)
int letkf_exclusive_scan_static(int n, const int* counts, int64_t* offs, void* stream);

/* gather packed local rows: rows_out[r][ne] = ens[idx[r]][ne] (double or
 * float via elem_bytes 8/4), dep_out[r] = dep[idx[r]] */
int letkf_gather_rows(int ne, int64_t nrows, const int* idx, const void* ens, const void* dep,
                      int elem_bytes, void* rows_out, void* dep_out, void* stream);

#ifdef __cplusplus
}
#endif
#endif
