/*
 * letkf_oracle.h -- CPU FP64 restatement of the reference LETKF analysis path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle of the CUDA path:
 * only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg / the
 * reference arm may load it.  The product path never calls into it.
 *
 * Parity status: UNPINNED against the reference itself.  The reference is
 * Fortran (takemasa-miyoshi/letkf), no Fortran compiler exists on either
 * machine, and the reference ships no tests, fixtures or golden outputs.
 * The restatement is pinned instead by known-answer tests from the maths
 * (nobsl=0 branch, column sums of W, 1^T wbar = 0, single-observation closed
 * form, agreement with the dense Kalman-gain posterior) and by an independent
 * LAPACK eigensolver cross-check.
 *
 * Every routine follows the reference loop order so that rounding matches a
 * gfortran build without FMA contraction (this file is compiled with
 * -ffp-contract=off).  Arrays are column-major with the reference's leading
 * dimensions; indices in the API are 0-based.
 */
#ifndef LETKF_ORACLE_H
#define LETKF_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* ---- numerics (common/netlibrs.f, common/common_mtx.f90, common/common_letkf.f90) ---- */
double oracle_pythag(double a, double b);
void oracle_tred2(int nm, int n, const double* a, double* d, double* e, double* z);
int oracle_tql2(int nm, int n, double* d, double* e, double* z);
int oracle_rs(int nm, int n, double* a, double* w, int matz, double* z, double* fv1, double* fv2);
/* returns 0 ok, 2 on the reference's STOP 2 conditions */
int oracle_mtx_eigen(int imode, int n, const double* a, double* eival, double* eivec, int* nrank_eff);
/* DGEMM('T','N') and DGEMM('N','T') with alpha=1, beta=0 (common/netlibblas.f loop order) */
void oracle_dgemm_tn(int m, int n, int k, const double* a, int lda, const double* b, int ldb, double* c, int ldc);
void oracle_dgemm_nt(int m, int n, int k, const double* a, int lda, const double* b, int ldb, double* c, int ldc);

/* letkf_core (common/common_letkf.f90:50-243).  transm, pao may be NULL
 * (absent); minfl may be NULL (absent).  Returns 0 ok, 2 eigensolver STOP,
 * 1 bad argument. */
int oracle_letkf_core(int ne, int nobs, int nobsl, const double* hdxb, const double* rdiag,
                      const double* rloc, const double* dep, double* parm_infl, double* trans,
                      double* transm, double* pao, int rdiag_wloc, const double* minfl);

/* Batched helper: npts points, each with a packed local-obs block (rows
 * offs[p]..offs[p+1]-1 of hdxb_rows, row-major [row][ne]).  Runs
 * oracle_letkf_core per point with OpenMP schedule(dynamic).  Outputs are
 * packed per point: trans[p*ne*ne] (col-major), transm[p*ne] (may be NULL),
 * pao (may be NULL).  status[p] gets each point's code. */
int oracle_letkf_core_batch(int ne, int npts, const int64_t* offs, const double* hdxb_rows,
                            const double* rdiag, const double* rloc, const double* dep,
                            double* parm_infl, double* trans, double* transm, double* pao,
                            int rdiag_wloc, double minfl, int nthreads, int* status);

/* ---- utilities (common/common.f90) ---- */
void oracle_com_distll_1(double alon, double alat, double blon, double blat, double* dist);

/* ---- SPEEDY lat/lon search (speedy/letkf/letkf_obs.f90, letkf_tools.f90) ---- */
/* Stable bucket sort of observations by latitude band then longitude cell.
 * lon[nlon], lat[nlat] grid axes.  perm[] receives, for each sorted slot, the
 * input obs index; nobsgrd[nlon*nlat] (column-major, i fastest) receives the
 * cumulative counts.  Returns the number of placed observations. */
int oracle_speedy_sort_obs(int nlon, int nlat, const double* lon, const double* lat, int nobs,
                           const double* obslon, const double* obslat, int* perm, int* nobsgrd);

typedef struct {
  int nlon, nlat;
  const double* lon;     /* [nlon] */
  const double* lat;     /* [nlat] */
  const int* nobsgrd;    /* [nlon*nlat] */
  int nobs;              /* number of sorted observations */
  const double* obselm;  /* sorted obs records [nobs] */
  const double* obslon;
  const double* obslat;
  const double* obslev;
  const double* obsdat;
  const double* obserr;
  double dist_zero, dist_zerov, dlat_zero, sigma_obs, sigma_obsv;
  const double* var_local; /* [7] row of var_local for this nvar: u,v,t,q,rh,ps,rain */
} oracle_speedy_obs;

/* obs_local for one (ij, ilev, nvar): returns nobsl, fills idx[] (0-based
 * sorted obs index, in the reference order), rloc[], rdiag[].  Returns -1 on
 * an unknown element id. */
int oracle_speedy_obs_local(const oracle_speedy_obs* o, double lon1, double lat1, double dlon_zero,
                            int ilev, double logpfm, int* idx, double* rloc, double* rdiag);

/* GFS obs_local (gfs/letkf/letkf_tools.f90:686-925) on the SPEEDY bucket layout */
typedef struct {
  double dist_zero, dist_zerov, dist_zero_rain, dist_zerov_rain;
  double sigma_obs, sigma_obsv, sigma_obs_rain, base_obsv_rain;
  const double* var_local; /* [6] (u/v, t/tv, q/rh, ps, rain, tc) or NULL */
} oracle_gfs_params;
int oracle_gfs_obs_local(const oracle_speedy_obs* o, const oracle_gfs_params* g, double rlon, double rlat,
                         double rlev, int* idx, double* rloc, double* rdiag);

/* ---- SCALE Cartesian search (scale/letkf/letkf_obs.f90, letkf_tools.f90) ---- */
/* obs classes used for the vertical / horizontal scale switch */
enum { ORC_CLS_DEFAULT = 0, ORC_CLS_PS = 1, ORC_CLS_RAIN = 2, ORC_CLS_RADAR_REF = 3,
       ORC_CLS_RADAR_VR = 4, ORC_CLS_RADAR_PRH = 5, ORC_CLS_TC = 6 };

/* Bucket sort by grid cell (scale/letkf/letkf_obs.f90:735-830), single subdomain.
 * obs_ri/obs_rj are grid coordinates (1-based), ihalo/jhalo subtracted as in
 * the reference.  perm[slot] = input index; nobsgrd[(nlon+1)*nlat] is the
 * 0:nlon x 1:nlat cumulative table (i fastest). */
void oracle_scale_sort_obs(int nlon, int nlat, int ihalo, int jhalo, int nobs, const double* obs_ri,
                           const double* obs_rj, int* perm, int* nobsgrd);

typedef struct {
  int nlon, nlat;
  const int* nobsgrd;     /* [(nlon+1)*nlat] */
  int nobs;
  const double* ri;       /* sorted obs arrays [nobs] */
  const double* rj;
  const double* lev;
  const double* dat;
  const double* err;
  const int* cls;         /* ORC_CLS_* per obs */
  const int* uid;         /* 0-based unique element id per obs (group index)   */
  const int* typ;         /* 0-based obs type per obs                          */
  const int* varloc_idx;  /* 0-based column of var_local per obs               */
  int nid, ntyp;
  double dx, dy, dlon_zero, dlat_zero;
  double sigma_obs, sigma_obsv, sigma_obs_rain, sigma_obsv_rain, base_obsv_rain;
  double sigma_obs_radar, sigma_obs_radar_noref, sigma_obsz_radar, radar_ref_thres_dbz;
  double sigma_obs_tc, sigma_obsv_tc;
  const double* var_local; /* row for this nvar [nvarloc], NULL when nvar <= 0 */
  int max_nobs_per_grid;  /* <=0 disables the limit */
} oracle_scale_obs;

int oracle_scale_obs_local(const oracle_scale_obs* o, double ri, double rj, double rlev, double rz,
                           int* idx, double* rloc, double* rdiag);

/* SCALE cutoff constants as the reference declares them (default-real literals) */
double oracle_scale_dist_zero_fac(void);
double oracle_scale_dist_zero_fac_square(void);

/* ---- Lorenz-96 selection (lorenz96/letkf/letkf.f90:220-254), nwindow=1 ---- */
int oracle_l96_select(int nx, int ny, const double* h /* ny x nx col-major */, int ix, double xlocal,
                      double tlocal, int* idx, double* rloc);
int oracle_l96_select_4d(int nx, int ny, int nslot, const double* h, int slot, int ix, double xlocal, double tlocal,
                         int* idx, double* rloc);
double oracle_com_correl(int n, const double* v1, const double* v2);
int oracle_l96_select_adaptive(int nx, int ny, int nslot, const double* h, const double* hdxf, const double* dxf,
                               int ne, int slot, int ix, double xlocal, double tlocal, int msw_local, double sa,
                               double sb, int* idx, double* rloc);

/* ---- sweeps (das_letkf loops) ---- */
/* Ensemble mean and perturbation, sequential member sum
 * (speedy/common/common_speedy.f90:335-370).  x is [npts][ne] row-major. */
void oracle_ensmean(int npts, int ne, const double* x, double* mean, double* pert);

/* SCALE-style grid loop over npts points (or the `subset` of nsub of them):
 * obs_local + letkf_core(transm, rdiag_wloc) + update of nv variables.
 * hdxf[nobs][ne] and odep[nobs] are in the sorted obs order; xb, xa are
 * [nv][npts][ne]; infl[npts] in/out.  Returns the number of failed points. */
int oracle_scale_sweep(const oracle_scale_obs* o, const double* hdxf, const double* odep, int ne, int nv, int npts,
                       const int* subset, int nsub, const double* pri, const double* prj, const double* prlev,
                       const double* prz, const double* xb, double* xa, double* infl, int* nobsl_out,
                       double minfl, int nthreads);

/* obs_local of npts points (OpenMP over points): cnt[p] = nobsl and the first
 * min(nobsl, cap) sorted indices and rloc in rows of cap entries */
int oracle_scale_obs_local_batch(const oracle_scale_obs* o, int npts, const double* pri, const double* prj,
                                 const double* prlev, const double* prz, int cap, int* cnt, int* idx_out,
                                 double* rloc_out, int nthreads);

/* relax_beta / RTPP / RTPS (scale/letkf/letkf_tools.f90:1182-1268) */
void oracle_weight_rtpp(int ne, const double* w, double alpha, double* wrlx);
void oracle_weight_rtps(int ne, const double* w, const double* pa, const double* xb, double alpha,
                        double* wrlx, double* infl);
double oracle_obs_analysis(int ne, const double* trans, double ybar, const double* hdxf, int mode,
                           double q_sprd_max, double* anal);
void oracle_efso(int ne, int npts, int nv, int nterm, const int64_t* offs, const int* idx, const double* rdiag,
                 const double* rloc, const double* hdxa, const double* fcst, const double* fcer, const int* term,
                 int nobs, const double* obsdep, double* djdy, double* obsense);


/* SCALE observation operator for conventional observations
 * (scale/obs/obsope_tools.f90:340-380, scale/common/common_obs_scale.f90:
 * 262-334, 969-1075): per (observation, member) phys2ijk then Trans_XtoY;
 * hx[n][m], qc_member[n][m] (may be NULL), qc[n] = the maximum over members
 * (may be NULL).  Layout in obs_operator_scale.c. */
int oracle_scale_obsope(int nlonh, int nlath, int nlev, int khalo, int ne, const double* v3d, int64_t v3d_mem,
                        int64_t v3d_var, const double* v2d, int64_t v2d_mem, int64_t v2d_var, int nobs,
                        const int* elem, const double* ri, const double* rj, const double* rlev, const double* rotc,
                        int stggrd, double ps_thres, double* hx, int* qc_member, int* qc);

/* SPEEDY observation operator (speedy/letkf/obsope.f90:53-104 with phys2ijk,
 * Trans_XtoY, calc_rh, itpl_2d/3d of speedy/common/common_obs_speedy.f90) */
double oracle_speedy_calc_rh(double t, double q, double p);
int oracle_speedy_obsope(int nlon, int nlat, int nlev, int ne, const double* lat, const double* sig,
                         const double* v3d, int64_t v3d_mem, int64_t v3d_rec, const double* v2d, int64_t v2d_mem,
                         int64_t v2d_rec, int nobs, const int* elem, const double* rlon, const double* rlat,
                         const double* rlev, const double* odat, double* hx, int* qc_member, int* qc);

#ifdef __cplusplus
}
#endif
#endif
