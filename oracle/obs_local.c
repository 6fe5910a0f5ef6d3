/*
 * obs_local.c -- CPU restatement of the reference local-observation search.
 * TEST INFRASTRUCTURE ONLY (the oracle of the CUDA search; never shipped).
 * Parity unpinned against the Fortran itself (no compiler, no golden data).
 *
 * Selected-observation lists and their order are the reference's; the CUDA
 * search must reproduce them bit-exactly.
 */
#include "letkf_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* common/common.f90:28,35 */
static const double PI = 3.1415926535;
static const double RE = 6371.3e3;

/* common/common.f90:401-424 */
void oracle_com_distll_1(double alon, double alat, double blon, double blat, double* dist) {
  const double r180 = 1.0 / 180.0;
  double lon1 = alon * PI * r180;
  double lon2 = blon * PI * r180;
  double lat1 = alat * PI * r180;
  double lat2 = blat * PI * r180;
  double cosd = sin(lat1) * sin(lat2) + cos(lat1) * cos(lat2) * cos(lon2 - lon1);
  cosd = fmin(1.0, cosd);
  cosd = fmax(-1.0, cosd);
  *dist = acos(cosd) * RE;
}

/* speedy/letkf/letkf_obs.f90:243-313.  Band j (1..nlat-1) holds
 * lat(j) <= obslat < lat(j+1); within a band, cell i holds lon(i) <= obslon <
 * lon(i+1) (cell nlon: lon(nlon) <= obslon < 360).  Input order is kept
 * inside each cell.  nobsgrd(:,nlat) stays 0 as in the reference. */
int oracle_speedy_sort_obs(int nlon, int nlat, const double* lon, const double* lat, int nobs,
                           const double* obslon, const double* obslat, int* perm, int* nobsgrd) {
  int* nj = (int*)calloc((size_t)nlat + 1, sizeof(int)); /* nj(0:nlat-1) -> index j */
  int* njs = (int*)calloc((size_t)nlat + 1, sizeof(int));
  int* band = (int*)malloc(sizeof(int) * (size_t)(nobs > 0 ? nobs : 1));
  int i, j, n, nn, placed = 0;
  memset(nobsgrd, 0, sizeof(int) * (size_t)nlon * nlat);
  for (j = 1; j <= nlat - 1; j++)
    for (n = 0; n < nobs; n++) {
      if (obslat[n] < lat[j - 1] || lat[j] <= obslat[n]) continue;
      nj[j] += 1;
    }
  for (j = 1; j <= nlat - 1; j++) {
    int s = 0;
    for (i = 0; i <= j - 1; i++) s += nj[i];
    njs[j] = s;
  }
  for (j = 1; j <= nlat - 1; j++) {
    nn = 0;
    for (n = 0; n < nobs; n++) {
      if (obslat[n] < lat[j - 1] || lat[j] <= obslat[n]) continue;
      band[njs[j] + nn] = n; /* tmp2 arrays */
      nn++;
    }
  }
  for (j = 1; j <= nlat - 1; j++) {
    if (nj[j] == 0) {
      for (i = 1; i <= nlon; i++) nobsgrd[(size_t)(j - 1) * nlon + (i - 1)] = njs[j];
      continue;
    }
    nn = 0;
    for (i = 1; i <= nlon; i++) {
      for (n = njs[j]; n < njs[j] + nj[j]; n++) {
        double x = obslon[band[n]];
        if (i < nlon) {
          if (x < lon[i - 1] || lon[i] <= x) continue;
        } else {
          if (x < lon[nlon - 1] || 360.0 <= x) continue;
        }
        perm[njs[j] + nn] = band[n];
        nn++;
      }
      nobsgrd[(size_t)(j - 1) * nlon + (i - 1)] = njs[j] + nn;
    }
    placed += nn;
  }
  free(nj); free(njs); free(band);
  return placed;
}

/* speedy/letkf/letkf_tools.f90:575-603 */
static void obs_local_sub(const oracle_speedy_obs* o, int imin, int imax, int jmin, int jmax, int* nn,
                          int* nobs_use) {
  int j, ib, ie, ip;
  const int nlon = o->nlon;
#define NOBSGRD(i, j) o->nobsgrd[(size_t)((j)-1) * nlon + ((i)-1)]
  for (j = jmin; j <= jmax; j++) {
    if (imin > 1) ib = NOBSGRD(imin - 1, j) + 1;
    else if (j > 1) ib = NOBSGRD(nlon, j - 1) + 1;
    else ib = 1;
    ie = NOBSGRD(imax, j);
    if (ie - ib + 1 == 0) continue;
    for (ip = ib; ip <= ie; ip++) {
      nobs_use[*nn - 1] = ip; /* 1-based obs index */
      *nn += 1;
    }
  }
#undef NOBSGRD
}

/* Fortran "DO idx=1,lim; IF(x < axis(idx+1)) EXIT; END DO": first idx with
 * x < axis(idx+1), else lim+1. */
static int first_below(double x, const double* axis, int lim) {
  int idx;
  for (idx = 1; idx <= lim; idx++)
    if (x < axis[idx]) return idx; /* axis(idx+1), 0-based axis[idx] */
  return lim + 1;
}

/* SPEEDY element ids (speedy/common/common_obs_speedy.f90:18-24) */
#define ID_U 2819
#define ID_V 2820
#define ID_T 3073
#define ID_Q 3330
#define ID_RH 3331
#define ID_PS 14593
#define ID_RAIN 9999

/* speedy/letkf/letkf_tools.f90:272-573 */
/* the candidate box of a point (speedy/letkf/letkf_tools.f90:297-452, the
 * same steps as gfs/letkf/letkf_tools.f90:709-825): sorted-observation
 * indices (1-based) into nobs_use, returns their number */
static int collect_box(const oracle_speedy_obs* o, double lon1, double lat1, double dlon_zero, double dlat_zero,
                       int* nobs_use) {
  const int nlon = o->nlon, nlat = o->nlat;
  const double* lon = o->lon;
  const double* lat = o->lat;
  double minlon, maxlon, minlat, maxlat;
  int imin, imax, jmin, jmax, nn;
  minlon = lon1 - dlon_zero;
  maxlon = lon1 + dlon_zero;
  minlat = lat1 - dlat_zero;
  maxlat = lat1 + dlat_zero;
  if (maxlon - minlon >= 360.0) {
    minlon = 0.0;
    maxlon = 360.0;
  }
  jmin = first_below(minlat, lat, nlat - 2);
  jmax = first_below(maxlat, lat, nlat - 2);
  nn = 1;
  if (minlon >= 0 && maxlon <= 360.0) {
    imin = first_below(minlon, lon, nlon - 1);
    imax = first_below(maxlon, lon, nlon - 1);
    obs_local_sub(o, imin, imax, jmin, jmax, &nn, nobs_use);
  } else if (minlon >= 0 && maxlon > 360.0) {
    imin = first_below(minlon, lon, nlon - 1);
    maxlon = maxlon - 360.0;
    if (maxlon > 360.0) {
      imin = 1;
      imax = nlon;
      obs_local_sub(o, imin, imax, jmin, jmax, &nn, nobs_use);
    } else {
      imax = first_below(maxlon, lon, nlon - 1);
      if (imax > imin) {
        imin = 1;
        imax = nlon;
        obs_local_sub(o, imin, imax, jmin, jmax, &nn, nobs_use);
      } else {
        imin = 1;
        obs_local_sub(o, imin, imax, jmin, jmax, &nn, nobs_use);
        imin = first_below(minlon, lon, nlon - 1);
        imax = nlon;
        obs_local_sub(o, imin, imax, jmin, jmax, &nn, nobs_use);
      }
    }
  } else if (minlon < 0 && maxlon <= 360.0) {
    imax = first_below(maxlon, lon, nlon - 1);
    minlon = minlon + 360.0;
    if (minlon < 0) {
      imin = 1;
      imax = nlon;
      obs_local_sub(o, imin, imax, jmin, jmax, &nn, nobs_use);
    } else {
      imin = first_below(minlon, lon, nlon - 1);
      if (imin < imax) {
        imin = 1;
        imax = nlon;
        obs_local_sub(o, imin, imax, jmin, jmax, &nn, nobs_use);
      } else {
        imin = 1;
        obs_local_sub(o, imin, imax, jmin, jmax, &nn, nobs_use);
        imin = first_below(minlon, lon, nlon - 1);
        imax = nlon;
        obs_local_sub(o, imin, imax, jmin, jmax, &nn, nobs_use);
      }
    }
  } else {
    maxlon = maxlon - 360.0;
    minlon = minlon + 360.0;
    if (maxlon > 360.0 || minlon < 0) {
      imin = 1;
      imax = nlon;
      obs_local_sub(o, imin, imax, jmin, jmax, &nn, nobs_use);
    } else {
      imin = first_below(minlon, lon, nlon - 1);
      imax = first_below(maxlon, lon, nlon - 1);
      if (imin > imax) {
        imin = 1;
        imax = nlon;
        obs_local_sub(o, imin, imax, jmin, jmax, &nn, nobs_use);
      } else {
        obs_local_sub(o, imin, imax, jmin, jmax, &nn, nobs_use);
      }
    }
  }
  return nn - 1;
}

int oracle_speedy_obs_local(const oracle_speedy_obs* o, double lon1, double lat1, double dlon_zero,
                            int ilev, double logpfm, int* idx, double* rloc, double* rdiag) {
  double dist, dlev;
  int n, nn, iobs, nobsl;
  int* nobs_use;
  if (o->nobs <= 0) return 0;
  nobs_use = (int*)malloc(sizeof(int) * (size_t)o->nobs);
  nn = collect_box(o, lon1, lat1, dlon_zero, o->dlat_zero, nobs_use);
  nobsl = 0;
  for (n = 1; n <= nn; n++) {
    int ob = nobs_use[n - 1] - 1; /* 0-based sorted index */
    int elm = (int)lround(o->obselm[ob]);
    if (elm == ID_PS && ilev > 1) dlev = fabs(log(o->obsdat[ob]) - logpfm);
    else if (elm != ID_PS) dlev = fabs(log(o->obslev[ob]) - logpfm);
    else dlev = 0.0;
    if (dlev > o->dist_zerov) continue;
    oracle_com_distll_1(o->obslon[ob], o->obslat[ob], lon1, lat1, &dist);
    if (dist > o->dist_zero) continue;
    switch (elm) {
      case ID_U: iobs = 1; break;
      case ID_V: iobs = 2; break;
      case ID_T: iobs = 3; break;
      case ID_Q: iobs = 4; break;
      case ID_RH: iobs = 5; break;
      case ID_PS: iobs = 6; break;
      case ID_RAIN: iobs = 7; break;
      default: free(nobs_use); return -1;
    }
    if (o->var_local[iobs - 1] < 2.2250738585072014e-308 /* TINY(real(8)) */) continue;
    idx[nobsl] = ob;
    rdiag[nobsl] = o->obserr[ob] * o->obserr[ob];
    {
      double a = dist / o->sigma_obs, b = dlev / o->sigma_obsv;
      rloc[nobsl] = exp(-0.5 * (a * a + b * b)) * o->var_local[iobs - 1];
    }
    nobsl++;
  }
  free(nobs_use);
  return nobsl;
}

/* scale/letkf/letkf_obs.f90:29-30: default-real (single precision) literals
 * stored in real(8) parameters. */
double oracle_scale_dist_zero_fac(void) { return (double)3.651483717f; }
double oracle_scale_dist_zero_fac_square(void) { return (double)13.33333333f; }

/* Fortran CEILING(x-0.5) for the cell index (letkf_obs.f90:751-763) */
static int ceil_half(double x) { return (int)ceil(x - 0.5); }

/* scale/letkf/letkf_obs.f90:735-830, one subdomain (ij_g2l is the identity) */
void oracle_scale_sort_obs(int nlon, int nlat, int ihalo, int jhalo, int nobs, const double* obs_ri,
                           const double* obs_rj, int* perm, int* nobsgrd) {
  int n, i, j;
  const int ld = nlon + 1;
#define G(i, j) nobsgrd[(size_t)((j)-1) * ld + (i)]
  int* nnext = (int*)malloc(sizeof(int) * (size_t)ld * nlat);
  memset(nobsgrd, 0, sizeof(int) * (size_t)ld * nlat);
  for (n = 0; n < nobs; n++) {
    i = ceil_half(obs_ri[n]) - ihalo;
    j = ceil_half(obs_rj[n]) - jhalo;
    if (i < 1) i = 1;
    if (i > nlon) i = nlon;
    if (j < 1) j = 1;
    if (j > nlat) j = nlat;
    G(i, j) += 1;
  }
  for (j = 1; j <= nlat; j++) {
    if (j > 1) G(0, j) = G(nlon, j - 1);
    for (i = 1; i <= nlon; i++) G(i, j) = G(i - 1, j) + G(i, j);
  }
  for (j = 1; j <= nlat; j++)
    for (i = 1; i <= nlon; i++) nnext[(size_t)(j - 1) * ld + i] = G(i - 1, j) + 1;
  for (n = 0; n < nobs; n++) {
    i = ceil_half(obs_ri[n]) - ihalo;
    j = ceil_half(obs_rj[n]) - jhalo;
    if (i < 1) i = 1;
    if (i > nlon) i = nlon;
    if (j < 1) j = 1;
    if (j > nlat) j = nlat;
    perm[nnext[(size_t)(j - 1) * ld + i] - 1] = n;
    nnext[(size_t)(j - 1) * ld + i] += 1;
  }
  free(nnext);
#undef G
}

static int ifloor(double x) { return (int)floor(x); }
static int iceil(double x) { return (int)ceil(x); }

/* scale/letkf/letkf_tools.f90:853-1178 with obs_choose (letkf_obs.f90:1054-1119),
 * MEM_NP = 1 and PRC_NUM_X = PRC_NUM_Y = 1. */
int oracle_scale_obs_local(const oracle_scale_obs* o, double ri, double rj, double rlev, double rz,
                           int* idx, double* rloc, double* rdiag) {
  const int nlon = o->nlon, nlat = o->nlat, ld = nlon + 1;
  const int M = o->max_nobs_per_grid;
  const double dzf2 = oracle_scale_dist_zero_fac_square();
  int imin1, imax1, jmin1, jmax1, j, ip, nobsl = 0;
  int *isort_t = NULL, *iob_t = NULL, *nobsl_t = NULL;
  double *rdiag_t = NULL, *rloc_t = NULL;
  const size_t ngrp = (size_t)o->nid * o->ntyp;
  if (M > 0) {
    isort_t = (int*)calloc((size_t)M * ngrp, sizeof(int));
    iob_t = (int*)calloc((size_t)M * ngrp, sizeof(int));
    rdiag_t = (double*)calloc((size_t)M * ngrp, sizeof(double));
    rloc_t = (double*)calloc((size_t)M * ngrp, sizeof(double));
  }
  nobsl_t = (int*)calloc(ngrp, sizeof(int));
#define G(i, j) o->nobsgrd[(size_t)((j)-1) * ld + (i)]
#define GRP(u, t) ((size_t)(t) * o->nid + (u))
  imin1 = ifloor(ri - o->dlon_zero);
  if (imin1 < 1) imin1 = 1;
  imax1 = iceil(ri + o->dlon_zero);
  if (imax1 > nlon) imax1 = nlon;
  jmin1 = ifloor(rj - o->dlat_zero);
  if (jmin1 < 1) jmin1 = 1;
  jmax1 = iceil(rj + o->dlat_zero);
  if (jmax1 > nlat) jmax1 = nlat;
  if (o->nobs > 0 && G(nlon, nlat) > 0 && imin1 <= imax1 && jmin1 <= jmax1) {
    for (j = jmin1; j <= jmax1; j++) {
      for (ip = G(imin1 - 1, j) + 1; ip <= G(imax1, j); ip++) {
        int ob = ip - 1;
        int vl = o->varloc_idx[ob];
        double nd_h, nd_v, ndist, nrloc, nrdiag, rdx, rdy;
        if (o->var_local) {
          if (o->var_local[vl] < 2.2250738585072014e-308 /* TINY(real(8)) */) continue;
        }
        rdx = (ri - o->ri[ob]) * o->dx;
        rdy = (rj - o->rj[ob]) * o->dy;
        nd_h = sqrt(rdx * rdx + rdy * rdy);
        switch (o->cls[ob]) {
          case ORC_CLS_PS:
            nd_h = nd_h / o->sigma_obs;
            nd_v = fabs(log(o->dat[ob]) - log(rlev)) / o->sigma_obsv;
            break;
          case ORC_CLS_RAIN:
            nd_h = nd_h / o->sigma_obs_rain;
            nd_v = fabs(log(o->base_obsv_rain) - log(rlev)) / o->sigma_obsv_rain;
            break;
          case ORC_CLS_RADAR_REF:
          case ORC_CLS_RADAR_VR:
          case ORC_CLS_RADAR_PRH:
            if (o->cls[ob] == ORC_CLS_RADAR_REF && o->dat[ob] <= o->radar_ref_thres_dbz + 1.0e-6)
              nd_h = nd_h / o->sigma_obs_radar_noref;
            else
              nd_h = nd_h / o->sigma_obs_radar;
            nd_v = fabs(o->lev[ob] - rz) / o->sigma_obsz_radar;
            break;
          case ORC_CLS_TC:
            nd_h = nd_h / o->sigma_obs_tc;
            nd_v = fabs(log(o->lev[ob]) - log(rlev)) / o->sigma_obsv_tc;
            break;
          default:
            nd_h = nd_h / o->sigma_obs;
            nd_v = fabs(log(o->lev[ob]) - log(rlev)) / o->sigma_obsv;
        }
        ndist = nd_h * nd_h + nd_v * nd_v;
        if (ndist > dzf2) continue;
        nrloc = exp(-0.5 * ndist);
        if (o->var_local) nrloc = nrloc * o->var_local[vl];
        nrdiag = o->err[ob] * o->err[ob] / nrloc;
        if (M <= 0) {
          idx[nobsl] = ob;
          rdiag[nobsl] = nrdiag;
          rloc[nobsl] = nrloc;
          nobsl++;
          nobsl_t[GRP(o->uid[ob], o->typ[ob])]++;
        } else {
          /* letkf_tools.f90:1072-1137: insertion into the per-(elem,type) best-M set */
          size_t g = GRP(o->uid[ob], o->typ[ob]);
          int* is = isort_t + g * M; /* isort_t(1:M) -> is[0..M-1], values are 1-based slots */
          int* ib = iob_t + g * M;
          double* rd = rdiag_t + g * M;
          double* rl = rloc_t + g * M;
          int s, ss;
          if (nobsl_t[g] >= M && nrdiag >= rd[is[M - 1] - 1]) continue;
          for (s = 1; s <= M; s++) {
            if (is[s - 1] == 0) {
              nobsl_t[g]++;
              is[s - 1] = nobsl_t[g];
              ib[is[s - 1] - 1] = ob;
              rd[is[s - 1] - 1] = nrdiag;
              rl[is[s - 1] - 1] = nrloc;
              break;
            } else if (nrdiag < rd[is[s - 1] - 1]) {
              if (nobsl_t[g] < M) {
                nobsl_t[g]++;
                for (ss = nobsl_t[g]; ss >= s + 1; ss--) is[ss - 1] = is[ss - 2];
                is[s - 1] = nobsl_t[g];
              } else {
                int tmp = is[M - 1];
                for (ss = M; ss >= s + 1; ss--) is[ss - 1] = is[ss - 2];
                is[s - 1] = tmp;
              }
              ib[is[s - 1] - 1] = ob;
              rd[is[s - 1] - 1] = nrdiag;
              rl[is[s - 1] - 1] = nrloc;
              break;
            }
          }
        }
      }
    }
  }
  if (M > 0) {
    /* letkf_tools.f90:1141-1156: slot order, grouped by type then element */
    int t, u, s;
    for (t = 0; t < o->ntyp; t++)
      for (u = 0; u < o->nid; u++) {
        size_t g = GRP(u, t);
        for (s = 1; s <= nobsl_t[g]; s++) {
          idx[nobsl] = iob_t[g * M + s - 1];
          rdiag[nobsl] = rdiag_t[g * M + s - 1];
          rloc[nobsl] = rloc_t[g * M + s - 1];
          nobsl++;
        }
      }
    free(isort_t); free(iob_t); free(rdiag_t); free(rloc_t);
  }
  free(nobsl_t);
#undef G
#undef GRP
  return nobsl;
}

/* lorenz96/letkf/letkf.f90:218-254 with nwindow = 1 (tdif = 0) and
 * msw_local = 0.  Returns ny_loc; idx[] holds the selected obs rows in order. */
int oracle_l96_select(int nx, int ny, const double* h, int ix, double xlocal, double tlocal, int* idx,
                      double* rloc) {
  const double xmaxloc = xlocal * 2.0 * sqrt(10.0 / 3.0);
  int i, j, ny_loc = 0;
  double tdif = 0.0;
  if (tlocal < 0.0) tdif = 0.0;
  for (i = 1; i <= ny; i++) {
    double mx = h[(size_t)0 * ny + (i - 1)];
    for (j = 2; j <= nx; j++)
      if (h[(size_t)(j - 1) * ny + (i - 1)] > mx) mx = h[(size_t)(j - 1) * ny + (i - 1)];
    for (j = 1; j <= nx; j++)
      if (mx == h[(size_t)(j - 1) * ny + (i - 1)]) break;
    {
      int a = abs(j - ix), b = nx - abs(j - ix);
      double dist = (double)(a < b ? a : b);
      if (dist < xmaxloc) {
        double r = exp(-0.5 * (dist / xlocal) * (dist / xlocal)) * exp(-0.5 * (tdif / tlocal) * (tdif / tlocal));
        ny_loc++;
        idx[ny_loc - 1] = i - 1;
        rloc[ny_loc - 1] = r;
        if (r < 0.0001) ny_loc--;
      }
    }
  }
  return ny_loc;
}

/* GFS element ids (gfs/common/common_obs_gfs.f90:48-61) */
#define GFS_U 2819
#define GFS_V 2820
#define GFS_T 3073
#define GFS_TV 3074
#define GFS_Q 3330
#define GFS_RH 3331
#define GFS_PS 14593
#define GFS_RAIN 19999
#define GFS_TCLON 99991
#define GFS_TCLAT 99992
#define GFS_TCMIP 99993

/* obs_local of the GFS driver (gfs/letkf/letkf_tools.f90:686-925) at a point
 * (rlon, rlat, pressure rlev): the SPEEDY box with dlat_zero = max(dist_zero,
 * dist_zero_rain) / pi / re * 180 and dlon_zero = dlat_zero / cos(rlat pi /
 * 180); vertical distance from ln(obsdat) for ps, ln(base_obsv_rain) (against
 * dist_zerov_rain) for rain, 0 for TC obs, ln(obslev) otherwise; horizontal
 * cut-off dist_zero_rain for rain; variable localisation over six classes when
 * var_local != NULL (element codes outside the GFS list are then not
 * selected: the reference leaves their class undefined). */
int oracle_gfs_obs_local(const oracle_speedy_obs* o, const oracle_gfs_params* g, double rlon, double rlat,
                         double rlev, int* idx, double* rloc, double* rdiag) {
  const double pi = 3.1415926535, re = 6371.3e3;
  double dlat_zero, dlon_zero, dist, dlev, logrlev;
  int n, nn, iobs = 0, nobsl;
  int* nobs_use;
  if (o->nobs <= 0) return 0;
  nobs_use = (int*)malloc(sizeof(int) * (size_t)o->nobs);
  dlat_zero = (g->dist_zero > g->dist_zero_rain ? g->dist_zero : g->dist_zero_rain) / pi / re * 180.0;
  dlon_zero = dlat_zero / cos(rlat * pi / 180.0);
  nn = collect_box(o, rlon, rlat, dlon_zero, dlat_zero, nobs_use);
  logrlev = log(rlev);
  nobsl = 0;
  for (n = 1; n <= nn; n++) {
    const int ob = nobs_use[n - 1] - 1;
    const int elm = (int)lround(o->obselm[ob]);
    if (elm == GFS_PS) {
      dlev = fabs(log(o->obsdat[ob]) - logrlev);
      if (dlev > g->dist_zerov) continue;
    } else if (elm == GFS_RAIN) {
      dlev = fabs(log(g->base_obsv_rain) - logrlev);
      if (dlev > g->dist_zerov_rain) continue;
    } else if (elm >= GFS_TCLON) {
      dlev = 0.0;
    } else {
      dlev = fabs(log(o->obslev[ob]) - logrlev);
      if (dlev > g->dist_zerov) continue;
    }
    oracle_com_distll_1(o->obslon[ob], o->obslat[ob], rlon, rlat, &dist);
    if (elm == GFS_RAIN) {
      if (dist > g->dist_zero_rain) continue;
    } else {
      if (dist > g->dist_zero) continue;
    }
    if (g->var_local) {
      switch (elm) {
        case GFS_U: case GFS_V: iobs = 1; break;
        case GFS_T: case GFS_TV: iobs = 2; break;
        case GFS_Q: case GFS_RH: iobs = 3; break;
        case GFS_PS: iobs = 4; break;
        case GFS_RAIN: iobs = 5; break;
        case GFS_TCLON: case GFS_TCLAT: case GFS_TCMIP: iobs = 6; break;
        default: iobs = 0; break;
      }
      if (iobs == 0 || g->var_local[iobs - 1] < 2.2250738585072014e-308) continue;
    }
    idx[nobsl] = ob;
    rdiag[nobsl] = o->obserr[ob] * o->obserr[ob];
    {
      const double a = dist / (elm == GFS_RAIN ? g->sigma_obs_rain : g->sigma_obs), b = dlev / g->sigma_obsv;
      rloc[nobsl] = exp(-0.5 * (a * a + b * b));
    }
    if (g->var_local) rloc[nobsl] = rloc[nobsl] * g->var_local[iobs - 1];
    nobsl++;
  }
  free(nobs_use);
  return nobsl;
}

/* 4D selection of the Lorenz-96 driver (lorenz96/letkf/letkf.f90:217-254):
 * for analysis slot `slot` (1-based nn) the observations of every slot n in
 * slot order, tdif = |nn - n| (0 when tlocal < 0), rloc = exp(-0.5 (dist /
 * xlocal)^2) exp(-0.5 (tdif / tlocal)^2), dropped below 1e-4.  h holds nslot
 * blocks of ny x nx (column-major); idx is the row n*ny + i (0-based) of the
 * slot-stacked observation arrays. */
int oracle_l96_select_4d(int nx, int ny, int nslot, const double* h, int slot, int ix, double xlocal, double tlocal,
                         int* idx, double* rloc) {
  const double xmaxloc = xlocal * 2.0 * sqrt(10.0 / 3.0);
  int n, i, j, ny_loc = 0;
  for (n = 1; n <= nslot; n++) {
    const double* hn = h + (size_t)(n - 1) * nx * ny;
    double tdif = (double)abs(slot - n);
    if (tlocal < 0.0) tdif = 0.0;
    for (i = 1; i <= ny; i++) {
      double mx = hn[(size_t)0 * ny + (i - 1)];
      for (j = 2; j <= nx; j++)
        if (hn[(size_t)(j - 1) * ny + (i - 1)] > mx) mx = hn[(size_t)(j - 1) * ny + (i - 1)];
      for (j = 1; j <= nx; j++)
        if (mx == hn[(size_t)(j - 1) * ny + (i - 1)]) break;
      {
        int a = abs(j - ix), b = nx - abs(j - ix);
        double dist = (double)(a < b ? a : b);
        if (dist < xmaxloc) {
          double r = exp(-0.5 * (dist / xlocal) * (dist / xlocal)) * exp(-0.5 * (tdif / tlocal) * (tdif / tlocal));
          ny_loc++;
          idx[ny_loc - 1] = (n - 1) * ny + (i - 1);
          rloc[ny_loc - 1] = r;
          if (r < 0.0001) ny_loc--;
        }
      }
    }
  }
  return ny_loc;
}

/* com_mean, com_stdev, com_covar, com_correl (common/common.f90:46-128):
 * sequential sums over n values. */
static double com_mean(int n, const double* v) {
  double s = 0.0;
  int i;
  for (i = 0; i < n; i++) s = s + v[i];
  return s / (double)n;
}

static double com_stdev(int n, const double* v) {
  const double m = com_mean(n, v);
  double s = 0.0;
  int i;
  for (i = 0; i < n; i++) {
    const double d = v[i] - m;
    s = s + d * d;
  }
  return sqrt(s / (double)(n - 1));
}

static double com_covar(int n, const double* v1, const double* v2) {
  const double m1 = com_mean(n, v1), m2 = com_mean(n, v2);
  double s = 0.0;
  int i;
  for (i = 0; i < n; i++) s = s + (v1[i] - m1) * (v2[i] - m2);
  return s / (double)(n - 1);
}

double oracle_com_correl(int n, const double* v1, const double* v2) {
  const double sd1 = com_stdev(n, v1), sd2 = com_stdev(n, v2);
  const double cov = com_covar(n, v1, v2);
  return cov / sd1 / sd2;
}

/* lorenz96/letkf/letkf.f90:217-254 with the localisation switch msw_local
 * (0 fixed, 1 adaptive, 2 both; :18-27).  hdxf holds the slot-stacked
 * obs-space perturbations [nslot*ny][ne] (row n*ny + i); dxf the first-guess
 * perturbations of point ix at the analysis slot [ne]; slot and ix 1-based.
 * nbv2 = CEILING(REAL(nbv)/2.0) (:76). */
int oracle_l96_select_adaptive(int nx, int ny, int nslot, const double* h, const double* hdxf, const double* dxf,
                               int ne, int slot, int ix, double xlocal, double tlocal, int msw_local, double sa,
                               double sb, int* idx, double* rloc) {
  const double xmaxloc = xlocal * 2.0 * sqrt(10.0 / 3.0);
  const int nbv2 = (int)ceil((double)(float)ne / 2.0);
  int n, i, j, ny_loc = 0;
  for (n = 1; n <= nslot; n++) {
    const double* hn = h + (size_t)(n - 1) * nx * ny;
    double tdif = (double)abs(slot - n);
    if (tlocal < 0.0) tdif = 0.0;
    for (i = 1; i <= ny; i++) {
      double mx = hn[(size_t)0 * ny + (i - 1)];
      for (j = 2; j <= nx; j++)
        if (hn[(size_t)(j - 1) * ny + (i - 1)] > mx) mx = hn[(size_t)(j - 1) * ny + (i - 1)];
      for (j = 1; j <= nx; j++)
        if (mx == hn[(size_t)(j - 1) * ny + (i - 1)]) break;
      {
        int a = abs(j - ix), b = nx - abs(j - ix);
        double dist = (double)(a < b ? a : b);
        if (dist < xmaxloc) {
          const int row = (n - 1) * ny + (i - 1);
          const double* hr = hdxf + (size_t)row * ne;
          double r;
          if (msw_local == 0) {
            r = exp(-0.5 * ((dist / xlocal) * (dist / xlocal))) * exp(-0.5 * ((tdif / tlocal) * (tdif / tlocal)));
          } else {
            const double c1 = oracle_com_correl(nbv2, hr, dxf);
            const double c2 = oracle_com_correl(ne - nbv2, hr + nbv2, dxf + nbv2);
            const double c3 = oracle_com_correl(ne, hr, dxf);
            const double wb = fabs(c3);
            const double wa = 1.0 - (0.5 * fabs(c1 - c2));
            r = pow(wa, sa) * pow(wb, sb);
            if (msw_local == 2)
              r = r * exp(-0.5 * ((dist / xlocal) * (dist / xlocal))) *
                  exp(-0.5 * ((tdif / tlocal) * (tdif / tlocal)));
          }
          ny_loc++;
          idx[ny_loc - 1] = row;
          rloc[ny_loc - 1] = r;
          if (r < 0.0001) ny_loc--;
        }
      }
    }
  }
  return ny_loc;
}

/* speedy/common/common_speedy.f90:335-370 and letkf_tools.f90:96-112 */
void oracle_ensmean(int npts, int ne, const double* x, double* mean, double* pert) {
  int p, m;
  for (p = 0; p < npts; p++) {
    double s = x[(size_t)p * ne + 0];
    for (m = 1; m < ne; m++) s = s + x[(size_t)p * ne + m];
    s = s / (double)ne;
    mean[p] = s;
    if (pert)
      for (m = 0; m < ne; m++) pert[(size_t)p * ne + m] = x[(size_t)p * ne + m] - s;
  }
}
