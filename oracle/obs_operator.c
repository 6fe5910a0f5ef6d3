/*
 * obs_operator.c -- CPU FP64 restatement of the SPEEDY observation operator
 * H(x) and of the driver rules around it.  TEST INFRASTRUCTURE ONLY (see
 * letkf_oracle.h): the oracle of letkf_speedy_obsope.
 *
 *   phys2ijk     speedy/common/common_obs_speedy.f90:137-206
 *   Trans_XtoY   speedy/common/common_obs_speedy.f90:29-80
 *   calc_rh      speedy/common/common_obs_speedy.f90:84-109
 *   itpl_2d/3d   speedy/common/common_obs_speedy.f90:210-280
 *   calc_pfull   speedy/common/common_speedy.f90:291-309 (p_full = ps * sig(k))
 *   driver       speedy/letkf/obsope.f90:53-104 (range checks, the u/v
 *                lowest-level clamp rk = 1.00001, missing ps skipped)
 *
 * Fields are one member's state with (lon, lat) planes, lon fastest:
 * v3d(i, j, k, n) at v3d[rec3 * (n * nlev + k) + j * nlon + i] and
 * v2d(i, j, n) at v2d[rec2 * n + j * nlon + i] (0-based i, j, k, n).
 * Indices below follow the reference's 1-based arithmetic and subtract 1 at
 * the array access.
 */
#include <math.h>
#include <stdint.h>

#include "letkf_oracle.h"

#define ID_U 2819
#define ID_V 2820
#define ID_T 3073
#define ID_Q 3330
#define ID_RH 3331
#define ID_PS 14593
#define ID_RAIN 9999

typedef struct {
  int nlon, nlat, nlev;
  const double* lat;
  const double* sig;
  const double* v3d;
  int64_t rec3;
  const double* v2d;
  int64_t rec2;
} member_t;

/* Fortran CEILING, saturated far outside any grid so that the range tests
 * below stay defined for huge or infinite arguments */
static long ceil_i(double x) {
  if (x >= 1.0e15) return 1000000000000000L;
  if (x <= -1.0e15) return -1000000000000000L;
  return (long)ceil(x);
}

static double v3(const member_t* s, int n, long i, long j, long k) {
  return s->v3d[s->rec3 * ((int64_t)n * s->nlev + (k - 1)) + (int64_t)(j - 1) * s->nlon + (i - 1)];
}
static double v2(const member_t* s, int n, long i, long j) {
  return s->v2d[s->rec2 * n + (int64_t)(j - 1) * s->nlon + (i - 1)];
}

/* calc_rh (speedy/common/common_obs_speedy.f90:84-109) */
double oracle_speedy_calc_rh(double t, double q, double p) {
  const double t0 = 273.15, e0c = 6.11, al = 17.3, bl = 237.3, e0i = 6.1121, ai = 22.587, bi = 273.86;
  const double e = q * p * 0.01 / (0.378 * q + 0.622);
  const double tc = t - t0;
  double es;
  if (tc >= 0.0)
    es = e0c * exp(al * tc / (bl + tc));
  else if (tc <= -15.0)
    es = e0i * exp(ai * tc / (bi + tc));
  else
    es = e0c * exp(al * tc / (bl + tc)) * (15.0 + tc) / 15.0 + e0i * exp(ai * tc / (bi + tc)) * (-tc) / 15.0;
  return e / es;
}

/* itpl_2d on four corner values c[jj][ii] (jj, ii in {0: j-1 / i-1, 1: j / i}) */
static double itpl2(const double c[2][2], double ai, double aj) {
  return c[0][0] * (1 - ai) * (1 - aj) + c[0][1] * ai * (1 - aj) + c[1][0] * (1 - ai) * aj + c[1][1] * ai * aj;
}

/* itpl_3d on eight corner values c[kk][jj][ii] */
static double itpl3(const double c[2][2][2], double ai, double aj, double ak) {
  return c[0][0][0] * (1 - ai) * (1 - aj) * (1 - ak) + c[0][0][1] * ai * (1 - aj) * (1 - ak) +
         c[0][1][0] * (1 - ai) * aj * (1 - ak) + c[0][1][1] * ai * aj * (1 - ak) +
         c[1][0][0] * (1 - ai) * (1 - aj) * ak + c[1][0][1] * ai * (1 - aj) * ak +
         c[1][1][0] * (1 - ai) * aj * ak + c[1][1][1] * ai * aj * ak;
}

/* column index of corner ii (0: i-1, 1: i) with the longitude wrap to column 1 */
static long col(long i, int ii, int nlon) { return ii == 0 ? i - 1 : (i <= nlon ? i : 1); }

/* phys2ijk (speedy/common/common_obs_speedy.f90:137-206) plus the obsope.f90
 * range rules.  Returns 1 with (ri, rj, rk) when the observation is usable
 * for this member, 0 when the driver would CYCLE.  A non-positive level of a
 * non-ps observation (log undefined) is also rejected. */
static int locate(const member_t* s, int elem, double rlon, double rlat, double rlev, double* ri_o, double* rj_o,
                  double* rk_o) {
  const int nlon = s->nlon, nlat = s->nlat, nlev = s->nlev;
  double ri, rj, rk;
  if (rlon == 0.0 || rlon == 360.0)
    ri = (double)(nlon + 1);
  else
    ri = rlon / 360.0 * (double)nlon + 1.0;
  if (isnan(ri) || ceil_i(ri) < 2 || nlon + 1 < ceil_i(ri)) return 0;
  int j;
  for (j = 1; j <= nlat; j++)
    if (rlat < s->lat[j - 1]) break;
  if (j == 1) {
    rj = (rlat + 90.0) / (s->lat[0] + 90.0);
  } else if (j == nlat + 1) {
    const double aj = (rlat - s->lat[nlat - 1]) / (90.0 - s->lat[nlat - 1]);
    rj = (double)nlat + aj;
  } else {
    const double aj = (rlat - s->lat[j - 2]) / (s->lat[j - 1] - s->lat[j - 2]);
    rj = (double)(j - 1) + aj;
  }
  if (isnan(rj) || ceil_i(rj) < 2 || nlat < ceil_i(rj)) return 0;
  if (elem == ID_PS) {
    rk = 0.0;
  } else {
    if (!(rlev > 0.0)) return 0;
    const long i = ceil_i(ri), jc = ceil_i(rj);
    const double ai = ri - (double)(i - 1), aj = rj - (double)(jc - 1);
    double ps[2][2];
    for (int jj = 0; jj < 2; jj++)
      for (int ii = 0; ii < 2; ii++) ps[jj][ii] = v2(s, 0, col(i, ii, nlon), jc - 1 + jj);
    double plev_prev = 0.0, plev_k = 0.0;
    int k;
    /* plev(k) = itpl_2d(LOG(p_full(:, :, k))), evaluated as the search needs it */
    for (k = 1; k <= nlev; k++) {
      double c[2][2];
      for (int jj = 0; jj < 2; jj++)
        for (int ii = 0; ii < 2; ii++) c[jj][ii] = log(ps[jj][ii] * s->sig[k - 1]);
      plev_prev = plev_k;
      plev_k = itpl2(c, ai, aj);
      if (k == 1) continue;
      if (k == nlev) break;           /* DO k=2,nlev-1 ran out: k = nlev */
      if (plev_k < log(rlev)) break;  /* EXIT */
    }
    if (nlev < 2) return 0;
    rk = log(rlev);
    const double ak = (rk - plev_prev) / (plev_k - plev_prev);
    rk = (double)(k - 1) + ak;
    if (isnan(rk)) return 0;
  }
  /* obsope.f90:70-93 */
  if (ceil_i(rk) > nlev) return 0;
  if (ceil_i(rk) < 2 && elem != ID_PS) {
    if (elem == ID_U || elem == ID_V)
      rk = 1.00001;
    else
      return 0;
  }
  *ri_o = ri;
  *rj_o = rj;
  *rk_o = rk;
  return 1;
}

/* Trans_XtoY (speedy/common/common_obs_speedy.f90:29-80).  Unknown element
 * codes leave yobs at the driver's initial 0. */
static double trans_xtoy(const member_t* s, int elem, double ri, double rj, double rk) {
  const int nlon = s->nlon;
  const long i = ceil_i(ri), j = ceil_i(rj);
  const double ai = ri - (double)(i - 1), aj = rj - (double)(j - 1);
  int var = -1;
  switch (elem) {
    case ID_U: var = 0; break;
    case ID_V: var = 1; break;
    case ID_T: var = 2; break;
    case ID_Q: var = 3; break;
    case ID_PS:
    case ID_RAIN: {
      double c[2][2];
      const int n = elem == ID_PS ? 0 : 1;
      for (int jj = 0; jj < 2; jj++)
        for (int ii = 0; ii < 2; ii++) c[jj][ii] = v2(s, n, col(i, ii, nlon), j - 1 + jj);
      return itpl2(c, ai, aj);
    }
    case ID_RH: break;
    default: return 0.0;
  }
  const long k = ceil_i(rk);
  const double ak = rk - (double)(k - 1);
  double c[2][2][2];
  for (int kk = 0; kk < 2; kk++)
    for (int jj = 0; jj < 2; jj++)
      for (int ii = 0; ii < 2; ii++) {
        const long ic = col(i, ii, nlon), jc = j - 1 + jj, kc = k - 1 + kk;
        if (var >= 0) {
          c[kk][jj][ii] = v3(s, var, ic, jc, kc);
        } else {
          const double p = v2(s, 0, ic, jc) * s->sig[kc - 1];
          c[kk][jj][ii] = oracle_speedy_calc_rh(v3(s, 2, ic, jc, kc), v3(s, 3, ic, jc, kc), p);
        }
      }
  return itpl3(c, ai, aj, ak);
}

int oracle_speedy_obsope(int nlon, int nlat, int nlev, int ne, const double* lat, const double* sig,
                         const double* v3d, int64_t v3d_mem, int64_t v3d_rec, const double* v2d, int64_t v2d_mem,
                         int64_t v2d_rec, int nobs, const int* elem, const double* rlon, const double* rlat,
                         const double* rlev, const double* odat, double* hx, int* qc_member, int* qc) {
  for (int n = 0; n < nobs; n++) {
    int qmin = 1;
    for (int m = 0; m < ne; m++) {
      const member_t s = {nlon, nlat, nlev, lat, sig, v3d + v3d_mem * m, v3d_rec, v2d + v2d_mem * m, v2d_rec};
      double ri, rj, rk, y = 0.0;
      int q = locate(&s, elem[n], rlon[n], rlat[n], rlev[n], &ri, &rj, &rk);
      if (q && elem[n] == ID_PS && odat[n] < -100.0) q = 0;
      if (q) y = trans_xtoy(&s, elem[n], ri, rj, rk);
      hx[(int64_t)n * ne + m] = y;
      if (qc_member) qc_member[(int64_t)n * ne + m] = q;
      if (q < qmin) qmin = q;
    }
    if (qc) qc[n] = qmin;
  }
  return 0;
}
