/*
 * obs_operator_scale.c -- CPU FP64 restatement of the SCALE observation
 * operator H(x) for conventional observations.  TEST INFRASTRUCTURE ONLY (see
 * letkf_oracle.h): the oracle of letkf_scale_obsope.
 *
 *   obsope_cal   scale/obs/obsope_tools.f90:340-380 (OBS_IN_FORMAT 1: phys2ijk,
 *                then Trans_XtoY where it kept qc good), :602-608 (qc over
 *                members: the maximum), val initialised to 0
 *                (scale/common/common_obs_scale.f90:1939)
 *   phys2ijk     scale/common/common_obs_scale.f90:969-1075
 *   Trans_XtoY   scale/common/common_obs_scale.f90:262-334
 *   prsadj       scale/common/common_obs_scale.f90:583-599
 *   itpl_2d, itpl_2d_column, itpl_3d   scale/common/common_obs_scale.f90:1254-1325
 *   constants    common/common.f90:28-38 (gg, rd, rv, fvirt, undef)
 *
 * One member's local domain with halos, k fastest as the reference's
 * v3dg(nlevh, nlonh, nlath, nv3dd): element (k, i, j, n) (1-based) at
 * v3d[n * var3 + ((j - 1) * nlonh + (i - 1)) * nlevh + (k - 1)], n = 0 u,
 * 1 v, 2 t, 3 q, 4 rh, 5 p; v2d (i, j, n) at v2d[n * var2 + (j - 1) * nlonh +
 * (i - 1)], n = 0 ps, 1 t2m, 2 q2m, 3 topo.  The u/v rotation coefficients of
 * the map projection (MPRJ_rotcoef, a SCALE-RM library routine) are inputs.
 *
 * Stencils: the reference takes i = CEILING(x) and reads i - 1 and i, so x = 1
 * exactly reads index 0, outside its array, with weight 0, and the staggered
 * u / v at ri - 0.5 < 1 (rj - 0.5 < 1) read it with a non-zero weight.  Here
 * the upper index is clamped to [2, n] and the weight follows (x - (i - 1)):
 * the same value, bit for bit, where the reference's outside term has weight
 * 0; an extrapolation from the edge columns for the staggered case.
 */
#include <math.h>
#include <stdint.h>

#include "letkf_oracle.h"

#define SC_U 2819
#define SC_V 2820
#define SC_T 3073
#define SC_TV 3074
#define SC_Q 3330
#define SC_RH 3331
#define SC_PS 14593

#define IQC_GOOD 0
#define IQC_PS_TER 10
#define IQC_OUT_VHI 20
#define IQC_OUT_VLO 21
#define IQC_OUT_H 22
#define IQC_OTYPE 90

static const double SC_GG = 9.81, SC_RD = 287.05, SC_RV = 461.50, SC_UNDEF = -9.99e33;

typedef struct {
  int nlonh, nlath, nlevh;
  const double* v3d;
  int64_t var3;
  const double* v2d;
  int64_t var2;
} sdom_t;

static long sc_ceil(double x) {
  if (x >= 1.0e15) return 1000000000000000L;
  if (x <= -1.0e15) return -1000000000000000L;
  return (long)ceil(x);
}

/* the stencil of coordinate x over 1..n: upper index i, weight *a of i */
static long stencil(double x, long n, double* a) {
  long i = sc_ceil(x);
  if (i < 2) i = 2;
  if (i > n) i = n;
  *a = x - (double)(i - 1);
  return i;
}

static double f3(const sdom_t* d, int n, long k, long i, long j) {
  return d->v3d[d->var3 * n + ((int64_t)(j - 1) * d->nlonh + (i - 1)) * d->nlevh + (k - 1)];
}
static double f2(const sdom_t* d, int n, long i, long j) {
  return d->v2d[d->var2 * n + (int64_t)(j - 1) * d->nlonh + (i - 1)];
}

/* itpl_2d (:1254-1274) on variable n of v2d */
static double itpl_2d(const sdom_t* d, int n, double ri, double rj) {
  double ai, aj;
  const long i = stencil(ri, d->nlonh, &ai), j = stencil(rj, d->nlath, &aj);
  return f2(d, n, i - 1, j - 1) * (1 - ai) * (1 - aj) + f2(d, n, i, j - 1) * ai * (1 - aj) +
         f2(d, n, i - 1, j) * (1 - ai) * aj + f2(d, n, i, j) * ai * aj;
}

/* itpl_3d (:1298-1325) as Trans_XtoY calls it, itpl_3d(v3d(:,:,:,n), rk,
 * ri, rj): its first coordinate runs over the levels */
static double itpl_3d(const sdom_t* d, int n, double rk, double ri, double rj) {
  double aa, ab, ac;
  const long a = stencil(rk, d->nlevh, &aa), b = stencil(ri, d->nlonh, &ab), c = stencil(rj, d->nlath, &ac);
  return f3(d, n, a - 1, b - 1, c - 1) * (1 - aa) * (1 - ab) * (1 - ac) +
         f3(d, n, a, b - 1, c - 1) * aa * (1 - ab) * (1 - ac) +
         f3(d, n, a - 1, b, c - 1) * (1 - aa) * ab * (1 - ac) + f3(d, n, a, b, c - 1) * aa * ab * (1 - ac) +
         f3(d, n, a - 1, b - 1, c) * (1 - aa) * (1 - ab) * ac + f3(d, n, a, b - 1, c) * aa * (1 - ab) * ac +
         f3(d, n, a - 1, b, c) * (1 - aa) * ab * ac + f3(d, n, a, b, c) * aa * ab * ac;
}

/* log pressure of level k bilinear in (ri, rj) (itpl_2d_column of
 * lnps = LOG(p_full) at the four columns, :1019-1020) */
static double lnp_at(const sdom_t* d, long k, long i, long j, double ai, double aj) {
  return log(f3(d, 5, k, i - 1, j - 1)) * (1 - ai) * (1 - aj) + log(f3(d, 5, k, i, j - 1)) * ai * (1 - aj) +
         log(f3(d, 5, k, i - 1, j)) * (1 - ai) * aj + log(f3(d, 5, k, i, j)) * ai * aj;
}

/* phys2ijk (:969-1075): rk of pressure rlev, or the rejection code */
static int phys2ijk(const sdom_t* d, int nlev, int khalo, int elem, double ri, double rj, double rlev, double* rk) {
  if (ri < 1.0 || ri > d->nlonh || rj < 1.0 || rj > d->nlath) {
    *rk = SC_UNDEF;
    return IQC_OUT_H;
  }
  if (elem > 9999) { /* surface observation */
    *rk = rlev;
    return IQC_GOOD;
  }
  double ai, aj;
  const long i = stencil(ri, d->nlonh, &ai), j = stencil(rj, d->nlath, &aj);
  const long top = nlev + khalo;
  long ks = 1 + khalo;
  for (long jj = j - 1; jj <= j; jj++)
    for (long ii = i - 1; ii <= i; ii++) {
      long k;
      for (k = 1 + khalo; k <= top; k++)
        if (f3(d, 5, k, ii, jj) >= 0.0) break;
      if (k > ks) ks = k;
    }
  const double lr = log(rlev);
  if (lr < lnp_at(d, top, i, j, ai, aj)) {
    *rk = SC_UNDEF;
    return IQC_OUT_VHI;
  }
  /* ks = top + 1 (no valid level in some column): plev(ks) is a halo level, as in the reference */
  if (lr > lnp_at(d, ks, i, j, ai, aj)) {
    *rk = SC_UNDEF;
    return IQC_OUT_VLO;
  }
  long k;
  for (k = ks + 1; k <= top; k++)
    if (lnp_at(d, k, i, j, ai, aj) < lr) break;
  const double pk = lnp_at(d, k, i, j, ai, aj), pk1 = lnp_at(d, k - 1, i, j, ai, aj);
  const double ak = (lr - pk1) / (pk - pk1);
  *rk = (double)(k - 1) + ak;
  return IQC_GOOD;
}

/* prsadj (:583-599) */
static double prsadj(double p, double dz, double t, double q) {
  const double gamma = 5.0e-3;
  if (dz != 0) {
    const double tv = t * (1.0 + 0.608 * q);
    p = p * pow((-gamma * dz + tv) / tv, SC_GG / (gamma * SC_RD));
  }
  return p;
}

/* Trans_XtoY (:262-334) */
static double trans_xtoy(const sdom_t* d, int elem, double ri, double rj, double rk, double rc1, double rc2,
                         int stggrd, double ps_thres, int* qc) {
  const double fvirt = SC_RV / SC_RD - 1.0;
  double y = SC_UNDEF, u, v, t, q, topo;
  *qc = IQC_GOOD;
  switch (elem) {
    case SC_U:
    case SC_V:
      if (stggrd == 1) {
        u = itpl_3d(d, 0, rk, ri - 0.5, rj);
        v = itpl_3d(d, 1, rk, ri, rj - 0.5);
      } else {
        u = itpl_3d(d, 0, rk, ri, rj);
        v = itpl_3d(d, 1, rk, ri, rj);
      }
      y = elem == SC_U ? u * rc1 - v * rc2 : u * rc2 + v * rc1;
      break;
    case SC_T: y = itpl_3d(d, 2, rk, ri, rj); break;
    case SC_TV:
      y = itpl_3d(d, 2, rk, ri, rj);
      q = itpl_3d(d, 3, rk, ri, rj);
      y = y * (1.0 + fvirt * q);
      break;
    case SC_Q: y = itpl_3d(d, 3, rk, ri, rj); break;
    case SC_PS:
      t = itpl_2d(d, 1, ri, rj);
      q = itpl_2d(d, 2, ri, rj);
      topo = itpl_2d(d, 3, ri, rj);
      y = itpl_2d(d, 0, ri, rj);
      y = prsadj(y, rk - topo, t, q);
      if (fabs(rk - topo) > ps_thres) *qc = IQC_PS_TER;
      break;
    case SC_RH: y = itpl_3d(d, 4, rk, ri, rj); break;
    default: *qc = IQC_OTYPE;
  }
  return y;
}

int oracle_scale_obsope(int nlonh, int nlath, int nlev, int khalo, int ne, const double* v3d, int64_t v3d_mem,
                        int64_t v3d_var, const double* v2d, int64_t v2d_mem, int64_t v2d_var, int nobs,
                        const int* elem, const double* ri, const double* rj, const double* rlev, const double* rotc,
                        int stggrd, double ps_thres, double* hx, int* qc_member, int* qc) {
  if (khalo < 2 || nlev < 2) return 1;
  for (int n = 0; n < nobs; n++) {
    int qmax = 0;
    for (int m = 0; m < ne; m++) {
      const sdom_t d = {nlonh, nlath, nlev + 2 * khalo, v3d + v3d_mem * m, v3d_var, v2d + v2d_mem * m, v2d_var};
      double rk, y = 0.0;
      int q = phys2ijk(&d, nlev, khalo, elem[n], ri[n], rj[n], rlev[n], &rk);
      if (q == IQC_GOOD)
        y = trans_xtoy(&d, elem[n], ri[n], rj[n], rk, rotc ? rotc[2 * n] : 1.0, rotc ? rotc[2 * n + 1] : 0.0,
                       stggrd, ps_thres, &q);
      hx[(int64_t)n * ne + m] = y;
      if (qc_member) qc_member[(int64_t)n * ne + m] = q;
      if (q > qmax) qmax = q;
    }
    if (qc) qc[n] = qmax;
  }
  return 0;
}
