/*
 * letkf_core.c -- CPU FP64 restatement of the reference numerics.
 * TEST INFRASTRUCTURE ONLY (the oracle of the CUDA path; never shipped).
 * Parity unpinned against the Fortran itself (no Fortran compiler, no
 * reference golden data); pinned by the maths known-answer tests in tests/.
 *
 * Each routine cites the reference file:line it follows.  Loops are written
 * with 1-based index macros so that every loop bound and operation order is
 * the reference's.
 */
#include "letkf_oracle.h"
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Fortran SIGN(a,b): |a| with the sign of b (gfortran honours -0.0). */
static double fsign(double a, double b) { return copysign(fabs(a), b); }

/* common/netlibrs.f:1-19 */
double oracle_pythag(double a, double b) {
  double p, r, s, t, u;
  p = fmax(fabs(a), fabs(b));
  if (p == 0.0) return p;
  r = fmin(fabs(a), fabs(b)) / p;
  r = r * r;
  for (;;) {
    t = 4.0 + r;
    if (t == 4.0) break;
    s = r / t;
    u = 1.0 + 2.0 * s;
    p = u * p;
    r = (s / u) * (s / u) * r;
  }
  return p;
}

/* common/netlibrs.f:520-683 (tred2: Householder reduction with accumulation) */
void oracle_tred2(int nm, int n, const double* a_, double* d_, double* e_, double* z_) {
#define A(i, j) a_[(size_t)((j)-1) * nm + ((i)-1)]
#define Z(i, j) z_[(size_t)((j)-1) * nm + ((i)-1)]
#define D(i) d_[(i)-1]
#define E(i) e_[(i)-1]
  int i, j, k, l, ii, jp1;
  double f, g, h, hh, scale;
  for (i = 1; i <= n; i++) {
    for (j = i; j <= n; j++) Z(j, i) = A(j, i);
    D(i) = A(n, i);
  }
  if (n != 1) {
    for (ii = 2; ii <= n; ii++) {
      i = n + 2 - ii;
      l = i - 1;
      h = 0.0;
      scale = 0.0;
      if (l < 2) goto L130;
      for (k = 1; k <= l; k++) scale = scale + fabs(D(k));
      if (scale != 0.0) goto L140;
    L130:
      E(i) = D(l);
      for (j = 1; j <= l; j++) {
        D(j) = Z(l, j);
        Z(i, j) = 0.0;
        Z(j, i) = 0.0;
      }
      goto L290;
    L140:
      for (k = 1; k <= l; k++) {
        D(k) = D(k) / scale;
        h = h + D(k) * D(k);
      }
      f = D(l);
      g = -fsign(sqrt(h), f);
      E(i) = scale * g;
      h = h - f * g;
      D(l) = f - g;
      for (j = 1; j <= l; j++) E(j) = 0.0;
      for (j = 1; j <= l; j++) {
        f = D(j);
        Z(j, i) = f;
        g = E(j) + Z(j, j) * f;
        jp1 = j + 1;
        if (l >= jp1) {
          for (k = jp1; k <= l; k++) {
            g = g + Z(k, j) * D(k);
            E(k) = E(k) + Z(k, j) * f;
          }
        }
        E(j) = g;
      }
      f = 0.0;
      for (j = 1; j <= l; j++) {
        E(j) = E(j) / h;
        f = f + E(j) * D(j);
      }
      hh = f / (h + h);
      for (j = 1; j <= l; j++) E(j) = E(j) - hh * D(j);
      for (j = 1; j <= l; j++) {
        f = D(j);
        g = E(j);
        for (k = j; k <= l; k++) Z(k, j) = Z(k, j) - f * E(k) - g * D(k);
        D(j) = Z(l, j);
        Z(i, j) = 0.0;
      }
    L290:
      D(i) = h;
    }
    for (i = 2; i <= n; i++) {
      l = i - 1;
      Z(n, l) = Z(l, l);
      Z(l, l) = 1.0;
      h = D(i);
      if (h != 0.0) {
        for (k = 1; k <= l; k++) D(k) = Z(k, i) / h;
        for (j = 1; j <= l; j++) {
          g = 0.0;
          for (k = 1; k <= l; k++) g = g + Z(k, i) * Z(k, j);
          for (k = 1; k <= l; k++) Z(k, j) = Z(k, j) - g * D(k);
        }
      }
      for (k = 1; k <= l; k++) Z(k, i) = 0.0;
    }
  }
  for (i = 1; i <= n; i++) {
    D(i) = Z(n, i);
    Z(n, i) = 0.0;
  }
  Z(n, n) = 1.0;
  E(1) = 0.0;
#undef A
}

/* common/netlibrs.f:215-384 (tql2: implicit QL with vectors, ascending sort) */
int oracle_tql2(int nm, int n, double* d_, double* e_, double* z_) {
  int i, j, k, l, m, ii, l1, l2, mml, ierr = 0;
  double c, c2, c3 = 0.0, dl1, el1, f, g, h, p, r, s, s2 = 0.0, tst1, tst2;
  if (n == 1) return 0;
  for (i = 2; i <= n; i++) E(i - 1) = E(i);
  f = 0.0;
  tst1 = 0.0;
  E(n) = 0.0;
  for (l = 1; l <= n; l++) {
    j = 0;
    h = fabs(D(l)) + fabs(E(l));
    if (tst1 < h) tst1 = h;
    for (m = l; m <= n; m++) {
      tst2 = tst1 + fabs(E(m));
      if (tst2 == tst1) break;
    }
    if (m > n) m = n; /* unreachable: e(n) is zero */
    if (m == l) goto L220;
  L130:
    if (j == 30) return l; /* ierr = l */
    j = j + 1;
    l1 = l + 1;
    l2 = l1 + 1;
    g = D(l);
    p = (D(l1) - g) / (2.0 * E(l));
    r = oracle_pythag(p, 1.0);
    D(l) = E(l) / (p + fsign(r, p));
    D(l1) = E(l) * (p + fsign(r, p));
    dl1 = D(l1);
    h = g - D(l);
    if (l2 <= n) {
      for (i = l2; i <= n; i++) D(i) = D(i) - h;
    }
    f = f + h;
    p = D(m);
    c = 1.0;
    c2 = c;
    el1 = E(l1);
    s = 0.0;
    mml = m - l;
    for (ii = 1; ii <= mml; ii++) {
      c3 = c2;
      c2 = c;
      s2 = s;
      i = m - ii;
      g = c * E(i);
      h = c * p;
      r = oracle_pythag(p, E(i));
      E(i + 1) = s * r;
      s = E(i) / r;
      c = p / r;
      p = c * D(i) - s * g;
      D(i + 1) = h + s * (c * g + s * D(i));
      for (k = 1; k <= n; k++) {
        h = Z(k, i + 1);
        Z(k, i + 1) = s * Z(k, i) + c * h;
        Z(k, i) = c * Z(k, i) - s * h;
      }
    }
    p = -s * s2 * c3 * el1 * E(l) / dl1;
    E(l) = s * p;
    D(l) = c * p;
    tst2 = tst1 + fabs(E(l));
    if (tst2 > tst1) goto L130;
  L220:
    D(l) = D(l) + f;
  }
  for (ii = 2; ii <= n; ii++) {
    i = ii - 1;
    k = i;
    p = D(i);
    for (j = ii; j <= n; j++) {
      if (D(j) >= p) continue;
      k = j;
      p = D(j);
    }
    if (k == i) continue;
    D(k) = D(i);
    D(i) = p;
    for (j = 1; j <= n; j++) {
      p = Z(j, i);
      Z(j, i) = Z(j, k);
      Z(j, k) = p;
    }
  }
  return ierr;
}
#undef Z
#undef D
#undef E

/* common/netlibrs.f:21-79 (matz != 0 branch only; letkf_core always asks for vectors) */
int oracle_rs(int nm, int n, double* a, double* w, int matz, double* z, double* fv1, double* fv2) {
  (void)fv2;
  if (n > nm) return 10 * n;
  if (matz == 0) return -1; /* eigenvalue-only branch (tred1/tql1) is not on the path */
  oracle_tred2(nm, n, a, w, fv1, z);
  return oracle_tql2(nm, n, w, fv1, z);
}

/* common/common_mtx.f90:41-99 */
int oracle_mtx_eigen(int imode, int n, const double* a, double* eival, double* eivec, int* nrank_eff) {
  double* a8 = (double*)malloc(sizeof(double) * (size_t)n * n);
  double* eival8 = (double*)malloc(sizeof(double) * n);
  double* eivec8 = (double*)calloc((size_t)n * n, sizeof(double));
  double* wrk1 = (double*)malloc(sizeof(double) * n);
  double* wrk2 = (double*)malloc(sizeof(double) * n);
  int ierr, i, j, r, st = 0;
  memcpy(a8, a, sizeof(double) * (size_t)n * n);
  ierr = oracle_rs(n, n, a8, eival8, imode, eivec8, wrk1, wrk2);
  if (ierr != 0) { st = 2; goto done; }
  *nrank_eff = n;
  if (eival8[n - 1] > 0) {
    double thr = fabs(eival8[n - 1]) * sqrt(DBL_EPSILON);
    for (i = 0; i < n; i++) {
      if (eival8[i] < thr) {
        *nrank_eff -= 1;
        eival8[i] = 0.0;
        for (r = 0; r < n; r++) eivec8[(size_t)i * n + r] = 0.0;
      }
    }
  } else {
    st = 2;
    goto done;
  }
  /* common_mtx.f90:80-91 reorder branch: writes the OUTPUT eivec (later
   * overwritten) and is entered only if eival8(1) /= 0 after truncation. */
  if (*nrank_eff < n && eival8[0] != 0) {
    j = 0;
    for (i = n; i >= 1; i--) {
      if (eival8[i - 1] == 0) {
        int src = n - *nrank_eff - j; /* 1-based */
        eival8[i - 1] = eival8[src - 1];
        for (r = 0; r < n; r++) eivec[(size_t)(i - 1) * n + r] = eivec8[(size_t)(src - 1) * n + r];
        eival8[src - 1] = 0.0;
        for (r = 0; r < n; r++) eivec8[(size_t)(src - 1) * n + r] = 0.0;
        j = j + 1;
      }
    }
  }
  for (i = 1; i <= n; i++) {
    eival[i - 1] = eival8[n - i];
    for (r = 0; r < n; r++) eivec[(size_t)(i - 1) * n + r] = eivec8[(size_t)(n - i) * n + r];
  }
done:
  free(a8); free(eival8); free(eivec8); free(wrk1); free(wrk2);
  return st;
}

/* common/netlibblas.f DGEMM, TRANSA='T', TRANSB='N', alpha=1, beta=0:
 * C(i,j) = sum_l A(l,i)*B(l,j), l ascending, then C = ALPHA*TEMP. */
void oracle_dgemm_tn(int m, int n, int k, const double* a, int lda, const double* b, int ldb, double* c, int ldc) {
  int i, j, l;
  if (m == 0 || n == 0) return;
  for (j = 0; j < n; j++)
    for (i = 0; i < m; i++) {
      double temp = 0.0;
      for (l = 0; l < k; l++) temp = temp + a[(size_t)i * lda + l] * b[(size_t)j * ldb + l];
      c[(size_t)j * ldc + i] = 1.0 * temp;
    }
}

/* common/netlibblas.f DGEMM, TRANSA='N', TRANSB='T', alpha=1, beta=0:
 * column j zeroed, then C(:,j) += (ALPHA*B(j,l))*A(:,l) for l ascending,
 * skipping B(j,l) == 0. */
void oracle_dgemm_nt(int m, int n, int k, const double* a, int lda, const double* b, int ldb, double* c, int ldc) {
  int i, j, l;
  if (m == 0 || n == 0) return;
  for (j = 0; j < n; j++) {
    for (i = 0; i < m; i++) c[(size_t)j * ldc + i] = 0.0;
    for (l = 0; l < k; l++) {
      double bjl = b[(size_t)l * ldb + j];
      if (bjl != 0.0) {
        double temp = 1.0 * bjl;
        for (i = 0; i < m; i++) c[(size_t)j * ldc + i] = c[(size_t)j * ldc + i] + temp * a[(size_t)l * lda + i];
      }
    }
  }
}

/* common/common_letkf.f90:50-243 */
int oracle_letkf_core(int ne, int nobs, int nobsl, const double* hdxb, const double* rdiag,
                      const double* rloc, const double* dep, double* parm_infl, double* trans,
                      double* transm, double* pao, int rdiag_wloc, const double* minfl) {
  const double sigma_b = 0.04;
  int i, j, st;
  if (ne < 1 || nobsl < 0 || nobs < nobsl || (nobsl > 0 && nobs < 1)) return 1;
  if (nobsl == 0) { /* :82-96 */
    for (j = 0; j < ne * ne; j++) trans[j] = 0.0;
    for (i = 0; i < ne; i++) trans[(size_t)i * ne + i] = sqrt(*parm_infl);
    if (transm) for (i = 0; i < ne; i++) transm[i] = 0.0;
    if (pao) {
      for (j = 0; j < ne * ne; j++) pao[j] = 0.0;
      for (i = 0; i < ne; i++) pao[(size_t)i * ne + i] = *parm_infl / (double)(ne - 1);
    }
    return 0;
  }
  size_t L = (size_t)nobsl, K = (size_t)ne;
  double* hdxb_rinv = (double*)malloc(sizeof(double) * L * K);
  double* hdxb_sec = (double*)malloc(sizeof(double) * L * K); /* hdxb(1:nobsl,:) temporary */
  double* eivec = (double*)malloc(sizeof(double) * K * K);
  double* eival = (double*)malloc(sizeof(double) * K);
  double* pa = (double*)malloc(sizeof(double) * K * K);
  double* work1 = (double*)malloc(sizeof(double) * K * K);
  double* work2 = (double*)malloc(sizeof(double) * K * L);
  double* work3 = (double*)malloc(sizeof(double) * K);
  double rho, parm[4], sigma_o, gain;
  int nrank;
  /* :101-113 */
  for (j = 0; j < ne; j++)
    for (i = 0; i < nobsl; i++) {
      double h = hdxb[(size_t)j * nobs + i];
      hdxb_sec[(size_t)j * L + i] = h;
      if (rdiag_wloc) hdxb_rinv[(size_t)j * L + i] = h / rdiag[i];
      else hdxb_rinv[(size_t)j * L + i] = h / rdiag[i] * rloc[i];
    }
  /* :117-118 */
  oracle_dgemm_tn(ne, ne, nobsl, hdxb_rinv, nobsl, hdxb_sec, nobsl, work1, ne);
  /* :130-138 */
  if (minfl) {
    if (*minfl > 0.0 && *parm_infl < *minfl) *parm_infl = *minfl;
  }
  rho = 1.0 / *parm_infl;
  for (i = 0; i < ne; i++) work1[(size_t)i * ne + i] = work1[(size_t)i * ne + i] + (double)(ne - 1) * rho;
  /* :142 */
  st = oracle_mtx_eigen(1, ne, work1, eival, eivec, &nrank);
  if (st != 0) goto done;
  /* :146-152 */
  for (j = 0; j < ne; j++)
    for (i = 0; i < ne; i++) work1[(size_t)j * ne + i] = eivec[(size_t)j * ne + i] / eival[j];
  oracle_dgemm_nt(ne, ne, ne, work1, ne, eivec, ne, pa, ne);
  /* :164 */
  oracle_dgemm_nt(ne, nobsl, ne, pa, ne, hdxb_rinv, nobsl, work2, ne);
  /* :177-182 */
  for (i = 0; i < ne; i++) {
    work3[i] = work2[i] * dep[0];
    for (j = 1; j < nobsl; j++) work3[i] = work3[i] + work2[(size_t)j * ne + i] * dep[j];
  }
  /* :186-193 */
  for (j = 0; j < ne; j++) {
    rho = sqrt((double)(ne - 1) / eival[j]);
    for (i = 0; i < ne; i++) work1[(size_t)j * ne + i] = eivec[(size_t)j * ne + i] * rho;
  }
  oracle_dgemm_nt(ne, ne, ne, work1, ne, eivec, ne, trans, ne);
  /* :205-214 */
  if (transm) {
    for (i = 0; i < ne; i++) transm[i] = work3[i];
  } else {
    for (j = 0; j < ne; j++)
      for (i = 0; i < ne; i++) trans[(size_t)j * ne + i] = trans[(size_t)j * ne + i] + work3[i];
  }
  if (pao) memcpy(pao, pa, sizeof(double) * K * K);
  /* :218-239 */
  parm[0] = parm[1] = parm[2] = parm[3] = 0.0;
  if (rdiag_wloc) {
    for (i = 0; i < nobsl; i++) parm[0] = parm[0] + dep[i] * dep[i] / rdiag[i];
  } else {
    for (i = 0; i < nobsl; i++) parm[0] = parm[0] + dep[i] * dep[i] / rdiag[i] * rloc[i];
  }
  for (j = 0; j < ne; j++)
    for (i = 0; i < nobsl; i++) parm[1] = parm[1] + hdxb_rinv[(size_t)j * L + i] * hdxb_sec[(size_t)j * L + i];
  parm[1] = parm[1] / (double)(ne - 1);
  for (i = 0; i < nobsl; i++) parm[2] = parm[2] + rloc[i];
  parm[3] = (parm[0] - parm[2]) / parm[1] - *parm_infl;
  {
    double t = (*parm_infl * parm[1] + parm[2]) / parm[1];
    sigma_o = 2.0 / parm[2] * (t * t);
  }
  gain = (sigma_b * sigma_b) / (sigma_o + sigma_b * sigma_b);
  *parm_infl = *parm_infl + gain * parm[3];
done:
  free(hdxb_rinv); free(hdxb_sec); free(eivec); free(eival); free(pa);
  free(work1); free(work2); free(work3);
  return st;
}

int oracle_letkf_core_batch(int ne, int npts, const int64_t* offs, const double* hdxb_rows,
                            const double* rdiag, const double* rloc, const double* dep,
                            double* parm_infl, double* trans, double* transm, double* pao,
                            int rdiag_wloc, double minfl, int nthreads, int* status) {
  int nbad = 0;
  int p;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
#pragma omp parallel for schedule(dynamic) reduction(+ : nbad)
  for (p = 0; p < npts; p++) {
    int64_t r0 = offs[p], nl = offs[p + 1] - offs[p];
    int nobsl = (int)nl;
    int nobs = nobsl > 0 ? nobsl : 1;
    double* h = (double*)malloc(sizeof(double) * (size_t)nobs * ne);
    int i, m;
    for (m = 0; m < ne; m++)
      for (i = 0; i < nobsl; i++) h[(size_t)m * nobs + i] = hdxb_rows[(size_t)(r0 + i) * ne + m];
    double mf = minfl;
    status[p] = oracle_letkf_core(ne, nobs, nobsl, h, rdiag + r0, rloc + r0, dep + r0, parm_infl + p,
                                  trans + (size_t)p * ne * ne, transm ? transm + (size_t)p * ne : NULL,
                                  pao ? pao + (size_t)p * ne * ne : NULL, rdiag_wloc, minfl > 0 ? &mf : NULL);
    if (status[p] != 0) nbad++;
    free(h);
  }
  return nbad;
}

/* scale/letkf/letkf_tools.f90:1224-1236 */
void oracle_weight_rtpp(int ne, const double* w, double alpha, double* wrlx) {
  int i, m;
  for (i = 0; i < ne * ne; i++) wrlx[i] = (1.0 - alpha) * w[i];
  for (m = 0; m < ne; m++) wrlx[(size_t)m * ne + m] = wrlx[(size_t)m * ne + m] + alpha;
}

/* scale/letkf/letkf_tools.f90:1240-1268 */
void oracle_weight_rtps(int ne, const double* w, const double* pa, const double* xb, double alpha,
                        double* wrlx, double* infl) {
  double var_g = 0.0, var_a = 0.0;
  int m, k, i;
  for (m = 0; m < ne; m++) {
    var_g = var_g + xb[m] * xb[m];
    for (k = 0; k < ne; k++) var_a = var_a + xb[k] * pa[(size_t)m * ne + k] * xb[m];
  }
  if (var_g > 0.0 && var_a > 0.0) {
    *infl = alpha * sqrt(var_g / (var_a * (double)(ne - 1))) - alpha + 1.0;
    for (i = 0; i < ne * ne; i++) wrlx[i] = w[i] * *infl;
  } else {
    for (i = 0; i < ne * ne; i++) wrlx[i] = w[i];
    *infl = 1.0;
  }
}

/* Observation-space analysis at one observation location
 * (gfs/letkf/letkf_tools.f90:466-497): trans (ne x ne, column-major, mean
 * weights merged, RTPP already applied by the caller), ybar = obsdat - obsdep,
 * hdxf = obshdxf(nn,:).  mode 0: update; 1: no update (q above the update
 * level); 2: update and relative-spread clip (q).  Writes anal[ne] and
 * returns the mean. */
double oracle_obs_analysis(int ne, const double* trans, double ybar, const double* hdxf, int mode,
                           double q_sprd_max, double* anal) {
  int m, k;
  double mean = 0.0;
  if (mode == 1) {
    for (m = 0; m < ne; m++) anal[m] = ybar + hdxf[m];
    return ybar;
  }
  for (m = 0; m < ne; m++) {
    anal[m] = ybar;
    for (k = 0; k < ne; k++) anal[m] = anal[m] + hdxf[k] * trans[(size_t)m * ne + k];
    mean = mean + anal[m];
  }
  mean = mean / (double)ne;
  if (mode == 2) {
    double sp = 0.0;
    double* qa = (double*)malloc(sizeof(double) * (size_t)ne);
    for (m = 0; m < ne; m++) {
      qa[m] = anal[m] - mean;
      sp = sp + qa[m] * qa[m];
    }
    sp = sqrt(sp / (double)(ne - 1)) / mean;
    if (sp > q_sprd_max)
      for (m = 0; m < ne; m++) anal[m] = mean + qa[m] * q_sprd_max / sp;
    free(qa);
  }
  return mean;
}

/* Observation sensitivity (EFSO, gfs/letkf/letkf_tools.f90:547-679) over
 * npts grid points with local lists offs/idx/rdiag/rloc (from obs_local):
 *   work1(t,m) = sum_v [term(v) == t] fcst(v,p,m) * fcer(v,p)
 *   djdy(t, idx) += sum_m work1(t,m) * hdxa(idx,m) / rdiag * rloc
 *   obsense(t, n) = djdy(t, n) * obsdep(n)
 * fcst [nv][npts][ne], fcer [nv][npts], term[nv] in 0..nterm-1 or -1,
 * hdxa [nobs][ne]; djdy and obsense [nobs][nterm] (zeroed here).  Points are
 * visited in order (the reference accumulates djdy in its loop order). */
void oracle_efso(int ne, int npts, int nv, int nterm, const int64_t* offs, const int* idx, const double* rdiag,
                 const double* rloc, const double* hdxa, const double* fcst, const double* fcer, const int* term,
                 int nobs, const double* obsdep, double* djdy, double* obsense) {
  int p, v, m, t;
  int64_t l;
  double* work1 = (double*)malloc(sizeof(double) * (size_t)nterm * ne);
  for (l = 0; l < (int64_t)nobs * nterm; l++) djdy[l] = 0.0;
  for (p = 0; p < npts; p++) {
    if (offs[p + 1] == offs[p]) continue;
    for (l = 0; l < (int64_t)nterm * ne; l++) work1[l] = 0.0;
    for (v = 0; v < nv; v++) {
      t = term[v];
      if (t < 0) continue;
      for (m = 0; m < ne; m++)
        work1[(size_t)t * ne + m] = work1[(size_t)t * ne + m] +
                                    fcst[((size_t)v * npts + p) * ne + m] * fcer[(size_t)v * npts + p];
    }
    for (l = offs[p]; l < offs[p + 1]; l++) {
      const int ob = idx[l];
      for (m = 0; m < ne; m++) {
        const double hr = hdxa[(size_t)ob * ne + m] / rdiag[l] * rloc[l];
        for (t = 0; t < nterm; t++) djdy[(size_t)ob * nterm + t] = djdy[(size_t)ob * nterm + t] + work1[(size_t)t * ne + m] * hr;
      }
    }
  }
  for (l = 0; l < (int64_t)nobs * nterm; l++) obsense[l] = djdy[l] * obsdep[l / nterm];
  free(work1);
}
