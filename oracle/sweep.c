/*
 * sweep.c -- CPU restatement of the SCALE-style das_letkf grid loop.
 * TEST INFRASTRUCTURE ONLY: the oracle of the GPU sweep and the timed CPU
 * baseline.  Parity unpinned against the Fortran itself.
 *
 * Per grid point (scale/letkf/letkf_tools.f90:175-251, OpenMP
 * SCHEDULE(DYNAMIC) over points as at :175):
 *   obs_local (letkf_tools.f90:853-1178)
 *   letkf_core(..., transm=, rdiag_wloc=.true., minfl=) (:199-206)
 *   relax_beta = 1 (no boundary buffer, no Q_UPDATE_TOP), no RTPP/RTPS
 *   transrlx(k,m) = (trans(k,m) + transm(k)) * beta, + (1-beta) on the diagonal (:237-243)
 *   anal(m) = mean + sum_k gues(k) transrlx(k,m) (:245-251)
 * with the mean / perturbations of ensmean_grd (speedy/common/common_speedy.f90:335-370).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "letkf_oracle.h"

int oracle_scale_sweep(const oracle_scale_obs* o, const double* hdxf, const double* odep, int ne, int nv, int npts,
                       const int* subset, int nsub, const double* pri, const double* prj, const double* prlev,
                       const double* prz, const double* xb, double* xa, double* infl, int* nobsl_out,
                       double minfl, int nthreads) {
  int nbad = 0;
  const int nwork = subset ? nsub : npts;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  /* scale/letkf/letkf_tools.f90:175-206: OpenMP over points, each thread with
   * its own obs_local outputs sized nobstotal (allocated once per thread, as
   * the reference's per-thread arrays are) */
#pragma omp parallel reduction(+ : nbad)
  {
    const int nmax = o->nobs > 0 ? o->nobs : 1;
    int* idx = (int*)malloc(sizeof(int) * nmax);
    double* rloc = (double*)malloc(sizeof(double) * nmax);
    double* rdiag = (double*)malloc(sizeof(double) * nmax);
    double* trans = (double*)malloc(sizeof(double) * (size_t)ne * ne);
    double* transm = (double*)malloc(sizeof(double) * ne);
    double* gues = (double*)malloc(sizeof(double) * ne);
    double *h = NULL, *dep = NULL;
    int hcap = 0, q;
#pragma omp for schedule(dynamic)
    for (q = 0; q < nwork; q++) {
      const int p = subset ? subset[q] : q;
      const int L = oracle_scale_obs_local(o, pri[p], prj[p], prlev[p], prz ? prz[p] : 0.0, idx, rloc, rdiag);
      const int ld = L > 0 ? L : 1;
      int i, m, k, v;
      if (ld > hcap) {
        free(h);
        free(dep);
        hcap = ld + ld / 4 + 64;
        h = (double*)malloc(sizeof(double) * (size_t)hcap * ne);
        dep = (double*)malloc(sizeof(double) * hcap);
      }
      for (i = 0; i < L; i++) {
        for (m = 0; m < ne; m++) h[(size_t)m * ld + i] = hdxf[(size_t)idx[i] * ne + m];
        dep[i] = odep[idx[i]];
      }
      double mf = minfl;
      int st = oracle_letkf_core(ne, ld, L, h, rdiag, rloc, dep, &infl[p], trans, transm, NULL, 1,
                                 minfl > 0 ? &mf : NULL);
      if (st != 0) nbad++;
      if (nobsl_out) nobsl_out[p] = L;
      for (v = 0; v < nv; v++) {
        const double* x = xb + ((size_t)v * npts + p) * ne;
        double mean = x[0];
        for (m = 1; m < ne; m++) mean = mean + x[m];
        mean = mean / (double)ne;
        for (m = 0; m < ne; m++) gues[m] = x[m] - mean;
        for (m = 0; m < ne; m++) {
          double a = mean;
          /* beta = 1: transrlx(k,m) = (trans(k,m) + transm(k)) * 1, diagonal + 0 */
          for (k = 0; k < ne; k++) a = a + gues[k] * ((trans[(size_t)m * ne + k] + transm[k]) * 1.0);
          xa[((size_t)v * npts + p) * ne + m] = a;
        }
      }
    }
    free(idx); free(rloc); free(rdiag); free(h); free(dep); free(trans); free(transm); free(gues);
  }
  return nbad;
}

int oracle_scale_obs_local_batch(const oracle_scale_obs* o, int npts, const double* pri, const double* prj,
                                 const double* prlev, const double* prz, int cap, int* cnt, int* idx_out,
                                 double* rloc_out, int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
#pragma omp parallel
  {
    const int nmax = o->nobs > 0 ? o->nobs : 1;
    int* idx = (int*)malloc(sizeof(int) * nmax);
    double* rloc = (double*)malloc(sizeof(double) * nmax);
    double* rdiag = (double*)malloc(sizeof(double) * nmax);
    int p;
#pragma omp for schedule(dynamic)
    for (p = 0; p < npts; p++) {
      const int L = oracle_scale_obs_local(o, pri[p], prj[p], prlev[p], prz ? prz[p] : 0.0, idx, rloc, rdiag);
      const int n = L < cap ? L : cap;
      cnt[p] = L;
      memcpy(idx_out + (size_t)p * cap, idx, sizeof(int) * (size_t)(n > 0 ? n : 0));
      memcpy(rloc_out + (size_t)p * cap, rloc, sizeof(double) * (size_t)(n > 0 ? n : 0));
    }
    free(idx); free(rloc); free(rdiag);
  }
  return 0;
}
