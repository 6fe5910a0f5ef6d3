// obs_operator.cu -- the SPEEDY observation operator H(x) on the device.
//
// For every (observation, member): phys2ijk (speedy/common/common_obs_speedy.f90:
// 137-206) maps (lon, lat, pressure) to fractional grid indices (ri, rj, rk)
// against that member's p_full = ps * sig(k) (speedy/common/common_speedy.f90:
// 291-309); the driver rules of speedy/letkf/obsope.f90:53-104 reject what is
// out of range (u/v below the lowest full level are clamped to rk = 1.00001,
// a missing ps value < -100 is skipped); Trans_XtoY (common_obs_speedy.f90:
// 29-80) interpolates u, v, t, q (trilinear), ps, rain (bilinear) or relative
// humidity (calc_rh at the eight corners, :84-109).  hx(n, m) = 0 and qc = 0
// where the driver would CYCLE; qc(n) is the minimum over members, as
// set_letkf_obs takes it (speedy/letkf/letkf_obs.f90:157-158).
//
// One warp per observation, members over the lanes, so the hx row is written
// coalesced.  Products and sums use the _rn intrinsics so that no multiply-add
// is contracted: the rounding follows the reference's expression order and
// only log/exp differ (by an ulp) from a host build.
#include "letkf_common.cuh"

namespace letkf {

constexpr int OBSOPE_NT = 256;
constexpr int ID_U = 2819, ID_V = 2820, ID_T = 3073, ID_Q = 3330, ID_RH = 3331, ID_PS = 14593, ID_RAIN = 9999;

struct SpeedyFields {
  int nlon, nlat, nlev, ne;
  const double* lat;  // [nlat] Gaussian latitudes (degrees), searched as the reference does
  const double* sig;  // [nlev] full-level sigma
  const double* v3d;  // v3d(i, j, k, n) of member m at v3d[m*mem3 + (n*nlev + k)*rec3 + j*nlon + i]
  int64_t mem3, rec3;
  const double* v2d;  // v2d(i, j, n) of member m at v2d[m*mem2 + n*rec2 + j*nlon + i]; n = 0 ps, 1 rain
  int64_t mem2, rec2;
};

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }

// Fortran CEILING, saturated far outside any grid
__device__ __forceinline__ long long ceil_i(double x) {
  if (x >= 1.0e15) return 1000000000000000LL;
  if (x <= -1.0e15) return -1000000000000000LL;
  return (long long)ceil(x);
}

// itpl_2d (common_obs_speedy.f90:210-237) on corners c[jj][ii]
__device__ __forceinline__ double itpl2(const double c[2][2], double ai, double aj) {
  const double bi = sub(1.0, ai), bj = sub(1.0, aj);
  double s = mul(mul(c[0][0], bi), bj);
  s = add(s, mul(mul(c[0][1], ai), bj));
  s = add(s, mul(mul(c[1][0], bi), aj));
  return add(s, mul(mul(c[1][1], ai), aj));
}

// itpl_3d (common_obs_speedy.f90:239-280) on corners c[kk][jj][ii]
__device__ __forceinline__ double itpl3(const double c[2][2][2], double ai, double aj, double ak) {
  const double bi = sub(1.0, ai), bj = sub(1.0, aj), bk = sub(1.0, ak);
  double s = mul(mul(mul(c[0][0][0], bi), bj), bk);
  s = add(s, mul(mul(mul(c[0][0][1], ai), bj), bk));
  s = add(s, mul(mul(mul(c[0][1][0], bi), aj), bk));
  s = add(s, mul(mul(mul(c[0][1][1], ai), aj), bk));
  s = add(s, mul(mul(mul(c[1][0][0], bi), bj), ak));
  s = add(s, mul(mul(mul(c[1][0][1], ai), bj), ak));
  s = add(s, mul(mul(mul(c[1][1][0], bi), aj), ak));
  return add(s, mul(mul(mul(c[1][1][1], ai), aj), ak));
}

// calc_rh (common_obs_speedy.f90:84-109)
__device__ double calc_rh(double t, double q, double p) {
  const double t0 = 273.15, e0c = 6.11, al = 17.3, bl = 237.3, e0i = 6.1121, ai = 22.587, bi = 273.86;
  const double e = mul(mul(q, p), 0.01) / add(mul(0.378, q), 0.622);
  const double tc = sub(t, t0);
  double es;
  if (tc >= 0.0) {
    es = mul(e0c, exp(mul(al, tc) / add(bl, tc)));
  } else if (tc <= -15.0) {
    es = mul(e0i, exp(mul(ai, tc) / add(bi, tc)));
  } else {
    const double wc = mul(mul(e0c, exp(mul(al, tc) / add(bl, tc))), add(15.0, tc)) / 15.0;
    const double wi = mul(mul(e0i, exp(mul(ai, tc) / add(bi, tc))), -tc) / 15.0;
    es = add(wc, wi);
  }
  return e / es;
}

// corner column (0: i-1, 1: i, wrapping to column 1 past nlon), 1-based
__device__ __forceinline__ long long col(long long i, int ii, int nlon) {
  return ii == 0 ? i - 1 : (i <= nlon ? i : 1);
}

__device__ __forceinline__ double f2(const SpeedyFields& f, int m, int n, long long i, long long j) {
  return f.v2d[(int64_t)m * f.mem2 + (int64_t)n * f.rec2 + (int64_t)(j - 1) * f.nlon + (i - 1)];
}
__device__ __forceinline__ double f3(const SpeedyFields& f, int m, int n, long long i, long long j, long long k) {
  return f.v3d[(int64_t)m * f.mem3 + ((int64_t)n * f.nlev + (k - 1)) * f.rec3 + (int64_t)(j - 1) * f.nlon + (i - 1)];
}

__global__ void __launch_bounds__(OBSOPE_NT) speedy_obsope_kernel(SpeedyFields f, int nobs,
                                                                   const int* __restrict__ elem,
                                                                   const double* __restrict__ rlon,
                                                                   const double* __restrict__ rlat,
                                                                   const double* __restrict__ rlev,
                                                                   const double* __restrict__ odat, double* hx,
                                                                   int* qc_member, int* qc) {
  const int lane = threadIdx.x & 31;
  const int nwarp = gridDim.x * (OBSOPE_NT / 32);
  for (int n = blockIdx.x * (OBSOPE_NT / 32) + (threadIdx.x >> 5); n < nobs; n += nwarp) {
    const int el = elem[n];
    const double lo = rlon[n], la = rlat[n], lev = rlev[n];
    // rlon -> ri, rlat -> rj (the same for every member)
    double ri;
    if (lo == 0.0 || lo == 360.0) ri = (double)(f.nlon + 1);
    else ri = add(mul(lo / 360.0, (double)f.nlon), 1.0);
    bool okh = !isnan(ri) && ceil_i(ri) >= 2 && ceil_i(ri) <= f.nlon + 1;
    double rj = 0.0;
    if (okh) {
      int j = 1;
      while (j <= f.nlat && !(la < f.lat[j - 1])) j++;
      if (j == 1) {
        rj = add(la, 90.0) / add(f.lat[0], 90.0);
      } else if (j == f.nlat + 1) {
        rj = add((double)f.nlat, sub(la, f.lat[f.nlat - 1]) / sub(90.0, f.lat[f.nlat - 1]));
      } else {
        rj = add((double)(j - 1), sub(la, f.lat[j - 2]) / sub(f.lat[j - 1], f.lat[j - 2]));
      }
      okh = !isnan(rj) && ceil_i(rj) >= 2 && ceil_i(rj) <= f.nlat;
    }
    const long long ic = okh ? ceil_i(ri) : 2, jc = okh ? ceil_i(rj) : 2;
    const double ai = sub(ri, (double)(ic - 1)), aj = sub(rj, (double)(jc - 1));
    const double loglev = (el != ID_PS && lev > 0.0) ? log(lev) : 0.0;
    int all = 1;
    for (int m = lane; m < f.ne; m += 32) {
      int q = okh;
      double rk = 0.0, y = 0.0;
      if (q && el != ID_PS) {
        if (!(lev > 0.0)) {
          q = 0;
        } else {
          double ps[2][2];
#pragma unroll
          for (int jj = 0; jj < 2; jj++)
#pragma unroll
            for (int ii = 0; ii < 2; ii++) ps[jj][ii] = f2(f, m, 0, col(ic, ii, f.nlon), jc - 1 + jj);
          double prev = 0.0, cur = 0.0;
          int k;
          for (k = 1; k <= f.nlev; k++) {  // plev(k) = itpl_2d(LOG(p_full(:, :, k))) as the search needs it
            const double sg = f.sig[k - 1];
            double c[2][2];
#pragma unroll
            for (int jj = 0; jj < 2; jj++)
#pragma unroll
              for (int ii = 0; ii < 2; ii++) c[jj][ii] = log(mul(ps[jj][ii], sg));
            prev = cur;
            cur = itpl2(c, ai, aj);
            if (k == 1) continue;
            if (k == f.nlev || cur < loglev) break;
          }
          rk = add((double)(k - 1), sub(loglev, prev) / sub(cur, prev));
          if (isnan(rk)) q = 0;
        }
      }
      if (q) {  // obsope.f90:70-96
        if (ceil_i(rk) > f.nlev) {
          q = 0;
        } else if (ceil_i(rk) < 2 && el != ID_PS) {
          if (el == ID_U || el == ID_V) rk = 1.00001;
          else q = 0;
        }
        if (el == ID_PS && odat[n] < -100.0) q = 0;
      }
      if (q) {  // Trans_XtoY
        if (el == ID_PS || el == ID_RAIN) {
          const int v = el == ID_PS ? 0 : 1;
          double c[2][2];
#pragma unroll
          for (int jj = 0; jj < 2; jj++)
#pragma unroll
            for (int ii = 0; ii < 2; ii++) c[jj][ii] = f2(f, m, v, col(ic, ii, f.nlon), jc - 1 + jj);
          y = itpl2(c, ai, aj);
        } else if (el == ID_U || el == ID_V || el == ID_T || el == ID_Q || el == ID_RH) {
          const int v = el == ID_U ? 0 : el == ID_V ? 1 : el == ID_T ? 2 : 3;
          const long long kc = ceil_i(rk);
          const double ak = sub(rk, (double)(kc - 1));
          double c[2][2][2];
#pragma unroll
          for (int kk = 0; kk < 2; kk++)
#pragma unroll
            for (int jj = 0; jj < 2; jj++)
#pragma unroll
              for (int ii = 0; ii < 2; ii++) {
                const long long i1 = col(ic, ii, f.nlon), j1 = jc - 1 + jj, k1 = kc - 1 + kk;
                if (el != ID_RH) {
                  c[kk][jj][ii] = f3(f, m, v, i1, j1, k1);
                } else {
                  const double p = mul(f2(f, m, 0, i1, j1), f.sig[k1 - 1]);
                  c[kk][jj][ii] = calc_rh(f3(f, m, 2, i1, j1, k1), f3(f, m, 3, i1, j1, k1), p);
                }
              }
          y = itpl3(c, ai, aj, ak);
        }
      }
      hx[(size_t)n * f.ne + m] = y;
      if (qc_member) qc_member[(size_t)n * f.ne + m] = q;
      all &= q;
    }
    all = __all_sync(0xffffffffu, all);
    if (qc && lane == 0) qc[n] = all;
  }
}

}  // namespace letkf

using namespace letkf;

extern "C" int letkf_speedy_obsope(int nlon, int nlat, int nlev, int ne, const double* lat, const double* sig,
                                   const double* v3d, int64_t v3d_mem_stride, int64_t v3d_rec_stride,
                                   const double* v2d, int64_t v2d_mem_stride, int64_t v2d_rec_stride, int nobs,
                                   const int* elem, const double* rlon, const double* rlat, const double* rlev,
                                   const double* odat, double* hx, int* qc_member, int* qc, void* stream) {
  if (nlon < 1 || nlat < 2 || nlev < 2 || ne < 1 || nobs < 0) return LETKF_ERR_ARG;
  if (!lat || !sig || !v3d || !v2d || v3d_rec_stride < (int64_t)nlat * nlon || v2d_rec_stride < (int64_t)nlat * nlon ||
      v3d_mem_stride < 0 || v2d_mem_stride < 0)
    return LETKF_ERR_ARG;
  if (nobs > 0 && (!elem || !rlon || !rlat || !rlev || !odat || !hx)) return LETKF_ERR_ARG;
  int nd = 0;
  if (cudaGetDeviceCount(&nd) != cudaSuccess || nd < 1) {
    cudaGetLastError();
    return LETKF_ERR_NOGPU;
  }
  if (nobs == 0) return LETKF_OK;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int per = OBSOPE_NT / 32;
  const int need = (nobs + per - 1) / per;
  const int grid = need < nsm * 8 ? need : nsm * 8;
  SpeedyFields f{nlon, nlat, nlev, ne, lat, sig, v3d, v3d_mem_stride, v3d_rec_stride, v2d, v2d_mem_stride,
                 v2d_rec_stride};
  speedy_obsope_kernel<<<grid, OBSOPE_NT, 0, (cudaStream_t)stream>>>(f, nobs, elem, rlon, rlat, rlev, odat, hx,
                                                                     qc_member, qc);
  note_launch();
  return cuda_status(cudaGetLastError());
}
