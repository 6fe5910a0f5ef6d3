// obs_search.cu -- local observation search kernels (bit-exact selection order).
//
// One thread per grid point scans its candidate bucket ranges in the
// reference order and applies the reference's tests in FP64:
//   SCALE  scale/letkf/letkf_tools.f90:853-1178 (+ obs_choose,
//          scale/letkf/letkf_obs.f90:1054-1119), MEM_NP = 1
//   SPEEDY speedy/letkf/letkf_tools.f90:272-603 (+ common/common.f90:401-424)
// Count pass (idx == NULL) writes nobsl[p]; fill pass writes the rows at
// offs[p].  The same predicate code runs in both passes.
#include <math.h>

#include "letkf_common.cuh"

namespace letkf {

// scale/letkf/letkf_obs.f90:29-30 keep these as default-real literals
__device__ __forceinline__ double scale_dzf2() { return (double)13.33333333f; }

struct ScaleParams {
  double dx, dy, dlon_zero, dlat_zero, sigma_obs, sigma_obsv, sigma_obs_rain, sigma_obsv_rain, base_obsv_rain,
      sigma_obs_radar, sigma_obs_radar_noref, sigma_obsz_radar, radar_ref_thres_dbz, sigma_obs_tc, sigma_obsv_tc;
};

// One warp per grid point: lane l tests candidates ib + l, ib + l + 32, ...
// of each row range; accepted ones are written in candidate order through a
// ballot prefix.  A candidate is first tested in FP32 and rejected there only
// where its normalised distance exceeds the cut-off by more than 1e-3
// (FP32 rounding of these terms is below 1e-5); every other candidate takes
// the reference's FP64 test.
__global__ void search_scale_kernel(int nlon, int nlat, const int* __restrict__ G, int nobs,
                                    const double* __restrict__ ori, const double* __restrict__ orj,
                                    const double* __restrict__ olev, const double* __restrict__ odat,
                                    const double* __restrict__ oerr, const int* __restrict__ ocls,
                                    const int* __restrict__ ovarloc, int npts, const double* __restrict__ pri,
                                    const double* __restrict__ prj, const double* __restrict__ prlev,
                                    const double* __restrict__ prz, const double* __restrict__ var_local,
                                    ScaleParams P, const int64_t* __restrict__ offs, int* nobsl, int* idx,
                                    double* rloc, double* rdiag) {
  const int p = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (p >= npts) return;
  const int lane = threadIdx.x & 31;
  const int ld = nlon + 1;
  const double ri = pri[p], rj = prj[p], rlev = prlev[p], rz = prz ? prz[p] : 0.0;
  const double logr = log(rlev);
  int imin = (int)floor(ri - P.dlon_zero);
  if (imin < 1) imin = 1;
  int imax = (int)ceil(ri + P.dlon_zero);
  if (imax > nlon) imax = nlon;
  int jmin = (int)floor(rj - P.dlat_zero);
  if (jmin < 1) jmin = 1;
  int jmax = (int)ceil(rj + P.dlat_zero);
  if (jmax > nlat) jmax = nlat;
  const double dzf2 = scale_dzf2();
  const float cut32 = (float)dzf2 * 1.001f;
  const float logr32 = (float)logr, rz32 = (float)rz;
  int cnt = 0;
  const int64_t base = idx ? offs[p] : 0;
  if (nobs > 0 && G[(size_t)(nlat - 1) * ld + nlon] > 0 && imin <= imax && jmin <= jmax) {
    for (int j = jmin; j <= jmax; j++) {
      const int ib = G[(size_t)(j - 1) * ld + imin - 1], ie = G[(size_t)(j - 1) * ld + imax];
      for (int ob0 = ib; ob0 < ie; ob0 += 32) {
        const int ob = ob0 + lane;
        bool ok = ob < ie;
        double ndist = 0.0;
        int vl = 0;
        if (ok) {
          vl = ovarloc[ob];
          if (var_local && var_local[vl] < 2.2250738585072014e-308) ok = false;
        }
        const int cls = ok ? ocls[ob] : 0;
        if (ok) {
          // FP32 pre-test (certain rejections only)
          const float hx = (float)((ri - ori[ob]) * P.dx), hy = (float)((rj - orj[ob]) * P.dy);
          float sh, vz;
          if (cls == 2) {
            sh = (float)P.sigma_obs_rain;
            vz = fabsf(__logf((float)P.base_obsv_rain) - logr32) / (float)P.sigma_obsv_rain;
          } else if (cls >= 3 && cls <= 5) {
            sh = (float)((cls == 3 && odat[ob] <= P.radar_ref_thres_dbz + 1.0e-6) ? P.sigma_obs_radar_noref
                                                                                 : P.sigma_obs_radar);
            vz = fabsf((float)olev[ob] - rz32) / (float)P.sigma_obsz_radar;
          } else if (cls == 6) {
            sh = (float)P.sigma_obs_tc;
            vz = fabsf(__logf((float)olev[ob]) - logr32) / (float)P.sigma_obsv_tc;
          } else {
            sh = (float)P.sigma_obs;
            vz = fabsf(__logf((float)(cls == 1 ? odat[ob] : olev[ob])) - logr32) / (float)P.sigma_obsv;
          }
          const float hh = (hx * hx + hy * hy) / (sh * sh);
          ok = !(hh + vz * vz > cut32);
        }
        if (ok) {
          const double rdx = (ri - ori[ob]) * P.dx, rdy = (rj - orj[ob]) * P.dy;
          double nd_h = sqrt(sumsq_rn(rdx, rdy)), nd_v;
          if (cls == 1) {
            nd_h = nd_h / P.sigma_obs;
            nd_v = fabs(log(odat[ob]) - logr) / P.sigma_obsv;
          } else if (cls == 2) {
            nd_h = nd_h / P.sigma_obs_rain;
            nd_v = fabs(log(P.base_obsv_rain) - logr) / P.sigma_obsv_rain;
          } else if (cls >= 3 && cls <= 5) {
            if (cls == 3 && odat[ob] <= P.radar_ref_thres_dbz + 1.0e-6)
              nd_h = nd_h / P.sigma_obs_radar_noref;
            else
              nd_h = nd_h / P.sigma_obs_radar;
            nd_v = fabs(olev[ob] - rz) / P.sigma_obsz_radar;
          } else if (cls == 6) {
            nd_h = nd_h / P.sigma_obs_tc;
            nd_v = fabs(log(olev[ob]) - logr) / P.sigma_obsv_tc;
          } else {
            nd_h = nd_h / P.sigma_obs;
            nd_v = fabs(log(olev[ob]) - logr) / P.sigma_obsv;
          }
          ndist = sumsq_rn(nd_h, nd_v);
          ok = !(ndist > dzf2);
        }
        const unsigned bal = __ballot_sync(0xffffffffu, ok);
        if (ok && idx) {
          const int64_t at = base + cnt + __popc(bal & ((1u << lane) - 1u));
          double nrloc = exp(-0.5 * ndist);
          if (var_local) nrloc = nrloc * var_local[vl];
          idx[at] = ob;
          rloc[at] = nrloc;
          rdiag[at] = oerr[ob] * oerr[ob] / nrloc;
        }
        cnt += __popc(bal);
      }
    }
  }
  if (!idx && lane == 0) nobsl[p] = cnt;
}

// common/common.f90:401-424 (pi and re of common/common.f90:28,35)
__device__ __forceinline__ double distll(double alon, double alat, double blon, double blat) {
  const double pi = 3.1415926535, re = 6371.3e3, r180 = 1.0 / 180.0;
  const double lon1 = alon * pi * r180, lon2 = blon * pi * r180;
  const double lat1 = alat * pi * r180, lat2 = blat * pi * r180;
  double cosd = __dadd_rn(__dmul_rn(sin(lat1), sin(lat2)), __dmul_rn(__dmul_rn(cos(lat1), cos(lat2)), cos(lon2 - lon1)));
  cosd = fmin(1.0, cosd);
  cosd = fmax(-1.0, cosd);
  return acos(cosd) * re;
}

__device__ __forceinline__ int first_below(double x, const double* axis, int lim) {
  for (int i = 1; i <= lim; i++)
    if (x < axis[i]) return i;
  return lim + 1;
}

struct SpeedyCtx {
  int nlon, nlat;
  const double *lon, *lat;
  const int* G;
  const double *elm, *olon, *olat, *olev, *odat, *oerr, *var_local;
  double dist_zero, dist_zerov, sigma_obs, sigma_obsv;
  // GFS variant (gfs/letkf/letkf_tools.f90:686-925)
  int gfs;
  double dist_zero_rain, dist_zerov_rain, sigma_obs_rain, base_obsv_rain;
  // FP32 pre-test of the horizontal distance: cos of the cut-off angles
  // dist_zero / re (-2 where the cut-off reaches the antipode)
  float cos_cut, cos_cut_rain;
};

// One warp per grid point: lane l tests candidates ib + l, ib + l + 32, ...;
// the accepted ones are written in candidate order (ballot prefix), so lists
// and their order are those of the reference's sequential loop.
struct WarpList {
  int* idx;
  double *rloc, *rdiag;
  int64_t base;
  int cnt;
  __device__ __forceinline__ void push(bool ok, int ob, double r, double rd) {
    const unsigned bal = __ballot_sync(0xffffffffu, ok);
    if (ok && idx) {
      const int64_t at = base + cnt + __popc(bal & ((1u << (threadIdx.x & 31)) - 1u));
      idx[at] = ob;
      rloc[at] = r;
      rdiag[at] = rd;
    }
    cnt += __popc(bal);
  }
};

// false only where the reference's FP64 test (common/common.f90:401-424:
// acos of the cosine of the angle, times re, against the cut-off) certainly
// rejects: the FP32 cosine is below the cut-off's by more than 1e-4 (FP32
// rounding of these terms is below 1e-6); every other candidate gets the
// FP64 test
__device__ __forceinline__ bool maybe_within(const SpeedyCtx& c, int ob, float s1, float c1, double lon1,
                                             float cos_cut) {
  constexpr double D2R = 3.1415926535 / 180.0;
  float s2, c2;
  sincosf((float)(c.olat[ob] * D2R), &s2, &c2);
  const float dl = (float)((c.olon[ob] - lon1) * D2R);
  const float cosd = s1 * s2 + c1 * c2 * cosf(dl);
  return cosd >= cos_cut - 1.0e-4f;
}

// GFS candidate test (gfs/letkf/letkf_tools.f90:833-915); logrlev = ln p of
// the point; var_local (6 classes) may be NULL (nvar = 0)
__device__ __forceinline__ void gfs_range(const SpeedyCtx& c, int ib, int ie, double lon1, double lat1, float s1,
                                          float c1, double logrlev, WarpList& out) {
  const int lane = threadIdx.x & 31;
  for (int ip0 = ib; ip0 <= ie; ip0 += 32) {
    const int ip = ip0 + lane;
    bool ok = false;
    int ob = ip - 1;
    double r = 0.0, rd = 0.0;
    if (ip <= ie) {
      const int elm = (int)llround(c.elm[ob]);
      ok = maybe_within(c, ob, s1, c1, lon1, elm == 19999 ? c.cos_cut_rain : c.cos_cut);
      double dlev = 0.0;
      if (ok) {
        if (elm == 14593) {
          dlev = fabs(log(c.odat[ob]) - logrlev);
          ok = !(dlev > c.dist_zerov);
        } else if (elm == 19999) {
          dlev = fabs(log(c.base_obsv_rain) - logrlev);
          ok = !(dlev > c.dist_zerov_rain);
        } else if (elm < 99991) {
          dlev = fabs(log(c.olev[ob]) - logrlev);
          ok = !(dlev > c.dist_zerov);
        }
      }
      double dist = 0.0;
      if (ok) {
        dist = distll(c.olon[ob], c.olat[ob], lon1, lat1);
        ok = !(dist > (elm == 19999 ? c.dist_zero_rain : c.dist_zero));
      }
      double vl = 1.0;
      if (ok && c.var_local) {
        int iobs;
        switch (elm) {
          case 2819: case 2820: iobs = 1; break;
          case 3073: case 3074: iobs = 2; break;
          case 3330: case 3331: iobs = 3; break;
          case 14593: iobs = 4; break;
          case 19999: iobs = 5; break;
          case 99991: case 99992: case 99993: iobs = 6; break;
          default: iobs = 0; break;  // class undefined in the reference: not selected
        }
        if (iobs == 0) ok = false;
        else {
          vl = c.var_local[iobs - 1];
          if (vl < 2.2250738585072014e-308) ok = false;
        }
      }
      if (ok && out.idx) {
        const double a = dist / (elm == 19999 ? c.sigma_obs_rain : c.sigma_obs), b = dlev / c.sigma_obsv;
        r = exp(-0.5 * (a * a + b * b));
        if (c.var_local) r = r * vl;
        rd = c.oerr[ob] * c.oerr[ob];
      }
    }
    out.push(ok, ob, r, rd);
  }
}

// Test candidates [ib, ie] (1-based, inclusive) for one point; appends.
__device__ __forceinline__ void speedy_range(const SpeedyCtx& c, int ib, int ie, double lon1, double lat1, float s1,
                                             float c1, int ilev, double logpfm, WarpList& out) {
  const int lane = threadIdx.x & 31;
  for (int ip0 = ib; ip0 <= ie; ip0 += 32) {
    const int ip = ip0 + lane;
    bool ok = false;
    int ob = ip - 1;
    double r = 0.0, rd = 0.0;
    if (ip <= ie) {
      const int elm = (int)llround(c.elm[ob]);
      ok = maybe_within(c, ob, s1, c1, lon1, c.cos_cut);
      double dlev = 0.0, dist = 0.0;
      if (ok) {
        if (elm == 14593 && ilev > 1) dlev = fabs(log(c.odat[ob]) - logpfm);
        else if (elm != 14593) dlev = fabs(log(c.olev[ob]) - logpfm);
        ok = !(dlev > c.dist_zerov);
      }
      if (ok) {
        dist = distll(c.olon[ob], c.olat[ob], lon1, lat1);
        ok = !(dist > c.dist_zero);
      }
      double vl = 0.0;
      if (ok) {
        int iobs;
        switch (elm) {
          case 2819: iobs = 1; break;
          case 2820: iobs = 2; break;
          case 3073: iobs = 3; break;
          case 3330: iobs = 4; break;
          case 3331: iobs = 5; break;
          case 14593: iobs = 6; break;
          default: iobs = 7; break;
        }
        vl = c.var_local[iobs - 1];
        ok = !(vl < 2.2250738585072014e-308);
      }
      if (ok && out.idx) {
        const double a = dist / c.sigma_obs, b = dlev / c.sigma_obsv;
        rd = c.oerr[ob] * c.oerr[ob];
        r = exp(-0.5 * (a * a + b * b)) * vl;
      }
    }
    out.push(ok, ob, r, rd);
  }
}

// speedy/letkf/letkf_tools.f90:575-603
__device__ __forceinline__ void speedy_sub(const SpeedyCtx& c, int imin, int imax, int jmin, int jmax, double lon1,
                                           double lat1, float s1, float c1, int ilev, double logpfm, WarpList& out) {
  const int nlon = c.nlon;
  for (int j = jmin; j <= jmax; j++) {
    int ib;
    if (imin > 1) ib = c.G[(size_t)(j - 1) * nlon + imin - 2] + 1;
    else if (j > 1) ib = c.G[(size_t)(j - 2) * nlon + nlon - 1] + 1;
    else ib = 1;
    const int ie = c.G[(size_t)(j - 1) * nlon + imax - 1];
    if (ie - ib + 1 == 0) continue;
    if (c.gfs) gfs_range(c, ib, ie, lon1, lat1, s1, c1, logpfm, out);
    else speedy_range(c, ib, ie, lon1, lat1, s1, c1, ilev, logpfm, out);
  }
}

__global__ void search_speedy_kernel(SpeedyCtx c, int npts, const double* __restrict__ plon,
                                     const double* __restrict__ plat, const double* __restrict__ pdlon,
                                     const int* __restrict__ pilev, const double* __restrict__ plogp, double dlat_zero,
                                     const int64_t* __restrict__ offs, int* nobsl, int* idx, double* rloc,
                                     double* rdiag) {
  const int p = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);  // one warp per point
  if (p >= npts) return;
  const int nlon = c.nlon, nlat = c.nlat;
  const double lon1 = plon[p], lat1 = plat[p];
  // SPEEDY: ln p_full of the point and its level; GFS: ln of the point's pressure
  const double logpfm = c.gfs ? log(plogp[p]) : plogp[p];
  const int ilev = c.gfs ? 0 : pilev[p];
  const double dlon = c.gfs ? dlat_zero / cos(lat1 * 3.1415926535 / 180.0) : pdlon[p];
  double minlon = lon1 - dlon, maxlon = lon1 + dlon;
  const double minlat = lat1 - dlat_zero, maxlat = lat1 + dlat_zero;
  if (maxlon - minlon >= 360.0) {
    minlon = 0.0;
    maxlon = 360.0;
  }
  const int jmin = first_below(minlat, c.lat, nlat - 2);
  const int jmax = first_below(maxlat, c.lat, nlat - 2);
  WarpList out;
  out.idx = idx;
  out.rloc = rloc;
  out.rdiag = rdiag;
  out.base = idx ? offs[p] : 0;
  out.cnt = 0;
  const float s1 = sinf((float)(lat1 * (3.1415926535 / 180.0))), c1 = cosf((float)(lat1 * (3.1415926535 / 180.0)));
  int imin, imax;
#define SUB(a, b) speedy_sub(c, (a), (b), jmin, jmax, lon1, lat1, s1, c1, ilev, logpfm, out)
  if (minlon >= 0 && maxlon <= 360.0) {
    imin = first_below(minlon, c.lon, nlon - 1);
    imax = first_below(maxlon, c.lon, nlon - 1);
    SUB(imin, imax);
  } else if (minlon >= 0 && maxlon > 360.0) {
    imin = first_below(minlon, c.lon, nlon - 1);
    maxlon = maxlon - 360.0;
    if (maxlon > 360.0) {
      SUB(1, nlon);
    } else {
      imax = first_below(maxlon, c.lon, nlon - 1);
      if (imax > imin) {
        SUB(1, nlon);
      } else {
        SUB(1, imax);
        imin = first_below(minlon, c.lon, nlon - 1);
        SUB(imin, nlon);
      }
    }
  } else if (minlon < 0 && maxlon <= 360.0) {
    imax = first_below(maxlon, c.lon, nlon - 1);
    minlon = minlon + 360.0;
    if (minlon < 0) {
      SUB(1, nlon);
    } else {
      imin = first_below(minlon, c.lon, nlon - 1);
      if (imin < imax) {
        SUB(1, nlon);
      } else {
        SUB(1, imax);
        imin = first_below(minlon, c.lon, nlon - 1);
        SUB(imin, nlon);
      }
    }
  } else {
    maxlon = maxlon - 360.0;
    minlon = minlon + 360.0;
    if (maxlon > 360.0 || minlon < 0) {
      SUB(1, nlon);
    } else {
      imin = first_below(minlon, c.lon, nlon - 1);
      imax = first_below(maxlon, c.lon, nlon - 1);
      if (imin > imax) SUB(1, nlon);
      else SUB(imin, imax);
    }
  }
#undef SUB
  if (!idx && (threadIdx.x & 31) == 0) nobsl[p] = out.cnt;
}

// cos of the angle dist / re (the FP32 pre-test's threshold)
static float cos_cut(double dist) {
  const double ang = dist / 6371.3e3;  // common/common.f90:35
  return ang >= 3.14159 ? -2.f : (float)cos(ang);
}

static void launch_speedy_warps(const SpeedyCtx& c, int npts, const double* plon, const double* plat,
                                const double* pdlon, const int* pilev, const double* plogp, double dlat_zero,
                                const int64_t* offs, int* nobsl, int* idx, double* rloc, double* rdiag,
                                cudaStream_t stream) {
  const int64_t threads = (int64_t)npts * 32;
  const int bs = 128;
  search_speedy_kernel<<<(unsigned)((threads + bs - 1) / bs), bs, 0, stream>>>(c, npts, plon, plat, pdlon, pilev,
                                                                               plogp, dlat_zero, offs, nobsl, idx,
                                                                               rloc, rdiag);
  note_launch();
}

int launch_search_scale(int nlon, int nlat, const int* G, int nobs, const double* ori, const double* orj,
                        const double* olev, const double* odat, const double* oerr, const int* ocls,
                        const int* ovarloc, int npts, const double* pri, const double* prj, const double* prlev,
                        const double* prz, const double* var_local, const double* params, const int64_t* offs,
                        int* nobsl, int* idx, double* rloc, double* rdiag, cudaStream_t stream) {
  if (npts <= 0) return npts == 0 ? LETKF_OK : LETKF_ERR_ARG;
  ScaleParams P;
  double* f = &P.dx;
  for (int i = 0; i < 15; i++) f[i] = params[i];
  const int64_t threads = (int64_t)npts * 32;  // one warp per point
  const int bs = 128;
  search_scale_kernel<<<(unsigned)((threads + bs - 1) / bs), bs, 0, stream>>>(
      nlon, nlat, G, nobs, ori, orj, olev, odat, oerr, ocls, ovarloc, npts, pri, prj, prlev, prz, var_local, P, offs,
      nobsl, idx, rloc, rdiag);
  note_launch();
  return cuda_status(cudaGetLastError());
}

int launch_search_speedy(int nlon, int nlat, const double* lon, const double* lat, const int* G, int nobs,
                         const double* elm, const double* olon, const double* olat, const double* olev,
                         const double* odat, const double* oerr, int npts, const double* plon, const double* plat,
                         const double* pdlon, const int* pilev, const double* plogp, const double* var_local,
                         const double* params, const int64_t* offs, int* nobsl, int* idx, double* rloc,
                         double* rdiag, cudaStream_t stream) {
  if (npts <= 0) return npts == 0 ? LETKF_OK : LETKF_ERR_ARG;
  SpeedyCtx c;
  c.nlon = nlon;
  c.nlat = nlat;
  c.lon = lon;
  c.lat = lat;
  c.G = G;
  c.elm = elm;
  c.olon = olon;
  c.olat = olat;
  c.olev = olev;
  c.odat = odat;
  c.oerr = oerr;
  c.var_local = var_local;
  c.dist_zero = params[0];
  c.dist_zerov = params[1];
  c.sigma_obs = params[3];
  c.sigma_obsv = params[4];
  c.gfs = 0;
  c.dist_zero_rain = c.dist_zerov_rain = c.sigma_obs_rain = c.base_obsv_rain = 0.0;
  c.cos_cut = cos_cut(c.dist_zero);
  c.cos_cut_rain = c.cos_cut;
  (void)nobs;
  launch_speedy_warps(c, npts, plon, plat, pdlon, pilev, plogp, params[2], offs, nobsl, idx, rloc, rdiag, stream);
  return cuda_status(cudaGetLastError());
}

int launch_search_gfs(int nlon, int nlat, const double* lon, const double* lat, const int* G, const double* elm,
                      const double* olon, const double* olat, const double* olev, const double* odat,
                      const double* oerr, int npts, const double* plon, const double* plat, const double* prlev,
                      const double* var_local, const double* params, const int64_t* offs, int* nobsl, int* idx,
                      double* rloc, double* rdiag, cudaStream_t stream) {
  if (npts <= 0) return npts == 0 ? LETKF_OK : LETKF_ERR_ARG;
  SpeedyCtx c;
  c.nlon = nlon;
  c.nlat = nlat;
  c.lon = lon;
  c.lat = lat;
  c.G = G;
  c.elm = elm;
  c.olon = olon;
  c.olat = olat;
  c.olev = olev;
  c.odat = odat;
  c.oerr = oerr;
  c.var_local = var_local;
  c.gfs = 1;
  c.dist_zero = params[0];
  c.dist_zerov = params[1];
  c.dist_zero_rain = params[2];
  c.dist_zerov_rain = params[3];
  c.sigma_obs = params[4];
  c.sigma_obsv = params[5];
  c.sigma_obs_rain = params[6];
  c.base_obsv_rain = params[7];
  const double dz = c.dist_zero > c.dist_zero_rain ? c.dist_zero : c.dist_zero_rain;
  const double dlat_zero = dz / 3.1415926535 / 6371.3e3 * 180.0;  // gfs/letkf/letkf_tools.f90:712
  c.cos_cut = cos_cut(c.dist_zero);
  c.cos_cut_rain = cos_cut(c.dist_zero_rain);
  launch_speedy_warps(c, npts, plon, plat, nullptr, nullptr, prlev, dlat_zero, offs, nobsl, idx, rloc, rdiag, stream);
  return cuda_status(cudaGetLastError());
}

// ---- exclusive scan of int32 counts into int64 offsets (three-phase) ----
constexpr int SCAN_BS = 1024;

__global__ void scan_blocks_kernel(int n, const int* __restrict__ in, int64_t* out, int64_t* bsum) {
  __shared__ int64_t s[SCAN_BS];
  const int i = blockIdx.x * SCAN_BS + threadIdx.x;
  s[threadIdx.x] = i < n ? (int64_t)in[i] : 0;
  __syncthreads();
  for (int o = 1; o < SCAN_BS; o <<= 1) {
    int64_t v = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
    __syncthreads();
    s[threadIdx.x] += v;
    __syncthreads();
  }
  if (i < n) out[i + 1] = s[threadIdx.x];  // inclusive into out[i+1]
  if (threadIdx.x == SCAN_BS - 1) bsum[blockIdx.x] = s[threadIdx.x];
}

// exclusive scan of the nb block sums by one block of SCAN_BS threads: each
// thread sums a contiguous chunk of ceil(nb / SCAN_BS) sums, the chunk totals
// are scanned in shared memory, and each thread rewrites its chunk
__global__ void scan_sums_kernel(int nb, int64_t* bsum) {
  __shared__ int64_t s[SCAN_BS];
  const int t = threadIdx.x;
  const int per = (nb + SCAN_BS - 1) / SCAN_BS;
  const int b0 = min(nb, t * per), b1 = min(nb, b0 + per);
  int64_t tot = 0;
  for (int b = b0; b < b1; b++) tot += bsum[b];
  s[t] = tot;
  __syncthreads();
  for (int o = 1; o < SCAN_BS; o <<= 1) {
    const int64_t v = t >= o ? s[t - o] : 0;
    __syncthreads();
    s[t] += v;
    __syncthreads();
  }
  int64_t run = s[t] - tot;
  for (int b = b0; b < b1; b++) {
    const int64_t v = bsum[b];
    bsum[b] = run;
    run += v;
  }
}

__global__ void scan_add_kernel(int n, int64_t* out, const int64_t* bsum) {
  const int i = blockIdx.x * SCAN_BS + threadIdx.x;
  if (i < n) out[i + 1] += bsum[blockIdx.x];
  if (i == 0) out[0] = 0;
}

int launch_exclusive_scan(int n, const int* counts, int64_t* offs, int64_t* scratch, cudaStream_t stream) {
  if (n <= 0) {
    cudaMemsetAsync(offs, 0, sizeof(int64_t), stream);
    return LETKF_OK;
  }
  const int nb = (n + SCAN_BS - 1) / SCAN_BS;
  scan_blocks_kernel<<<nb, SCAN_BS, 0, stream>>>(n, counts, offs, scratch);
  scan_sums_kernel<<<1, SCAN_BS, 0, stream>>>(nb, scratch);
  scan_add_kernel<<<nb, SCAN_BS, 0, stream>>>(n, offs, scratch);
  note_launch();
  note_launch();
  note_launch();
  return cuda_status(cudaGetLastError());
}

template <typename T>
__global__ void gather_rows_kernel(int ne, int64_t nrows, const int* __restrict__ idx, const T* __restrict__ ens,
                                   const T* __restrict__ dep, T* rows_out, T* dep_out) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t tot = nrows * ne;
  if (t < tot) {
    const int64_t r = t / ne;
    const int m = (int)(t - r * ne);
    rows_out[t] = ens[(size_t)idx[r] * ne + m];
    if (m == 0 && dep) dep_out[r] = dep[idx[r]];
  }
}

int launch_gather_rows(int ne, int64_t nrows, const int* idx, const void* ens, const void* dep, int elem_bytes,
                       void* rows_out, void* dep_out, cudaStream_t stream) {
  if (nrows <= 0) return LETKF_OK;
  const int64_t tot = nrows * ne;
  const int bs = 256;
  const unsigned grid = (unsigned)((tot + bs - 1) / bs);
  if (elem_bytes == 8)
    gather_rows_kernel<double><<<grid, bs, 0, stream>>>(ne, nrows, idx, (const double*)ens, (const double*)dep,
                                                        (double*)rows_out, (double*)dep_out);
  else if (elem_bytes == 4)
    gather_rows_kernel<float><<<grid, bs, 0, stream>>>(ne, nrows, idx, (const float*)ens, (const float*)dep,
                                                       (float*)rows_out, (float*)dep_out);
  else
    return LETKF_ERR_ARG;
  note_launch();
  return cuda_status(cudaGetLastError());
}

}  // namespace letkf
