// sweep_search.cuh -- CTA-wide local observation search of the fused sweeps.
//
// The SCALE search (scale/letkf/letkf_tools.f90:853-1178) for one grid point:
// the candidate ranges of obs_choose (scale/letkf/letkf_obs.f90:1054-1119) are
// flattened over the CTA, every candidate is tested with an FP32 filter and the
// ambiguous band |ndist - cutoff| < 1e-3 cutoff is re-tested with the
// reference's FP64 formula.  Accepted observations are compacted, in the
// reference order, into a pending list (index, weight rloc/err^2, departure,
// rloc); `flush(nr)` consumes the first nr entries whenever CH are pending and
// once more for the remainder.  Returns the number of accepted observations.
// With probe >= 0 the accepted entries are also written, in emitted order, to
// the selection probe of SweepArgs (slot `probe`).
#pragma once
#include "sweep_args.cuh"

namespace letkf {

constexpr int SW_MAXROWS = 128;
constexpr float SW_BAND = 1.0e-3f;

// exact FP64 SCALE test (scale/letkf/letkf_tools.f90:961-1022); returns ndist
__device__ __forceinline__ double scale_ndist_exact(const SweepArgs& a, int ob, double ri, double rj, double logr,
                                                    double rz) {
  const SweepScaleParams& P = a.P;
  const double rdx = (ri - a.ori[ob]) * P.dx, rdy = (rj - a.orj[ob]) * P.dy;
  double nd_h = sqrt(sumsq_rn(rdx, rdy)), nd_v;
  const int cls = a.ocls[ob];
  if (cls == 1) {
    nd_h = nd_h / P.sigma_obs;
    nd_v = fabs(log(a.odat[ob]) - logr) / P.sigma_obsv;
  } else if (cls == 2) {
    nd_h = nd_h / P.sigma_obs_rain;
    nd_v = fabs(log(P.base_obsv_rain) - logr) / P.sigma_obsv_rain;
  } else if (cls >= 3 && cls <= 5) {
    if (cls == 3 && a.odat[ob] <= P.radar_ref_thres_dbz + 1.0e-6)
      nd_h = nd_h / P.sigma_obs_radar_noref;
    else
      nd_h = nd_h / P.sigma_obs_radar;
    nd_v = fabs(a.olev[ob] - rz) / P.sigma_obsz_radar;
  } else if (cls == 6) {
    nd_h = nd_h / P.sigma_obs_tc;
    nd_v = fabs(log(a.olev[ob]) - logr) / P.sigma_obsv_tc;
  } else {
    nd_h = nd_h / P.sigma_obs;
    nd_v = fabs(log(a.olev[ob]) - logr) / P.sigma_obsv;
  }
  return sumsq_rn(nd_h, nd_v);
}

struct SearchSmem {
  int* pidx;    // [CH + CPT*NT]
  float* pw;    // weight rloc / err^2
  float* pd;    // departure
  float* pr;    // rloc
  int* rowib;   // [SW_MAXROWS]
  int* rowpre;  // [SW_MAXROWS + 1]
  int* wcnt;    // [CPT*NT/32 + 1]
};

// One pass over the candidates of a grid point.  Each batch tests CPT*NT
// candidates (CPT per thread, candidate base + g*NT + tid in group g), so the
// batches and their barriers are CPT times fewer; accepted observations are
// compacted group by group, which keeps the reference's candidate order.
template <int NT, int CH, int CPT = 1, typename Flush>
__device__ int sweep_search(const SweepArgs& a, double ri, double rj, double logr, double rz, const SearchSmem& s,
                            int probe, Flush&& flush) {
  constexpr int NW = NT / 32;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int ld = a.nlon + 1;
  const float dzf2 = 13.33333333f;  // scale/letkf/letkf_obs.f90:30 (default-real literal)
  const double dzf2d = (double)13.33333333f;
  const float band_lo = dzf2 * (1.f - SW_BAND), band_hi = dzf2 * (1.f + SW_BAND);
  const float dx2 = (float)(a.P.dx * a.P.dx), dy2 = (float)(a.P.dy * a.P.dy);
  const float rif = (float)ri, rjf = (float)rj, logrf = (float)logr, rzf = (float)rz;
  int imin = (int)floor(ri - a.P.dlon_zero), imax = (int)ceil(ri + a.P.dlon_zero);
  int jmin = (int)floor(rj - a.P.dlat_zero), jmax = (int)ceil(rj + a.P.dlat_zero);
  imin = max(imin, 1);
  imax = min(imax, a.nlon);
  jmin = max(jmin, 1);
  jmax = min(jmax, a.nlat);
  int pend = 0, L = 0;
  const bool any = a.nobs > 0 && a.G[(size_t)(a.nlat - 1) * ld + a.nlon] > 0 && imin <= imax && jmin <= jmax;
  for (int jb = jmin; any && jb <= jmax; jb += SW_MAXROWS) {
    const int nrow = min(SW_MAXROWS, jmax - jb + 1);
    __syncthreads();
    for (int r = tid; r < nrow; r += NT) {
      const int j = jb + r;
      const int ib = a.G[(size_t)(j - 1) * ld + imin - 1], ie = a.G[(size_t)(j - 1) * ld + imax];
      s.rowib[r] = ib;
      s.rowpre[r + 1] = ie - ib;
    }
    __syncthreads();
    if (tid == 0) {
      s.rowpre[0] = 0;
      for (int r = 1; r <= nrow; r++) s.rowpre[r] += s.rowpre[r - 1];
    }
    __syncthreads();
    const int ncand = s.rowpre[nrow];
    for (int base = 0; base < ncand; base += CPT * NT) {
      int obg[CPT], before[CPT];
      bool okg[CPT];
      float wg[CPT], dg[CPT], rg[CPT];
#pragma unroll
      for (int g = 0; g < CPT; g++) {
        const int c = base + g * NT + tid;
        int ob = -1;
        bool ok_acc = false;
        float w = 0.f, dv = 0.f, rl = 0.f;
        if (c < ncand) {
          int lo = 0, hi = nrow - 1;  // rowpre[lo] <= c < rowpre[lo+1]
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (s.rowpre[mid] <= c) lo = mid;
            else hi = mid - 1;
          }
          ob = s.rowib[lo] + (c - s.rowpre[lo]);
          const int meta = a.obsMeta[ob];
          if (!(meta & 2)) {
            const float4 f = a.obsF[ob];
            const float di = rif - f.x, dj = rjf - f.y;
            const float h2 = (di * di * dx2 + dj * dj * dy2) * f.w;
            const float4 q = a.obsA[ob];
            const float vv = ((meta & 1) ? rzf : logrf) - f.z;
            float nd = h2 + vv * vv * q.x;
            bool ok = nd <= band_lo;
            if (!ok && nd <= band_hi) {
              const double ndd = scale_ndist_exact(a, ob, ri, rj, logr, rz);
              ok = !(ndd > dzf2d);
              nd = (float)ndd;
            }
            if (ok) {
              ok_acc = true;
              rl = __expf(-0.5f * nd) * q.w;
              w = rl * q.y;
              dv = q.z;
            }
          }
        }
        const unsigned bal = __ballot_sync(0xffffffffu, ok_acc);
        before[g] = __popc(bal & ((1u << lane) - 1u));
        if (lane == 0) s.wcnt[g * NW + wid] = __popc(bal);
        obg[g] = ob;
        okg[g] = ok_acc;
        wg[g] = w;
        dg[g] = dv;
        rg[g] = rl;
      }
      __syncthreads();
      if (tid == 0) {
        int t = 0;
        for (int k = 0; k < CPT * NW; k++) {
          const int v = s.wcnt[k];
          s.wcnt[k] = t;
          t += v;
        }
        s.wcnt[CPT * NW] = t;
      }
      __syncthreads();
#pragma unroll
      for (int g = 0; g < CPT; g++)
        if (okg[g]) {
          const int rel = s.wcnt[g * NW + wid] + before[g];
          const int slot = pend + rel;
          s.pidx[slot] = obg[g];
          s.pw[slot] = wg[g];
          s.pd[slot] = dg[g];
          s.pr[slot] = rg[g];
          if (probe >= 0 && L + rel < a.probe_cap) {
            const size_t at = (size_t)probe * a.probe_cap + (L + rel);
            a.probe_idx[at] = obg[g];
            a.probe_rloc[at] = rg[g];
          }
        }
      pend += s.wcnt[CPT * NW];
      L += s.wcnt[CPT * NW];
      __syncthreads();
      while (pend >= CH) {
        flush(CH);
        __syncthreads();
        // move the tail (fewer than CPT*NT entries) to the front
        const int rest = pend - CH;
        int i0[CPT];
        float w0[CPT], d0[CPT], r0[CPT];
#pragma unroll
        for (int g = 0; g < CPT; g++) {
          const int t = g * NT + tid;
          if (t < rest) {
            i0[g] = s.pidx[CH + t];
            w0[g] = s.pw[CH + t];
            d0[g] = s.pd[CH + t];
            r0[g] = s.pr[CH + t];
          }
        }
        __syncthreads();
#pragma unroll
        for (int g = 0; g < CPT; g++) {
          const int t = g * NT + tid;
          if (t < rest) {
            s.pidx[t] = i0[g];
            s.pw[t] = w0[g];
            s.pd[t] = d0[g];
            s.pr[t] = r0[g];
          }
        }
        pend = rest;
        __syncthreads();
      }
    }
  }
  if (pend > 0) {
    flush(pend);
    __syncthreads();
  }
  if (probe >= 0 && threadIdx.x == 0) a.probe_count[probe] = L;
  return L;
}

// List mode: the point's local observations come from a list made by another
// search (for instance the MAX_NOBS_PER_GRID selection) instead of the scan
// above; they are fed to `flush` in stages of CH, in list order, with the same
// pending-list entries (index, weight rloc / err^2, departure, rloc).
template <int NT, int CH, typename Flush>
__device__ int sweep_list(const SweepArgs& a, int q, const SearchSmem& s, Flush&& flush) {
  const int tid = threadIdx.x;
  const int64_t o0 = a.list_offs[q], o1 = a.list_offs[q + 1];
  for (int64_t b = o0; b < o1; b += CH) {
    const int nr = (int)min((int64_t)CH, o1 - b);
    __syncthreads();
    for (int t = tid; t < nr; t += NT) {
      const int ob = a.list_idx[b + t];
      const float rl = (float)a.list_rloc[b + t];
      const float4 q4 = a.obsA[ob];
      s.pidx[t] = ob;
      s.pr[t] = rl;
      s.pw[t] = rl * q4.y;
      s.pd[t] = q4.z;
    }
    __syncthreads();
    flush(nr);
    __syncthreads();
  }
  return (int)(o1 - o0);
}

}  // namespace letkf
