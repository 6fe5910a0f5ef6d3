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
  int* wcnt;    // [2 * (CPT*NT/32 + 1)]: accepted, then column-cache survivors
};

// The FP32 filter's terms, written with explicit roundings so that the direct
// scan and the column cache below give the same bits: the horizontal term
// h2 = (di^2 dx^2 + dj^2 dy^2) / sigma_h^2 and nd = h2 + vv^2 / sigma_v^2.
__device__ __forceinline__ float sw_h2(float rif, float rjf, float dx2, float dy2, const float4& f) {
  const float di = rif - f.x, dj = rjf - f.y;
  return __fmul_rn(__fmaf_rn(__fmul_rn(di, di), dx2, __fmul_rn(__fmul_rn(dj, dj), dy2)), f.w);
}
__device__ __forceinline__ float sw_nd(float h2, float vv, float qx) { return __fmaf_rn(__fmul_rn(vv, vv), qx, h2); }

// One candidate's outcome: accepted (ok) with its pending-list entry, and for
// the column cache whether it survives the horizontal test (sv) with its
// 32-byte entry (e0, e1)
struct SwCand {
  int ob;
  bool ok, sv;
  float w, d, r;
  int4 e0, e1;
};

// Column cache.  The horizontal part of the test depends on (ri, rj) only, so
// the points of one column (the levels of a grid column, consecutive in the
// processing order) share it.  The first point of a column scans the
// candidate ranges as usual and also keeps, in candidate order, every
// candidate whose horizontal term alone does not exceed the band's upper edge
// as two int4: (ob | vertical-coordinate bit << 31, h2, vertical coordinate,
// 1/sigma_v^2) and (rloc factor, 1/err^2, departure, 0), so that a cached
// level reads nothing else; any other candidate has nd >= h2 > band_hi at every level
// (nd = h2 + a non-negative term, rounded monotonically) and is rejected.  The
// next points of the column read only that list and apply the vertical test,
// with the same FP32 terms and the same FP64 re-test of the band, so the
// accepted lists, their order and the FP32 weights are the direct scan's.
struct SwCache {
  int4* ent;  // [2 * cap] or NULL (no cache)
  int cap;    // entries
};

// Compaction of one batch of CPT*NT evaluated candidates: accepted ones go to
// the pending list (and the probe) in candidate order, survivors to the
// column cache; flush(CH) consumes the pending list in stages of CH.
template <int NT, int CH, int CPT, typename Flush>
__device__ __forceinline__ void sw_compact(const SweepArgs& a, const SearchSmem& s, int probe, const SwCand (&cg)[CPT],
                                           int& pend, int& L, const SwCache& cache, int& nsurv, Flush& flush) {
  const bool BUILD = cache.ent != nullptr;  // uniform
  constexpr int NW = NT / 32;
  constexpr int SV = CPT * NW + 1;  // survivors' counts follow the accepted ones
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const unsigned below = (1u << lane) - 1u;
  int before[CPT], sbefore[CPT];
#pragma unroll
  for (int g = 0; g < CPT; g++) {
    const unsigned bal = __ballot_sync(0xffffffffu, cg[g].ok);
    before[g] = __popc(bal & below);
    if (lane == 0) s.wcnt[g * NW + wid] = __popc(bal);
    if (BUILD) {
      const unsigned sb = __ballot_sync(0xffffffffu, cg[g].sv);
      sbefore[g] = __popc(sb & below);
      if (lane == 0) s.wcnt[SV + g * NW + wid] = __popc(sb);
    }
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
    if (BUILD) {
      t = 0;
      for (int k = 0; k < CPT * NW; k++) {
        const int v = s.wcnt[SV + k];
        s.wcnt[SV + k] = t;
        t += v;
      }
      s.wcnt[SV + CPT * NW] = t;
    }
  }
  __syncthreads();
#pragma unroll
  for (int g = 0; g < CPT; g++) {
    if (cg[g].ok) {
      const int rel = s.wcnt[g * NW + wid] + before[g];
      const int slot = pend + rel;
      s.pidx[slot] = cg[g].ob;
      s.pw[slot] = cg[g].w;
      s.pd[slot] = cg[g].d;
      s.pr[slot] = cg[g].r;
      if (probe >= 0 && L + rel < a.probe_cap) {
        const size_t at = (size_t)probe * a.probe_cap + (L + rel);
        a.probe_idx[at] = cg[g].ob;
        a.probe_rloc[at] = cg[g].r;
      }
    }
    if (BUILD && cg[g].sv) {
      const int at = nsurv + s.wcnt[SV + g * NW + wid] + sbefore[g];
      if (at < cache.cap) {
        cache.ent[2 * at] = cg[g].e0;
        cache.ent[2 * at + 1] = cg[g].e1;
      }
    }
  }
  pend += s.wcnt[CPT * NW];
  L += s.wcnt[CPT * NW];
  if (BUILD) nsurv += s.wcnt[SV + CPT * NW];
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

// The FP32 filter with the FP64 re-test of the band |nd - cutoff| < 1e-3
// cutoff: whether the candidate is accepted, and in nd_out the nd its rloc is
// computed from (the FP64 value rounded to FP32 where the re-test ran)
__device__ __forceinline__ bool sw_accept(const SweepArgs& a, int ob, float nd, double ri, double rj, double logr,
                                          double rz, float& nd_out) {
  const float dzf2 = 13.33333333f;  // scale/letkf/letkf_obs.f90:30 (default-real literal)
  const float band_lo = dzf2 * (1.f - SW_BAND), band_hi = dzf2 * (1.f + SW_BAND);
  bool ok = nd <= band_lo;
  if (!ok && nd <= band_hi) {
    const double ndd = scale_ndist_exact(a, ob, ri, rj, logr, rz);
    ok = !(ndd > (double)dzf2);
    nd = (float)ndd;
  }
  nd_out = nd;
  return ok;
}

// One pass over the candidates of a grid point.  Each batch tests CPT*NT
// candidates (CPT per thread, candidate base + g*NT + tid in group g), so the
// batches and their barriers are CPT times fewer; accepted observations are
// compacted group by group, which keeps the reference's candidate order.
// With cache.ent set, the column cache of this point's (ri, rj) is written
// on the way; *nsurv receives its length (above cache.cap: not usable).
template <int NT, int CH, int CPT, typename Flush>
__device__ int sweep_search(const SweepArgs& a, double ri, double rj, double logr, double rz, const SearchSmem& s,
                            int probe, Flush&& flush, const SwCache& cache = SwCache{nullptr, 0},
                            int* nsurv_out = nullptr) {
  const bool BUILD = cache.ent != nullptr;  // uniform
  const int tid = threadIdx.x;
  const int ld = a.nlon + 1;
  const float band_hi = 13.33333333f * (1.f + SW_BAND);
  const float dx2 = (float)(a.P.dx * a.P.dx), dy2 = (float)(a.P.dy * a.P.dy);
  const float rif = (float)ri, rjf = (float)rj, logrf = (float)logr, rzf = (float)rz;
  int imin = (int)floor(ri - a.P.dlon_zero), imax = (int)ceil(ri + a.P.dlon_zero);
  int jmin = (int)floor(rj - a.P.dlat_zero), jmax = (int)ceil(rj + a.P.dlat_zero);
  imin = max(imin, 1);
  imax = min(imax, a.nlon);
  jmin = max(jmin, 1);
  jmax = min(jmax, a.nlat);
  int pend = 0, L = 0, nsurv = 0;
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
      SwCand cg[CPT];
#pragma unroll
      for (int g = 0; g < CPT; g++) {
        const int c = base + g * NT + tid;
        SwCand& o = cg[g];
        o.ob = -1;
        o.ok = o.sv = false;
        o.w = o.d = o.r = 0.f;
        if (c < ncand) {
          int lo = 0, hi = nrow - 1;  // rowpre[lo] <= c < rowpre[lo+1]
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (s.rowpre[mid] <= c) lo = mid;
            else hi = mid - 1;
          }
          const int ob = s.rowib[lo] + (c - s.rowpre[lo]);
          o.ob = ob;
          const int meta = a.obsMeta[ob];
          if (!(meta & 2)) {
            const float4 f = a.obsF[ob];
            const float h2 = sw_h2(rif, rjf, dx2, dy2, f);
            const float4 q = a.obsA[ob];
            const float vv = ((meta & 1) ? rzf : logrf) - f.z;
            float nd;
            if (sw_accept(a, ob, sw_nd(h2, vv, q.x), ri, rj, logr, rz, nd)) {
              o.ok = true;
              o.r = __expf(-0.5f * nd) * q.w;
              o.w = o.r * q.y;
              o.d = q.z;
            }
            if (BUILD) {
              o.sv = h2 <= band_hi;
              o.e0 = make_int4((int)((unsigned)ob | ((unsigned)(meta & 1) << 31)), __float_as_int(h2),
                               __float_as_int(f.z), __float_as_int(q.x));
              o.e1 = make_int4(__float_as_int(q.w), __float_as_int(q.y), __float_as_int(q.z), 0);
            }
          }
        }
      }
      sw_compact<NT, CH, CPT>(a, s, probe, cg, pend, L, cache, nsurv, flush);
    }
  }
  if (pend > 0) {
    flush(pend);
    __syncthreads();
  }
  if (probe >= 0 && threadIdx.x == 0) a.probe_count[probe] = L;
  if (nsurv_out) *nsurv_out = nsurv;
  return L;
}

// A point whose column cache holds n entries (see SwCache): the vertical
// test over the cached horizontal survivors, in their (candidate) order.  The
// next batch's entries are loaded before this batch's compaction barriers.
template <int NT, int CH, typename Flush>
__device__ int sweep_search_cached(const SweepArgs& a, const int4* __restrict__ ent, int n, double ri, double rj,
                                   double logr, double rz, const SearchSmem& s, int probe, Flush&& flush) {
  const int tid = threadIdx.x;
  const float logrf = (float)logr, rzf = (float)rz;
  int pend = 0, L = 0, nsurv = 0;
  const SwCache none{nullptr, 0};
  int4 e0 = make_int4(0, 0, 0, 0), e1 = e0;
  if (tid < n) {
    e0 = ent[2 * tid];
    e1 = ent[2 * tid + 1];
  }
  for (int base = 0; base < n; base += NT) {
    SwCand cg[1];
    SwCand& o = cg[0];
    const int c = base + tid;
    int4 f0 = make_int4(0, 0, 0, 0), f1 = f0;
    if (c + NT < n) {
      f0 = ent[2 * (c + NT)];
      f1 = ent[2 * (c + NT) + 1];
    }
    o.ob = -1;
    o.ok = o.sv = false;
    o.w = o.d = o.r = 0.f;
    if (c < n) {
      const int ob = e0.x & 0x7fffffff;
      o.ob = ob;
      const float vv = ((e0.x < 0) ? rzf : logrf) - __int_as_float(e0.z);
      float nd;
      if (sw_accept(a, ob, sw_nd(__int_as_float(e0.y), vv, __int_as_float(e0.w)), ri, rj, logr, rz, nd)) {
        o.ok = true;
        o.r = __expf(-0.5f * nd) * __int_as_float(e1.x);
        o.w = o.r * __int_as_float(e1.y);
        o.d = __int_as_float(e1.z);
      }
    }
    sw_compact<NT, CH, 1>(a, s, probe, cg, pend, L, none, nsurv, flush);
    e0 = f0;
    e1 = f1;
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
