// sweep_mixed.cu -- fused mixed-precision analysis sweep (Cartesian search).
//
// One persistent launch analyses every grid point of a sweep.  A CTA takes
// the next point from an atomic work counter (points pre-ordered in column
// tiles so that concurrently resident points share their observations in L2)
// and runs, without leaving the SM:
//   1. the SCALE local search (scale/letkf/letkf_tools.f90:853-1178): the
//      candidate cells of obs_choose (scale/letkf/letkf_obs.f90:1054-1119)
//      flattened over the CTA, tested with an FP32 filter whose ambiguous band
//      (|ndist - cutoff| < 1e-3 cutoff) is re-tested with the reference's FP64
//      formula, so the accepted set is the reference's; accepted obs are
//      compacted in the reference order into a pending list;
//   2. streaming Gram accumulation Yb^T diag(w) Yb with w = rloc / err^2
//      (both the SPEEDY (rdiag, rloc) and the SCALE (rdiag = err^2/rloc,
//      rdiag_wloc) conventions give this weight), the departure product and
//      the inflation sums, from rows gathered out of the obs ensemble;
//   3. inflation on the diagonal, parallel Jacobi eigensolver, W and wbar
//      (common/common_letkf.f90:125-214);
//   4. the ensemble update of every variable (scale/letkf/letkf_tools.f90:
//      237-251 with beta = 1): mean and mean increment in FP64, perturbation
//      part in FP32; and the adaptive inflation update (:218-239).
#include <math.h>

#include "mixed_core.cuh"
#include "sweep_args.cuh"

namespace letkf {

constexpr int SW_MAXROWS = 128;
constexpr float SW_BAND = 1.0e-3f;

// exact FP64 SCALE test (letkf_tools.f90:961-1022); returns ndist
__device__ double scale_ndist_exact(const SweepArgs& a, int ob, double ri, double rj, double logr, double rz) {
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

template <int NP>
struct SweepSmem {
  using S = MixedSmem<NP>;
  static constexpr int NT = MixedCfg<NP>::NT;
  static constexpr int CH = S::CH;
  static constexpr int PCAP = CH + NT;        // pending list capacity
  // search-phase tables, aliased with the Newton-Schulz product T (NSSmem::T)
  static constexpr int U = S::TOTAL;
  static constexpr int PIDX = U;              // int [PCAP]
  static constexpr int PW = PIDX + PCAP;      // float [PCAP]
  static constexpr int PD = PW + PCAP;
  static constexpr int PR = PD + PCAP;
  static constexpr int ROWIB = PR + PCAP;     // int [SW_MAXROWS]
  static constexpr int ROWPRE = ROWIB + SW_MAXROWS;  // int [SW_MAXROWS+1]
  static constexpr int WCNT = ROWPRE + SW_MAXROWS + 1;  // int [NT/32 + 1]
  static constexpr int TAIL = WCNT + NT / 32 + 2 - U;
  static constexpr int USIZE = TAIL > NP * NP ? TAIL : NP * NP;
  static constexpr int MEAN = (U + USIZE + 1) & ~1;  // double [16]
  static constexpr int CTRL = MEAN + 32;      // int [8]
  static constexpr int TOTAL = CTRL + 8;
  static constexpr size_t BYTES = sizeof(float) * (size_t)TOTAL;
};

template <int NP>
__global__ void __launch_bounds__(MixedCfg<NP>::NT, MixedCfg<NP>::MINB) sweep_mixed_kernel(SweepArgs a) {
  using C = MixedCfg<NP>;
  using S = MixedSmem<NP>;
  using W = SweepSmem<NP>;
  constexpr int NT = C::NT, CH = S::CH;
  extern __shared__ __align__(16) float sm[];
  int* pidx = reinterpret_cast<int*>(sm + W::PIDX);
  float* pw = sm + W::PW;
  float* pd = sm + W::PD;
  float* pr = sm + W::PR;
  int* rowib = reinterpret_cast<int*>(sm + W::ROWIB);
  int* rowpre = reinterpret_cast<int*>(sm + W::ROWPRE);
  int* wcnt = reinterpret_cast<int*>(sm + W::WCNT);
  double* meanv = reinterpret_cast<double*>(sm + W::MEAN);
  int* ctrl = reinterpret_cast<int*>(sm + W::CTRL);
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int n = a.n, nv = a.nv, ld = a.nlon + 1;
  const float dzf2 = 13.33333333f;
  const double dzf2d = (double)13.33333333f;
  const float band_lo = dzf2 * (1.f - SW_BAND), band_hi = dzf2 * (1.f + SW_BAND);
  const float dx2 = (float)(a.P.dx * a.P.dx), dy2 = (float)(a.P.dy * a.P.dy);

  const int npts_work = a.npts_dev ? *a.npts_dev : a.nwork;
  for (;;) {
    __syncthreads();
    if (tid == 0) ctrl[0] = atomicAdd(a.counter, 1);
    __syncthreads();
    const int q = ctrl[0];
    if (q >= npts_work) break;
    const int qq = a.qmap ? a.qmap[q] : q;  // position in `order` (and in the list of list mode)
    const int pt = a.order[qq];
    const double ri = a.pri[pt], rj = a.prj[pt], rz = a.prz ? a.prz[pt] : 0.0;
    const double logr = a.plogr[pt];
    const float rif = (float)ri, rjf = (float)rj, logrf = (float)logr, rzf = (float)rz;
    int imin = (int)floor(ri - a.P.dlon_zero), imax = (int)ceil(ri + a.P.dlon_zero);
    int jmin = (int)floor(rj - a.P.dlat_zero), jmax = (int)ceil(rj + a.P.dlat_zero);
    imin = max(imin, 1);
    imax = min(imax, a.nlon);
    jmin = max(jmin, 1);
    jmax = min(jmax, a.nlat);
    GramAcc<NP> acc;
    acc.zero();
    int pend = 0, L = 0;
    const int probe = a.probe_slot ? a.probe_slot[pt] : -1;
    // list mode: the point's local observations come from a list (for instance
    // the MAX_NOBS_PER_GRID selection), staged CH at a time in list order
    if (a.list_offs) {
      const int64_t o0 = a.list_offs[qq], o1 = a.list_offs[qq + 1];
      for (int64_t b = o0; b < o1; b += CH) {
        const int nr = (int)min((int64_t)CH, o1 - b);
        __syncthreads();
        for (int t = tid; t < nr; t += NT) {
          const int ob = a.list_idx[b + t];
          const float rl = (float)a.list_rloc[b + t];
          const float4 g4 = a.obsA[ob];
          pidx[t] = ob;
          pr[t] = rl;
          pw[t] = rl * g4.y;
          pd[t] = g4.z;
        }
        __syncthreads();
        for (int t = tid; t < CH * NP; t += NT) {
          const int r = t / NP, m = t - r * NP;
          const float y = (r < nr && m < n) ? a.ens_obs[(size_t)pidx[r] * n + m] : 0.f;
          sm[S::Y + t] = y;
          sm[S::YW + t] = r < nr ? y * pw[r] : 0.f;
        }
        if (tid < nr) {
          sm[S::WR + tid] = pw[tid];
          sm[S::DR + tid] = pd[tid];
          sm[S::RL + tid] = pr[tid];
        }
        __syncthreads();
        gram_chunk<NP>(sm, nr, acc);
      }
      L = (int)(o1 - o0);
    }
    const bool any = !a.list_offs && a.nobs > 0 && a.G[(size_t)(a.nlat - 1) * ld + a.nlon] > 0 && imin <= imax &&
                     jmin <= jmax;
    for (int jb = jmin; any && jb <= jmax; jb += SW_MAXROWS) {
      const int nrow = min(SW_MAXROWS, jmax - jb + 1);
      // row table: candidate ranges of obs_choose in row order
      for (int r = tid; r < nrow; r += NT) {
        const int j = jb + r;
        const int ib = a.G[(size_t)(j - 1) * ld + imin - 1], ie = a.G[(size_t)(j - 1) * ld + imax];
        rowib[r] = ib;
        rowpre[r + 1] = ie - ib;
      }
      __syncthreads();
      if (tid == 0) {
        rowpre[0] = 0;
        for (int r = 1; r <= nrow; r++) rowpre[r] += rowpre[r - 1];
      }
      __syncthreads();
      const int ncand = rowpre[nrow];
      for (int base = 0; base < ncand; base += NT) {
        const int c = base + tid;
        int ob = -1;
        bool acc_ok = false;
        float w = 0.f, dv = 0.f, rl = 0.f;
        if (c < ncand) {
          int lo = 0, hi = nrow - 1;  // rowpre[lo] <= c < rowpre[lo+1]
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (rowpre[mid] <= c) lo = mid;
            else hi = mid - 1;
          }
          ob = rowib[lo] + (c - rowpre[lo]);
          const int meta = a.obsMeta[ob];
          if (!(meta & 2)) {
            const float4 f = a.obsF[ob];
            const float di = rif - f.x, dj = rjf - f.y;
            const float h2 = (di * di * dx2 + dj * dj * dy2) * f.w;
            const float4 g = a.obsA[ob];
            const float vv = ((meta & 1) ? rzf : logrf) - f.z;
            float nd = h2 + vv * vv * g.x;
            bool ok = nd <= band_lo;
            if (!ok && nd <= band_hi) {
              const double ndd = scale_ndist_exact(a, ob, ri, rj, logr, rz);
              ok = !(ndd > dzf2d);
              nd = (float)ndd;
            }
            if (ok) {
              acc_ok = true;
              rl = __expf(-0.5f * nd) * g.w;
              w = rl * g.y;
              dv = g.z;
            }
          }
        }
        // order-preserving block compaction
        const unsigned bal = __ballot_sync(0xffffffffu, acc_ok);
        const int before = __popc(bal & ((1u << lane) - 1u));
        if (lane == 0) wcnt[wid] = __popc(bal);
        __syncthreads();
        if (tid == 0) {
          int s = 0;
          for (int k = 0; k < NT / 32; k++) {
            const int t = wcnt[k];
            wcnt[k] = s;
            s += t;
          }
          wcnt[NT / 32] = s;
        }
        __syncthreads();
        if (acc_ok) {
          const int rel = wcnt[wid] + before;
          const int slot = pend + rel;
          pidx[slot] = ob;
          pw[slot] = w;
          pd[slot] = dv;
          pr[slot] = rl;
          if (probe >= 0 && L + rel < a.probe_cap) {
            const size_t at = (size_t)probe * a.probe_cap + (L + rel);
            a.probe_idx[at] = ob;
            a.probe_rloc[at] = rl;
          }
        }
        pend += wcnt[NT / 32];
        L += wcnt[NT / 32];
        __syncthreads();
        while (pend >= CH) {
          // flush CH rows: gather, weight, accumulate
          for (int t = tid; t < CH * NP; t += NT) {
            const int r = t / NP, m = t - r * NP;
            const float y = m < n ? a.ens_obs[(size_t)pidx[r] * n + m] : 0.f;
            sm[S::Y + t] = y;
            sm[S::YW + t] = y * pw[r];
          }
          if (tid < CH) {
            sm[S::WR + tid] = pw[tid];
            sm[S::DR + tid] = pd[tid];
            sm[S::RL + tid] = pr[tid];
          }
          __syncthreads();
          gram_chunk<NP>(sm, CH, acc);
          __syncthreads();
          const int rest = pend - CH;
          int i0 = 0, i1 = 0;
          float w0 = 0, w1 = 0, d0 = 0, d1 = 0, r0 = 0, r1 = 0;
          // move the tail (at most NT entries) to the front
          if (tid < rest) {
            i0 = pidx[CH + tid];
            w0 = pw[CH + tid];
            d0 = pd[CH + tid];
            r0 = pr[CH + tid];
          }
          if (tid + NT < rest) {
            i1 = pidx[CH + NT + tid];
            w1 = pw[CH + NT + tid];
            d1 = pd[CH + NT + tid];
            r1 = pr[CH + NT + tid];
          }
          __syncthreads();
          if (tid < rest) {
            pidx[tid] = i0;
            pw[tid] = w0;
            pd[tid] = d0;
            pr[tid] = r0;
          }
          if (tid + NT < rest) {
            pidx[NT + tid] = i1;
            pw[NT + tid] = w1;
            pd[NT + tid] = d1;
            pr[NT + tid] = r1;
          }
          pend = rest;
          __syncthreads();
        }
      }
    }
    if (pend > 0) {
      for (int t = tid; t < CH * NP; t += NT) {
        const int r = t / NP, m = t - r * NP;
        const float y = (r < pend && m < n) ? a.ens_obs[(size_t)pidx[r] * n + m] : 0.f;
        sm[S::Y + t] = y;
        sm[S::YW + t] = r < pend ? y * pw[r] : 0.f;
      }
      if (tid < pend) {
        sm[S::WR + tid] = pw[tid];
        sm[S::DR + tid] = pd[tid];
        sm[S::RL + tid] = pr[tid];
      }
      __syncthreads();
      gram_chunk<NP>(sm, pend, acc);
    }
    if (probe >= 0 && tid == 0) a.probe_count[probe] = L;
    // ---- core ----
    double infl = a.infl[pt];
    int sweeps = 0;
    const double trace = gram_finish<NP>(sm, acc);  // syncs
    if (L > 0) {
      if (a.minfl > 0.0 && infl < a.minfl) infl = a.minfl;
      const float cdiag = (float)((double)(n - 1) / infl);
      for (int i = tid; i < NP; i += NT) sm[S::A + i * NP + i] += cdiag;
      __syncthreads();
      int st = LETKF_OK;
      if (a.use_ns && cdiag > 0.f && trace < 1.0e6 * (double)cdiag) {
        // Newton-Schulz: spectrum within [c, c + tr(G)], far from the
        // mtx_eigen truncation threshold lambda_max * sqrt(eps)
        int its = 0;
        bool ok = false;
        const float s = ns_invsqrt<NP>(sm, cdiag, a.max_ns_iter, &its, a.ns_cond_max, &ok);
        if (!ok) {
          // spectrum bound beyond the iteration's range, or no convergence:
          // the point goes to the Jacobi pass (ok is uniform over the CTA)
          if (tid == 0) {
            a.defer_list[atomicAdd(a.defer_count, 1)] = a.list_offs ? qq : pt;
            if (a.defer_total) atomicAdd(a.defer_total, 1);
            if (a.nobsl_out) a.nobsl_out[pt] = L;
          }
          continue;
        }
        sweeps = its;
        const float* Z = sm + S::V;
        if (tid < NP) {
          float acc_g = 0.f;
          for (int j = 0; j < NP; j++) acc_g = fmaf(Z[j * NP + tid], sm[S::B + j], acc_g);
          sm[S::G + tid] = acc_g;
        }
        __syncthreads();
        if (tid < NP) {
          float acc_w = 0.f;
          for (int j = 0; j < NP; j++) acc_w = fmaf(Z[j * NP + tid], sm[S::G + j], acc_w);
          sm[S::WB + tid] = acc_w / s;
        }
        const float coef = sqrtf((float)(n - 1) / s);
        for (int idx = tid; idx < NP * NP; idx += NT) sm[S::A + idx] = coef * Z[idx];
        if (tid == 0) a.status[pt] = LETKF_OK;
      } else {
        sweeps = jacobi_eig<NP>(sm, a.max_sweeps);
        st = eig_postprocess<NP>(sm, n);
        if (st != LETKF_OK) {
          // reference STOP 2: flag the point and leave the background unchanged
          for (int i = tid; i < NP; i += NT) {
            sm[S::FQ + i] = 0.f;
            sm[S::WB + i] = 0.f;
          }
          if (tid == 0) a.status[pt] = st;
        } else if (tid == 0) {
          a.status[pt] = LETKF_OK;
        }
        __syncthreads();
        // W into registers, then into sm[A] (row k = background member, column m)
        float wt[C::TR][C::TC];
        constexpr int NTI = NP / C::TR;
        const int wi0 = (tid % NTI) * C::TR, wj0 = (tid / NTI) * C::TC;
        form_w<NP>(sm, [&](int i, int j, float v) { wt[i - wi0][j - wj0] = v; });
        __syncthreads();
#pragma unroll
        for (int r = 0; r < C::TR; r++)
#pragma unroll
          for (int c = 0; c < C::TC; c++) sm[S::A + (wi0 + r) * NP + wj0 + c] = wt[r][c];
      }
      if (st == LETKF_OK && tid == 0) a.infl[pt] = infl_update(n, infl, acc.p1, trace, acc.p3);
      // st is uniform over the CTA; the W tiles above are written by other threads
      __syncthreads();
      if (st != LETKF_OK)
        for (int idx = tid; idx < NP * NP; idx += NT) sm[S::A + idx] = (idx / NP == idx % NP) ? 1.f : 0.f;
    } else {
      const float sq = (float)sqrt(infl);
      for (int idx = tid; idx < NP * NP; idx += NT) sm[S::A + idx] = (idx / NP == idx % NP) ? sq : 0.f;
      for (int i = tid; i < NP; i += NT) sm[S::WB + i] = 0.f;
      if (tid == 0) a.status[pt] = LETKF_OK;
    }
    if (tid == 0) {
      if (a.nobsl_out) a.nobsl_out[pt] = L;
      if (a.sweeps_out) a.sweeps_out[pt] = sweeps;
    }
    __syncthreads();
    // ---- update: xa = mean + xp (W + wbar 1^T) ----
    float* xs = sm + S::V;  // nv * NP staged members (V is free now)
    for (int t = tid; t < nv * n; t += NT) {
      const int v = t / n, m = t - v * n;
      xs[v * NP + m] = a.xb[((size_t)v * a.npts + pt) * n + m];
    }
    __syncthreads();
    // mean: FP64 member sum, then an unevaluated FP32 pair mh + ml (xs - mh is
    // exact for members within a factor of two of the mean); the increment
    // accumulated in FP64; the analysis mean kept as a pair for the stores
    float* meanf = reinterpret_cast<float*>(meanv + 8);  // [v] = {hi, lo}
    for (int v = wid; v < nv; v += NT / 32) {
      double sx = 0.0;
      for (int m = lane; m < n; m += 32) sx += (double)xs[v * NP + m];
      const double mean = warp_sum(sx) / (double)n;
      const float mh = (float)mean, ml = (float)(mean - (double)mh);
      double dlt = 0.0;
      for (int m = lane; m < n; m += 32) {
        const float xp = (xs[v * NP + m] - mh) - ml;
        xs[v * NP + m] = xp;
        dlt = fma((double)xp, (double)sm[S::WB + m], dlt);
      }
      dlt = warp_sum(dlt);
      if (lane == 0) {
        const double am = mean + dlt;
        const float ah = (float)am;
        meanf[2 * v] = ah;
        meanf[2 * v + 1] = (float)(am - (double)ah);
      }
    }
    __syncthreads();
    for (int t = tid; t < nv * n; t += NT) {
      const int v = t / n, m = t - v * n;
      float s = 0.f;
      const float* xp = xs + v * NP;
      for (int k = 0; k < n; k++) s = fmaf(xp[k], sm[S::A + k * NP + m], s);
      a.xa[((size_t)v * a.npts + pt) * n + m] = meanf[2 * v] + (s + meanf[2 * v + 1]);
    }
  }
}

template <int NP>
static std::atomic<uint32_t>& mixed_attr() {
  static std::atomic<uint32_t> done{0};
  return done;
}

template <int NP>
static int prepare_np() {
  return cuda_status(set_smem_once(sweep_mixed_kernel<NP>, SweepSmem<NP>::BYTES, mixed_attr<NP>()));
}

int prepare_sweep_mixed(int n) {
  if (n <= 32) return prepare_np<32>();
  if (n <= 64) return prepare_np<64>();
  return prepare_np<128>();
}

template <int NP>
static int launch_sweep_np(const SweepArgs& a, cudaStream_t stream, int grid_cap) {
  auto kern = sweep_mixed_kernel<NP>;
  constexpr size_t bytes = SweepSmem<NP>::BYTES;
  cudaError_t err = set_smem_once(kern, bytes, mixed_attr<NP>());
  if (err != cudaSuccess) return cuda_status(err);
  int dev = 0, nsm = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, MixedCfg<NP>::NT, bytes);
  if (per_sm < 1) per_sm = 1;
  int grid = nsm * per_sm;
  if (grid_cap > 0 && grid > grid_cap) grid = grid_cap;
  if (grid_cap < 0) grid = grid / -grid_cap > 0 ? grid / -grid_cap : 1;  // a 1/v share of the resident CTAs
  if (grid > a.nwork) grid = a.nwork > 0 ? a.nwork : 1;
  kern<<<grid, MixedCfg<NP>::NT, bytes, stream>>>(a);
  note_launch();
  return cuda_status(cudaGetLastError());
}

int launch_sweep_mixed(const SweepArgs& a, cudaStream_t stream, int grid_cap) {
  if (a.n < 2 || a.nv < 1 || a.nv > 8) return LETKF_ERR_ARG;
  if (a.n > LETKF_MAX_NE) return LETKF_ERR_CAPACITY;
  if (a.nwork == 0) return LETKF_OK;
  if (a.n <= 32) return launch_sweep_np<32>(a, stream, grid_cap);
  if (a.n <= 64) return launch_sweep_np<64>(a, stream, grid_cap);
  return launch_sweep_np<128>(a, stream, grid_cap);
}

// ---- observation preparation for the sweep ----
__global__ void sweep_prep_obs_kernel(int nobs, const double* __restrict__ ri, const double* __restrict__ rj,
                                      const double* __restrict__ lev, const double* __restrict__ dat,
                                      const double* __restrict__ err, const double* __restrict__ dep,
                                      const int* __restrict__ cls, const int* __restrict__ varloc,
                                      const double* __restrict__ var_local, SweepScaleParams P, float4* obsF,
                                      float4* obsA, int* meta) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nobs) return;
  const int c = cls[i];
  double sh, sv, vc;
  int kind = 0;
  if (c == 1) {
    sh = P.sigma_obs;
    sv = P.sigma_obsv;
    vc = log(dat[i]);
  } else if (c == 2) {
    sh = P.sigma_obs_rain;
    sv = P.sigma_obsv_rain;
    vc = log(P.base_obsv_rain);
  } else if (c >= 3 && c <= 5) {
    sh = (c == 3 && dat[i] <= P.radar_ref_thres_dbz + 1.0e-6) ? P.sigma_obs_radar_noref : P.sigma_obs_radar;
    sv = P.sigma_obsz_radar;
    vc = lev[i];
    kind = 1;
  } else if (c == 6) {
    sh = P.sigma_obs_tc;
    sv = P.sigma_obsv_tc;
    vc = log(lev[i]);
  } else {
    sh = P.sigma_obs;
    sv = P.sigma_obsv;
    vc = log(lev[i]);
  }
  double vlw = 1.0;
  int rej = 0;
  if (var_local) {
    vlw = var_local[varloc[i]];
    rej = vlw < 2.2250738585072014e-308;
  }
  obsF[i] = make_float4((float)ri[i], (float)rj[i], (float)vc, (float)(1.0 / (sh * sh)));
  obsA[i] = make_float4((float)(1.0 / (sv * sv)), (float)(1.0 / (err[i] * err[i])), (float)dep[i], (float)vlw);
  meta[i] = kind | (rej << 1);
}

int launch_sweep_prep_obs(int nobs, const double* ri, const double* rj, const double* lev, const double* dat,
                          const double* err, const double* dep, const int* cls, const int* varloc,
                          const double* var_local, const double* params, float4* obsF, float4* obsA, int* meta,
                          cudaStream_t stream) {
  if (nobs <= 0) return LETKF_OK;
  SweepScaleParams P;
  double* f = &P.dx;
  for (int i = 0; i < 15; i++) f[i] = params[i];
  sweep_prep_obs_kernel<<<(nobs + 255) / 256, 256, 0, stream>>>(nobs, ri, rj, lev, dat, err, dep, cls, varloc,
                                                                 var_local, P, obsF, obsA, meta);
  note_launch();
  return cuda_status(cudaGetLastError());
}

}  // namespace letkf
