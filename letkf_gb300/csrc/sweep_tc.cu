// sweep_tc.cu -- fused analysis sweep with the contractions on the tcgen05 tensor cores.
//
// Same work as sweep_mixed.cu (search, Gram, transform, update per grid point,
// one persistent launch), for ensembles up to 64 members, with the two
// contraction stages issued as tcgen05.mma from shared-memory descriptors
// and FP32 accumulation in tensor memory:
//
//  * Gram  G = Ywᵀ Y (common/common_letkf.f90:101-118): every stage of 24
//    accepted observations is staged K-major as A = [Yw_hi; Yw_lo] (128 x 24
//    TF32) with B = Y_hi and B = Y_lo (64 x 24); two M=128 MMAs accumulate
//    D0 = A Y_hiᵀ and D1 = A Y_loᵀ in tensor memory, and G is the sum of their
//    four 64 x 64 blocks, i.e. the product of the two-term TF32 splits (about
//    1e-6 relative).  Staging of stage c+1 overlaps the MMAs of stage c (two
//    24 KB buffers, one mbarrier each).
//  * Newton-Schulz  A^(-1/2): the iterates Y, Z commute, so one iteration is
//    T = Z Y and [Y;Z] <- 1.5 [Y;Z] - 0.5 [Y;Z] T: two M=128 MMA groups with
//    the stacked operand S = [Y;Z] (128 x 64) and B = Y or T (64 x 64), each
//    as the three split products hi.hi + hi.lo + lo.hi of BF16 splits.
//  * An uncoupled FP32 step anchored to the exact A (kept in tensor memory)
//    restores FP32 accuracy after the 16-bit phase.
//
// Points where the transform needs mtx_eigen's truncation semantics (c <= 0 or
// tr(G) >= 1e6 c) are appended to a deferred list for the Jacobi pass.
#include <cuda_bf16.h>

#include "mixed_core.cuh"
#include "sweep_search.cuh"
#include "tc_sm100.cuh"

namespace letkf {

constexpr int TC_NT = 128;
constexpr int TC_CH = 24;  // observations per Gram stage
constexpr int TC_NP = 64;
constexpr int TC_CPT = 1;  // search candidates per thread and batch (2 measured 0.7 % slower)
constexpr uint32_t TC_TMEM_COLS = 128;
constexpr uint32_t TC_WAIT = 1u << 22;
constexpr int TC_POLISH_MAX = 8;  // FP32 iterations at most

// byte offsets in dynamic shared memory
struct TcLayout {
  // operand region, 48 KB, reused by phase
  static constexpr int STG = 0;           // two Gram stages of 24 KB
  static constexpr int STG_A = 0;         //   A = [Yw_hi^T; Yw_lo^T]: 128 x 24 tf32 (12 KB)
  static constexpr int STG_BH = 12288;    //   Y_hi^T: 64 x 24 tf32 (6 KB)
  static constexpr int STG_BL = 18432;    //   Y_lo^T
  static constexpr int STG_SIZE = 24576;
  static constexpr int S_HI = 0;          // Newton-Schulz S = [Y; Z]: 128 x 64 bf16 (16 KB)
  static constexpr int S_LO = 16384;
  static constexpr int B_HI = 32768;      // B = Y or T: 64 x 64 bf16 (8 KB)
  static constexpr int B_LO = 40960;
  static constexpr int GTMP = 32768;      // Gram in FP32, 64 x 64, swizzled rows (gsw; over B)
  static constexpr int WMAT = 32768;      // transform W in FP32, 64 x 64 row-major (over B)
  static constexpr int XS = 0;            // update staging, nv x 64 FP32 (over S)
  static constexpr int YF = 0;            // FP32 polish: Y (64 x 64), Z, T row-major
  static constexpr int ZF = 16384;
  static constexpr int TF = 32768;
  static constexpr int OPER_END = 49152;
  // small data
  static constexpr int VB = OPER_END;            // float[64] departure product
  static constexpr int VBP = VB + 256;           // float[128] partial departure products
  static constexpr int VWB = VBP + 512;          // float[64] wbar
  static constexpr int VG = VWB + 256;           // float[64]
  static constexpr int VX = VG + 256;            // float[64] power iteration
  static constexpr int VY = VX + 256;            // float[64]
  static constexpr int RED = VY + 256;           // float[64]
  static constexpr int PCAP = TC_CH + TC_CPT * TC_NT;  // pending-list entries
  static constexpr int PIDX = RED + 256;         // int[PCAP]
  static constexpr int PW = PIDX + 4 * PCAP;
  static constexpr int PD = PW + 4 * PCAP;
  static constexpr int PR = PD + 4 * PCAP;
  static constexpr int ROWIB = PR + 4 * PCAP;
  static constexpr int ROWPRE = ROWIB + 4 * SW_MAXROWS;
  static constexpr int WCNT = ROWPRE + 4 * (SW_MAXROWS + 1);
  static constexpr int MEAN = ((WCNT + 4 * 2 * (TC_CPT * TC_NT / 32 + 1)) + 7) & ~7;  // double[16]
  static constexpr int MBAR = MEAN + 128;        // uint64[5]: Gram stages 0/1, products, background rows, drain
  static constexpr int TMEMH = MBAR + 40;        // uint32
  static constexpr int CTRL = TMEMH + 8;         // int[4]: position, scratch
  static constexpr int CKEY = CTRL + 16;         // double[2]: the column-cache point (ri, rj)
  static constexpr int RUN = CKEY + 16;          // int[4]: run of positions [next, end), column-cache length
  static constexpr int TOTAL = RUN + 16;
};

// sum_j M[j][c] x[j] for a 64 x 64 row-major matrix in shared memory (column
// c read as consecutive lanes); four partial sums keep the loads in flight
__device__ __forceinline__ float col_dot64(const float* M, const float* x, int c) {
  float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
#pragma unroll 4
  for (int j = 0; j < 64; j += 4) {
    a0 = fmaf(M[j * 64 + c], x[j], a0);
    a1 = fmaf(M[(j + 1) * 64 + c], x[j + 1], a1);
    a2 = fmaf(M[(j + 2) * 64 + c], x[j + 2], a2);
    a3 = fmaf(M[(j + 3) * 64 + c], x[j + 3], a3);
  }
  return (a0 + a1) + (a2 + a3);
}

// The Gram in shared memory: 64 x 64 FP32, row r's 4-float column groups XOR-ed
// by r & 7 (element (r, c) at r * 64 + (c ^ 4 (r & 7))).  Rows read or written
// one per lane as float4, columns one per lane, the diagonal and the
// symmetrising diagonal walk then all fall in distinct banks.
__device__ __forceinline__ int gsw(int r, int c) { return r * 64 + (c ^ ((r & 7) << 2)); }

// (M x)[c] for the swizzled Gram M (symmetric: column c read as row c)
__device__ __forceinline__ float col_dot64_g(const float* M, const float* x, int c) {
  float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
#pragma unroll 4
  for (int j = 0; j < 64; j += 4) {
    a0 = fmaf(M[gsw(j, c)], x[j], a0);
    a1 = fmaf(M[gsw(j + 1, c)], x[j + 1], a1);
    a2 = fmaf(M[gsw(j + 2, c)], x[j + 2], a2);
    a3 = fmaf(M[gsw(j + 3, c)], x[j + 3], a3);
  }
  return (a0 + a1) + (a2 + a3);
}

// 12 MMAs: D = S_hi B_hi + S_hi B_lo + S_lo B_hi over K = 64 (4 steps of 16)
__device__ __forceinline__ void ns_mma(uint32_t d, uint32_t s_hi, uint32_t s_lo, uint32_t b_hi, uint32_t b_lo,
                                       uint32_t idesc) {
#pragma unroll
  for (int pass = 0; pass < 3; pass++) {
    const uint32_t sa = pass == 2 ? s_lo : s_hi;
    const uint32_t sb = pass == 1 ? b_lo : b_hi;
#pragma unroll
    for (int s = 0; s < 4; s++)
      tc::mma_bf16(d, tc::smem_desc(sa + s * 256, 128, 1024), tc::smem_desc(sb + s * 256, 128, 1024), idesc,
                   (pass == 0 && s == 0) ? 0u : 1u);
  }
}

__global__ void __launch_bounds__(TC_NT, 4) sweep_tc_kernel(SweepArgs a) {
  using L = TcLayout;
  extern __shared__ __align__(1024) unsigned char sm[];
  float* vb = reinterpret_cast<float*>(sm + L::VB);
  float* vbp = reinterpret_cast<float*>(sm + L::VBP);
  float* vwb = reinterpret_cast<float*>(sm + L::VWB);
  float* vg = reinterpret_cast<float*>(sm + L::VG);
  float* vx = reinterpret_cast<float*>(sm + L::VX);
  float* vy = reinterpret_cast<float*>(sm + L::VY);
  float* red = reinterpret_cast<float*>(sm + L::RED);
  double* meanv = reinterpret_cast<double*>(sm + L::MEAN);
  uint64_t* mbar = reinterpret_cast<uint64_t*>(sm + L::MBAR);
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(sm + L::TMEMH);
  int* ctrl = reinterpret_cast<int*>(sm + L::CTRL);
  SearchSmem ss;
  ss.pidx = reinterpret_cast<int*>(sm + L::PIDX);
  ss.pw = reinterpret_cast<float*>(sm + L::PW);
  ss.pd = reinterpret_cast<float*>(sm + L::PD);
  ss.pr = reinterpret_cast<float*>(sm + L::PR);
  ss.rowib = reinterpret_cast<int*>(sm + L::ROWIB);
  ss.rowpre = reinterpret_cast<int*>(sm + L::ROWPRE);
  ss.wcnt = reinterpret_cast<int*>(sm + L::WCNT);
  float* Gt = reinterpret_cast<float*>(sm + L::GTMP);
  float* Wm = reinterpret_cast<float*>(sm + L::WMAT);
  float* xs = reinterpret_cast<float*>(sm + L::XS);

  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int n = a.n, nv = a.nv;
  const uint32_t sbase = tc::smem_u32(sm);
  const uint32_t idesc = tc::idesc_bf16(128, 64);    // Newton-Schulz products
  const uint32_t idesc_g = tc::idesc_tf32(128, 64);  // Gram

  if (tid == 0) {
    tc::mbar_init(&mbar[0], 1);
    tc::mbar_init(&mbar[1], 1);
    tc::mbar_init(&mbar[2], 1);
    tc::mbar_init(&mbar[3], 1);
    tc::mbar_init(&mbar[4], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    int* rn = reinterpret_cast<int*>(sm + L::RUN);
    rn[0] = rn[1] = 0;
    rn[2] = -2;
    double* ck = reinterpret_cast<double*>(sm + L::CKEY);
    ck[0] = ck[1] = __longlong_as_double(0x7ff8000000000000ll);  // NaN: equal to no point
  }
  if (wid == 0) tc::tmem_alloc(tmem_holder, TC_TMEM_COLS);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = *tmem_holder;
  const uint32_t D0 = tbase, D1 = tbase + 64;
  const uint32_t lane_off = (uint32_t)(wid * 32) << 16;
  const int r = tid;  // the tile row this thread owns in TMEM / S
  // mbarrier phase parities (bit i: barrier i) and the Gram stages with MMAs in
  // flight (bit b: stage buffer b), as bit masks so that a stage index known
  // only at run time does not put them in local memory
  uint32_t par = 0u;
  bool xb_outst = false;  // a TMA copy of background rows is in flight
  uint32_t outst = 0u;
  int tmo = 0;  // this thread saw a bounded wait give up
  const int npts_work = a.npts_dev ? *a.npts_dev : a.nwork;
  const double inv_n = 1.0 / (double)n;  // one FP64 division per kernel, not per variable and point

  // A wait that gives up still flips its parity, so that control flow stays
  // the same in every thread; the drain below then waits (with a long bound)
  // for what the timed-out wait left in flight before TMEM is released.
  uint32_t xb_lost = 0u;  // bit 1: a background-row copy whose wait gave up; bit 0: its phase parity
  auto wait_bar = [&](int i) {
    const uint32_t pb = (par >> i) & 1u;
    if (!tc::mbar_wait(&mbar[i], pb, TC_WAIT)) {
      tmo = 1;
      if (i == 3) xb_lost = 2u | pb;
    }
    par ^= 1u << i;
  };

  // failure injection: a wait on a barrier that nothing arrives at gives up
  // after the given polls; the CTA then processes no point
  if (a.fault_wait_polls > 0u && !tc::mbar_wait(&mbar[4], 0u, a.fault_wait_polls)) tmo = 1;
  const bool skip_all = __syncthreads_or(tmo);  // uniform over the CTA
  if (skip_all) tmo = 1;

  // The CTA takes runs of consecutive order positions [run[0], run[1]), of
  // col_unit positions until the end of the work nears.  Column cache of the search (state in shared memory, uniform over
  // the CTA): run[2] entries for the point column ckey = (ri, rj); -1: it did
  // not fit, -2: none.
  const bool col = a.col_ent != nullptr && !a.list_offs && (int)blockIdx.x < a.col_slots;
  double* ckey = reinterpret_cast<double*>(sm + L::CKEY);
  int* run = reinterpret_cast<int*>(sm + L::RUN);
  for (; !skip_all;) {
    __syncthreads();
    if (tid == 0) {
      if (run[0] >= run[1]) {
        // guided self-scheduling over the positions: runs of col_unit while
        // more than four runs per CTA remain, shorter ones towards the end
        int len = a.col_unit > 1 ? a.col_unit : 1;
        const int left = npts_work - *reinterpret_cast<volatile int*>(a.counter);
        const int share = left / (4 * (int)gridDim.x);
        if (share < len) len = share > 1 ? share : 1;
        const int s0 = atomicAdd(a.counter, len);
        run[0] = min(s0, npts_work);
        run[1] = (int)min((int64_t)s0 + len, (int64_t)npts_work);
      }
      ctrl[0] = run[0]++;
    }
    __syncthreads();
    const int q = ctrl[0];
    if (q >= npts_work) break;
    const int qq = a.qmap ? a.qmap[q] : q;  // position in `order` (and in the list of list mode)
    const int pt = a.order[qq];
    const double ri = a.pri[pt], rj = a.prj[pt], rz = a.prz ? a.prz[pt] : 0.0;
    const double logr = a.plogr[pt];

    // ---- search + Gram on the tensor cores ----
    const int m = tid & 63, hh = tid >> 6;
    float bpart = 0.f, p1 = 0.f, p3 = 0.f;
    int chunk = 0;
    bool first = true;
    auto flush = [&](int nr) {
      const int buf = chunk & 1;
      if ((outst >> buf) & 1u) {
        wait_bar(buf);
        outst &= ~(1u << buf);
      }
      tc::fence_after_sync();
      unsigned char* stg = sm + L::STG + buf * L::STG_SIZE;
      constexpr int KH = TC_CH / 2;  // observations per thread: member m, half hh
      float yv[KH], wv[KH];
#pragma unroll
      for (int kk = 0; kk < KH; kk++) {
        const int k = hh * KH + kk;
        float y = 0.f, w = 0.f, dd = 0.f;
        if (k < nr) {
          w = ss.pw[k];
          dd = ss.pd[k];
          if (m < n) y = a.ens_obs[(size_t)ss.pidx[k] * n + m];
        }
        yv[kk] = y;
        wv[kk] = y * w;
        bpart = fmaf(wv[kk], dd, bpart);
      }
#pragma unroll
      for (int g = 0; g < KH / 4; g++) {
        float4 h, l;
        const uint32_t off = tc::kmajor_off(m, hh * KH + g * 4, TC_CH);
        split4_tf32(wv + 4 * g, h, l);
        *reinterpret_cast<float4*>(stg + L::STG_A + off) = h;
        *reinterpret_cast<float4*>(stg + L::STG_A + tc::kmajor_off(64 + m, hh * KH + g * 4, TC_CH)) = l;
        split4_tf32(yv + 4 * g, h, l);
        *reinterpret_cast<float4*>(stg + L::STG_BH + off) = h;
        *reinterpret_cast<float4*>(stg + L::STG_BL + off) = l;
      }
      for (int k = tid; k < nr; k += TC_NT) {
        const float dd = ss.pd[k];
        p1 = fmaf(dd * dd, ss.pw[k], p1);
        p3 += ss.pr[k];
      }
      tc::fence_smem_async();
      tc::fence_before_sync();
      __syncthreads();
      if (tid == 0) {
        tc::fence_after_sync();
        const uint32_t sa = sbase + L::STG + buf * L::STG_SIZE;
        constexpr uint32_t SBO = TC_CH * 32;  // bytes between 8-row core-matrix groups
#pragma unroll
        for (int s = 0; s < TC_CH / 8; s++)
          tc::mma_tf32(D0, tc::smem_desc(sa + L::STG_A + s * 256, 128, SBO),
                       tc::smem_desc(sa + L::STG_BH + s * 256, 128, SBO), idesc_g, (first && s == 0) ? 0u : 1u);
#pragma unroll
        for (int s = 0; s < TC_CH / 8; s++)
          tc::mma_tf32(D1, tc::smem_desc(sa + L::STG_A + s * 256, 128, SBO),
                       tc::smem_desc(sa + L::STG_BL + s * 256, 128, SBO), idesc_g, (first && s == 0) ? 0u : 1u);
        tc::mma_commit(&mbar[buf]);
      }
      outst |= 1u << buf;
      first = false;
      chunk++;
    };
    const int probe = a.probe_slot ? a.probe_slot[pt] : -1;
    int Lp;
    const bool same_col = col && ri == ckey[0] && rj == ckey[1];
    const int cn = run[2];
    if (a.list_offs) {
      Lp = sweep_list<TC_NT, TC_CH>(a, qq, ss, flush);
    } else if (same_col && cn >= 0) {
      Lp = sweep_search_cached<TC_NT, TC_CH>(a, a.col_ent + (size_t)blockIdx.x * a.col_cap * 2, cn, ri, rj, logr,
                                             rz, ss, probe, flush);
    } else if (col && !same_col) {
      int nsv = 0;
      const SwCache cache{a.col_ent + (size_t)blockIdx.x * a.col_cap * 2, a.col_cap};
      Lp = sweep_search<TC_NT, TC_CH, TC_CPT>(a, ri, rj, logr, rz, ss, probe, flush, cache, &nsv);
      if (tid == 0) {  // read by the next point, after the barriers in between
        ckey[0] = ri;
        ckey[1] = rj;
        run[2] = nsv <= a.col_cap ? nsv : -1;
      }
    } else {  // no cache, or this column's did not fit
      Lp = sweep_search<TC_NT, TC_CH, TC_CPT>(a, ri, rj, logr, rz, ss, probe, flush);
    }
    for (int b = 0; b < 2; b++)
      if ((outst >> b) & 1u) {
        wait_bar(b);
        outst &= ~(1u << b);
      }
    tc::fence_after_sync();
    if (__syncthreads_or(tmo)) {
      tmo = 1;
      break;
    }
    // TMA: fetch this point's background rows (nv x n floats) into the
    // search's pending-list area, which is free until the next point; the
    // copy overlaps the transform and is consumed by the update
    if (a.xb_bulk) {
      tc::fence_smem_async();
      __syncthreads();
      if (tid == 0) {
        const uint32_t row = (uint32_t)n * 4u;
        tc::mbar_arrive_expect_tx(&mbar[3], row * (uint32_t)nv);
        for (int v = 0; v < nv; v++)
          tc::bulk_g2s(sbase + L::PIDX + v * row, a.xb + ((size_t)v * a.npts + pt) * n, row, &mbar[3]);
      }
      xb_outst = true;
    }

    double infl = a.infl[pt];
    bool deferred = false;
    if (Lp > 0) {
      if (a.minfl > 0.0 && infl < a.minfl) infl = a.minfl;
      // c = (k-1)/rho: one FP64 division by one thread, read after the barrier below
      if (tid == 0) reinterpret_cast<float*>(ctrl)[1] = (float)((double)(n - 1) / infl);
      // G = D0[r] + D0[r+64] + D1[r] + D1[r+64]: warps 2-3 first, then warps 0-1 add
      if (wid >= 2) {
#pragma unroll 1
        for (int c0 = 0; c0 < 64; c0 += 16) {
          float v0[16], v1[16];
          tc::tmem_ld16(D0 + lane_off + c0, v0);
          tc::tmem_ld16(D1 + lane_off + c0, v1);
#pragma unroll
          for (int j = 0; j < 16; j += 4)
            *reinterpret_cast<float4*>(Gt + gsw(r - 64, c0 + j)) =
                make_float4(v0[j] + v1[j], v0[j + 1] + v1[j + 1], v0[j + 2] + v1[j + 2], v0[j + 3] + v1[j + 3]);
        }
      }
      vbp[tid] = bpart;
      __syncthreads();
      const float cdiag = reinterpret_cast<const float*>(ctrl)[1];
      if (wid < 2) {
#pragma unroll 1
        for (int c0 = 0; c0 < 64; c0 += 16) {
          float v0[16], v1[16];
          tc::tmem_ld16(D0 + lane_off + c0, v0);
          tc::tmem_ld16(D1 + lane_off + c0, v1);
#pragma unroll
          for (int j = 0; j < 16; j += 4) {
            float4* dst = reinterpret_cast<float4*>(Gt + gsw(r, c0 + j));
            float4 g = *dst;
            g.x += v0[j] + v1[j];
            g.y += v0[j + 1] + v1[j + 1];
            g.z += v0[j + 2] + v1[j + 2];
            g.w += v0[j + 3] + v1[j + 3];
            *dst = g;
          }
        }
        vb[r] = vbp[r] + vbp[r + 64];
      }
      tc::fence_before_sync();
      __syncthreads();
      // symmetrise (pairs owned by one thread) and take the trace.  The pairs
      // are walked along diagonals, (i, i + d mod 64) for d = 1..32, so the 32
      // lanes of a warp touch 32 distinct banks for both the element and its
      // mirror (a row-by-row walk reads the mirror at a 64-float stride).
      for (int t = tid; t < 32 * 64; t += TC_NT) {
        const int d = 1 + (t >> 6), i = t & 63;
        if (d == 32 && i >= 32) continue;
        const int j = (i + d) & 63;
        const float v = 0.5f * (Gt[gsw(i, j)] + Gt[gsw(j, i)]);
        Gt[gsw(i, j)] = v;
        Gt[gsw(j, i)] = v;
      }
      __syncthreads();
      float sums[3] = {tid < 64 ? Gt[gsw(tid, tid)] : 0.f, p1, p3};
      block_sum_k<float, TC_NT, 3>(sums, red);
      const float trace = sums[0];
      p1 = sums[1];
      p3 = sums[2];
      if (!(cdiag > 0.f) || !((double)trace < 1.0e6 * (double)cdiag)) {
        deferred = true;  // needs the eigensolver with mtx_eigen's truncation
      } else {
        if (tid < 64) Gt[gsw(tid, tid)] += cdiag;
        __syncthreads();
        // keep the exact FP32 A in the Gram's second accumulator (lanes 0..63 of
        // columns 64..127); the Newton-Schulz products only use columns 0..63
        if (wid < 2) {
#pragma unroll 1
          for (int c0 = 0; c0 < 64; c0 += 16) {
            float v[16];
#pragma unroll
            for (int j = 0; j < 16; j += 4) {
              const float4 g = *reinterpret_cast<const float4*>(Gt + gsw(r, c0 + j));
              v[j] = g.x;
              v[j + 1] = g.y;
              v[j + 2] = g.z;
              v[j + 3] = g.w;
            }
            tc::tmem_st16(D1 + lane_off + c0, v);
          }
        }
        tc::fence_before_sync();
        // scaling s: power iteration guarded by the Gershgorin bound (s >= lambda_max / 2)
        float gsum = 0.f;
        if (tid < 64) {
          float g0 = 0.f, g1 = 0.f, g2 = 0.f, g3 = 0.f;
#pragma unroll 4
          for (int j = 0; j < 64; j += 4) {
            g0 += fabsf(Gt[gsw(j, tid)]);
            g1 += fabsf(Gt[gsw(j + 1, tid)]);
            g2 += fabsf(Gt[gsw(j + 2, tid)]);
            g3 += fabsf(Gt[gsw(j + 3, tid)]);
          }
          gsum = (g0 + g1) + (g2 + g3);
          vx[tid] = Gt[gsw(tid, tid)] * (1.f + 0.25f * __sinf(1.7f * tid));
        }
        gsum = warp_max(gsum);
        __syncthreads();
        if (lane == 0) red[wid] = gsum;
        __syncthreads();
        const float gmax = fmaxf(fmaxf(red[0], red[1]), fmaxf(red[2], red[3]));
        __syncthreads();
        float lam = 0.f, fro = 0.f;
        if (a.tc_scale_bound) {
          // s = min(||A||_F, Gershgorin) >= lambda_max: every eigenvalue of A/s is <= 1
          float f2 = 0.f;
          if (tid < 64) {
            float q0 = 0.f, q1 = 0.f, q2 = 0.f, q3 = 0.f;
#pragma unroll 4
            for (int j = 0; j < 64; j += 4) {
              const float x0 = Gt[gsw(j, tid)], x1 = Gt[gsw(j + 1, tid)];
              const float x2 = Gt[gsw(j + 2, tid)], x3 = Gt[gsw(j + 3, tid)];
              q0 = fmaf(x0, x0, q0);
              q1 = fmaf(x1, x1, q1);
              q2 = fmaf(x2, x2, q2);
              q3 = fmaf(x3, x3, q3);
            }
            f2 = (q0 + q1) + (q2 + q3);
          }
          fro = sqrtf(block_sum<float, TC_NT>(f2, red));
        }
        for (int it = 0; it < (a.tc_scale_bound ? 0 : 8); it++) {
          float part = 0.f, xx = 0.f;
          if (tid < 64) {
            const float acc = col_dot64_g(Gt, vx, tid);
            vy[tid] = acc;
            part = acc * acc;
            xx = vx[tid] * vx[tid];
          }
          float q2[2] = {part, xx};
          block_sum_k<float, TC_NT, 2>(q2, red);
          const float nrm2 = q2[0], x2 = q2[1];
          lam = sqrtf(nrm2 / fmaxf(x2, 1e-30f));
          const float inv = rsqrtf(fmaxf(nrm2, 1e-30f));
          if (tid < 64) vx[tid] = vy[tid] * inv;
          __syncthreads();
        }
        const float s = a.tc_scale_bound ? fminf(fro, gmax) : fmaxf(1.05f * lam, 0.5f * gmax);
        const float inv_s = 1.f / s;
        // S = [A/s ; I] split into bf16 hi / lo (row r per thread)
#pragma unroll 1
        for (int c0 = 0; c0 < 64; c0 += 8) {
          float v[8];
          if (r < 64) {
            const float4 x0 = *reinterpret_cast<const float4*>(Gt + gsw(r, c0));
            const float4 x1 = *reinterpret_cast<const float4*>(Gt + gsw(r, c0 + 4));
            v[0] = x0.x * inv_s; v[1] = x0.y * inv_s; v[2] = x0.z * inv_s; v[3] = x0.w * inv_s;
            v[4] = x1.x * inv_s; v[5] = x1.y * inv_s; v[6] = x1.z * inv_s; v[7] = x1.w * inv_s;
          } else {
#pragma unroll
            for (int j = 0; j < 8; j++) v[j] = (r - 64 == c0 + j) ? 1.f : 0.f;
          }
          uint4 h, l;
          split8(v, h, l);
          const uint32_t off = tc::kmajor_off_bf16(r, c0, 64);
          *reinterpret_cast<uint4*>(sm + L::S_HI + off) = h;
          *reinterpret_cast<uint4*>(sm + L::S_LO + off) = l;
        }
        tc::fence_smem_async();
        tc::fence_before_sync();
        __syncthreads();
        const float coef = sqrtf((float)(n - 1) / s);
        // ok: Z is certified (the probe or the polish residual against the exact
        // A is small).  A spectrum bound s / c beyond what the 16-bit products
        // resolve skips the iteration; that point, and one whose certificate
        // fails (no convergence, a non-finite residual), goes to the Jacobi pass.
        bool ok = a.ns_cond_max > 0.f ? (s < a.ns_cond_max * cdiag) : true;
        int it = 0;
        if (ok) {
        // tensor-core phase: the iterations that move the small eigenvalues of
        // ZY towards 1; stop once ||ZY - I||_F^2 < tc_ns_tol (or after TC_NS_MAX).
        // Spectrum scaling: with X = ZY = (A/s) Z^2 and f(x) = x (3 - x)^2 / 4,
        // the step S <- sqrt(a) S (3I - aX) / 2 maps every eigenvalue x of X to
        // f(a x).  With s = min(||A||_F, Gershgorin) >= lambda_max the spectrum
        // starts in [lo, 1] and every step is scaled; with the power-iteration
        // scale the first step is plain (a = 1; x <= gmax / s <= 2), which
        // leaves the spectrum in [lo, 1].  A scaled step takes the a that balances
        // f(a lo) = f(a (1 + d)), a = 3 (1 - sqrt(l)) / (1 - l^1.5) / (1 + d)
        // with l = lo / (1 + d), which multiplies the small eigenvalues by about
        // 6.75 per step instead of 2.25.  lo starts from the diagonal shift
        // (A >= c I; 0.9 c covers the Gram's rounding) and follows f; an
        // eigenvalue below lo only converges later, and the margin d = 0.02
        // keeps a x < 3 for the rounding of the 16-bit products.
        float lo = 0.9f * cdiag * inv_s;
        const float lo_top = f_ns(fminf(gmax * inv_s, 2.f));
        const int tc_max = a.tc_ns_max;
        for (bool done = tc_max <= 0; !done; it++) {
          if (it == tc_max - 1) done = true;
          // T = Z Y  (rows 64..127 of S Y)
          if (tid == 0) {
            tc::fence_after_sync();
            // B = Y read in place: rows 0..63 of S have the K-major offsets of a
            // 64 x 64 operand with the same strides
            ns_mma(D0, sbase + L::S_HI, sbase + L::S_LO, sbase + L::S_HI, sbase + L::S_LO, idesc);
            tc::mma_commit(&mbar[2]);
          }
          wait_bar(2);
          tc::fence_after_sync();
          float e2 = 0.f;
          if (wid >= 2) {
#pragma unroll 1
            for (int c0 = 0; c0 < 64; c0 += 16) {
              float v[16];
              tc::tmem_ld16(D0 + lane_off + c0, v);
#pragma unroll
              for (int j = 0; j < 16; j++) {
                const float dlt = v[j] - ((r - 64 == c0 + j) ? 1.f : 0.f);
                e2 = fmaf(dlt, dlt, e2);
              }
#pragma unroll
              for (int g = 0; g < 2; g++) {
                uint4 h, l;
                split8(v + 8 * g, h, l);
                const uint32_t off = tc::kmajor_off_bf16(r - 64, c0 + 8 * g, 64);
                *reinterpret_cast<uint4*>(sm + L::B_HI + off) = h;
                *reinterpret_cast<uint4*>(sm + L::B_LO + off) = l;
              }
            }
          }
          // ||ZY - I||^2 from warps 2 and 3 (rows 64..127), summed across the
          // barrier that publishes the B operand
          e2 = warp_sum(e2);
          if (lane == 0 && wid >= 2) red[wid] = e2;
          tc::fence_smem_async();
          tc::fence_before_sync();
          __syncthreads();
          if (red[2] + red[3] < a.tc_ns_tol) done = true;
          // [Y;Z] T
          if (tid == 0) {
            tc::fence_after_sync();
            ns_mma(D0, sbase + L::S_HI, sbase + L::S_LO, sbase + L::B_HI, sbase + L::B_LO, idesc);
            tc::mma_commit(&mbar[2]);
          }
          wait_bar(2);
          tc::fence_after_sync();
          if (__syncthreads_or(tmo)) {
            tmo = 1;
            break;
          }
          // S <- sqrt(a) (1.5 S - 0.5 a S X) (each thread rewrites only its own row)
          float ka = 1.5f, kb = 0.5f;
          if (it == 0 && !a.tc_scale_bound) {
            lo = fminf(f_ns(lo), lo_top);
          } else if (a.tc_ns_scaled) {
            const float al = ns_scale(lo);
            const float sa = sqrtf(al);
            ka = 1.5f * sa;
            kb = 0.5f * al * sa;
            lo = f_ns(al * lo);
          } else {
            lo = f_ns(lo);
          }
#pragma unroll 1
          for (int c0 = 0; c0 < 64; c0 += 16) {
            float v[16];
            tc::tmem_ld16(D0 + lane_off + c0, v);
#pragma unroll
            for (int g = 0; g < 2; g++) {
              const uint32_t off = tc::kmajor_off_bf16(r, c0 + 8 * g, 64);
              float sh[8], sl[8], sn[8];
              unpack8(*reinterpret_cast<const uint4*>(sm + L::S_HI + off), sh);
              unpack8(*reinterpret_cast<const uint4*>(sm + L::S_LO + off), sl);
#pragma unroll
              for (int j = 0; j < 8; j++) sn[j] = ka * (sh[j] + sl[j]) - kb * v[8 * g + j];
              uint4 h, l;
              split8(sn, h, l);
              *reinterpret_cast<uint4*>(sm + L::S_HI + off) = h;
              *reinterpret_cast<uint4*>(sm + L::S_LO + off) = l;
            }
          }
          // the new S is the next step's operands (generic stores -> async proxy)
          tc::fence_smem_async();
          tc::fence_before_sync();
          __syncthreads();
        }
        if (tmo) break;
        if (a.tc_polish) {
          // Tensor-core polish: the anchored step Q = Z (A/s) Z^T,
          // Z <- Z - Z (Q - I) / 2, as three stacked 3-term bf16 products
          // D = S B^T with S = [scratch; Z] (Z stays in rows 64..127):
          //   B = A/s (exact A from TMEM)      -> rows 64..127: P = Z A/s
          //   S rows 0..63 = P, B = Z          -> rows 0..63:   Q = P Z^T
          //   B = R = Q - I                    -> rows 64..127: Z R
          // R is small, so its 16-bit split is ample; Z's own 16-bit rounding
          // is what the step measures and corrects.  Ends after the step whose
          // ||Q - I||_F^2 fell below 1e-6 (the FP32 accumulation in TMEM
          // leaves about 1e-7), at most TC_POLISH_MAX steps.
          int pit = 0;
          for (bool last = false; !last && !tmo;) {
            // B <- A / s (row r of A from TMEM lanes 0..63)
            if (wid < 2) {
#pragma unroll 1
              for (int c0 = 0; c0 < 64; c0 += 16) {
                float v[16];
                tc::tmem_ld16(D1 + lane_off + c0, v);
#pragma unroll
                for (int j = 0; j < 16; j++) v[j] *= inv_s;
#pragma unroll
                for (int g = 0; g < 2; g++) {
                  uint4 h, l;
                  split8(v + 8 * g, h, l);
                  const uint32_t off = tc::kmajor_off_bf16(r, c0 + 8 * g, 64);
                  *reinterpret_cast<uint4*>(sm + L::B_HI + off) = h;
                  *reinterpret_cast<uint4*>(sm + L::B_LO + off) = l;
                }
              }
            }
            tc::fence_smem_async();
            tc::fence_before_sync();
            __syncthreads();
            if (tid == 0) {
              tc::fence_after_sync();
              ns_mma(D0, sbase + L::S_HI, sbase + L::S_LO, sbase + L::B_HI, sbase + L::B_LO, idesc);
              tc::mma_commit(&mbar[2]);
            }
            wait_bar(2);
            tc::fence_after_sync();
            // S rows 0..63 <- P (from rows 64..127 of D); B <- Z
            if (wid >= 2) {
#pragma unroll 1
              for (int c0 = 0; c0 < 64; c0 += 16) {
                float v[16];
                tc::tmem_ld16(D0 + lane_off + c0, v);
#pragma unroll
                for (int g = 0; g < 2; g++) {
                  uint4 h, l;
                  split8(v + 8 * g, h, l);
                  const uint32_t off = tc::kmajor_off_bf16(r - 64, c0 + 8 * g, 64);
                  *reinterpret_cast<uint4*>(sm + L::S_HI + off) = h;
                  *reinterpret_cast<uint4*>(sm + L::S_LO + off) = l;
                }
              }
            }
            for (int i = tid; i < 8192 / 16; i += TC_NT) {
              reinterpret_cast<uint4*>(sm + L::B_HI)[i] = reinterpret_cast<const uint4*>(sm + L::S_HI + 8192)[i];
              reinterpret_cast<uint4*>(sm + L::B_LO)[i] = reinterpret_cast<const uint4*>(sm + L::S_LO + 8192)[i];
            }
            tc::fence_smem_async();
            tc::fence_before_sync();
            __syncthreads();
            if (tid == 0) {
              tc::fence_after_sync();
              ns_mma(D0, sbase + L::S_HI, sbase + L::S_LO, sbase + L::B_HI, sbase + L::B_LO, idesc);
              tc::mma_commit(&mbar[2]);
            }
            wait_bar(2);
            tc::fence_after_sync();
            // B <- R = Q - I (rows 0..63 of D); ||R||_F^2
            float e2 = 0.f;
            if (wid < 2) {
#pragma unroll 1
              for (int c0 = 0; c0 < 64; c0 += 16) {
                float v[16];
                tc::tmem_ld16(D0 + lane_off + c0, v);
#pragma unroll
                for (int j = 0; j < 16; j++) {
                  v[j] -= (r == c0 + j) ? 1.f : 0.f;
                  e2 = fmaf(v[j], v[j], e2);
                }
#pragma unroll
                for (int g = 0; g < 2; g++) {
                  uint4 h, l;
                  split8(v + 8 * g, h, l);
                  const uint32_t off = tc::kmajor_off_bf16(r, c0 + 8 * g, 64);
                  *reinterpret_cast<uint4*>(sm + L::B_HI + off) = h;
                  *reinterpret_cast<uint4*>(sm + L::B_LO + off) = l;
                }
              }
            }
            tc::fence_smem_async();
            tc::fence_before_sync();
            e2 = block_sum<float, TC_NT>(e2, red);
            pit++;
            ok = e2 < 1.0e-6f;
            last = ok || pit >= TC_POLISH_MAX;
            if (tid == 0) {
              tc::fence_after_sync();
              ns_mma(D0, sbase + L::S_HI, sbase + L::S_LO, sbase + L::B_HI, sbase + L::B_LO, idesc);
              tc::mma_commit(&mbar[2]);
            }
            wait_bar(2);
            tc::fence_after_sync();
            if (__syncthreads_or(tmo)) {
              tmo = 1;
              break;
            }
            // Z <- Z - Z R / 2 (rows 64..127); the last step writes W = coef Z
            if (wid >= 2) {
#pragma unroll 1
              for (int c0 = 0; c0 < 64; c0 += 16) {
                float v[16];
                tc::tmem_ld16(D0 + lane_off + c0, v);
#pragma unroll
                for (int g = 0; g < 2; g++) {
                  const uint32_t off = tc::kmajor_off_bf16(r, c0 + 8 * g, 64);
                  float sh[8], sl[8], zn[8];
                  unpack8(*reinterpret_cast<const uint4*>(sm + L::S_HI + off), sh);
                  unpack8(*reinterpret_cast<const uint4*>(sm + L::S_LO + off), sl);
#pragma unroll
                  for (int j = 0; j < 8; j++) zn[j] = (sh[j] + sl[j]) - 0.5f * v[8 * g + j];
                  if (last) {
                    float* dst = Wm + (r - 64) * 64 + c0 + 8 * g;
#pragma unroll
                    for (int j = 0; j < 8; j++) dst[j] = coef * zn[j];
                  } else {
                    uint4 h, l;
                    split8(zn, h, l);
                    *reinterpret_cast<uint4*>(sm + L::S_HI + off) = h;
                    *reinterpret_cast<uint4*>(sm + L::S_LO + off) = l;
                  }
                }
              }
            }
            tc::fence_before_sync();
            __syncthreads();
          }
          if (tmo) break;
          // W symmetric, as the reference's V diag(.) V^T is
          for (int idx = tid; idx < 64 * 64; idx += TC_NT) {
            const int i = idx >> 6, j = idx & 63;
            if (i < j) {
              const float v = 0.5f * (Wm[i * 64 + j] + Wm[j * 64 + i]);
              Wm[i * 64 + j] = v;
              Wm[j * 64 + i] = v;
            }
          }
          __syncthreads();
          it += pit;
        } else {
          // FP32 polish.  The coupled iteration never looks at A again, so the
          // 16-bit rounding of the tensor-core phase shifts the matrix it is
          // converging for.  Finish with the uncoupled iteration
          //   Q = Z (A/s) Z,  Z <- (3 Z - Q Z) / 2,
          // which references the exact A (kept in TMEM) at every step and so
          // converges to (A/s)^(-1/2) from the tensor-core estimate.
          // Z goes to the free B area (it becomes W in place there: TF == WMAT),
          // so rows of S are converted straight out of their 16-bit split; A / s
          // overwrites S_HI once every row of S has been read
          static_assert(L::TF == L::WMAT, "Z is scaled into W in place");
          float* Zf = reinterpret_cast<float*>(sm + L::TF);
          float* Af = reinterpret_cast<float*>(sm + L::YF);  // A / s
          float* Pf = reinterpret_cast<float*>(sm + L::ZF);  // A Z, then Q; the probe vectors
          if (r >= 64) {
            float* dst = Zf + (r - 64) * 64;
  #pragma unroll 1
            for (int c0 = 0; c0 < 64; c0 += 8) {
              const uint32_t off = tc::kmajor_off_bf16(r, c0, 64);
              float sh[8], sl[8];
              unpack8(*reinterpret_cast<const uint4*>(sm + L::S_HI + off), sh);
              unpack8(*reinterpret_cast<const uint4*>(sm + L::S_LO + off), sl);
              *reinterpret_cast<float4*>(dst + c0) = make_float4(sh[0] + sl[0], sh[1] + sl[1], sh[2] + sl[2], sh[3] + sl[3]);
              *reinterpret_cast<float4*>(dst + c0 + 4) =
                  make_float4(sh[4] + sl[4], sh[5] + sl[5], sh[6] + sl[6], sh[7] + sl[7]);
            }
          }
          __syncthreads();
          if (r < 64) {
  #pragma unroll 1
            for (int c0 = 0; c0 < 64; c0 += 16) {
              float v[16];
              tc::tmem_ld16(D1 + lane_off + c0, v);
  #pragma unroll
              for (int j = 0; j < 16; j++) Af[r * 64 + c0 + j] = v[j] * inv_s;
            }
          }
          tc::fence_before_sync();
          __syncthreads();
          // Probe of the anchored residual, three matvecs: e = ||Z (A/s) Z p - p||^2
          // / ||p||^2 for a fixed pseudo-random p.  With Z = (A/s)^(-1/2) (I + E),
          // Z (A/s) Z p - p = 2 E p to first order, so e estimates 4 ||E p||^2 /
          // ||p||^2, the relative error the transform would carry into the
          // analysis; a point whose estimate is below the probe tolerance already
          // has the accuracy the polish would restore.  Z and A are symmetric, so
          // the products read columns (consecutive lanes, no bank conflicts).
          bool polish = true;
          if (a.polish_probe > 0.f) {
            float* pv = Pf;
            float* pu = Pf + 64;
            float* pw = Pf + 128;
            if (tid < 64) pv[tid] = probe_component(tid);
            __syncthreads();
            if (tid < 64) pu[tid] = col_dot64(Zf, pv, tid);
            __syncthreads();
            if (tid < 64) pw[tid] = col_dot64(Af, pu, tid);
            __syncthreads();
            float q2[2] = {0.f, 0.f};
            if (tid < 64) {
              const float d = col_dot64(Zf, pw, tid) - pv[tid];
              q2[0] = d * d;
              q2[1] = pv[tid] * pv[tid];
            }
            block_sum_k<float, TC_NT, 2>(q2, red);
            polish = !(q2[0] < a.polish_probe * q2[1]);  // a NaN residual polishes
          }
          if (polish)
            it += ns_polish<TC_NP>(Af, Zf, Pf, red, tc_max > 0 ? TC_POLISH_MAX : a.max_ns_iter, a.polish_tol, &ok);
          for (int idx = tid; idx < 64 * 64; idx += TC_NT) Wm[idx] = coef * Zf[idx];
          __syncthreads();
        }
        }  // ok: Newton-Schulz attempted
        if (tmo) break;
        if (!ok) {
          deferred = true;
        } else {
          // wbar = Z (Z b) / s with Z = W / coef (W symmetric: column reads);
          // meanwhile a thread of the upper half, idle here, does the FP64
          // inflation update
          if (tid < 64) {
            const float acc = col_dot64(Wm, vb, tid);
            vg[tid] = acc / coef;
          } else if (tid == 64) {
            a.infl[pt] = infl_update(n, infl, (double)p1, (double)trace, (double)p3);
            a.status[pt] = LETKF_OK;
            if (a.sweeps_out) a.sweeps_out[pt] = it;
          }
          __syncthreads();
          if (tid < 64) {
            const float acc = col_dot64(Wm, vg, tid);
            vwb[tid] = acc / (coef * s);
          }
        }
      }
    } else {
      const float sq = (float)sqrt(infl);
      for (int idx = tid; idx < 64 * 64; idx += TC_NT) Wm[idx] = ((idx >> 6) == (idx & 63)) ? sq : 0.f;
      if (tid < 64) vwb[tid] = 0.f;
      if (tid == 0) {
        a.status[pt] = LETKF_OK;
        if (a.sweeps_out) a.sweeps_out[pt] = 0;
      }
    }
    if (tid == 0 && a.nobsl_out) a.nobsl_out[pt] = Lp;
    if (deferred) {
      if (tid == 0) {
        a.defer_list[atomicAdd(a.defer_count, 1)] = a.list_offs ? qq : pt;
        if (a.defer_total) atomicAdd(a.defer_total, 1);
      }
      if (xb_outst) {
        wait_bar(3);
        xb_outst = false;
      }
      continue;
    }
    __syncthreads();
    // ---- update: xa = mean + xp (W + wbar 1^T); FP64 mean and mean increment ----
    if (xb_outst) {
      wait_bar(3);
      xb_outst = false;
      const float* xin = reinterpret_cast<const float*>(sm + L::PIDX);
      for (int t = tid; t < nv * n; t += TC_NT) {
        const int v = t / n, mm = t - v * n;
        xs[v * 64 + mm] = xin[t];
      }
    } else {
      for (int t = tid; t < nv * n; t += TC_NT) {
        const int v = t / n, mm = t - v * n;
        xs[v * 64 + mm] = a.xb[((size_t)v * a.npts + pt) * n + mm];
      }
    }
    __syncthreads();
    // The member sum and the mean-increment accumulation stay FP64; centring
    // and the stores run in FP32 on the mean as an unevaluated pair mh + ml
    // (GB300's FP64 pipe is narrow): xs - mh is exact for members within a
    // factor of two of the mean and ml carries the rest; the analysis mean
    // (mean + increment) is kept as a pair again for the stores.
    float* meanf = reinterpret_cast<float*>(meanv + 8);  // [v] = {hi, lo}
    for (int v = wid; v < nv; v += TC_NT / 32) {
      double sx = 0.0;
      for (int mm = lane; mm < n; mm += 32) sx += (double)xs[v * 64 + mm];
      const double mean = warp_sum(sx) * inv_n;
      const float mh = (float)mean, ml = (float)(mean - (double)mh);
      double dlt = 0.0;
      for (int mm = lane; mm < n; mm += 32) {
        const float xp = (xs[v * 64 + mm] - mh) - ml;
        xs[v * 64 + mm] = xp;
        dlt = fma((double)xp, (double)vwb[mm], dlt);
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
    {
      // thread: member mm, variables vg, vg + 2, ... (up to four); one W load
      // feeds every variable and the sums run in k order as before
      const int mm = tid & 63, vg = tid >> 6;
      if (mm < n) {
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 2
        for (int k = 0; k < n; k++) {
          const float w = Wm[k * 64 + mm];
#pragma unroll
          for (int j = 0; j < 4; j++)
            if (vg + 2 * j < nv) acc[j] = fmaf(xs[(vg + 2 * j) * 64 + k], w, acc[j]);
        }
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const int v = vg + 2 * j;
          if (v < nv) a.xa[((size_t)v * a.npts + pt) * n + mm] = meanf[2 * v] + (acc[j] + meanf[2 * v + 1]);
        }
      }
    }
  }
  // drain (bounded), report, release tensor memory
  for (int b = 0; b < 2; b++)
    if ((outst >> b) & 1u) wait_bar(b);
  if (xb_outst) wait_bar(3);
  if (__syncthreads_or(tmo)) {
    // a wait gave up: before TMEM and shared memory are released, every MMA
    // this CTA issued (one commit on the drain barrier tracks all of them)
    // and a background-row copy whose wait gave up must have landed; both
    // always complete, so these waits end
    if (tid == 0) {
      tc::fence_after_sync();
      tc::mma_commit(&mbar[4]);
      if (a.err_flag) atomicExch(a.err_flag, 1);
    }
    tc::mbar_wait(&mbar[4], 0u, TC_WAIT);
    if (xb_lost) tc::mbar_wait(&mbar[3], xb_lost & 1u, TC_WAIT);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (wid == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tbase, TC_TMEM_COLS);
  }
}

static std::atomic<uint32_t> g_tc_attr{0};

int prepare_sweep_tc() {
  return cuda_status(set_smem_once(sweep_tc_kernel, TcLayout::TOTAL, g_tc_attr));
}

int launch_sweep_tc(const SweepArgs& a, cudaStream_t stream, int grid_cap) {
  if (a.n < 2 || a.n > TC_NP || a.nv < 1 || a.nv > 8) return LETKF_ERR_ARG;
  if (a.nwork == 0) return LETKF_OK;
  constexpr size_t bytes = TcLayout::TOTAL;
  cudaError_t err = set_smem_once(sweep_tc_kernel, bytes, g_tc_attr);
  if (err != cudaSuccess) return cuda_status(err);
  int dev = 0, nsm = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  {
    // residency from the registers and shared memory the kernel uses (the
    // occupancy query reports one CTA per SM for this tensor-memory kernel)
    cudaFuncAttributes fa;
    int smem_sm = 0, regs_sm = 0;
    if (cudaFuncGetAttributes(&fa, sweep_tc_kernel) != cudaSuccess) return LETKF_ERR_CUDA;
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
    const int by_smem = smem_sm / (int)(bytes + fa.sharedSizeBytes + 1024);
    const int by_regs = regs_sm / (TC_NT * (fa.numRegs > 0 ? fa.numRegs : 128));
    per_sm = by_smem < by_regs ? by_smem : by_regs;
    if (per_sm < 1) per_sm = 1;
  }
  // tensor memory: 512 columns per SM
  if (per_sm > (int)(512 / TC_TMEM_COLS)) per_sm = 512 / TC_TMEM_COLS;
  int grid = nsm * per_sm;
  if (grid_cap > 0 && grid > grid_cap) grid = grid_cap;
  if (grid_cap < 0) grid = grid / -grid_cap > 0 ? grid / -grid_cap : 1;  // a 1/v share of the resident CTAs
  if (grid > a.nwork) grid = a.nwork;
  sweep_tc_kernel<<<grid, TC_NT, bytes, stream>>>(a);
  note_launch();
  return cuda_status(cudaGetLastError());
}

}  // namespace letkf
