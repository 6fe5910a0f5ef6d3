// sweep_tc128.cu -- fused analysis sweep on the tcgen05 tensor cores for 64 < k <= 128.
//
// The per-point work of sweep_tc.cu (search, Gram, Newton-Schulz transform,
// update; scale/letkf/letkf_tools.f90:853-1178 with common/common_letkf.f90:
// 50-243) at ensemble sizes up to 128, where the k x k matrices fill a whole
// 128 x 128 MMA tile.  One CTA of 256 threads per SM (the operands take 192 KB
// of shared memory and the accumulators all 512 TMEM columns):
//
//  * Gram  G = Ywᵀ Y: stages of 32 accepted observations staged K-major as
//    TF32 hi / lo splits of Yw and Y (128 x 32 each); three MMAs per K step
//    (hi.hi + hi.lo + lo.hi, M = N = 128) accumulate into TMEM columns 0..127.
//    Staging of stage c+1 overlaps the MMAs of stage c (two 64 KB buffers).
//  * A = G + (k-1)/rho I is kept exactly in TMEM columns 256..383.
//  * Coupled Newton-Schulz on BF16 hi / lo splits of Y and Z (128 x 128 each):
//    T = Z Y (columns 0..127), then Y T and Z T (columns 0..127, 128..255),
//    each product the three split terms over K = 128, spectrum-scaled steps.
//  * the anchored probe and FP32 polish (ns_polish<128>), wbar, inflation and
//    the update as in sweep_tc.cu.
// TMEM lanes are split by warp quadrant: warp w reads rows 32 (w % 4) ..
// +31, and warps w and w + 4 take the two column halves of those rows.
#include "mixed_core.cuh"
#include "sweep_search.cuh"
#include "tc_sm100.cuh"

namespace letkf {

constexpr int T8_NT = 256;
constexpr int T8_NP = 128;
constexpr int T8_CH = 32;  // observations per Gram stage
constexpr uint32_t T8_TMEM_COLS = 512;
constexpr uint32_t T8_WAIT = 1u << 22;
constexpr int T8_POLISH_MAX = 8;

struct T8Layout {
  // operand region, 192 KB, reused by phase
  static constexpr int STG = 0;            // two Gram stages of 64 KB
  static constexpr int STG_AH = 0;         //   Yw_hi: 128 x 32 tf32 (16 KB)
  static constexpr int STG_AL = 16384;     //   Yw_lo
  static constexpr int STG_BH = 32768;     //   Y_hi
  static constexpr int STG_BL = 49152;     //   Y_lo
  static constexpr int STG_SIZE = 65536;
  static constexpr int Y_HI = 0;           // Newton-Schulz Y: 128 x 128 bf16 (32 KB)
  static constexpr int Y_LO = 32768;
  static constexpr int Z_HI = 65536;       // Z
  static constexpr int Z_LO = 98304;
  static constexpr int B_HI = 131072;      // B = Y or T
  static constexpr int B_LO = 163840;
  static constexpr int GTMP = 131072;      // Gram in FP32, 128 x 128, swizzled rows (over B)
  static constexpr int AF = 0;             // FP32 polish: A / s (over Y)
  static constexpr int PF = 65536;         //   scratch (over Z)
  static constexpr int ZF = 131072;        //   Z, then W in place (over B)
  static constexpr int WMAT = ZF;
  static constexpr int XS = 0;             // update staging, nv x 128 FP32 (over A / s)
  static constexpr int OPER_END = 196608;
  // small data
  static constexpr int VB = OPER_END;                 // float[128] departure product
  static constexpr int VBP = VB + 512;                // float[256] partial departure products
  static constexpr int VWB = VBP + 1024;              // float[128] wbar
  static constexpr int VG = VWB + 512;                // float[128]
  static constexpr int RED = VG + 512;                // float[64]
  static constexpr int PCAP = T8_CH + T8_NT;          // pending-list entries
  static constexpr int PIDX = RED + 256;              // int[PCAP]
  static constexpr int PW = PIDX + 4 * PCAP;
  static constexpr int PD = PW + 4 * PCAP;
  static constexpr int PR = PD + 4 * PCAP;
  static constexpr int ROWIB = PR + 4 * PCAP;
  static constexpr int ROWPRE = ROWIB + 4 * SW_MAXROWS;
  static constexpr int WCNT = ROWPRE + 4 * (SW_MAXROWS + 1);
  static constexpr int MEAN = ((WCNT + 4 * 2 * (T8_NT / 32 + 1)) + 7) & ~7;  // double[16]
  static constexpr int MBAR = MEAN + 128;             // uint64[5]: Gram stages 0/1, products, rows, drain
  static constexpr int TMEMH = MBAR + 40;
  static constexpr int CTRL = TMEMH + 8;              // int[4]: position, scratch
  static constexpr int CKEY = CTRL + 16;              // double[2]: the column-cache point (ri, rj)
  static constexpr int RUN = CKEY + 16;               // int[4]: run of positions [next, end), column-cache length
  static constexpr int TOTAL = RUN + 16;
  static_assert(4 * PCAP >= 8 * 128, "background rows (nv <= 8, ne <= 128) fit the pending-list area");
};

// the 128 x 128 FP32 Gram, row r's 4-float column groups XOR-ed by r & 7
__device__ __forceinline__ int gsw8(int r, int c) { return r * 128 + (c ^ ((r & 7) << 2)); }

// sum_j M[j][c] x[j] for a 128 x 128 row-major matrix (column c as consecutive lanes)
__device__ __forceinline__ float col_dot128(const float* M, const float* x, int c) {
  float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
#pragma unroll 4
  for (int j = 0; j < 128; j += 4) {
    a0 = fmaf(M[j * 128 + c], x[j], a0);
    a1 = fmaf(M[(j + 1) * 128 + c], x[j + 1], a1);
    a2 = fmaf(M[(j + 2) * 128 + c], x[j + 2], a2);
    a3 = fmaf(M[(j + 3) * 128 + c], x[j + 3], a3);
  }
  return (a0 + a1) + (a2 + a3);
}

// D = X_hi B_hi + X_hi B_lo + X_lo B_hi over K = 128 (8 steps of 16): 24 MMAs
__device__ __forceinline__ void ns_mma128(uint32_t d, uint32_t x_hi, uint32_t x_lo, uint32_t b_hi, uint32_t b_lo,
                                          uint32_t idesc) {
#pragma unroll
  for (int pass = 0; pass < 3; pass++) {
    const uint32_t sa = pass == 2 ? x_lo : x_hi;
    const uint32_t sb = pass == 1 ? b_lo : b_hi;
#pragma unroll
    for (int s = 0; s < 8; s++)
      tc::mma_bf16(d, tc::smem_desc(sa + s * 256, 128, 2048), tc::smem_desc(sb + s * 256, 128, 2048), idesc,
                   (pass == 0 && s == 0) ? 0u : 1u);
  }
}

__global__ void __launch_bounds__(T8_NT, 1) sweep_tc128_kernel(SweepArgs a) {
  using L = T8Layout;
  extern __shared__ __align__(1024) unsigned char sm[];
  float* vb = reinterpret_cast<float*>(sm + L::VB);
  float* vbp = reinterpret_cast<float*>(sm + L::VBP);
  float* vwb = reinterpret_cast<float*>(sm + L::VWB);
  float* vg = reinterpret_cast<float*>(sm + L::VG);
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
  const uint32_t idesc = tc::idesc_bf16(128, 128);
  const uint32_t idesc_g = tc::idesc_tf32(128, 128);

  if (tid == 0) {
    for (int i = 0; i < 5; i++) tc::mbar_init(&mbar[i], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    int* rn = reinterpret_cast<int*>(sm + L::RUN);
    rn[0] = rn[1] = 0;
    rn[2] = -2;
    double* ck = reinterpret_cast<double*>(sm + L::CKEY);
    ck[0] = ck[1] = __longlong_as_double(0x7ff8000000000000ll);  // NaN: equal to no point
  }
  if (wid == 0) tc::tmem_alloc(tmem_holder, T8_TMEM_COLS);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = *tmem_holder;
  const uint32_t DG = tbase, DY = tbase, DZ = tbase + 128, DA = tbase + 256;
  const int quad = wid & 3, half = wid >> 2;
  const int r = quad * 32 + lane;  // the TMEM lane / operand row this thread owns
  const int cbase = half * 64;     // and its 64 columns
  const uint32_t lane_off = (uint32_t)(quad * 32) << 16;
  uint32_t par = 0u, outst = 0u, xb_lost = 0u;
  bool xb_outst = false;
  int tmo = 0;
  const int npts_work = a.npts_dev ? *a.npts_dev : a.nwork;
  const double inv_n = 1.0 / (double)n;

  auto wait_bar = [&](int i) {
    const uint32_t pb = (par >> i) & 1u;
    if (!tc::mbar_wait(&mbar[i], pb, T8_WAIT)) {
      tmo = 1;
      if (i == 3) xb_lost = 2u | pb;
    }
    par ^= 1u << i;
  };
  if (a.fault_wait_polls > 0u && !tc::mbar_wait(&mbar[4], 0u, a.fault_wait_polls)) tmo = 1;
  const bool skip_all = __syncthreads_or(tmo);
  if (skip_all) tmo = 1;

  // runs of consecutive order positions and the column cache of the search,
  // as in the k <= 64 sweep (sweep_tc.cu)
  const bool col = a.col_ent != nullptr && !a.list_offs && (int)blockIdx.x < a.col_slots;
  double* ckey = reinterpret_cast<double*>(sm + L::CKEY);
  int* run = reinterpret_cast<int*>(sm + L::RUN);
  for (; !skip_all;) {
    __syncthreads();
    if (tid == 0) {
      if (run[0] >= run[1]) {
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
    const int qq = a.qmap ? a.qmap[q] : q;
    const int pt = a.order[qq];
    const double ri = a.pri[pt], rj = a.prj[pt], rz = a.prz ? a.prz[pt] : 0.0;
    const double logr = a.plogr[pt];

    // ---- search + Gram on the tensor cores ----
    const int m = tid & 127, hh = tid >> 7;
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
      constexpr int KH = T8_CH / 2;  // observations per thread: member m, half hh
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
        const uint32_t off = tc::kmajor_off(m, hh * KH + g * 4, T8_CH);
        split4_tf32(wv + 4 * g, h, l);
        *reinterpret_cast<float4*>(stg + L::STG_AH + off) = h;
        *reinterpret_cast<float4*>(stg + L::STG_AL + off) = l;
        split4_tf32(yv + 4 * g, h, l);
        *reinterpret_cast<float4*>(stg + L::STG_BH + off) = h;
        *reinterpret_cast<float4*>(stg + L::STG_BL + off) = l;
      }
      for (int k = tid; k < nr; k += T8_NT) {
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
        constexpr uint32_t SBO = T8_CH * 32;
#pragma unroll
        for (int s = 0; s < T8_CH / 8; s++) {
          const uint64_t ah = tc::smem_desc(sa + L::STG_AH + s * 256, 128, SBO);
          const uint64_t al = tc::smem_desc(sa + L::STG_AL + s * 256, 128, SBO);
          const uint64_t bh = tc::smem_desc(sa + L::STG_BH + s * 256, 128, SBO);
          const uint64_t bl = tc::smem_desc(sa + L::STG_BL + s * 256, 128, SBO);
          tc::mma_tf32(DG, ah, bh, idesc_g, (first && s == 0) ? 0u : 1u);
          tc::mma_tf32(DG, ah, bl, idesc_g, 1u);
          tc::mma_tf32(DG, al, bh, idesc_g, 1u);
        }
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
      Lp = sweep_list<T8_NT, T8_CH>(a, qq, ss, flush);
    } else if (same_col && cn >= 0) {
      Lp = sweep_search_cached<T8_NT, T8_CH>(a, a.col_ent + (size_t)blockIdx.x * a.col_cap * 2, cn, ri, rj, logr,
                                             rz, ss, probe, flush);
    } else if (col && !same_col) {
      int nsv = 0;
      const SwCache cache{a.col_ent + (size_t)blockIdx.x * a.col_cap * 2, a.col_cap};
      Lp = sweep_search<T8_NT, T8_CH, 1>(a, ri, rj, logr, rz, ss, probe, flush, cache, &nsv);
      if (tid == 0) {  // read by the next point, after the barriers in between
        ckey[0] = ri;
        ckey[1] = rj;
        run[2] = nsv <= a.col_cap ? nsv : -1;
      }
    } else {  // no cache, or this column's did not fit
      Lp = sweep_search<T8_NT, T8_CH, 1>(a, ri, rj, logr, rz, ss, probe, flush);
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
    // TMA: this point's background rows into the pending-list area (free
    // until the next point), consumed by the update
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
      if (tid == 0) reinterpret_cast<float*>(ctrl)[1] = (float)((double)(n - 1) / infl);
      // G: this thread's row r, columns cbase .. cbase + 63
#pragma unroll
      for (int c0 = 0; c0 < 64; c0 += 16) {
        float v[16];
        tc::tmem_ld16(DG + lane_off + cbase + c0, v);
#pragma unroll
        for (int j = 0; j < 16; j += 4)
          *reinterpret_cast<float4*>(Gt + gsw8(r, cbase + c0 + j)) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
      }
      vbp[tid] = bpart;
      tc::fence_before_sync();
      __syncthreads();
      const float cdiag = reinterpret_cast<const float*>(ctrl)[1];
      if (tid < 128) vb[tid] = vbp[tid] + vbp[tid + 128];
      // symmetrise along diagonals (i, i + d mod 128), d = 1..64
      for (int t = tid; t < 64 * 128; t += T8_NT) {
        const int d = 1 + (t >> 7), i = t & 127;
        if (d == 64 && i >= 64) continue;
        const int j = (i + d) & 127;
        const float v = 0.5f * (Gt[gsw8(i, j)] + Gt[gsw8(j, i)]);
        Gt[gsw8(i, j)] = v;
        Gt[gsw8(j, i)] = v;
      }
      __syncthreads();
      float sums[3] = {tid < 128 ? Gt[gsw8(tid, tid)] : 0.f, p1, p3};
      block_sum_k<float, T8_NT, 3>(sums, red);
      const float trace = sums[0];
      p1 = sums[1];
      p3 = sums[2];
      if (!(cdiag > 0.f) || !((double)trace < 1.0e6 * (double)cdiag)) {
        deferred = true;  // needs the eigensolver with mtx_eigen's truncation
      } else {
        if (tid < 128) Gt[gsw8(tid, tid)] += cdiag;
        __syncthreads();
        // exact FP32 A into TMEM columns 256..383 (row r, this thread's half)
#pragma unroll
        for (int c0 = 0; c0 < 64; c0 += 16) {
          float v[16];
#pragma unroll
          for (int j = 0; j < 16; j += 4) {
            const float4 g = *reinterpret_cast<const float4*>(Gt + gsw8(r, cbase + c0 + j));
            v[j] = g.x;
            v[j + 1] = g.y;
            v[j + 2] = g.z;
            v[j + 3] = g.w;
          }
          tc::tmem_st16(DA + lane_off + cbase + c0, v);
        }
        tc::fence_before_sync();
        // scale s = min(||A||_F, Gershgorin) >= lambda_max
        float gsum = 0.f, f2 = 0.f;
        if (tid < 128) {
          float g0 = 0.f, g1 = 0.f, q0 = 0.f, q1 = 0.f;
#pragma unroll 4
          for (int j = 0; j < 128; j += 2) {
            const float x0 = Gt[gsw8(j, tid)], x1 = Gt[gsw8(j + 1, tid)];
            g0 += fabsf(x0);
            g1 += fabsf(x1);
            q0 = fmaf(x0, x0, q0);
            q1 = fmaf(x1, x1, q1);
          }
          gsum = g0 + g1;
          f2 = q0 + q1;
        }
        gsum = warp_max(gsum);
        if (lane == 0) red[32 + wid] = gsum;
        const float fro = sqrtf(block_sum<float, T8_NT>(f2, red));
        float gmax = 0.f;
#pragma unroll
        for (int w = 0; w < T8_NT / 32; w++) gmax = fmaxf(gmax, red[32 + w]);
        const float s = fminf(fro, gmax);
        const float inv_s = 1.f / s;
        // Y = A / s and Z = I as bf16 hi / lo splits (row r, this thread's half)
#pragma unroll
        for (int c0 = 0; c0 < 64; c0 += 8) {
          const int c = cbase + c0;
          float v[8], e[8];
          const float4 x0 = *reinterpret_cast<const float4*>(Gt + gsw8(r, c));
          const float4 x1 = *reinterpret_cast<const float4*>(Gt + gsw8(r, c + 4));
          v[0] = x0.x * inv_s; v[1] = x0.y * inv_s; v[2] = x0.z * inv_s; v[3] = x0.w * inv_s;
          v[4] = x1.x * inv_s; v[5] = x1.y * inv_s; v[6] = x1.z * inv_s; v[7] = x1.w * inv_s;
#pragma unroll
          for (int j = 0; j < 8; j++) e[j] = (r == c + j) ? 1.f : 0.f;
          uint4 h, l;
          const uint32_t off = tc::kmajor_off_bf16(r, c, 128);
          split8(v, h, l);
          *reinterpret_cast<uint4*>(sm + L::Y_HI + off) = h;
          *reinterpret_cast<uint4*>(sm + L::Y_LO + off) = l;
          split8(e, h, l);
          *reinterpret_cast<uint4*>(sm + L::Z_HI + off) = h;
          *reinterpret_cast<uint4*>(sm + L::Z_LO + off) = l;
        }
        tc::fence_smem_async();
        tc::fence_before_sync();
        __syncthreads();
        const float coef = sqrtf((float)(n - 1) / s);
        bool ok = a.ns_cond_max > 0.f ? (s < a.ns_cond_max * cdiag) : true;
        int it = 0;
        if (ok) {
          // spectrum-scaled coupled iteration (see sweep_tc.cu): the spectrum of
          // ZY starts in [lo, 1]; each step S <- sqrt(al) S (3I - al ZY) / 2
          float lo = 0.9f * cdiag * inv_s;
          const int tc_max = a.tc_ns_max;
          for (bool done = tc_max <= 0; !done; it++) {
            if (it == tc_max - 1) done = true;
            // T = Z Y (B = Y: symmetric)
            if (tid == 0) {
              tc::fence_after_sync();
              ns_mma128(DY, sbase + L::Z_HI, sbase + L::Z_LO, sbase + L::Y_HI, sbase + L::Y_LO, idesc);
              tc::mma_commit(&mbar[2]);
            }
            wait_bar(2);
            tc::fence_after_sync();
            float e2 = 0.f;
#pragma unroll
            for (int c0 = 0; c0 < 64; c0 += 16) {
              float v[16];
              tc::tmem_ld16(DY + lane_off + cbase + c0, v);
#pragma unroll
              for (int j = 0; j < 16; j++) {
                const float dlt = v[j] - ((r == cbase + c0 + j) ? 1.f : 0.f);
                e2 = fmaf(dlt, dlt, e2);
              }
#pragma unroll
              for (int g = 0; g < 2; g++) {
                uint4 h, l;
                split8(v + 8 * g, h, l);
                const uint32_t off = tc::kmajor_off_bf16(r, cbase + c0 + 8 * g, 128);
                *reinterpret_cast<uint4*>(sm + L::B_HI + off) = h;
                *reinterpret_cast<uint4*>(sm + L::B_LO + off) = l;
              }
            }
            tc::fence_smem_async();
            tc::fence_before_sync();
            e2 = block_sum<float, T8_NT>(e2, red);  // also the barrier that publishes B
            if (e2 < a.tc_ns_tol) done = true;
            // Y T and Z T
            if (tid == 0) {
              tc::fence_after_sync();
              ns_mma128(DY, sbase + L::Y_HI, sbase + L::Y_LO, sbase + L::B_HI, sbase + L::B_LO, idesc);
              ns_mma128(DZ, sbase + L::Z_HI, sbase + L::Z_LO, sbase + L::B_HI, sbase + L::B_LO, idesc);
              tc::mma_commit(&mbar[2]);
            }
            wait_bar(2);
            tc::fence_after_sync();
            if (__syncthreads_or(tmo)) {
              tmo = 1;
              break;
            }
            float ka = 1.5f, kb = 0.5f;
            if (a.tc_ns_scaled) {
              const float al = ns_scale(lo);
              const float sa = sqrtf(al);
              ka = 1.5f * sa;
              kb = 0.5f * al * sa;
              lo = f_ns(al * lo);
            } else {
              lo = f_ns(lo);
            }
            // Y <- ka Y - kb Y T, Z <- ka Z - kb Z T (each thread its own row and half)
#pragma unroll
            for (int mtx = 0; mtx < 2; mtx++) {
              const uint32_t D = mtx ? DZ : DY;
              const int HI = mtx ? L::Z_HI : L::Y_HI, LO = mtx ? L::Z_LO : L::Y_LO;
#pragma unroll
              for (int c0 = 0; c0 < 64; c0 += 16) {
                float v[16];
                tc::tmem_ld16(D + lane_off + cbase + c0, v);
#pragma unroll
                for (int g = 0; g < 2; g++) {
                  const uint32_t off = tc::kmajor_off_bf16(r, cbase + c0 + 8 * g, 128);
                  float sh[8], sl[8], sn[8];
                  unpack8(*reinterpret_cast<const uint4*>(sm + HI + off), sh);
                  unpack8(*reinterpret_cast<const uint4*>(sm + LO + off), sl);
#pragma unroll
                  for (int j = 0; j < 8; j++) sn[j] = ka * (sh[j] + sl[j]) - kb * v[8 * g + j];
                  uint4 h, l;
                  split8(sn, h, l);
                  *reinterpret_cast<uint4*>(sm + HI + off) = h;
                  *reinterpret_cast<uint4*>(sm + LO + off) = l;
                }
              }
            }
            tc::fence_smem_async();
            tc::fence_before_sync();
            __syncthreads();
          }
          if (tmo) break;
          // FP32 polish anchored to the exact A (as in sweep_tc.cu): Z to FP32
          // (over B), A / s from TMEM (over Y), probe, polish where needed
          float* Zf = reinterpret_cast<float*>(sm + L::ZF);
          float* Af = reinterpret_cast<float*>(sm + L::AF);
          float* Pf = reinterpret_cast<float*>(sm + L::PF);
#pragma unroll
          for (int c0 = 0; c0 < 64; c0 += 8) {
            const int c = cbase + c0;
            const uint32_t off = tc::kmajor_off_bf16(r, c, 128);
            float sh[8], sl[8];
            unpack8(*reinterpret_cast<const uint4*>(sm + L::Z_HI + off), sh);
            unpack8(*reinterpret_cast<const uint4*>(sm + L::Z_LO + off), sl);
            *reinterpret_cast<float4*>(Zf + r * 128 + c) =
                make_float4(sh[0] + sl[0], sh[1] + sl[1], sh[2] + sl[2], sh[3] + sl[3]);
            *reinterpret_cast<float4*>(Zf + r * 128 + c + 4) =
                make_float4(sh[4] + sl[4], sh[5] + sl[5], sh[6] + sl[6], sh[7] + sl[7]);
          }
#pragma unroll
          for (int c0 = 0; c0 < 64; c0 += 16) {
            float v[16];
            tc::tmem_ld16(DA + lane_off + cbase + c0, v);
#pragma unroll
            for (int j = 0; j < 16; j += 4)
              *reinterpret_cast<float4*>(Af + r * 128 + cbase + c0 + j) =
                  make_float4(v[j] * inv_s, v[j + 1] * inv_s, v[j + 2] * inv_s, v[j + 3] * inv_s);
          }
          tc::fence_before_sync();
          __syncthreads();
          bool polish = true;
          if (a.polish_probe > 0.f) {
            float* pv = Pf;
            float* pu = Pf + 128;
            float* pw = Pf + 256;
            if (tid < 128) pv[tid] = probe_component(tid);
            __syncthreads();
            if (tid < 128) pu[tid] = col_dot128(Zf, pv, tid);
            __syncthreads();
            if (tid < 128) pw[tid] = col_dot128(Af, pu, tid);
            __syncthreads();
            float q2[2] = {0.f, 0.f};
            if (tid < 128) {
              const float d = col_dot128(Zf, pw, tid) - pv[tid];
              q2[0] = d * d;
              q2[1] = pv[tid] * pv[tid];
            }
            block_sum_k<float, T8_NT, 2>(q2, red);
            polish = !(q2[0] < a.polish_probe * q2[1]);
          }
          if (polish)
            it += ns_polish<T8_NP>(Af, Zf, Pf, red, tc_max > 0 ? T8_POLISH_MAX : a.max_ns_iter, a.polish_tol, &ok);
          for (int idx = tid; idx < 128 * 128; idx += T8_NT) Wm[idx] = coef * Zf[idx];
          __syncthreads();
        }
        if (tmo) break;
        if (!ok) {
          deferred = true;
        } else {
          if (tid < 128) {
            vg[tid] = col_dot128(Wm, vb, tid) / coef;
          } else if (tid == 128) {
            a.infl[pt] = infl_update(n, infl, (double)p1, (double)trace, (double)p3);
            a.status[pt] = LETKF_OK;
            if (a.sweeps_out) a.sweeps_out[pt] = it;
          }
          __syncthreads();
          if (tid < 128) vwb[tid] = col_dot128(Wm, vg, tid) / (coef * s);
        }
      }
    } else {
      const float sq = (float)sqrt(infl);
      for (int idx = tid; idx < 128 * 128; idx += T8_NT) Wm[idx] = ((idx >> 7) == (idx & 127)) ? sq : 0.f;
      if (tid < 128) vwb[tid] = 0.f;
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
    // ---- update: xa = mean + xp (W + wbar 1^T); FP64 member sum and mean increment ----
    if (xb_outst) {
      wait_bar(3);
      xb_outst = false;
      const float* xin = reinterpret_cast<const float*>(sm + L::PIDX);
      for (int t = tid; t < nv * n; t += T8_NT) {
        const int v = t / n, mm = t - v * n;
        xs[v * 128 + mm] = xin[t];
      }
    } else {
      for (int t = tid; t < nv * n; t += T8_NT) {
        const int v = t / n, mm = t - v * n;
        xs[v * 128 + mm] = a.xb[((size_t)v * a.npts + pt) * n + mm];
      }
    }
    __syncthreads();
    float* meanf = reinterpret_cast<float*>(meanv + 8);  // [v] = {hi, lo}
    for (int v = wid; v < nv; v += T8_NT / 32) {
      double sx = 0.0;
      for (int mm = lane; mm < n; mm += 32) sx += (double)xs[v * 128 + mm];
      const double mean = warp_sum(sx) * inv_n;
      const float mh = (float)mean, ml = (float)(mean - (double)mh);
      double dlt = 0.0;
      for (int mm = lane; mm < n; mm += 32) {
        const float xp = (xs[v * 128 + mm] - mh) - ml;
        xs[v * 128 + mm] = xp;
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
      // thread: member mm, variables vgp, vgp + 2, ... (up to four)
      const int mm = tid & 127, vgp = tid >> 7;
      if (mm < n) {
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 2
        for (int k = 0; k < n; k++) {
          const float w = Wm[k * 128 + mm];
#pragma unroll
          for (int j = 0; j < 4; j++)
            if (vgp + 2 * j < nv) acc[j] = fmaf(xs[(vgp + 2 * j) * 128 + k], w, acc[j]);
        }
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const int v = vgp + 2 * j;
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
    if (tid == 0) {
      tc::fence_after_sync();
      tc::mma_commit(&mbar[4]);
      if (a.err_flag) atomicExch(a.err_flag, 1);
    }
    tc::mbar_wait(&mbar[4], 0u, T8_WAIT);
    if (xb_lost) tc::mbar_wait(&mbar[3], xb_lost & 1u, T8_WAIT);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (wid == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tbase, T8_TMEM_COLS);
  }
}

static std::atomic<uint32_t> g_t8_attr{0};

int prepare_sweep_tc128() { return cuda_status(set_smem_once(sweep_tc128_kernel, T8Layout::TOTAL, g_t8_attr)); }

int launch_sweep_tc128(const SweepArgs& a, cudaStream_t stream, int grid_cap) {
  if (a.n < 2 || a.n > T8_NP || a.nv < 1 || a.nv > 8) return LETKF_ERR_ARG;
  if (a.nwork == 0) return LETKF_OK;
  constexpr size_t bytes = T8Layout::TOTAL;
  cudaError_t err = set_smem_once(sweep_tc128_kernel, bytes, g_t8_attr);
  if (err != cudaSuccess) return cuda_status(err);
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  // one CTA per SM: its shared memory and all 512 TMEM columns
  int grid = nsm;
  if (grid_cap > 0 && grid > grid_cap) grid = grid_cap;
  if (grid_cap < 0) grid = grid / -grid_cap > 0 ? grid / -grid_cap : 1;  // a 1/v share of the resident CTAs
  if (grid > a.nwork) grid = a.nwork;
  sweep_tc128_kernel<<<grid, T8_NT, bytes, stream>>>(a);
  note_launch();
  return cuda_status(cudaGetLastError());
}

}  // namespace letkf
