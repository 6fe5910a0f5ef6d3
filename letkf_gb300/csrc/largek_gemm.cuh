// largek_gemm.cuh -- batched tcgen05 GEMM for the large-ensemble core.
//
// One CTA computes a 128 x 128 tile of one point's product with the
// accumulator in tensor memory (128 columns).  Operands are FP32 in global
// memory and enter the tensor core as three-term TF32 splits
// (x = hi + lo, hi = x with the low 13 mantissa bits cleared):
//   acc = A_hi B_hi + A_hi B_lo + A_lo B_hi        (about 1e-6 relative)
// staged K-major (SWIZZLE_NONE core matrices of 8 rows x 16 bytes) in two
// 32 KB stages (K = 16) so the staging of stage c+1 overlaps the MMAs of
// stage c; 64 KB per CTA lets three CTAs share an SM (384 TMEM columns), so
// one CTA's MMAs also overlap another's global loads.
//
// Modes:
//   LK_GRAM   out = Ywᵀ Y over the point's local rows (K = its L, Yw = w_l y_l):
//             rows of the packed FP32 [nrows][ne] array, or with ridx rows
//             ridx[l] of the observation ensemble (FP32 rows, or BF16 rows16),
//             so that no per-point copies are made however long the list
//   LK_T      out = X Y and e2[b] += ||out - I||²_F   (Newton-Schulz residual)
//   LK_AXPBY  out = alpha X Y + beta D   (alpha, beta per point when alpha_b,
//             beta_b are set;
//             D may be NULL: out = alpha X Y)
// X, Y, D, out are [batch][kp][kp] row-major; B(n, k) = Y[k][n], so no operand
// needs to be symmetric.  Points with active[b] == 0 copy D to out (AXPBY) or
// return (other modes).
#pragma once
#include "letkf_common.cuh"
#include "tc_sm100.cuh"

namespace letkf {

constexpr int LK_NT = 256;
constexpr int LK_TILE = 128;
constexpr int LK_KC = 16;                // K per stage
constexpr int LK_OPER = 8192;            // one 128 x 16 TF32 operand
constexpr int LK_STAGE = 4 * LK_OPER;    // A_hi, A_lo, B_hi, B_lo
constexpr int LK_SMEM = 2 * LK_STAGE + 64;
constexpr uint32_t LK_TMEM_COLS = 128;
constexpr uint32_t LK_WAIT = 1u << 22;

enum { LK_GRAM = 0, LK_T = 1, LK_AXPBY = 2 };

struct LkGemmArgs {
  int kp;                 // padded matrix size (multiple of 128)
  int64_t mstride;        // kp * kp
  const float* X;
  const float* Y;
  const float* D;
  float alpha, beta;
  const float* alpha_b;   // [batch] or NULL
  const float* beta_b;    // [batch] or NULL
  float* out;
  float* e2;              // [batch] (LK_T)
  const int* active;      // [batch] or NULL
  // LK_GRAM
  const float* rows;      // [nrows][ne], or [nobs][ne] with ridx
  const __nv_bfloat16* rows16;  // [nobs][ne] BF16 rows (with ridx; rows is then NULL)
  const int* ridx;        // [nrows] observation of each list entry, or NULL (packed rows)
  const float* wts;       // [nrows] weight of each row (rloc / rdiag)
  const int64_t* offs;    // [batch + 1] rows of point b: offs[b] .. offs[b+1]-1
  int ne;
  int* err_flag;
};

// split 4 values into TF32 hi (low 13 mantissa bits cleared) and remainder
__device__ __forceinline__ void lk_split4(const float (&v)[4], float4& hi, float4& lo) {
  float h[4];
#pragma unroll
  for (int j = 0; j < 4; j++) h[j] = __uint_as_float(__float_as_uint(v[j]) & 0xFFFFE000u);
  hi = make_float4(h[0], h[1], h[2], h[3]);
  lo = make_float4(v[0] - h[0], v[1] - h[1], v[2] - h[2], v[3] - h[3]);
}

__device__ __forceinline__ void lk_store(unsigned char* hi_base, unsigned char* lo_base, int r, int kk,
                                         const float (&v)[4]) {
  float4 h, l;
  lk_split4(v, h, l);
  const uint32_t off = tc::kmajor_off(r, kk, LK_KC);
  *reinterpret_cast<float4*>(hi_base + off) = h;
  *reinterpret_cast<float4*>(lo_base + off) = l;
}

template <int MODE>
__global__ void __launch_bounds__(LK_NT, 3) largek_gemm_kernel(LkGemmArgs a) {
  extern __shared__ __align__(1024) unsigned char sm[];
  uint64_t* mbar = reinterpret_cast<uint64_t*>(sm + 2 * LK_STAGE);
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(sm + 2 * LK_STAGE + 16);
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int b = blockIdx.z;
  const int m0 = blockIdx.y * LK_TILE, n0 = blockIdx.x * LK_TILE;
  const int kp = a.kp;
  const size_t mo = (size_t)b * a.mstride;
  const bool act = a.active == nullptr || a.active[b] != 0;
  if (!act) {
    if (MODE == LK_AXPBY && a.D) {  // keep the converged state in the output buffer
      for (int t = tid; t < LK_TILE * LK_TILE / 4; t += LK_NT) {
        const int r = t / (LK_TILE / 4), c4 = t % (LK_TILE / 4);
        const size_t idx = mo + (size_t)(m0 + r) * kp + n0 + 4 * c4;
        *reinterpret_cast<float4*>(a.out + idx) = *reinterpret_cast<const float4*>(a.D + idx);
      }
    }
    return;
  }
  int nk;
  int64_t r0 = 0;
  int L = 0;
  if (MODE == LK_GRAM) {
    r0 = a.offs[b];
    L = (int)(a.offs[b + 1] - r0);
    nk = (L + LK_KC - 1) / LK_KC;
  } else {
    nk = kp / LK_KC;
  }
  if (tid == 0) {
    tc::mbar_init(&mbar[0], 1);
    tc::mbar_init(&mbar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (wid == 0) tc::tmem_alloc(tmem_holder, LK_TMEM_COLS);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tacc = *tmem_holder;
  const uint32_t sbase = tc::smem_u32(sm);
  const uint32_t idesc = tc::idesc_tf32(128, 128);
  // phase parities and stages with MMAs in flight as bit masks (bit = stage
  // buffer): the buffer index is known only at run time, and arrays indexed by
  // it would live in local memory
  uint32_t par = 0u, outst = 0u;
  int tmo = 0;
  const int r = tid & 127, h = tid >> 7;  // staging: row r, K half h (8 values)

  // stage values of this thread: rows r of A and B, K half h (8 values each);
  // the next stage's loads are issued before this stage is split and stored,
  // so their latency overlaps the staging, the barrier and the MMA issue
  float va[8], vb[8];
  auto load_stage = [&](int c, float (&xa)[8], float (&xb)[8]) {
    const int k0 = c * LK_KC + h * 8;
    if (MODE == LK_GRAM) {
      // A(m, l) = w_l y_l[m], B(n, l) = y_l[n]; rows beyond L or members beyond ne are 0
#pragma unroll
      for (int j = 0; j < 8; j++) {
        const int l = k0 + j;
        float ya = 0.f, yb = 0.f;
        if (l < L) {
          const size_t ri = a.ridx ? (size_t)a.ridx[r0 + l] : (size_t)(r0 + l);
          const float w = a.wts[r0 + l];
          if (a.rows16) {
            const __nv_bfloat16* row = a.rows16 + ri * a.ne;
            if (m0 + r < a.ne) ya = w * __bfloat162float(row[m0 + r]);
            if (n0 + r < a.ne) yb = __bfloat162float(row[n0 + r]);
          } else {
            const float* row = a.rows + ri * a.ne;
            if (m0 + r < a.ne) ya = w * row[m0 + r];
            if (n0 + r < a.ne) yb = row[n0 + r];
          }
        }
        xa[j] = ya;
        xb[j] = yb;
      }
    } else {
      const float4 x0 = *reinterpret_cast<const float4*>(a.X + mo + (size_t)(m0 + r) * kp + k0);
      const float4 x1 = *reinterpret_cast<const float4*>(a.X + mo + (size_t)(m0 + r) * kp + k0 + 4);
      xa[0] = x0.x;
      xa[1] = x0.y;
      xa[2] = x0.z;
      xa[3] = x0.w;
      xa[4] = x1.x;
      xa[5] = x1.y;
      xa[6] = x1.z;
      xa[7] = x1.w;
#pragma unroll
      for (int j = 0; j < 8; j++) xb[j] = a.Y[mo + (size_t)(k0 + j) * kp + n0 + r];
    }
  };
  if (nk > 0) load_stage(0, va, vb);

  for (int c = 0; c < nk; c++) {
    const int buf = c & 1;
    float ca[8], cb[8];
#pragma unroll
    for (int j = 0; j < 8; j++) {
      ca[j] = va[j];
      cb[j] = vb[j];
    }
    if (c + 1 < nk) load_stage(c + 1, va, vb);
    if ((outst >> buf) & 1u) {
      if (!tc::mbar_wait(&mbar[buf], (par >> buf) & 1u, LK_WAIT)) tmo = 1;
      par ^= 1u << buf;
      outst &= ~(1u << buf);
    }
    tc::fence_after_sync();
    unsigned char* st = sm + buf * LK_STAGE;
#pragma unroll
    for (int g = 0; g < 2; g++) {
      const int kk = h * 8 + g * 4;
      const float qa[4] = {ca[4 * g], ca[4 * g + 1], ca[4 * g + 2], ca[4 * g + 3]};
      const float qb[4] = {cb[4 * g], cb[4 * g + 1], cb[4 * g + 2], cb[4 * g + 3]};
      lk_store(st, st + LK_OPER, r, kk, qa);
      lk_store(st + 2 * LK_OPER, st + 3 * LK_OPER, r, kk, qb);
    }
    tc::fence_smem_async();
    tc::fence_before_sync();
    if (__syncthreads_or(tmo)) {  // a bounded wait gave up: issue nothing more
      tmo = 1;
      break;
    }
    if (tid == 0) {
      tc::fence_after_sync();
      const uint32_t s0 = sbase + buf * LK_STAGE;
#pragma unroll
      for (int pass = 0; pass < 3; pass++) {
        const uint32_t sa = s0 + (pass == 2 ? LK_OPER : 0);
        const uint32_t sb = s0 + 2 * LK_OPER + (pass == 1 ? LK_OPER : 0);
#pragma unroll
        for (int s = 0; s < LK_KC / 8; s++)
          tc::mma_tf32(tacc, tc::smem_desc(sa + s * 256, 128, LK_KC * 32), tc::smem_desc(sb + s * 256, 128, LK_KC * 32),
                       idesc, (c == 0 && pass == 0 && s == 0) ? 0u : 1u);
      }
      tc::mma_commit(&mbar[buf]);
    }
    outst |= 1u << buf;
  }
  for (int q = 0; q < 2; q++)
    if ((outst >> q) & 1u) {
      if (!tc::mbar_wait(&mbar[q], (par >> q) & 1u, LK_WAIT)) tmo = 1;
      par ^= 1u << q;
      outst &= ~(1u << q);
    }
  tc::fence_after_sync();
  const bool bad = __syncthreads_or(tmo) != 0;
  if (bad) {
    if (tid == 0 && a.err_flag) atomicExch(a.err_flag, 1);
  } else {
    // epilogue: warp w reads TMEM lanes 32 (w % 4) .. +31 (rows), columns 64 (w / 4) .. +63
    const int row = 32 * (wid & 3) + lane;
    const int cb = 64 * (wid >> 2);
    const uint32_t taddr = tacc + ((uint32_t)(32 * (wid & 3)) << 16) + (uint32_t)cb;
    float e2 = 0.f;
    const size_t orow = mo + (size_t)(m0 + row) * kp + n0 + cb;
#pragma unroll 1
    for (int c0 = 0; c0 < 64; c0 += 16) {
      float v[16];
      if (nk > 0) {
        tc::tmem_ld16(taddr + c0, v);
      } else {
#pragma unroll
        for (int j = 0; j < 16; j++) v[j] = 0.f;
      }
      float* dst = a.out + orow + c0;
      if (MODE == LK_AXPBY) {
        const float al = a.alpha_b ? a.alpha_b[b] : a.alpha;
        const float be = a.beta_b ? a.beta_b[b] : a.beta;
        if (a.D) {
          const float* dd = a.D + orow + c0;
#pragma unroll
          for (int j = 0; j < 16; j += 4) {
            const float4 d4 = *reinterpret_cast<const float4*>(dd + j);
            *reinterpret_cast<float4*>(dst + j) =
                make_float4(al * v[j] + be * d4.x, al * v[j + 1] + be * d4.y, al * v[j + 2] + be * d4.z,
                            al * v[j + 3] + be * d4.w);
          }
        } else {
#pragma unroll
          for (int j = 0; j < 16; j += 4)
            *reinterpret_cast<float4*>(dst + j) = make_float4(al * v[j], al * v[j + 1], al * v[j + 2], al * v[j + 3]);
        }
      } else {
        if (MODE == LK_T) {
#pragma unroll
          for (int j = 0; j < 16; j++) {
            const float dl = v[j] - ((m0 + row == n0 + cb + c0 + j) ? 1.f : 0.f);
            e2 = fmaf(dl, dl, e2);
          }
        }
#pragma unroll
        for (int j = 0; j < 16; j += 4)
          *reinterpret_cast<float4*>(dst + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
      }
    }
    if (MODE == LK_T) {
      e2 = warp_sum(e2);
      if (lane == 0) atomicAdd(&a.e2[b], e2);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (wid == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tacc, LK_TMEM_COLS);
  }
}

}  // namespace letkf
