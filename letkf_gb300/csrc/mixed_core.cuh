// mixed_core.cuh -- FP32 building blocks of the mixed-precision LETKF core.
//
// The k x k problem is padded to NP (32, 64 or 128) with zero perturbations,
// so the padded block of A = Yb^T R^-1 Yb + (k-1)/rho I is c*I and decouples
// from the real block: its eigenvectors have no components in rows < k and
// drop out of W and wbar.
//
//   gram_*     register-tiled FP32 accumulation of Yb^T diag(w) Yb, the
//              departure product Yb^T diag(w) dep and the inflation sums
//              (common/common_letkf.f90:101-118, 218-233)
//   jacobi_*   parallel cyclic Jacobi eigensolver (round-robin pairing, NP/2
//              disjoint rotations per round) replacing mtx_eigen / EISPACK rs
//              (common/common_mtx.f90:41-99)
//   form_w     W = V diag(sqrt((k-1)/lambda)) V^T and wbar = V diag(1/lambda) V^T b
//              (common/common_letkf.f90:146-193)
#pragma once
#include "letkf_common.cuh"

namespace letkf {

template <int NP>
struct MixedCfg;
template <>
struct MixedCfg<32> {
  static constexpr int NT = 64, TR = 4, TC = 4, CH = 32, MINB = 6;
};
template <>
struct MixedCfg<64> {
  static constexpr int NT = 128, TR = 8, TC = 4, CH = 32, MINB = 4;
};
template <>
struct MixedCfg<128> {
  static constexpr int NT = 256, TR = 8, TC = 8, CH = 16, MINB = 1;
};

// Shared-memory layout (floats) of one point's mixed core.
template <int NP>
struct MixedSmem {
  static constexpr int CH = MixedCfg<NP>::CH;
  static constexpr int NBLK = (NP / 2) * (NP / 2 + 1) / 2;  // upper 2x2 blocks incl. diagonal
  // Y / YW (staged rows, Gram phase only) share V's space when they fit
  static constexpr bool ALIAS = 2 * CH * NP <= NP * NP;
  static constexpr int A = 0;                       // NP*NP row-major work matrix
  static constexpr int V = A + NP * NP;             // NP*NP eigenvectors, column-major V[q*NP+i]
  static constexpr int Y = ALIAS ? V : V + NP * NP; // CH*NP staged rows
  static constexpr int YW = Y + CH * NP;            // CH*NP weighted rows
  static constexpr int B = ALIAS ? V + NP * NP : YW + CH * NP;  // NP departure product
  static constexpr int LAM = B + NP;                // NP  eigenvalues
  static constexpr int FQ = LAM + NP;               // NP  sqrt((k-1)/lambda)
  static constexpr int IQ = FQ + NP;                // NP  1/lambda
  static constexpr int G = IQ + NP;                 // NP  scratch vector
  static constexpr int WB = G + NP;                 // NP  wbar
  static constexpr int ROT = WB + NP;               // 2*(NP/2) rotation c, s
  static constexpr int PAIR = ROT + NP;             // NP/2 packed (p | q<<8) as int
  static constexpr int BLK = PAIR + NP / 2;         // NBLK packed (s1 | s2<<8) as int
  static constexpr int WR = BLK + NBLK;             // CH weights
  static constexpr int DR = WR + CH;                // CH departures
  static constexpr int RL = DR + CH;                // CH rloc
  static constexpr int RED = RL + CH;               // 64 reduction scratch
  static constexpr int TOTAL = RED + 64;
  static constexpr size_t BYTES = sizeof(float) * (size_t)TOTAL;
};

// Thread-owned Gram tile accumulators.
template <int NP>
struct GramAcc {
  static constexpr int TR = MixedCfg<NP>::TR, TC = MixedCfg<NP>::TC;
  float a[TR][TC];
  float bacc;
  float p1, p3;  // per-thread partial inflation sums; block totals after gram_finish
  __device__ void zero() {
#pragma unroll
    for (int r = 0; r < TR; r++)
#pragma unroll
      for (int c = 0; c < TC; c++) a[r][c] = 0.f;
    bacc = 0.f;
    p1 = 0.f;
    p3 = 0.f;
  }
};

// Accumulate nr staged rows (sm[Y], sm[YW], sm[WR], sm[DR], sm[RL]) into acc.
template <int NP>
__device__ __forceinline__ void gram_chunk(const float* sm, int nr, GramAcc<NP>& acc) {
  using C = MixedCfg<NP>;
  using S = MixedSmem<NP>;
  constexpr int NTI = NP / C::TR;
  const int tid = threadIdx.x;
  const int i0 = (tid % NTI) * C::TR, j0 = (tid / NTI) * C::TC;
  const float* yw = sm + S::YW;
  const float* y = sm + S::Y;
  for (int r = 0; r < nr; r++) {
    float av[C::TR], bv[C::TC];
#pragma unroll
    for (int q = 0; q < C::TR; q += 4) {
      float4 t = *reinterpret_cast<const float4*>(yw + r * NP + i0 + q);
      av[q] = t.x;
      av[q + 1] = t.y;
      av[q + 2] = t.z;
      av[q + 3] = t.w;
    }
#pragma unroll
    for (int q = 0; q < C::TC; q += 4) {
      float4 t = *reinterpret_cast<const float4*>(y + r * NP + j0 + q);
      bv[q] = t.x;
      bv[q + 1] = t.y;
      bv[q + 2] = t.z;
      bv[q + 3] = t.w;
    }
#pragma unroll
    for (int a = 0; a < C::TR; a++)
#pragma unroll
      for (int b = 0; b < C::TC; b++) acc.a[a][b] = fmaf(av[a], bv[b], acc.a[a][b]);
  }
  if (tid < NP) {
    float s = acc.bacc;
    for (int r = 0; r < nr; r++) s = fmaf(yw[r * NP + tid], sm[S::DR + r], s);
    acc.bacc = s;
  }
  if (tid < nr) {  // one staged row per thread (CH <= NT)
    const float dd = sm[S::DR + tid];
    acc.p1 = fmaf(dd * dd, sm[S::WR + tid], acc.p1);
    acc.p3 += sm[S::RL + tid];
  }
}

// Write the Gram tiles into sm[A] (symmetrised from the lower triangle), the
// departure product into sm[B], reduce the inflation sums into acc.p1 / acc.p3
// of every thread, and return trace(Gram) in FP64 (all threads).
template <int NP>
__device__ __forceinline__ double gram_finish(float* sm, GramAcc<NP>& acc) {
  using C = MixedCfg<NP>;
  using S = MixedSmem<NP>;
  constexpr int NTI = NP / C::TR;
  const int tid = threadIdx.x;
  const int i0 = (tid % NTI) * C::TR, j0 = (tid / NTI) * C::TC;
  float* A = sm + S::A;
  __syncthreads();
#pragma unroll
  for (int a = 0; a < C::TR; a++)
#pragma unroll
    for (int b = 0; b < C::TC; b++) A[(i0 + a) * NP + j0 + b] = acc.a[a][b];
  if (tid < NP) sm[S::B + tid] = acc.bacc;
  __syncthreads();
  // mirror the lower triangle onto the upper one, walking the pairs along
  // diagonals (i, i + d mod NP), d = 1..NP/2, so a warp's lanes read and write
  // distinct banks (a row walk reads the mirror at an NP-float stride)
  for (int t = tid; t < (NP / 2) * NP; t += C::NT) {
    const int d = 1 + t / NP, i = t - (d - 1) * NP;
    if (d == NP / 2 && i >= NP / 2) continue;
    const int j = (i + d) & (NP - 1);
    const int lo = i < j ? i : j, hi = i < j ? j : i;
    A[lo * NP + hi] = A[hi * NP + lo];
  }
  float tr = 0.f;
  for (int i = tid; i < NP; i += C::NT) tr += A[i * NP + i];
  float* red = sm + S::RED;
  const float trace = block_sum<float, C::NT>(tr, red);
  acc.p1 = block_sum<float, C::NT>(acc.p1, red);
  acc.p3 = block_sum<float, C::NT>(acc.p3, red);
  return (double)trace;
}

// Parallel cyclic Jacobi on sm[A] (symmetric, NP x NP), eigenvectors into
// sm[V] (column-major), eigenvalues into sm[LAM].  Returns the sweeps used.
template <int NP>
__device__ int jacobi_eig(float* sm, int max_sweeps) {
  using C = MixedCfg<NP>;
  using S = MixedSmem<NP>;
  constexpr int HP = NP / 2;
  const int tid = threadIdx.x;
  float* A = sm + S::A;
  float* V = sm + S::V;
  float* rot = sm + S::ROT;
  int* pair = reinterpret_cast<int*>(sm + S::PAIR);
  int* blk = reinterpret_cast<int*>(sm + S::BLK);
  // identity V; block table (upper triangle of the pair grid)
  for (int idx = tid; idx < NP * NP; idx += C::NT) V[idx] = (idx / NP == idx % NP) ? 1.f : 0.f;
  for (int b = tid; b < S::NBLK; b += C::NT) {
    // invert b -> (s1 <= s2) over rows s1 = 0..HP-1
    int s1 = 0, rem = b;
    while (rem >= HP - s1) {
      rem -= HP - s1;
      s1++;
    }
    blk[b] = s1 | ((s1 + rem) << 8);
  }
  __syncthreads();
  int sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    // convergence: every |a_ij| <= eps * sqrt(|a_ii a_jj|)
    int bad = 0;
    for (int idx = tid; idx < NP * NP; idx += C::NT) {
      const int i = idx / NP, j = idx - i * NP;
      if (i < j) {
        const float aij = fabsf(A[idx]);
        const float thr = 1.0e-7f * sqrtf(fabsf(A[i * NP + i]) * fabsf(A[j * NP + j]));
        bad |= (aij > thr);
      }
    }
    if (!__syncthreads_or(bad)) break;
    for (int r = 0; r < NP - 1; ++r) {
      if (tid < HP) {
        int p, q;
        if (tid == 0) {
          p = r;
          q = NP - 1;
        } else {
          p = (r + tid) % (NP - 1);
          q = (r - tid + NP - 1) % (NP - 1);
        }
        const float app = A[p * NP + p], aqq = A[q * NP + q], apq = A[p * NP + q];
        float c = 1.f, s = 0.f;
        if (apq != 0.f) {
          const float theta = (aqq - app) / (2.f * apq);
          const float t = copysignf(1.f, theta) / (fabsf(theta) + sqrtf(fmaf(theta, theta, 1.f)));
          c = rsqrtf(fmaf(t, t, 1.f));
          s = t * c;
        }
        rot[2 * tid] = c;
        rot[2 * tid + 1] = s;
        pair[tid] = p | (q << 8);
      }
      __syncthreads();
      // A <- J^T A J on 2x2 blocks (s1 <= s2), mirrored
      for (int b = tid; b < S::NBLK; b += C::NT) {
        const int code = blk[b];
        const int s1 = code & 0xff, s2 = code >> 8;
        const int pq1 = pair[s1], pq2 = pair[s2];
        const int p1 = pq1 & 0xff, q1 = pq1 >> 8, p2 = pq2 & 0xff, q2 = pq2 >> 8;
        const float c1 = rot[2 * s1], sn1 = rot[2 * s1 + 1];
        if (s1 == s2) {
          const float app = A[p1 * NP + p1], aqq = A[q1 * NP + q1], apq = A[p1 * NP + q1];
          const float t = (c1 != 0.f) ? sn1 / c1 : 0.f;
          A[p1 * NP + p1] = app - t * apq;
          A[q1 * NP + q1] = aqq + t * apq;
          A[p1 * NP + q1] = 0.f;
          A[q1 * NP + p1] = 0.f;
        } else {
          const float c2 = rot[2 * s2], sn2 = rot[2 * s2 + 1];
          const float x00 = A[p1 * NP + p2], x01 = A[p1 * NP + q2];
          const float x10 = A[q1 * NP + p2], x11 = A[q1 * NP + q2];
          const float y00 = c2 * x00 - sn2 * x01, y01 = sn2 * x00 + c2 * x01;
          const float y10 = c2 * x10 - sn2 * x11, y11 = sn2 * x10 + c2 * x11;
          const float z00 = c1 * y00 - sn1 * y10, z01 = c1 * y01 - sn1 * y11;
          const float z10 = sn1 * y00 + c1 * y10, z11 = sn1 * y01 + c1 * y11;
          A[p1 * NP + p2] = z00;
          A[p1 * NP + q2] = z01;
          A[q1 * NP + p2] = z10;
          A[q1 * NP + q2] = z11;
          A[p2 * NP + p1] = z00;
          A[q2 * NP + p1] = z01;
          A[p2 * NP + q1] = z10;
          A[q2 * NP + q1] = z11;
        }
      }
      // V <- V J (columns p, q)
      for (int e = tid; e < NP * HP; e += C::NT) {
        const int i = e % NP, s = e / NP;
        const int pq = pair[s];
        const int p = pq & 0xff, q = pq >> 8;
        const float c = rot[2 * s], sn = rot[2 * s + 1];
        const float vp = V[p * NP + i], vq = V[q * NP + i];
        V[p * NP + i] = c * vp - sn * vq;
        V[q * NP + i] = sn * vp + c * vq;
      }
      __syncthreads();
    }
  }
  for (int i = tid; i < NP; i += C::NT) sm[S::LAM + i] = A[i * NP + i];
  __syncthreads();
  return sweep;
}

// ---------------------------------------------------------------------------
// Newton-Schulz inverse square root (GEMM-only replacement of the eigensolve
// for the fused sweep).  A = Gram + c I is SPD with every eigenvalue >= c, so
// with s >= lambda_max / 2 the coupled iteration
//   T = Z Y,  Y <- Y (3I - T) / 2,  Z <- (3I - T) Z / 2,   Y0 = A / s, Z0 = I
// converges to Y = (A/s)^(1/2), Z = (A/s)^(-1/2).  Then
//   W    = sqrt((k-1)/s) Z          = sqrt((k-1) Pa)     (common_letkf.f90:186-193)
//   wbar = Z (Z b) / s              = Pa hdxb_rinv^T dep (:146-182)
// All iterates are polynomials in A, hence symmetric and commuting, so every
// product reads its left factor by rows of the symmetric storage.
// ---------------------------------------------------------------------------
template <int NP>
struct NSSmem {
  using S = MixedSmem<NP>;
  static constexpr int T = S::TOTAL;          // NP*NP product T = Z Y
  static constexpr int TOTAL = T + NP * NP;
};

// acc = X Yb for this thread's TR x TC tile (X, Yb symmetric, row-major, ld NP)
template <int NP>
__device__ __forceinline__ void sym_gemm_tile(const float* X, const float* Yb, int i0, int j0,
                                              float (&acc)[MixedCfg<NP>::TR][MixedCfg<NP>::TC]) {
  using C = MixedCfg<NP>;
#pragma unroll
  for (int a = 0; a < C::TR; a++)
#pragma unroll
    for (int b = 0; b < C::TC; b++) acc[a][b] = 0.f;
#pragma unroll 4
  for (int k = 0; k < NP; k++) {
    float av[C::TR], bv[C::TC];
#pragma unroll
    for (int t = 0; t < C::TR; t += 4) {
      const float4 x = *reinterpret_cast<const float4*>(X + k * NP + i0 + t);
      av[t] = x.x;
      av[t + 1] = x.y;
      av[t + 2] = x.z;
      av[t + 3] = x.w;
    }
#pragma unroll
    for (int t = 0; t < C::TC; t += 4) {
      const float4 y = *reinterpret_cast<const float4*>(Yb + k * NP + j0 + t);
      bv[t] = y.x;
      bv[t + 1] = y.y;
      bv[t + 2] = y.z;
      bv[t + 3] = y.w;
    }
#pragma unroll
    for (int a = 0; a < C::TR; a++)
#pragma unroll
      for (int b = 0; b < C::TC; b++) acc[a][b] = fmaf(av[a], bv[b], acc[a][b]);
  }
}

// Coupled Newton-Schulz iterations in FP32 on row-major symmetric Y, Z with
// scratch T (NP x NP each), until ||ZY - I||_F < 1e-4 plus one more step (the
// quadratic convergence then reaches the FP32 floor) or max_iter.  Returns the
// iterations done; Y, Z hold the last iterate.
template <int NP>
__device__ int ns_iterate(float* Y, float* Z, float* T, float* redf, int max_iter, float lo = -1.f,
                           bool* conv = nullptr) {
  // lo >= 0: the spectrum of ZY starts in [lo, 1] and every step is
  // spectrum-scaled (Y' = sqrt(a) Y (3I - aT) / 2, likewise Z; see ns_scale);
  // lo < 0: plain steps
  using C = MixedCfg<NP>;
  constexpr int NTI = NP / C::TR;
  const int tid = threadIdx.x;
  const int i0 = (tid % NTI) * C::TR, j0 = (tid / NTI) * C::TC;
  float acc[C::TR][C::TC];
  int it = 0;
  bool last = false;
  for (; it < max_iter; it++) {
    // T = Z Y and ||T - I||_F^2
    sym_gemm_tile<NP>(Z, Y, i0, j0, acc);
    float e2 = 0.f;
#pragma unroll
    for (int a = 0; a < C::TR; a++)
#pragma unroll
      for (int b = 0; b < C::TC; b++) {
        T[(i0 + a) * NP + j0 + b] = acc[a][b];
        const float d = acc[a][b] - ((i0 + a) == (j0 + b) ? 1.f : 0.f);
        e2 = fmaf(d, d, e2);
      }
    e2 = block_sum<float, C::NT>(e2, redf);  // also publishes T
    if (e2 < 1.0e-8f) last = true;
    float ka = 1.5f, kb = 0.5f;
    if (lo >= 0.f) {
      const float al = ns_scale(lo);
      const float sa = sqrtf(al);
      ka = 1.5f * sa;
      kb = 0.5f * al * sa;
      lo = f_ns(al * lo);
    }
    // Y' = ka Y - kb Y T ; Z' = ka Z - kb T Z
    float ynew[C::TR][C::TC];
    sym_gemm_tile<NP>(Y, T, i0, j0, acc);
#pragma unroll
    for (int a = 0; a < C::TR; a++)
#pragma unroll
      for (int b = 0; b < C::TC; b++) ynew[a][b] = ka * Y[(i0 + a) * NP + j0 + b] - kb * acc[a][b];
    sym_gemm_tile<NP>(T, Z, i0, j0, acc);
#pragma unroll
    for (int a = 0; a < C::TR; a++)
#pragma unroll
      for (int b = 0; b < C::TC; b++) acc[a][b] = ka * Z[(i0 + a) * NP + j0 + b] - kb * acc[a][b];
    __syncthreads();
#pragma unroll
    for (int a = 0; a < C::TR; a++)
#pragma unroll
      for (int b = 0; b < C::TC; b++) {
        Y[(i0 + a) * NP + j0 + b] = ynew[a][b];
        Z[(i0 + a) * NP + j0 + b] = acc[a][b];
      }
    __syncthreads();
    if (last) {
      it++;
      break;
    }
  }
  if (conv) *conv = last;  // uniform: e2 is a block sum
  return it;
}

// Uncoupled Newton-Schulz refinement of Z ~ As^(-1/2) for symmetric As:
//   P = As Z, Q = Z P (= Z As Z, symmetric), Z <- 1.5 Z - 0.5 Q Z, then Z is
// symmetrised.  Stops after the step following ||Q - I||_F < 1e-4 or after
// max_iter; returns the iterations done.  P is scratch (NP x NP).
template <int NP>
__device__ int ns_polish(const float* As, float* Z, float* P, float* redf, int max_iter, float tol = 1.0e-8f,
                         bool* conv = nullptr) {
  using C = MixedCfg<NP>;
  constexpr int NTI = NP / C::TR;
  const int tid = threadIdx.x;
  const int i0 = (tid % NTI) * C::TR, j0 = (tid / NTI) * C::TC;
  float acc[C::TR][C::TC];
  int it = 0;
  bool last = false;
  for (; it < max_iter; it++) {
    sym_gemm_tile<NP>(As, Z, i0, j0, acc);  // As Z
#pragma unroll
    for (int a = 0; a < C::TR; a++)
#pragma unroll
      for (int b = 0; b < C::TC; b++) P[(i0 + a) * NP + j0 + b] = acc[a][b];
    __syncthreads();
    sym_gemm_tile<NP>(Z, P, i0, j0, acc);   // Z^T (As Z)
    float e2 = 0.f;
#pragma unroll
    for (int a = 0; a < C::TR; a++)
#pragma unroll
      for (int b = 0; b < C::TC; b++) {
        const float d = acc[a][b] - ((i0 + a) == (j0 + b) ? 1.f : 0.f);
        e2 = fmaf(d, d, e2);
      }
    __syncthreads();
#pragma unroll
    for (int a = 0; a < C::TR; a++)
#pragma unroll
      for (int b = 0; b < C::TC; b++) P[(i0 + a) * NP + j0 + b] = acc[a][b];
    e2 = block_sum<float, C::NT>(e2, redf);  // also publishes Q
    if (e2 < tol) last = true;
    sym_gemm_tile<NP>(P, Z, i0, j0, acc);   // Q Z
#pragma unroll
    for (int a = 0; a < C::TR; a++)
#pragma unroll
      for (int b = 0; b < C::TC; b++) acc[a][b] = 1.5f * Z[(i0 + a) * NP + j0 + b] - 0.5f * acc[a][b];
    __syncthreads();
#pragma unroll
    for (int a = 0; a < C::TR; a++)
#pragma unroll
      for (int b = 0; b < C::TC; b++) Z[(i0 + a) * NP + j0 + b] = acc[a][b];
    __syncthreads();
    // symmetrise: the mirror of this thread's tile is TC rows of TR contiguous
    // values (float4 reads, no bank conflicts); Z <- (Z + Z^T) / 2
    float mir[C::TR][C::TC];
#pragma unroll
    for (int b = 0; b < C::TC; b++)
#pragma unroll
      for (int t = 0; t < C::TR; t += 4) {
        const float4 x = *reinterpret_cast<const float4*>(Z + (j0 + b) * NP + i0 + t);
        mir[t][b] = x.x;
        mir[t + 1][b] = x.y;
        mir[t + 2][b] = x.z;
        mir[t + 3][b] = x.w;
      }
    __syncthreads();
#pragma unroll
    for (int a = 0; a < C::TR; a++)
#pragma unroll
      for (int b = 0; b < C::TC; b++) Z[(i0 + a) * NP + j0 + b] = 0.5f * (acc[a][b] + mir[a][b]);
    __syncthreads();
    if (last) {
      it++;
      break;
    }
  }
  if (conv) *conv = last;
  return it;
}

// Newton-Schulz on sm[A] (SPD, all eigenvalues >= cdiag > 0).  Leaves
// Z = (A/s)^(-1/2) in sm[V] (row-major, symmetric), scratch in sm[NS::T], and
// returns s (> 0); *iters gets the iterations used.  *ok (may be NULL) tells
// whether Z is good: false when the spectrum bound s / cdiag is not below
// cond_max (> 0; A is then left untouched) or when the iteration did not
// converge within max_iter (A is then overwritten).  Either way the caller
// needs the eigensolver for this point.
template <int NP>
__device__ float ns_invsqrt(float* sm, float cdiag, int max_iter, int* iters, float cond_max = 0.f,
                            bool* ok = nullptr) {
  using C = MixedCfg<NP>;
  using S = MixedSmem<NP>;
  using N = NSSmem<NP>;
  constexpr int NTI = NP / C::TR;
  const int tid = threadIdx.x;
  float* A = sm + S::A;
  float* Z = sm + S::V;
  float* T = sm + N::T;
  float* redf = sm + S::RED;
  // s = min(Gershgorin, ||A||_F) >= lambda_max, so the spectrum of A/s lies in
  // [c/s, 1] and every Newton-Schulz step can be spectrum-scaled.  A is
  // symmetric: row i is read as column i (consecutive lanes, no bank conflicts).
  float g = 0.f, f2 = 0.f;
  if (tid < NP) {
    float s = 0.f, q = 0.f;
    for (int j = 0; j < NP; j++) {
      const float x = A[j * NP + tid];
      s += fabsf(x);
      q = fmaf(x, x, q);
    }
    g = s;
    f2 = q;
  }
  g = warp_max(g);
  __syncthreads();
  if ((tid & 31) == 0) redf[tid >> 5] = g;
  __syncthreads();
  float gmax = redf[0];
  for (int w = 1; w < C::NT / 32; w++) gmax = fmaxf(gmax, redf[w]);
  __syncthreads();
  const float fro = sqrtf(block_sum<float, C::NT>(f2, redf));
  const float s = fminf(gmax, fro);
  if (cond_max > 0.f && !(s < cond_max * cdiag)) {
    if (iters) *iters = 0;
    if (ok) *ok = false;
    return s;
  }
  const float inv_s = 1.f / s;
  // Y0 = A/s (in place), Z0 = I
  for (int idx = tid; idx < NP * NP; idx += C::NT) {
    A[idx] *= inv_s;
    Z[idx] = (idx / NP == idx % NP) ? 1.f : 0.f;
  }
  __syncthreads();
  bool conv = false;
  const int it = ns_iterate<NP>(A, Z, T, redf, max_iter, 0.9f * cdiag * inv_s, &conv);
  if (iters) *iters = it;
  if (ok) *ok = conv;
  return s;
}

// From sm[V], sm[LAM], sm[B]: fq, 1/lambda, wbar into sm[FQ], sm[IQ], sm[WB];
// returns 0 ok, LETKF_ERR_EIG when all eigenvalues are <= 0.
template <int NP>
__device__ int eig_postprocess(float* sm, int n) {
  using C = MixedCfg<NP>;
  using S = MixedSmem<NP>;
  const int tid = threadIdx.x;
  float* V = sm + S::V;
  float lmax = -INFINITY;
  for (int i = tid; i < NP; i += C::NT) lmax = fmaxf(lmax, sm[S::LAM + i]);
  lmax = warp_max(lmax);
  float* redf = sm + S::RED;
  __syncthreads();
  if ((tid & 31) == 0) redf[tid >> 5] = lmax;
  __syncthreads();
  lmax = redf[0];
  for (int w = 1; w < C::NT / 32; w++) lmax = fmaxf(lmax, redf[w]);
  if (!(lmax > 0.f)) return LETKF_ERR_EIG;
  const float thr = fabsf(lmax) * 1.4901161193847656e-08f;
  for (int q = tid; q < NP; q += C::NT) {
    const float lam = sm[S::LAM + q];
    const bool keep = !(lam < thr);
    sm[S::FQ + q] = keep ? sqrtf((float)(n - 1) / lam) : 0.f;
    sm[S::IQ + q] = keep ? 1.f / lam : 0.f;
  }
  __syncthreads();
  for (int q = tid; q < NP; q += C::NT) {
    float acc = 0.f;
    for (int i = 0; i < NP; i++) acc = fmaf(V[q * NP + i], sm[S::B + i], acc);
    sm[S::G + q] = acc * sm[S::IQ + q];
  }
  __syncthreads();
  for (int i = tid; i < NP; i += C::NT) {
    float acc = 0.f;
    for (int q = 0; q < NP; q++) acc = fmaf(V[q * NP + i], sm[S::G + q], acc);
    sm[S::WB + i] = acc;
  }
  __syncthreads();
  return LETKF_OK;
}

// W tile of this thread: W[i][j] = sum_q V[q][i] fq[q] V[q][j].  Uses sm[A] as
// scratch for Vf = V * fq.  out(i, j) is called for every i, j < NP.
template <int NP, typename Out>
__device__ __forceinline__ void form_w(float* sm, Out out) {
  using C = MixedCfg<NP>;
  using S = MixedSmem<NP>;
  constexpr int NTI = NP / C::TR;
  const int tid = threadIdx.x;
  float* Vf = sm + S::A;
  const float* V = sm + S::V;
  for (int idx = tid; idx < NP * NP; idx += C::NT) Vf[idx] = V[idx] * sm[S::FQ + idx / NP];
  __syncthreads();
  const int i0 = (tid % NTI) * C::TR, j0 = (tid / NTI) * C::TC;
  float acc[C::TR][C::TC];
#pragma unroll
  for (int a = 0; a < C::TR; a++)
#pragma unroll
    for (int b = 0; b < C::TC; b++) acc[a][b] = 0.f;
  for (int q = 0; q < NP; q++) {
    float av[C::TR], bv[C::TC];
#pragma unroll
    for (int t = 0; t < C::TR; t += 4) {
      float4 x = *reinterpret_cast<const float4*>(Vf + q * NP + i0 + t);
      av[t] = x.x;
      av[t + 1] = x.y;
      av[t + 2] = x.z;
      av[t + 3] = x.w;
    }
#pragma unroll
    for (int t = 0; t < C::TC; t += 4) {
      float4 x = *reinterpret_cast<const float4*>(V + q * NP + j0 + t);
      bv[t] = x.x;
      bv[t + 1] = x.y;
      bv[t + 2] = x.z;
      bv[t + 3] = x.w;
    }
#pragma unroll
    for (int a = 0; a < C::TR; a++)
#pragma unroll
      for (int b = 0; b < C::TC; b++) acc[a][b] = fmaf(av[a], bv[b], acc[a][b]);
  }
#pragma unroll
  for (int a = 0; a < C::TR; a++)
#pragma unroll
    for (int b = 0; b < C::TC; b++) out(i0 + a, j0 + b, acc[a][b]);
}

// Adaptive inflation (common/common_letkf.f90:218-239) from FP64 sums.
// component j of the fixed probe vector of the transform certificates: a
// multiplicative hash of j mapped to [-1, 1), so the vector has weight in
// every eigen-direction of a point's A
__device__ __forceinline__ float probe_component(int j) {
  const uint32_t h = (uint32_t)(j + 1) * 2654435761u;
  return (float)(h >> 8) * (2.0f / 16777216.0f) - 1.0f;
}

__device__ __forceinline__ double infl_update(int n, double infl, double p1, double trace, double p3) {
  const double q2 = trace / (double)(n - 1);
  const double q4 = (p1 - p3) / q2 - infl;
  const double t = (infl * q2 + p3) / q2;
  const double sigma_o = 2.0 / p3 * (t * t);
  const double gain = (kSigmaB * kSigmaB) / (sigma_o + kSigmaB * kSigmaB);
  return infl + gain * q4;
}

}  // namespace letkf
