// largek.cu -- batched LETKF core for large ensembles (k up to 512 and beyond).
//
// Same contract as letkf_core_batch_mixed (common/common_letkf.f90:50-243 per
// point: Gram, transform W = sqrt((k-1) Pa), wbar = Pa Ywᵀ dep, adaptive
// inflation), for ensembles whose k x k matrices do not fit on chip.  Per
// batch of points the matrices live in HBM (k padded to kp, a multiple of 128)
// and every dense product runs on the tensor cores (largek_gemm.cuh):
//   1. G = Ywᵀ Y            (tcgen05, three-term TF32, K = the point's L)
//   2. A = G + (k-1)/rho I, padded with the same diagonal; scale s = 1.05 x a
//      power-iteration estimate of lambda_max (tight: fewer iterations); a
//      point whose residual grows restarts once from the Gershgorin bound,
//      which always converges; Y0 = A/s, Z0 = I
//   3. coupled Newton-Schulz  T = Z Y, Y <- b Y + a Y T, Z <- b Z + a T Z
//      until ||T - I||² < tol (per-point active flags); the first step is
//      plain (a = -0.5, b = 1.5), later ones spectrum-scaled per point
//      (a = -0.5 g sqrt(g), b = 1.5 sqrt(g) with the step scale g from the
//      tracked lower spectral bound, as in the tensor-core sweep); a
//      residual above what a spectrum in [lo, 1] allows restarts the point
//   4. two uncoupled steps anchored to A:  Z <- 1.5 Z - 0.5 (Z (A/s) Z) Z,
//      symmetrised; then a certificate: the anchored residual
//      ||Z (A/s) Z p - p||^2 / ||p||^2 for a fixed probe p must be below 1e-6,
//      else the point is reported as not converged (LETKF_ERR_EIG)
//   5. W = sqrt((k-1)/s) Z, wbar = Z (Z Ywᵀdep) / s, inflation update.
// Points with no local observations take the nobsl = 0 branch; points with
// c <= 0 or tr(G) >= 1e6 c (where mtx_eigen's truncation could act) are
// reported with LETKF_ERR_CAPACITY and an identity transform.
#include <vector>

#include "largek_gemm.cuh"
#include "mixed_core.cuh"

namespace letkf {

constexpr int LKP_NT = 256;
constexpr float LK_NS_TOL = 1.0e-4f;  // ||ZY - I||_F^2 at which the coupled phase stops
constexpr int LK_NS_MAX = 40;
constexpr int LK_POLISH = 2;
constexpr float LK_CERT_TOL = 1.0e-6f;  // anchored probe residual a finished transform must reach

struct LkPoint {  // per-point scalars of a batch
  double s, c, p1, p3, trace, infl;
  float gmax;     // Gershgorin bound of lambda_max
  float e2_prev;  // residual of the previous iteration
  int kind;       // 0 transform, 1 no observations, 2 unsupported spectrum, 3 no convergence
  int restarted;  // 1 after the restart from the Gershgorin scale
  float lo;       // lower bound of the spectrum of ZY (0.9 c / s at the start)
  int steps;      // Newton-Schulz steps since the (re)start
};

__global__ void lk_weights_kernel(int64_t n, const float* __restrict__ rdiag, const float* __restrict__ rloc,
                                  int wloc, float* __restrict__ w) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) w[i] = wloc ? 1.0f / rdiag[i] : rloc[i] / rdiag[i];
}

// per point: p1, p3, b = Ywᵀ dep, trace, branch, A = G + cI, s, Y0, Z0
__global__ void __launch_bounds__(LKP_NT) lk_prep_kernel(int ne, int kp, const int64_t* __restrict__ offs,
                                                          const float* __restrict__ rows,
                                                          const __nv_bfloat16* __restrict__ rows16,
                                                          const int* __restrict__ ridx,
                                                          const float* __restrict__ w,
                                                          const float* __restrict__ dep,
                                                          const float* __restrict__ rloc, const double* infl_in,
                                                          double minfl, float* G, float* Y, float* Z,
                                                          float* bvec, float* inv_s, LkPoint* pt, int* active) {
  __shared__ double red[LKP_NT / 32];
  __shared__ __align__(16) float xv[1024];
  __shared__ __align__(16) float yv[1024];
  __shared__ float redf[LKP_NT / 32];
  const int b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int64_t r0 = offs[b];
  const int L = (int)(offs[b + 1] - r0);
  const size_t mo = (size_t)b * kp * kp;
  float* A = G + mo;
  auto bsum = [&](double v) {
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    double t = 0.0;
    for (int i = 0; i < LKP_NT / 32; i++) t += red[i];
    return t;
  };
  // list entry e: its row (packed, or observation ridx[e]) and departure
  auto row_of = [&](int64_t e) -> size_t { return ridx ? (size_t)ridx[e] : (size_t)e; };
  auto dep_of = [&](int64_t e) -> float { return dep[row_of(e)]; };
  double p1 = 0.0, p3 = 0.0;
  for (int l = tid; l < L; l += LKP_NT) {
    const double d = dep_of(r0 + l);
    p1 += d * d * (double)w[r0 + l];
    p3 += (double)rloc[r0 + l];
  }
  p1 = bsum(p1);
  p3 = bsum(p3);
  for (int m = tid; m < kp; m += LKP_NT) {
    float acc = 0.f;
    if (m < ne) {
      if (rows16)
        for (int l = 0; l < L; l++)
          acc = fmaf(w[r0 + l] * dep_of(r0 + l), __bfloat162float(rows16[row_of(r0 + l) * ne + m]), acc);
      else
        for (int l = 0; l < L; l++) acc = fmaf(w[r0 + l] * dep_of(r0 + l), rows[row_of(r0 + l) * ne + m], acc);
    }
    bvec[(size_t)b * kp + m] = acc;
  }
  double tr = 0.0;
  for (int m = tid; m < ne; m += LKP_NT) tr += (double)A[(size_t)m * kp + m];
  tr = bsum(tr);
  double infl = infl_in[b];
  int kind = 0;
  double c = 0.0;
  if (L == 0) {
    kind = 1;
  } else {
    if (minfl > 0.0 && infl < minfl) infl = minfl;
    c = (double)(ne - 1) / infl;
    if (!(c > 0.0) || !(tr < 1.0e6 * c)) kind = 2;
  }
  if (tid == 0) {
    LkPoint q;
    q.s = 1.0;
    q.c = c;
    q.p1 = p1;
    q.p3 = p3;
    q.trace = tr;
    q.infl = infl;
    q.gmax = 0.f;
    q.e2_prev = INFINITY;
    q.kind = kind;
    q.restarted = 0;
    q.lo = 0.f;
    q.steps = 0;
    pt[b] = q;
    active[b] = kind == 0;
  }
  if (kind != 0) return;
  const float cf = (float)c;
  for (int m = tid; m < kp; m += LKP_NT) A[(size_t)m * kp + m] = (m < ne ? A[(size_t)m * kp + m] : 0.f) + cf;
  __syncthreads();
  // Gershgorin bound and power iteration (s >= lambda_max / 2 keeps Newton-Schulz convergent);
  // one warp per row, the lanes over 16-byte column groups (coalesced row reads)
  const int kp4 = kp / 4;
  float gmax = 0.f;
  for (int m = wid; m < kp; m += LKP_NT / 32) {
    const float4* row4 = reinterpret_cast<const float4*>(A + (size_t)m * kp);
    float g = 0.f;
    for (int j4 = lane; j4 < kp4; j4 += 32) {
      const float4 x = row4[j4];
      g += (fabsf(x.x) + fabsf(x.y)) + (fabsf(x.z) + fabsf(x.w));
    }
    gmax = fmaxf(gmax, warp_sum(g));
  }
  for (int m = tid; m < kp; m += LKP_NT) xv[m] = A[(size_t)m * kp + m] * (1.f + 0.25f * __sinf(1.7f * m));
  __syncthreads();
  if (lane == 0) redf[wid] = gmax;
  __syncthreads();
  gmax = 0.f;
  for (int i = 0; i < LKP_NT / 32; i++) gmax = fmaxf(gmax, redf[i]);
  float lam = 0.f;
  const float4* xv4 = reinterpret_cast<const float4*>(xv);
  for (int it = 0; it < 8; it++) {
    for (int m = wid; m < kp; m += LKP_NT / 32) {
      const float4* row4 = reinterpret_cast<const float4*>(A + (size_t)m * kp);
      float acc = 0.f;
      for (int j4 = lane; j4 < kp4; j4 += 32) {
        const float4 x = row4[j4], v = xv4[j4];
        acc = fmaf(x.x, v.x, fmaf(x.y, v.y, fmaf(x.z, v.z, fmaf(x.w, v.w, acc))));
      }
      acc = warp_sum(acc);
      if (lane == 0) yv[m] = acc;
    }
    __syncthreads();
    double nrm2 = 0.0, x2 = 0.0;
    for (int m = tid; m < kp; m += LKP_NT) {
      nrm2 += (double)yv[m] * yv[m];
      x2 += (double)xv[m] * xv[m];
    }
    nrm2 = bsum(nrm2);
    x2 = bsum(x2);
    lam = (float)sqrt(nrm2 / fmax(x2, 1e-300));
    const float inv = (float)(1.0 / sqrt(fmax(nrm2, 1e-300)));
    for (int m = tid; m < kp; m += LKP_NT) xv[m] = yv[m] * inv;
    __syncthreads();
  }
  const float s = lam > 0.f ? 1.05f * lam : gmax;
  const float is = 1.f / s;
  if (tid == 0) {
    pt[b].s = (double)s;
    pt[b].gmax = gmax;
    pt[b].lo = 0.9f * (float)(c / (double)s);
    pt[b].steps = 0;
    inv_s[b] = is;
  }
  float* Yb = Y + mo;
  float* Zb = Z + mo;
  for (int64_t idx = tid; idx < (int64_t)kp * kp; idx += LKP_NT) {
    const int i = (int)(idx / kp), j = (int)(idx - (int64_t)i * kp);
    Yb[idx] = A[idx] * is;
    Zb[idx] = i == j ? 1.f : 0.f;
  }
}

// Converged points leave the coupled phase.  With the spectrum of ZY in
// [lo, u] (u = gmax / s before the first step, 1 + d after it) the residual
// is at most kp max((1 - lo)^2, (u - 1)^2); a residual above that, or not
// finite, restarts the point once from the Gershgorin scale (counts[1]); a
// second failure, or a point still iterating at the cap (last != 0), fails
// the point.  Points that go on get this step's coefficients (alpha_b,
// beta_b) and their bound follows f.  counts[0] = points still iterating.
__global__ void lk_check_kernel(int nb, int kp, const float* __restrict__ e2, int* active, int* counts, LkPoint* pt,
                                int* restart, int last, float* alpha_b, float* beta_b) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb || !active[b]) return;
  const float r = e2[b];
  LkPoint q = pt[b];
  const float u = q.steps == 0 ? q.gmax * (float)(1.0 / q.s) : 1.02f;
  const float d0 = 1.f - q.lo, d1 = u - 1.f;
  const float bound = (float)kp * fmaxf(d0 * d0, d1 * d1) * 1.05f + 1.0e-3f;
  const bool bad = !isfinite(r) || r > bound;
  if (bad && !q.restarted) {
    q.restarted = 1;
    q.e2_prev = INFINITY;
    restart[b] = 1;
    active[b] = 0;  // left alone by this iteration's updates, reset and reactivated after them
    atomicAdd(&counts[0], 1);
    atomicAdd(&counts[1], 1);
  } else if (bad || (last && !(r < LK_NS_TOL))) {
    q.kind = 3;
    active[b] = 0;
  } else if (r < LK_NS_TOL) {
    active[b] = 0;
  } else {
    float g = 1.f;
    if (q.steps == 0) {
      // plain first step: with s = 1.05 x the power estimate the top of the
      // spectrum is near 1 (f(1) = 1), so the bound follows the bottom; a
      // power estimate far below lambda_max shows as a residual above the
      // bound and restarts the point from the Gershgorin scale (top <= 1)
      q.lo = f_ns(q.lo);
    } else {
      g = ns_scale(q.lo);
      q.lo = f_ns(g * q.lo);
    }
    const float sg = sqrtf(g);
    alpha_b[b] = -0.5f * g * sg;
    beta_b[b] = 1.5f * sg;
    q.steps++;
    q.e2_prev = r;
    atomicAdd(&counts[0], 1);
  }
  pt[b] = q;
}

// restart flagged points from s = Gershgorin bound: Y = A/s, Z = I, active again
__global__ void lk_restart_kernel(int kp, const float* __restrict__ G, float* Y, float* Z, float* inv_s, LkPoint* pt,
                                  int* restart, int* active) {
  const int b = blockIdx.y;
  if (!restart[b]) return;
  const size_t mo = (size_t)b * kp * kp;
  const float s = pt[b].gmax, is = 1.f / s;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < (int64_t)kp * kp;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(idx / kp), j = (int)(idx - (int64_t)i * kp);
    Y[mo + idx] = G[mo + idx] * is;
    Z[mo + idx] = i == j ? 1.f : 0.f;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    pt[b].s = (double)s;
    pt[b].lo = 0.9f * (float)(pt[b].c / (double)s);
    pt[b].steps = 0;
    inv_s[b] = is;
    active[b] = 1;
  }
}

__global__ void lk_reactivate_kernel(int nb, const LkPoint* __restrict__ pt, int* active) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < nb) active[b] = pt[b].kind == 0;
}

// Certificate of a finished transform, three matvecs against the exact A (G
// holds A): e = ||Z (A/s) Z p - p||^2 / ||p||^2 for the fixed probe vector p on
// the ensemble coordinates.  With Z = (A/s)^(-1/2) (I + E) the residual is
// 2 E p to first order; a point with e not below tol (or not finite) is
// reported as not converged instead of returning its transform.  Column
// reads of the symmetric matrices keep the loads coalesced.
__global__ void __launch_bounds__(LKP_NT) lk_certify_kernel(int ne, int kp, const float* __restrict__ Z,
                                                             const float* __restrict__ G,
                                                             const float* __restrict__ inv_s, LkPoint* pt,
                                                             float tol) {
  __shared__ float vp[LETKF_LARGEK_MAX_NE], vu[LETKF_LARGEK_MAX_NE], vw[LETKF_LARGEK_MAX_NE];
  __shared__ float red[2 * (LKP_NT / 32)];
  const int b = blockIdx.x, tid = threadIdx.x;
  if (pt[b].kind != 0) return;
  const size_t mo = (size_t)b * kp * kp;
  const float* Zb = Z + mo;
  const float* Ab = G + mo;
  const float is = inv_s[b];
  for (int i = tid; i < kp; i += LKP_NT) vp[i] = i < ne ? probe_component(i) : 0.f;
  __syncthreads();
  for (int i = tid; i < kp; i += LKP_NT) {
    float acc = 0.f;
    for (int j = 0; j < kp; j++) acc = fmaf(Zb[(size_t)j * kp + i], vp[j], acc);
    vu[i] = acc;
  }
  __syncthreads();
  for (int i = tid; i < kp; i += LKP_NT) {
    float acc = 0.f;
    for (int j = 0; j < kp; j++) acc = fmaf(Ab[(size_t)j * kp + i], vu[j], acc);
    vw[i] = acc * is;
  }
  __syncthreads();
  float e = 0.f, pn = 0.f;
  for (int i = tid; i < kp; i += LKP_NT) {
    float acc = 0.f;
    for (int j = 0; j < kp; j++) acc = fmaf(Zb[(size_t)j * kp + i], vw[j], acc);
    const float d = acc - vp[i];
    e = fmaf(d, d, e);
    pn = fmaf(vp[i], vp[i], pn);
  }
  e = warp_sum(e);
  pn = warp_sum(pn);
  if ((tid & 31) == 0) {
    red[tid >> 5] = e;
    red[LKP_NT / 32 + (tid >> 5)] = pn;
  }
  __syncthreads();
  if (tid == 0) {
    float es = 0.f, ps = 0.f;
    for (int w = 0; w < LKP_NT / 32; w++) {
      es += red[w];
      ps += red[LKP_NT / 32 + w];
    }
    if (!(es < tol * ps)) pt[b].kind = 3;
  }
}

// Z <- (Zn + Znᵀ) / 2 for active points
__global__ void lk_symmetrize_kernel(int kp, const float* __restrict__ Zn, float* Z, const int* __restrict__ active) {
  const int b = blockIdx.y;
  if (!active[b]) return;
  const size_t mo = (size_t)b * kp * kp;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < (int64_t)kp * kp;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(idx / kp), j = (int)(idx - (int64_t)i * kp);
    Z[mo + idx] = 0.5f * (Zn[mo + idx] + Zn[mo + (size_t)j * kp + i]);
  }
}

// W, wbar, inflation, status for the points of a batch
__global__ void __launch_bounds__(LKP_NT) lk_finalize_kernel(int ne, int kp, const float* __restrict__ Z,
                                                              const float* __restrict__ bvec,
                                                              const LkPoint* __restrict__ pt, double* infl,
                                                              float* trans, float* transm, int* status) {
  __shared__ float g[1024];
  const int b = blockIdx.x, tid = threadIdx.x;
  const LkPoint q = pt[b];
  float* tr = trans + (size_t)b * ne * ne;
  if (q.kind != 0) {
    const float d = q.kind == 1 ? (float)sqrt(q.infl) : 1.f;
    for (int idx = tid; idx < ne * ne; idx += LKP_NT) tr[idx] = (idx / ne == idx % ne) ? d : 0.f;
    if (transm)
      for (int m = tid; m < ne; m += LKP_NT) transm[(size_t)b * ne + m] = 0.f;
    if (tid == 0) status[b] = q.kind == 1 ? LETKF_OK : (q.kind == 2 ? LETKF_ERR_CAPACITY : LETKF_ERR_EIG);
    return;
  }
  const float* Zb = Z + (size_t)b * kp * kp;
  const float* bv = bvec + (size_t)b * kp;
  for (int m = tid; m < ne; m += LKP_NT) {
    float acc = 0.f;
    for (int j = 0; j < ne; j++) acc = fmaf(Zb[(size_t)m * kp + j], bv[j], acc);
    g[m] = acc;
  }
  __syncthreads();
  const float inv_s = (float)(1.0 / q.s);
  if (transm)
    for (int m = tid; m < ne; m += LKP_NT) {
      float acc = 0.f;
      for (int j = 0; j < ne; j++) acc = fmaf(Zb[(size_t)m * kp + j], g[j], acc);
      transm[(size_t)b * ne + m] = acc * inv_s;
    }
  const float coef = (float)sqrt((double)(ne - 1) / q.s);
  // trans(k, m) = W[k][m] at column-major index m * ne + k (W symmetric)
  for (int idx = tid; idx < ne * ne; idx += LKP_NT) {
    const int m = idx / ne, k = idx - m * ne;
    tr[idx] = coef * Zb[(size_t)k * kp + m];
  }
  if (tid == 0) {
    infl[b] = infl_update(ne, q.infl, q.p1, q.trace, q.p3);
    status[b] = LETKF_OK;
  }
}

// xa(p,m,v) = mean + sum_k xb'(k) (trans(k,m) + transm(k)) for any ne: the
// product in FP32 from 32-row tiles of trans staged through shared memory,
// the mean and the mean increment in FP64 (as the fused sweeps)
constexpr int LKU_KT = 32;

// floats before the FP64 array of lk_update_kernel's shared memory (8-byte aligned)
__host__ __device__ constexpr int lku_base_floats(int nv, int ne) {
  return (nv * ne + LKU_KT * (ne + 1) + 1) & ~1;
}

// BF == false: xb, xa [nv][npts][ne] FP32 members.  BF == true: members
// stored as an FP32 mean xmean [nv][npts] plus BF16 perturbations xb
// [nv][npts][ne]; the analysis likewise (amean = mean + xb' transm in FP64,
// xa = xb' trans rounded to BF16)
template <bool BF>
__global__ void __launch_bounds__(LKP_NT) lk_update_kernel(int ne, int npts, int nv, const void* __restrict__ xb_,
                                                            const float* __restrict__ xmean,
                                                            const float* __restrict__ trans,
                                                            const float* __restrict__ transm, void* xa_,
                                                            float* amean) {
  extern __shared__ __align__(16) float su[];
  const int ld = ne + 1;                   // padded row of the staged tile (conflict-free columns)
  float* xs = su;                          // [nv][ne] perturbations
  float* tt = xs + nv * ne;                // [LKU_KT][ld] trans(k0 + kk, m)
  double* base = reinterpret_cast<double*>(su + lku_base_floats(nv, ne));  // [nv] mean + increment
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  for (int p = blockIdx.x; p < npts; p += gridDim.x) {
    __syncthreads();
    for (int t = tid; t < nv * ne; t += LKP_NT) {
      const int v = t / ne, m = t - v * ne;
      const size_t at = ((size_t)v * npts + p) * ne + m;
      xs[t] = BF ? __bfloat162float(reinterpret_cast<const __nv_bfloat16*>(xb_)[at])
                 : reinterpret_cast<const float*>(xb_)[at];
    }
    __syncthreads();
    for (int v = wid; v < nv; v += LKP_NT / 32) {
      double sx = 0.0;
      for (int m = lane; m < ne; m += 32) sx += (double)xs[v * ne + m];
      const double mean = warp_sum(sx) / (double)ne;  // of the members (BF: of the stored perturbations)
      double dl = 0.0;
      for (int m = lane; m < ne; m += 32) {
        const float x = (float)((double)xs[v * ne + m] - mean);
        xs[v * ne + m] = x;
        if (transm) dl += (double)x * (double)transm[(size_t)p * ne + m];
      }
      dl = warp_sum(dl);
      if (lane == 0) {
        if (BF) {
          base[v] = 0.0;
          amean[(size_t)v * npts + p] = (float)((double)xmean[(size_t)v * npts + p] + mean + dl);
        } else {
          base[v] = mean + dl;
        }
      }
    }
    float acc[8][2];
#pragma unroll
    for (int v = 0; v < 8; v++) acc[v][0] = acc[v][1] = 0.f;
    const float* tp = trans + (size_t)p * ne * ne;
    for (int k0 = 0; k0 < ne; k0 += LKU_KT) {
      const int kn = min(LKU_KT, ne - k0);
      __syncthreads();
      // column m of trans is contiguous in k: each thread copies whole runs
      for (int t = tid; t < kn * ne; t += LKP_NT) {
        const int m = t / kn, kk = t - m * kn;
        tt[kk * ld + m] = tp[(size_t)m * ne + k0 + kk];
      }
      __syncthreads();
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int m = tid + h * LKP_NT;
        if (m >= ne) continue;
        for (int kk = 0; kk < kn; kk++) {
          const float w = tt[kk * ld + m];
#pragma unroll
          for (int v = 0; v < 8; v++)
            if (v < nv) acc[v][h] = fmaf(xs[v * ne + k0 + kk], w, acc[v][h]);
        }
      }
    }
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int m = tid + h * LKP_NT;
      if (m >= ne) continue;
#pragma unroll
      for (int v = 0; v < 8; v++)
        if (v < nv) {
          const size_t at = ((size_t)v * npts + p) * ne + m;
          if (BF)
            reinterpret_cast<__nv_bfloat16*>(xa_)[at] = __float2bfloat16_rn(acc[v][h]);
          else
            reinterpret_cast<float*>(xa_)[at] = (float)(base[v] + (double)acc[v][h]);
        }
    }
  }
}

template <bool BF>
static int launch_lk_update(int ne, int npts, int nv, const void* xb, const float* xmean, const float* trans,
                            const float* transm, void* xa, float* amean, cudaStream_t stream) {
  const size_t smem = sizeof(float) * (size_t)lku_base_floats(nv, ne) + sizeof(double) * 8;
  cudaError_t e = cudaFuncSetAttribute(lk_update_kernel<BF>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_status(e);
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int grid = npts < nsm * 4 ? npts : nsm * 4;
  lk_update_kernel<BF><<<grid, LKP_NT, smem, stream>>>(ne, npts, nv, xb, xmean, trans, transm, xa, amean);
  note_launch();
  return cuda_status(cudaGetLastError());
}

template <int MODE>
static int lk_gemm(const LkGemmArgs& a, int nb, cudaStream_t s) {
  static_assert(LK_SMEM <= 227 * 1024, "shared memory");
  cudaError_t e = cudaFuncSetAttribute(largek_gemm_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, LK_SMEM);
  if (e != cudaSuccess) return cuda_status(e);
  dim3 grid(a.kp / LK_TILE, a.kp / LK_TILE, nb);
  largek_gemm_kernel<MODE><<<grid, LK_NT, LK_SMEM, s>>>(a);
  note_launch();
  return cuda_status(cudaGetLastError());
}

}  // namespace letkf

using namespace letkf;

extern "C" int letkf_update_mixed(int ne, int npts, int nv, const float* xb, const float* trans,
                                  const float* transm, float* xa, void* stream) {
  if (ne < 2 || npts < 0 || nv < 1 || nv > 8 || !xb || !trans || !xa) return LETKF_ERR_ARG;
  if (ne > 2 * LKP_NT) return LETKF_ERR_CAPACITY;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return LETKF_ERR_NOGPU;
  }
  if (npts == 0) return LETKF_OK;
  return launch_lk_update<false>(ne, npts, nv, xb, nullptr, trans, transm, xa, nullptr, (cudaStream_t)stream);
}

extern "C" int letkf_update_bf16(int ne, int npts, int nv, const float* xmean, const void* xpert,
                                 const float* trans, const float* transm, float* amean, void* apert, void* stream) {
  if (ne < 2 || npts < 0 || nv < 1 || nv > 8 || !xmean || !xpert || !trans || !amean || !apert) return LETKF_ERR_ARG;
  if (ne > 2 * LKP_NT) return LETKF_ERR_CAPACITY;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return LETKF_ERR_NOGPU;
  }
  if (npts == 0) return LETKF_OK;
  return launch_lk_update<true>(ne, npts, nv, xpert, xmean, trans, transm, apert, amean, (cudaStream_t)stream);
}

namespace letkf {
int largek_fp64_pass(int ne, int npts, const int64_t* offs, const float* rows, const __nv_bfloat16* rows16,
                     const int* ridx, const float* rdiag, const float* rloc, const float* dep, double* parm_infl,
                     float* trans, float* transm, int rdiag_wloc, double minfl, int* status, cudaStream_t s);
}  // namespace letkf

// the large-ensemble core over packed rows (rows, dep per list entry) or over
// index lists into the observation ensemble (ridx; FP32 rows or BF16 rows16,
// dep per observation)
static int largek_core(int ne, int npts, const int64_t* offs, const float* rows, const __nv_bfloat16* rows16,
                       const int* ridx, const float* rdiag, const float* rloc, const float* dep, double* parm_infl,
                       float* trans, float* transm, int rdiag_wloc, double minfl, int* status, void* stream) {
  if (ne < 2 || npts < 0 || !offs || !parm_infl || !trans || !status) return LETKF_ERR_ARG;
  if (ne > LETKF_LARGEK_MAX_NE) return LETKF_ERR_CAPACITY;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return LETKF_ERR_NOGPU;
  }
  if (npts == 0) return LETKF_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const int kp = (ne + LK_TILE - 1) / LK_TILE * LK_TILE;
  const size_t mat = (size_t)kp * kp;
  // batch: six kp x kp FP32 matrices per point, at most 1.5 GB
  int B = (int)std::min<size_t>((size_t)npts, std::max<size_t>(1, (size_t)(1536u << 20) / (6 * mat * 4)));
  int64_t nrows = 0;
  if (cudaMemcpyAsync(&nrows, offs + npts, sizeof(int64_t), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return LETKF_ERR_CUDA;
  float *w = nullptr, *G = nullptr, *Y = nullptr, *Z = nullptr, *Yn = nullptr, *Zn = nullptr, *T = nullptr;
  float *bvec = nullptr, *e2 = nullptr, *inv_s = nullptr, *alphas = nullptr, *betas = nullptr;
  int *active = nullptr, *count = nullptr, *err = nullptr, *restart = nullptr;
  LkPoint* pt = nullptr;
  bool ok = true;
  auto A = [&](auto** p, size_t bytes) { ok = ok && cudaMallocAsync((void**)p, bytes, s) == cudaSuccess; };
  A(&w, sizeof(float) * (size_t)std::max<int64_t>(nrows, 1));
  A(&G, sizeof(float) * mat * B);
  A(&Y, sizeof(float) * mat * B);
  A(&Z, sizeof(float) * mat * B);
  A(&Yn, sizeof(float) * mat * B);
  A(&Zn, sizeof(float) * mat * B);
  A(&T, sizeof(float) * mat * B);
  A(&bvec, sizeof(float) * (size_t)kp * B);
  A(&e2, sizeof(float) * B);
  A(&inv_s, sizeof(float) * B);
  A(&alphas, sizeof(float) * B);
  A(&betas, sizeof(float) * B);
  A(&active, sizeof(int) * B);
  A(&count, 2 * sizeof(int));
  A(&restart, sizeof(int) * B);
  A(&err, sizeof(int));
  A(&pt, sizeof(LkPoint) * B);
  int st = ok ? LETKF_OK : LETKF_ERR_CUDA;
  if (st == LETKF_OK) st = cuda_status(cudaMemsetAsync(err, 0, sizeof(int), s));
  if (st == LETKF_OK && nrows > 0) {
    lk_weights_kernel<<<(unsigned)((nrows + 255) / 256), 256, 0, s>>>(nrows, rdiag, rloc, rdiag_wloc, w);
    note_launch();
  }
  for (int p0 = 0; p0 < npts && st == LETKF_OK; p0 += B) {
    const int nb = std::min(B, npts - p0);
    LkGemmArgs g;
    memset(&g, 0, sizeof(g));
    g.kp = kp;
    g.mstride = (int64_t)mat;
    g.err_flag = err;
    // 1. Gram
    g.out = G;
    g.rows = rows;
    g.rows16 = rows16;
    g.ridx = ridx;
    g.wts = w;
    g.offs = offs + p0;
    g.ne = ne;
    st = lk_gemm<LK_GRAM>(g, nb, s);
    if (st) break;
    // 2. prep
    lk_prep_kernel<<<nb, LKP_NT, 0, s>>>(ne, kp, offs + p0, rows, rows16, ridx, w, dep, rloc, parm_infl + p0, minfl,
                                         G, Y, Z, bvec, inv_s, pt, active);
    note_launch();
    // 3. coupled Newton-Schulz
    g.rows = nullptr;
    g.rows16 = nullptr;
    g.ridx = nullptr;
    g.wts = nullptr;
    g.offs = nullptr;
    g.active = active;
    cudaMemsetAsync(restart, 0, sizeof(int) * nb, s);
    for (int it = 0; it < LK_NS_MAX && st == LETKF_OK; it++) {
      cudaMemsetAsync(e2, 0, sizeof(float) * nb, s);
      cudaMemsetAsync(count, 0, 2 * sizeof(int), s);
      g.X = Z;
      g.Y = Y;
      g.D = nullptr;
      g.out = T;
      g.e2 = e2;
      st = lk_gemm<LK_T>(g, nb, s);
      if (st) break;
      lk_check_kernel<<<(nb + 127) / 128, 128, 0, s>>>(nb, kp, e2, active, count, pt, restart, it == LK_NS_MAX - 1,
                                                       alphas, betas);
      note_launch();
      int h_count[2] = {0, 0};
      cudaMemcpyAsync(h_count, count, 2 * sizeof(int), cudaMemcpyDeviceToHost, s);
      st = cuda_status(cudaStreamSynchronize(s));
      if (st || h_count[0] == 0) break;
      g.alpha_b = alphas;  // per-point step coefficients
      g.beta_b = betas;
      g.X = Y;  // Y <- b Y + a Y T
      g.Y = T;
      g.D = Y;
      g.out = Yn;
      st = lk_gemm<LK_AXPBY>(g, nb, s);
      if (st) break;
      g.X = T;  // Z <- b Z + a T Z
      g.Y = Z;
      g.D = Z;
      g.out = Zn;
      st = lk_gemm<LK_AXPBY>(g, nb, s);
      g.alpha_b = nullptr;
      g.beta_b = nullptr;
      std::swap(Y, Yn);
      std::swap(Z, Zn);
      if (st == LETKF_OK && h_count[1] > 0) {  // restarted points: Y0, Z0 from the Gershgorin scale
        dim3 rg(64, nb);
        lk_restart_kernel<<<rg, 256, 0, s>>>(kp, G, Y, Z, inv_s, pt, restart, active);
        note_launch();
        cudaMemsetAsync(restart, 0, sizeof(int) * nb, s);
      }
    }
    g.alpha_b = nullptr;
    g.beta_b = nullptr;
    // 4. uncoupled steps anchored to A (G holds A)
    lk_reactivate_kernel<<<(nb + 127) / 128, 128, 0, s>>>(nb, pt, active);
    note_launch();
    for (int it = 0; it < LK_POLISH && st == LETKF_OK; it++) {
      g.alpha_b = inv_s;  // P = (A / s) Z  (into T)
      g.alpha = 1.f;
      g.beta = 0.f;
      g.X = G;
      g.Y = Z;
      g.D = nullptr;
      g.out = T;
      st = lk_gemm<LK_AXPBY>(g, nb, s);
      if (st) break;
      g.alpha_b = nullptr;  // Q = Z P  (into Yn)
      g.X = Z;
      g.Y = T;
      g.out = Yn;
      st = lk_gemm<LK_AXPBY>(g, nb, s);
      if (st) break;
      g.alpha = -0.5f;  // Zn = 1.5 Z - 0.5 Q Z
      g.beta = 1.5f;
      g.X = Yn;
      g.Y = Z;
      g.D = Z;
      g.out = Zn;
      st = lk_gemm<LK_AXPBY>(g, nb, s);
      if (st) break;
      dim3 sg(64, nb);
      lk_symmetrize_kernel<<<sg, 256, 0, s>>>(kp, Zn, Z, active);
      note_launch();
    }
    // certificate of every transform against the exact A
    if (st == LETKF_OK) {
      lk_certify_kernel<<<nb, LKP_NT, 0, s>>>(ne, kp, Z, G, inv_s, pt, LK_CERT_TOL);
      note_launch();
    }
    // 5. transform, mean weights, inflation
    lk_finalize_kernel<<<nb, LKP_NT, 0, s>>>(ne, kp, Z, bvec, pt, parm_infl + p0, trans + (size_t)p0 * ne * ne,
                                             transm ? transm + (size_t)p0 * ne : nullptr, status + p0);
    note_launch();
  }
  int h_err = 0;
  if (st == LETKF_OK) {
    cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost, s);
    st = cuda_status(cudaStreamSynchronize(s));
    if (st == LETKF_OK && h_err) st = LETKF_ERR_TIMEOUT;
  }
  void* fr[] = {w, G, Y, Z, Yn, Zn, T, bvec, e2, inv_s, alphas, betas, active, count, err, pt, restart};
  for (void* p : fr)
    if (p) cudaFreeAsync(p, s);
  // points whose mixed-precision transform did not certify: the FP64 pass
  if (st == LETKF_OK)
    st = largek_fp64_pass(ne, npts, offs, rows, rows16, ridx, rdiag, rloc, dep, parm_infl, trans, transm, rdiag_wloc,
                          minfl, status, s);
  return st;
}

extern "C" int letkf_core_batch_largek(int ne, int npts, const int64_t* offs, const float* rows, const float* rdiag,
                                       const float* rloc, const float* dep, double* parm_infl, float* trans,
                                       float* transm, int rdiag_wloc, double minfl, int* status, void* stream) {
  return largek_core(ne, npts, offs, rows, nullptr, nullptr, rdiag, rloc, dep, parm_infl, trans, transm, rdiag_wloc,
                     minfl, status, stream);
}

extern "C" int letkf_core_batch_largek_indexed(int ne, int npts, const int64_t* offs, const int* idx,
                                               const void* ens_obs, int ens_bf16, const float* dep_obs,
                                               const float* rdiag, const float* rloc, double* parm_infl,
                                               float* trans, float* transm, int rdiag_wloc, double minfl,
                                               int* status, void* stream) {
  if (!ens_obs || !dep_obs || !idx) return LETKF_ERR_ARG;
  return largek_core(ne, npts, offs, ens_bf16 ? nullptr : (const float*)ens_obs,
                     ens_bf16 ? (const __nv_bfloat16*)ens_obs : nullptr, idx, rdiag, rloc, dep_obs, parm_infl, trans,
                     transm, rdiag_wloc, minfl, status, stream);
}
