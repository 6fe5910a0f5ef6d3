// largek_fp64.cu -- FP64 pass of the large-ensemble core for points the
// mixed-precision transform cannot certify.
//
// The large-k core (largek.cu) forms the Gram and the Newton-Schulz products
// from TF32 / BF16 splits with FP32 accumulation, about 1e-6 relative.  Where
// lambda_max / c of A = Gram + (k-1)/rho I reaches about 1e3..1e4 (long local
// lists, small observation errors), the smallest eigen-directions of W are
// then not resolved and the core reports LETKF_ERR_EIG.  This pass redoes those
// points in FP64, the reference's precision (common/common_letkf.f90:101-239):
//   1. rows of the point gathered in FP64 and scaled, B = sqrt(w) Y with
//      w = rloc / rdiag (1 / rdiag with rdiag_wloc), G = Bᵀ B by cuBLAS DGEMM
//      (measured 2.4x faster than DSYRK's triangle here, which computes half
//      the products) and b = Bᵀ (sqrt(w) dep) by DGEMV;
//   2. A = G + cI, s = Gershgorin bound, Y0 = A / s, Z0 = I;
//   3. coupled Newton-Schulz in FP64, batched over the points (cuBLAS
//      strided-batched DGEMM), spectrum-scaled steps from the lower bound
//      0.9 c / s, until ||ZY - I||_F^2 < 1e-24;
//   4. certificate ||Z (A/s) Z - I||_F^2 < 1e-16, then W = sqrt((k-1)/s) Z,
//      wbar = Z (Z b) / s and the adaptive inflation (:218-239).
// The core reports LETKF_ERR_CAPACITY where tr(G) >= 1e6 c, a cheap sufficient
// test that mtx_eigen's truncation (common/common_mtx.f90:66-72: eigenvalues
// below lambda_max sqrt(eps) are dropped) cannot act.  Every eigenvalue of A is
// at least c, so truncation needs lambda_max > c / sqrt(eps) = 6.7e7 c: this
// pass takes those points too and keeps the flag only where the sharper upper
// bound min(Gershgorin, ||A||_F) of lambda_max reaches 3e7 c, or where c <= 0.
#include <cublas_v2.h>

#include <vector>

#include "mixed_core.cuh"

namespace letkf {

constexpr int L64_NT = 256;
constexpr int L64_NS_MAX = 60;
constexpr double L64_NS_TOL = 1.0e-24;
constexpr double L64_CERT_TOL = 1.0e-16;
// lambda_max bound / c from which mtx_eigen's truncation could act (half of 1 / sqrt(eps))
constexpr double L64_TRUNC_RATIO = 3.0e7;

struct L64Point {
  double s, c, p1, p3, trace, infl, lo;
  int done, skip;
};

// Bc [L][ne] (column-major ne x L): the point's rows in FP64 times sqrt(w),
// and sqrt(w) dep per list entry
__global__ void l64_gather_kernel(int ne, int L, int64_t r0, const float* __restrict__ rows,
                                  const __nv_bfloat16* __restrict__ rows16, const int* __restrict__ ridx,
                                  const float* __restrict__ rdiag, const float* __restrict__ rloc,
                                  const float* __restrict__ dep, int wloc, double* Bc, double* e64) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)L * ne) return;
  const int64_t l = t / ne;
  const int m = (int)(t - l * ne);
  const int64_t e = r0 + l;
  const size_t ri = ridx ? (size_t)ridx[e] : (size_t)e;
  const double sw = sqrt(wloc ? 1.0 / (double)rdiag[e] : (double)rloc[e] / (double)rdiag[e]);
  const double y = rows16 ? (double)__bfloat162float(rows16[ri * ne + m]) : (double)rows[ri * ne + m];
  Bc[t] = sw * y;
  if (m == 0) e64[l] = sw * (double)dep[ri];
}

// p1 = sum dep^2 w, p3 = sum rloc over the point's entries
__global__ void l64_sums_kernel(int L, int64_t r0, const float* __restrict__ rloc, const double* __restrict__ e64,
                                double* out) {
  __shared__ double red[L64_NT / 32];
  double p1 = 0.0, p3 = 0.0;
  for (int l = threadIdx.x; l < L; l += L64_NT) {
    p1 += e64[l] * e64[l];
    p3 += (double)rloc[r0 + l];
  }
  p1 = block_sum<double, L64_NT>(p1, red);
  p3 = block_sum<double, L64_NT>(p3, red);
  if (threadIdx.x == 0) {
    out[0] = p1;
    out[1] = p3;
  }
}

// G's upper triangle from its lower one (exactly symmetric), A = G + cI (in place), s,
// Y0 = A / s, Z0 = I, the point's scalars
__global__ void l64_prep_kernel(int ne, double* G, double* Y, double* Z, const double* __restrict__ sums,
                                const double* __restrict__ infl_in, double minfl, L64Point* pt) {
  __shared__ double red[L64_NT / 32];
  __shared__ double gmx[L64_NT / 32];
  const int b = blockIdx.x, tid = threadIdx.x;
  const size_t mo = (size_t)b * ne * ne;
  double* A = G + mo;
  for (size_t idx = tid; idx < (size_t)ne * ne; idx += L64_NT) {
    const int j = (int)(idx / ne), m = (int)(idx - (size_t)j * ne);  // row m, column j
    if (m < j) A[idx] = A[(size_t)m * ne + j];
  }
  __syncthreads();
  double tr = 0.0;
  for (int m = tid; m < ne; m += L64_NT) tr += A[(size_t)m * ne + m];
  tr = block_sum<double, L64_NT>(tr, red);
  double infl = infl_in[b];
  if (minfl > 0.0 && infl < minfl) infl = minfl;
  const double c = (double)(ne - 1) / infl;
  for (int m = tid; m < ne; m += L64_NT) A[(size_t)m * ne + m] += c;
  __syncthreads();
  double g = 0.0;  // Gershgorin: largest absolute row sum
  for (int m = tid; m < ne; m += L64_NT) {
    double r = 0.0;
    for (int j = 0; j < ne; j++) r += fabs(A[(size_t)j * ne + m]);
    g = fmax(g, r);
  }
  g = warp_max(g);
  if ((tid & 31) == 0) gmx[tid >> 5] = g;
  double f2 = 0.0;  // ||A||_F^2
  for (size_t idx = tid; idx < (size_t)ne * ne; idx += L64_NT) f2 += A[idx] * A[idx];
  f2 = block_sum<double, L64_NT>(f2, red);  // (its barriers publish gmx)
  double s = 0.0;
  for (int w = 0; w < L64_NT / 32; w++) s = fmax(s, gmx[w]);
  // c <= 0, or truncation in mtx_eigen possible: the point keeps the core's flag
  const bool skip = !(c > 0.0) || !(fmin(s, sqrt(f2)) < L64_TRUNC_RATIO * c);
  if (skip) s = 1.0;
  const double inv_s = 1.0 / s;
  for (size_t idx = tid; idx < (size_t)ne * ne; idx += L64_NT) {
    const int m = (int)(idx / ne), j = (int)(idx - (size_t)m * ne);
    Y[mo + idx] = A[idx] * inv_s;
    Z[mo + idx] = m == j ? 1.0 : 0.0;
  }
  if (tid == 0) {
    L64Point q;
    q.s = s;
    q.c = c;
    q.p1 = sums[2 * b];
    q.p3 = sums[2 * b + 1];
    q.trace = tr;
    q.infl = infl;
    q.lo = 0.9 * c * inv_s;
    q.done = skip ? 1 : 0;
    q.skip = skip ? 1 : 0;
    pt[b] = q;
  }
}

// ||T - I||^2; the step matrix M = sqrt(a) (3I - aT) / 2 (I once converged)
__global__ void l64_step_kernel(int ne, const double* __restrict__ T, double* M, L64Point* pt, int* active) {
  __shared__ double red[L64_NT / 32];
  const int b = blockIdx.x, tid = threadIdx.x;
  const size_t mo = (size_t)b * ne * ne;
  double e2 = 0.0;
  for (size_t idx = tid; idx < (size_t)ne * ne; idx += L64_NT) {
    const int m = (int)(idx / ne), j = (int)(idx - (size_t)m * ne);
    const double d = T[mo + idx] - (m == j ? 1.0 : 0.0);
    e2 += d * d;
  }
  e2 = block_sum<double, L64_NT>(e2, red);
  L64Point q = pt[b];
  const bool done = q.done || !(e2 >= L64_NS_TOL);  // a NaN residual ends the point (not certified)
  double ka = 1.0, kb = 0.0;
  if (!done) {
    // balanced scale of the step from the lower bound lo of the spectrum of ZY
    // (as ns_scale in FP32): f(a lo) = f(a (1 + d)), d = 0.02
    const double d1 = 1.02;
    const double l = fmin(fmax(q.lo / d1, 0.0), 0.999);
    const double r = sqrt(l);
    const double al = fmax(3.0 * (1.0 - r) / ((1.0 - l * r) * d1), 1.0);
    const double sa = sqrt(al);
    ka = 1.5 * sa;
    kb = 0.5 * al * sa;
    const double x = al * q.lo, t3 = 3.0 - x;
    q.lo = 0.25 * x * t3 * t3;
  }
  for (size_t idx = tid; idx < (size_t)ne * ne; idx += L64_NT) {
    const int m = (int)(idx / ne), j = (int)(idx - (size_t)m * ne);
    M[mo + idx] = (m == j ? ka : 0.0) - kb * T[mo + idx];
  }
  if (tid == 0) {
    q.done = done ? 1 : 0;
    pt[b] = q;
    if (!done) atomicAdd(active, 1);
  }
}

// certificate on Q = Z (A Z) / s, then W, wbar, inflation
__global__ void l64_finalize_kernel(int ne, const double* __restrict__ Q, const double* __restrict__ Z,
                                    const double* __restrict__ bvec, L64Point* pt, const int* __restrict__ which,
                                    double* infl, float* trans, float* transm, int* status) {
  __shared__ double red[L64_NT / 32];
  extern __shared__ double g[];
  const int b = blockIdx.x, tid = threadIdx.x;
  const size_t mo = (size_t)b * ne * ne;
  const L64Point q = pt[b];
  if (q.skip) return;
  const double inv_s = 1.0 / q.s;
  double e2 = 0.0;
  for (size_t idx = tid; idx < (size_t)ne * ne; idx += L64_NT) {
    const int m = (int)(idx / ne), j = (int)(idx - (size_t)m * ne);
    const double d = Q[mo + idx] * inv_s - (m == j ? 1.0 : 0.0);
    e2 += d * d;
  }
  e2 = block_sum<double, L64_NT>(e2, red);
  if (!(e2 < L64_CERT_TOL)) return;  // keeps the core's status and identity
  const int p = which[b];
  const double* Zb = Z + mo;
  const double* bv = bvec + (size_t)b * ne;
  for (int m = tid; m < ne; m += L64_NT) {
    double acc = 0.0;
    for (int j = 0; j < ne; j++) acc += Zb[(size_t)j * ne + m] * bv[j];
    g[m] = acc;
  }
  __syncthreads();
  if (transm)
    for (int m = tid; m < ne; m += L64_NT) {
      double acc = 0.0;
      for (int j = 0; j < ne; j++) acc += Zb[(size_t)j * ne + m] * g[j];
      transm[(size_t)p * ne + m] = (float)(acc * inv_s);
    }
  const double coef = sqrt((double)(ne - 1) * inv_s);
  float* tr = trans + (size_t)p * ne * ne;
  // trans(k, m) = W[k][m] at column-major index m * ne + k; Z is column-major too
  for (size_t idx = tid; idx < (size_t)ne * ne; idx += L64_NT) tr[idx] = (float)(coef * Zb[idx]);
  if (tid == 0) {
    infl[p] = infl_update(ne, q.infl, q.p1, q.trace, q.p3);
    status[p] = LETKF_OK;
  }
}

static int cublas_status(cublasStatus_t e) { return e == CUBLAS_STATUS_SUCCESS ? LETKF_OK : LETKF_ERR_CUDA; }

// The FP64 pass over the points whose status is LETKF_ERR_EIG or
// LETKF_ERR_CAPACITY after the mixed-precision core; their parm_infl is still
// the input value.
int largek_fp64_pass(int ne, int npts, const int64_t* offs, const float* rows, const __nv_bfloat16* rows16,
                     const int* ridx, const float* rdiag, const float* rloc, const float* dep, double* parm_infl,
                     float* trans, float* transm, int rdiag_wloc, double minfl, int* status, cudaStream_t s) {
  std::vector<int> st(npts);
  std::vector<int64_t> ho(npts + 1);
  cudaMemcpyAsync(st.data(), status, sizeof(int) * npts, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(ho.data(), offs, sizeof(int64_t) * (npts + 1), cudaMemcpyDeviceToHost, s);
  int rc = cuda_status(cudaStreamSynchronize(s));
  if (rc != LETKF_OK) return rc;
  std::vector<int> todo;
  int64_t lmax = 0;
  for (int p = 0; p < npts; p++)
    if ((st[p] == LETKF_ERR_EIG || st[p] == LETKF_ERR_CAPACITY) && ho[p + 1] > ho[p]) {
      todo.push_back(p);
      lmax = std::max(lmax, ho[p + 1] - ho[p]);
    }
  if (todo.empty()) return LETKF_OK;
  cublasHandle_t hb = nullptr;
  if (cublasCreate(&hb) != CUBLAS_STATUS_SUCCESS) return LETKF_ERR_CUDA;
  cublasSetStream(hb, s);
  const size_t mat = (size_t)ne * ne;
  const int R = (int)std::min<size_t>(todo.size(), 32);  // points per group
  double *Bc = nullptr, *e64 = nullptr, *G = nullptr, *Y = nullptr, *Z = nullptr;
  double *T = nullptr, *M = nullptr, *Yn = nullptr, *Zn = nullptr, *bvec = nullptr, *sums = nullptr, *pinf = nullptr;
  int *active = nullptr, *which = nullptr;
  L64Point* pt = nullptr;
  bool okm = true;
  auto A = [&](auto** p, size_t bytes) { okm = okm && cudaMallocAsync((void**)p, bytes, s) == cudaSuccess; };
  A(&Bc, sizeof(double) * (size_t)lmax * ne);
  A(&e64, sizeof(double) * (size_t)lmax);
  for (double** p : {&G, &Y, &Z, &T, &M, &Yn, &Zn}) A(p, sizeof(double) * mat * R);
  A(&bvec, sizeof(double) * (size_t)ne * R);
  A(&sums, sizeof(double) * 2 * R);
  A(&pinf, sizeof(double) * R);
  A(&active, sizeof(int));
  A(&which, sizeof(int) * R);
  A(&pt, sizeof(L64Point) * R);
  rc = okm ? LETKF_OK : LETKF_ERR_CUDA;
  const double one = 1.0, zero = 0.0;
  for (size_t g0 = 0; g0 < todo.size() && rc == LETKF_OK; g0 += R) {
    const int nb = (int)std::min<size_t>(R, todo.size() - g0);
    cudaMemcpyAsync(which, todo.data() + g0, sizeof(int) * nb, cudaMemcpyHostToDevice, s);
    // 1. Gram, departure product and sums, one point at a time
    for (int j = 0; j < nb && rc == LETKF_OK; j++) {
      const int p = todo[g0 + j];
      const int64_t r0 = ho[p];
      const int L = (int)(ho[p + 1] - r0);
      const int64_t tot = (int64_t)L * ne;
      l64_gather_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(ne, L, r0, rows, rows16, ridx, rdiag, rloc,
                                                                       dep, rdiag_wloc, Bc, e64);
      l64_sums_kernel<<<1, L64_NT, 0, s>>>(L, r0, rloc, e64, sums + 2 * j);
      note_launch();
      note_launch();
      cudaMemcpyAsync(pinf + j, parm_infl + p, sizeof(double), cudaMemcpyDeviceToDevice, s);
      rc = cublas_status(cublasDgemm(hb, CUBLAS_OP_N, CUBLAS_OP_T, ne, ne, L, &one, Bc, ne, Bc, ne, &zero,
                                     G + (size_t)j * mat, ne));
      if (rc == LETKF_OK)
        rc = cublas_status(cublasDgemv(hb, CUBLAS_OP_N, ne, L, &one, Bc, ne, e64, 1, &zero, bvec + (size_t)j * ne, 1));
    }
    if (rc != LETKF_OK) break;
    // 2. A, s, Y0, Z0
    l64_prep_kernel<<<nb, L64_NT, 0, s>>>(ne, G, Y, Z, sums, pinf, minfl, pt);
    note_launch();
    // 3. coupled Newton-Schulz: T = Z Y, M = sqrt(a)(3I - aT)/2, Y <- Y M, Z <- M Z
    for (int it = 0; it < L64_NS_MAX && rc == LETKF_OK; it++) {
      rc = cublas_status(cublasDgemmStridedBatched(hb, CUBLAS_OP_N, CUBLAS_OP_N, ne, ne, ne, &one, Z, ne, mat, Y, ne,
                                                   mat, &zero, T, ne, mat, nb));
      if (rc != LETKF_OK) break;
      cudaMemsetAsync(active, 0, sizeof(int), s);
      l64_step_kernel<<<nb, L64_NT, 0, s>>>(ne, T, M, pt, active);
      note_launch();
      int h_active = 0;
      cudaMemcpyAsync(&h_active, active, sizeof(int), cudaMemcpyDeviceToHost, s);
      rc = cuda_status(cudaStreamSynchronize(s));
      if (rc != LETKF_OK || h_active == 0) break;
      rc = cublas_status(cublasDgemmStridedBatched(hb, CUBLAS_OP_N, CUBLAS_OP_N, ne, ne, ne, &one, Y, ne, mat, M, ne,
                                                   mat, &zero, Yn, ne, mat, nb));
      if (rc == LETKF_OK)
        rc = cublas_status(cublasDgemmStridedBatched(hb, CUBLAS_OP_N, CUBLAS_OP_N, ne, ne, ne, &one, M, ne, mat, Z,
                                                     ne, mat, &zero, Zn, ne, mat, nb));
      std::swap(Y, Yn);
      std::swap(Z, Zn);
    }
    if (rc != LETKF_OK) break;
    // 4. certificate against A: Q = Z (A Z), then W, wbar, inflation
    rc = cublas_status(cublasDgemmStridedBatched(hb, CUBLAS_OP_N, CUBLAS_OP_N, ne, ne, ne, &one, G, ne, mat, Z, ne,
                                                 mat, &zero, T, ne, mat, nb));
    if (rc == LETKF_OK)
      rc = cublas_status(cublasDgemmStridedBatched(hb, CUBLAS_OP_N, CUBLAS_OP_N, ne, ne, ne, &one, Z, ne, mat, T, ne,
                                                   mat, &zero, M, ne, mat, nb));
    if (rc != LETKF_OK) break;
    l64_finalize_kernel<<<nb, L64_NT, sizeof(double) * ne, s>>>(ne, M, Z, bvec, pt, which, parm_infl, trans, transm,
                                                                 status);
    note_launch();
    rc = cuda_status(cudaGetLastError());
  }
  const int rc2 = cuda_status(cudaStreamSynchronize(s));
  void* fr[] = {Bc, e64, G, Y, Z, T, M, Yn, Zn, bvec, sums, pinf, active, which, pt};
  for (void* p : fr)
    if (p) cudaFreeAsync(p, s);
  cublasDestroy(hb);
  return rc != LETKF_OK ? rc : rc2;
}

}  // namespace letkf
