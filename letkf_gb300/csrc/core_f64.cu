// core_f64.cu -- FP64 plain form of letkf_core on the GPU.
//
// One CTA per grid point (persistent over the batch).  The k x k work matrix
// lives in shared memory; the steps are those of common/common_letkf.f90:50-243:
//   hdxb_rinv weighting (:101-113) and the Gram DGEMM (:117) accumulated in
//   staged row chunks, covariance inflation on the diagonal (:125-138),
//   mtx_eigen (common/common_mtx.f90:41-99) as EISPACK tred2 + tql2
//   (common/netlibrs.f:520-683, :215-384) parallelised over the CTA, then
//   Pa, the symmetric square root T and the mean weights (:146-214) formed
//   from the eigenpairs on chip, and the adaptive inflation update (:218-239).
//
// Differences from the reference that only change rounding:
//   * the Gram and the dot products use FMA and per-thread summation order;
//   * wbar is formed as Pa (hdxb_rinv^T dep) instead of (Pa hdxb_rinv^T) dep;
//   * the eigenpairs are used unsorted (tql2's final selection sort only
//     permutes terms of sums that do not depend on the order).
// Truncated eigenpairs (lambda < lambda_max * sqrt(eps)) drop out of Pa and T,
// which is what the reference DGEMM's "IF (B(J,L).NE.ZERO)" skip makes of the
// zeroed eigenvectors.
#include <math.h>

#include "letkf_common.cuh"

namespace letkf {

constexpr int F64_NT = 256;  // threads per point
constexpr int F64_CH = 16;   // obs rows staged per chunk

__host__ __device__ inline size_t f64_smem_doubles(int n) {
  return (size_t)n * n + 7 * (size_t)n + 2 * (size_t)F64_CH * n + 3 * F64_CH + 32;
}

// EISPACK pythag (common/netlibrs.f:1-19)
__device__ double pythag_d(double a, double b) {
  double p = fmax(fabs(a), fabs(b));
  if (p == 0.0) return p;
  double r = fmin(fabs(a), fabs(b)) / p;
  r = r * r;
  for (int it = 0; it < 64; ++it) {
    double t = 4.0 + r;
    if (t == 4.0) break;
    double s = r / t;
    double u = 1.0 + 2.0 * s;
    p = u * p;
    r = (s / u) * (s / u) * r;
  }
  return p;
}

struct QLState {
  int l, j, m, phase;  // phase 0: new l, 1: iterate
  double f, tst1;
};

// Scalar part of tql2 (thread 0 only).  Advances to the next QL sweep, writes
// its rotations to cs[2*(i-1)], cs[2*(i-1)+1] (c, s) for i = l..m-1 and
// returns 1 with [lo, hi) = [l, m); returns 0 when done, -l on non-convergence.
__device__ int ql_advance(QLState& st, int n, double* d_, double* e_, double* cs, int& lo, int& hi) {
#define D(i) d_[(i)-1]
#define E(i) e_[(i)-1]
  for (;;) {
    if (st.phase == 0) {
      if (st.l > n) return 0;
      const int l = st.l;
      st.j = 0;
      double h = fabs(D(l)) + fabs(E(l));
      if (st.tst1 < h) st.tst1 = h;
      int m;
      for (m = l; m <= n; m++) {
        double tst2 = st.tst1 + fabs(E(m));
        if (tst2 == st.tst1) break;
      }
      if (m > n) m = n;
      st.m = m;
      if (m == l) {
        D(l) = D(l) + st.f;
        st.l++;
        continue;
      }
      st.phase = 1;
    }
    // one QL iteration on [l, m]
    const int l = st.l, m = st.m;
    if (st.j == 30) return -l;
    st.j++;
    const int l1 = l + 1, l2 = l1 + 1;
    double g = D(l);
    double p = (D(l1) - g) / (2.0 * E(l));
    double r = pythag_d(p, 1.0);
    D(l) = E(l) / (p + fsign(r, p));
    D(l1) = E(l) * (p + fsign(r, p));
    const double dl1 = D(l1);
    double h = g - D(l);
    for (int i = l2; i <= n; i++) D(i) = D(i) - h;
    st.f = st.f + h;
    p = D(m);
    double c = 1.0, c2 = c, c3 = c, s = 0.0, s2 = 0.0;
    const double el1 = E(l1);
    for (int i = m - 1; i >= l; i--) {
      c3 = c2;
      c2 = c;
      s2 = s;
      g = c * E(i);
      h = c * p;
      r = pythag_d(p, E(i));
      E(i + 1) = s * r;
      s = E(i) / r;
      c = p / r;
      p = c * D(i) - s * g;
      D(i + 1) = h + s * (c * g + s * D(i));
      cs[2 * (i - 1)] = c;
      cs[2 * (i - 1) + 1] = s;
    }
    p = -s * s2 * c3 * el1 * E(l) / dl1;
    E(l) = s * p;
    D(l) = c * p;
    lo = l;
    hi = m;
    double tst2 = st.tst1 + fabs(E(l));
    if (!(tst2 > st.tst1)) {
      D(l) = D(l) + st.f;
      st.l++;
      st.phase = 0;
    }
    return 1;
  }
#undef D
#undef E
}

__global__ void __launch_bounds__(F64_NT) core_f64_kernel(int n, int npts, const int64_t* __restrict__ offs,
                                                           const double* __restrict__ rows,
                                                           const double* __restrict__ rdiag,
                                                           const double* __restrict__ rloc,
                                                           const double* __restrict__ dep, double* parm_infl,
                                                           double* trans, double* transm, double* pao,
                                                           int rdiag_wloc, double minfl, int* status) {
  extern __shared__ __align__(16) double sm[];
  double* Zm = sm;               // n*n, column-major, ld = n
  double* d = Zm + n * n;        // n
  double* e = d + n;             // n
  double* g = e + n;             // n
  double* bv = g + n;            // n   hdxb_rinv^T dep
  double* cs = bv + n;           // 2n  rotation log
  double* fq = cs + 2 * n;       // n   per-eigenpair factor
  double* Yc = fq + n;           // CH*n staged rows
  double* Yw = Yc + F64_CH * n;  // CH*n weighted rows
  double* wr = Yw + F64_CH * n;  // CH
  double* dr = wr + F64_CH;      // CH
  double* rl = dr + F64_CH;      // CH
  double* red = rl + F64_CH;     // 32
  __shared__ double sc[4];
  __shared__ int cmd[3];
  const int tid = threadIdx.x;
#define Z(i, j) Zm[(size_t)((j)-1) * n + ((i)-1)]
#define D(i) d[(i)-1]
#define E(i) e[(i)-1]

  for (int p = blockIdx.x; p < npts; p += gridDim.x) {
    const int64_t r0 = offs[p];
    const int L = (int)(offs[p + 1] - r0);
    double infl = parm_infl[p];
    double* T = trans + (size_t)p * n * n;
    if (L == 0) {  // common_letkf.f90:82-96
      const double sq = sqrt(infl);
      for (int idx = tid; idx < n * n; idx += F64_NT) {
        int j = idx / n, i = idx - j * n;
        T[idx] = (i == j) ? sq : 0.0;
        if (pao) pao[(size_t)p * n * n + idx] = (i == j) ? infl / (double)(n - 1) : 0.0;
      }
      if (transm)
        for (int i = tid; i < n; i += F64_NT) transm[(size_t)p * n + i] = 0.0;
      if (tid == 0) status[p] = LETKF_OK;
      continue;
    }
    // ---- weighting + Gram (lower triangle) + hdxb_rinv^T dep ----
    for (int idx = tid; idx < n * n; idx += F64_NT) Zm[idx] = 0.0;
    double bacc = 0.0, p1 = 0.0, p3 = 0.0;
    for (int c0 = 0; c0 < L; c0 += F64_CH) {
      const int nr = min(F64_CH, L - c0);
      __syncthreads();
      const double* src = rows + (size_t)(r0 + c0) * n;
      for (int t = tid; t < nr * n; t += F64_NT) Yc[t] = src[t];
      if (tid < nr) {
        const double rd = rdiag[r0 + c0 + tid], rlc = rloc[r0 + c0 + tid];
        wr[tid] = rdiag_wloc ? 1.0 / rd : rlc / rd;
        dr[tid] = dep[r0 + c0 + tid];
        rl[tid] = rlc;
      }
      __syncthreads();
      for (int t = tid; t < nr * n; t += F64_NT) Yw[t] = Yc[t] * wr[t / n];
      __syncthreads();
      for (int idx = tid; idx < n * n; idx += F64_NT) {
        const int j = idx / n, i = idx - j * n;
        if (i < j) continue;
        double acc = Zm[idx];
        for (int r = 0; r < nr; r++) acc = fma(Yw[r * n + i], Yc[r * n + j], acc);
        Zm[idx] = acc;
      }
      if (tid < n)
        for (int r = 0; r < nr; r++) bacc = fma(Yw[r * n + tid], dr[r], bacc);
      if (tid == 0)
        for (int r = 0; r < nr; r++) {
          p1 = p1 + dr[r] * dr[r] * wr[r];
          p3 = p3 + rl[r];
        }
    }
    if (tid < n) bv[tid] = bacc;
    __syncthreads();
    // ---- inflation on the diagonal (:125-138); p2 = trace(Gram)/(ne-1) ----
    double p2 = 0.0;
    for (int i = tid; i < n; i += F64_NT) p2 += Zm[(size_t)i * n + i];
    p2 = block_sum<double, F64_NT>(p2, red);
    if (minfl > 0.0 && infl < minfl) infl = minfl;
    {
      const double rho = 1.0 / infl;
      for (int i = tid; i < n; i += F64_NT) Zm[(size_t)i * n + i] += (double)(n - 1) * rho;
    }
    __syncthreads();
    // ---- tred2 ----
    for (int i = tid + 1; i <= n; i += F64_NT) D(i) = Z(n, i);
    __syncthreads();
    if (n != 1) {
      for (int ii = 2; ii <= n; ii++) {
        const int i = n + 2 - ii, l = i - 1;
        double h = 0.0, scale = 0.0;
        if (l >= 2) {
          double s = 0.0;
          for (int k = tid + 1; k <= l; k += F64_NT) s += fabs(D(k));
          scale = block_sum<double, F64_NT>(s, red);
        }
        if (l < 2 || scale == 0.0) {
          if (tid == 0) E(i) = D(l);
          __syncthreads();
          for (int j = tid + 1; j <= l; j += F64_NT) {
            D(j) = Z(l, j);
            Z(i, j) = 0.0;
            Z(j, i) = 0.0;
          }
        } else {
          double s = 0.0;
          for (int k = tid + 1; k <= l; k += F64_NT) {
            const double v = D(k) / scale;
            D(k) = v;
            s += v * v;
          }
          h = block_sum<double, F64_NT>(s, red);  // syncs: D(k) visible
          const double f = D(l);
          const double gg = -fsign(sqrt(h), f);
          h = h - f * gg;
          __syncthreads();
          if (tid == 0) {
            E(i) = scale * gg;
            D(l) = f - gg;
          }
          __syncthreads();
          // form a*u into g(j); store u in column i
          for (int j = tid + 1; j <= l; j += F64_NT) {
            double acc = 0.0;
            for (int k = 1; k <= j; k++) acc = fma(Z(j, k), D(k), acc);
            for (int k = j + 1; k <= l; k++) acc = fma(Z(k, j), D(k), acc);
            g[j - 1] = acc;
            Z(j, i) = D(j);
          }
          __syncthreads();
          double fs = 0.0;
          for (int j = tid + 1; j <= l; j += F64_NT) {
            const double v = g[j - 1] / h;
            E(j) = v;
            fs += v * D(j);
          }
          fs = block_sum<double, F64_NT>(fs, red);
          const double hh = fs / (h + h);
          for (int j = tid + 1; j <= l; j += F64_NT) E(j) = E(j) - hh * D(j);
          __syncthreads();
          // reduced a (lower triangle 1 <= j <= k <= l)
          for (int idx = tid; idx < l * l; idx += F64_NT) {
            const int j = idx / l + 1, k = idx - (j - 1) * l + 1;
            if (k < j) continue;
            Z(k, j) = Z(k, j) - D(j) * E(k) - E(j) * D(k);
          }
          __syncthreads();
          for (int j = tid + 1; j <= l; j += F64_NT) {
            D(j) = Z(l, j);
            Z(i, j) = 0.0;
          }
        }
        __syncthreads();
        if (tid == 0) D(i) = h;
        __syncthreads();
      }
      // accumulation of transformation matrices
      for (int i = 2; i <= n; i++) {
        const int l = i - 1;
        if (tid == 0) {
          Z(n, l) = Z(l, l);
          Z(l, l) = 1.0;
        }
        __syncthreads();
        const double h = D(i);
        if (h != 0.0) {
          for (int k = tid + 1; k <= l; k += F64_NT) D(k) = Z(k, i) / h;
          for (int j = tid + 1; j <= l; j += F64_NT) {
            double acc = 0.0;
            for (int k = 1; k <= l; k++) acc = fma(Z(k, i), Z(k, j), acc);
            g[j - 1] = acc;
          }
          __syncthreads();
          for (int idx = tid; idx < l * l; idx += F64_NT) {
            const int j = idx / l + 1, k = idx - (j - 1) * l + 1;
            Z(k, j) = Z(k, j) - g[j - 1] * D(k);
          }
          __syncthreads();
        }
        for (int k = tid + 1; k <= l; k += F64_NT) Z(k, i) = 0.0;
        __syncthreads();
      }
    }
    for (int i = tid + 1; i <= n; i += F64_NT) D(i) = Z(n, i);
    __syncthreads();
    for (int i = tid + 1; i <= n; i += F64_NT) Z(n, i) = 0.0;
    __syncthreads();
    if (tid == 0) {
      Z(n, n) = 1.0;
      E(1) = 0.0;
    }
    __syncthreads();
    // ---- tql2: scalar chain on thread 0, rotations applied by rows ----
    if (tid == 0) {
      for (int i = 2; i <= n; i++) E(i - 1) = E(i);
      E(n) = 0.0;
    }
    QLState st;
    st.l = 1;
    st.j = 0;
    st.m = 1;
    st.phase = 0;
    st.f = 0.0;
    st.tst1 = 0.0;
    int eig_err = 0;
    for (;;) {
      if (tid == 0) {
        int lo = 0, hi = 0;
        int r = (n == 1) ? 0 : ql_advance(st, n, d, e, cs, lo, hi);
        cmd[0] = r;
        cmd[1] = lo;
        cmd[2] = hi;
      }
      __syncthreads();
      const int r = cmd[0], lo = cmd[1], hi = cmd[2];
      if (r <= 0) {
        eig_err = r < 0;
        break;
      }
      for (int row = tid + 1; row <= n; row += F64_NT) {
        double zi1 = Z(row, hi);
        for (int i = hi - 1; i >= lo; i--) {
          const double c = cs[2 * (i - 1)], s = cs[2 * (i - 1) + 1];
          const double zi = Z(row, i);
          Z(row, i + 1) = s * zi + c * zi1;
          zi1 = c * zi - s * zi1;
        }
        Z(row, lo) = zi1;
      }
      __syncthreads();
    }
    __syncthreads();
    // ---- mtx_eigen truncation test (common_mtx.f90:66-78) ----
    double lmax = -INFINITY;
    for (int i = tid; i < n; i += F64_NT) lmax = fmax(lmax, d[i]);
    {
      lmax = warp_max(lmax);
      __syncthreads();
      if ((tid & 31) == 0) red[tid >> 5] = lmax;
      __syncthreads();
      if (tid == 0) {
        double mx = red[0];
        for (int w = 1; w < F64_NT / 32; w++) mx = fmax(mx, red[w]);
        sc[0] = mx;
      }
      __syncthreads();
      lmax = sc[0];
    }
    if (eig_err || !(lmax > 0.0)) {
      for (int idx = tid; idx < n * n; idx += F64_NT) T[idx] = NAN;
      if (tid == 0) status[p] = LETKF_ERR_EIG;
      __syncthreads();
      continue;
    }
    const double thr = fabs(lmax) * 1.4901161193847656e-08;  // sqrt(EPSILON(1d0))
    // fq = sqrt((ne-1)/lambda), cs[q] = 1/lambda (0 when truncated)
    for (int q = tid; q < n; q += F64_NT) {
      const double lam = d[q];
      const bool keep = !(lam < thr);
      fq[q] = keep ? sqrt((double)(n - 1) / lam) : 0.0;
      cs[q] = keep ? 1.0 / lam : 0.0;
    }
    __syncthreads();
    // g = diag(1/lambda) V^T b
    for (int q = tid; q < n; q += F64_NT) {
      double acc = 0.0;
      for (int i = 0; i < n; i++) acc = fma(Zm[(size_t)q * n + i], bv[i], acc);
      g[q] = acc * cs[q];
    }
    __syncthreads();
    // wbar = V g  (into e)
    for (int i = tid; i < n; i += F64_NT) {
      double acc = 0.0;
      for (int q = 0; q < n; q++) acc = fma(Zm[(size_t)q * n + i], g[q], acc);
      e[i] = acc;
    }
    __syncthreads();
    // T = V diag(fq) V^T (+ wbar), Pa = V diag(1/lambda) V^T
    for (int idx = tid; idx < n * n; idx += F64_NT) {
      const int j = idx / n, i = idx - j * n;
      double acc = 0.0, pacc = 0.0;
      for (int q = 0; q < n; q++) {
        const double vv = Zm[(size_t)q * n + i] * Zm[(size_t)q * n + j];
        acc = fma(vv, fq[q], acc);
        pacc = fma(vv, cs[q], pacc);
      }
      T[idx] = transm ? acc : acc + e[i];
      if (pao) pao[(size_t)p * n * n + idx] = pacc;
    }
    if (transm)
      for (int i = tid; i < n; i += F64_NT) transm[(size_t)p * n + i] = e[i];
    // ---- adaptive inflation (:218-239) ----
    if (tid == 0) {
      const double q2 = p2 / (double)(n - 1);
      const double q4 = (p1 - p3) / q2 - infl;
      const double t = (infl * q2 + p3) / q2;
      const double sigma_o = 2.0 / p3 * (t * t);
      const double gain = (kSigmaB * kSigmaB) / (sigma_o + kSigmaB * kSigmaB);
      parm_infl[p] = infl + gain * q4;
      status[p] = LETKF_OK;
    }
    __syncthreads();
  }
#undef Z
#undef D
#undef E
}

int launch_core_f64(int ne, int npts, const int64_t* offs, const double* rows, const double* rdiag,
                    const double* rloc, const double* dep, double* parm_infl, double* trans, double* transm,
                    double* pao, int rdiag_wloc, double minfl, int* status, cudaStream_t stream) {
  if (ne < 2 || ne > LETKF_MAX_NE || npts < 0) return ne > LETKF_MAX_NE ? LETKF_ERR_CAPACITY : LETKF_ERR_ARG;
  if (npts == 0) return LETKF_OK;
  const size_t smem = f64_smem_doubles(ne) * sizeof(double);
  cudaError_t err = cudaFuncSetAttribute(core_f64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return cuda_status(err);
  int dev = 0, nsm = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, core_f64_kernel, F64_NT, smem);
  if (per_sm < 1) per_sm = 1;
  int grid = nsm * per_sm;
  if (grid > npts) grid = npts;
  core_f64_kernel<<<grid, F64_NT, smem, stream>>>(ne, npts, offs, rows, rdiag, rloc, dep, parm_infl, trans, transm,
                                                   pao, rdiag_wloc, minfl, status);
  note_launch();
  return cuda_status(cudaGetLastError());
}

}  // namespace letkf
