// core_mixed.cu -- batched mixed-precision letkf_core on packed local rows.
//
// One CTA per point (persistent grid).  FP32 Gram on chip; the transform by
// spectrum-scaled Newton-Schulz (W = sqrt((k-1)/s) (A/s)^(-1/2),
// wbar = Z (Z b) / s) where mtx_eigen's truncation cannot act (c > 0 and
// tr(G) < 1e6 c) and the iteration converges, else the parallel Jacobi
// eigensolver with the reference's truncation; FP64 for the inflation sums.  Outputs FP32 trans / transm with
// the semantics of common/common_letkf.f90:50-243 (transm present: trans = T,
// transm = wbar; absent: trans = T + wbar 1^T).
#include "mixed_core.cuh"

namespace letkf {

template <int NP>
__global__ void __launch_bounds__(MixedCfg<NP>::NT) core_mixed_kernel(
    int n, int npts, const int64_t* __restrict__ offs, const float* __restrict__ rows,
    const float* __restrict__ rdiag, const float* __restrict__ rloc, const float* __restrict__ dep,
    double* parm_infl, float* trans, float* transm, int rdiag_wloc, double minfl, int* status, int max_sweeps,
    int use_ns) {
  using C = MixedCfg<NP>;
  using S = MixedSmem<NP>;
  extern __shared__ __align__(16) float sm[];
  const int tid = threadIdx.x;
  for (int p = blockIdx.x; p < npts; p += gridDim.x) {
    const int64_t r0 = offs[p];
    const int L = (int)(offs[p + 1] - r0);
    double infl = parm_infl[p];
    float* T = trans + (size_t)p * n * n;
    if (L == 0) {
      const float sq = (float)sqrt(infl);
      for (int idx = tid; idx < n * n; idx += C::NT) T[idx] = (idx / n == idx % n) ? sq : 0.f;
      if (transm)
        for (int i = tid; i < n; i += C::NT) transm[(size_t)p * n + i] = 0.f;
      if (tid == 0) status[p] = LETKF_OK;
      continue;
    }
    // Newton-Schulz first where it applies; a point it does not converge for
    // is done again with the eigensolver (its Gram recomputed: the iteration
    // overwrote A)
    bool try_ns = use_ns != 0;
  gram_again:
    GramAcc<NP> acc;
    acc.zero();
    for (int c0 = 0; c0 < L; c0 += S::CH) {
      const int nr = min(S::CH, L - c0);
      __syncthreads();
      for (int t = tid; t < S::CH * NP; t += C::NT) {
        const int r = t / NP, m = t - r * NP;
        sm[S::Y + t] = (r < nr && m < n) ? rows[(size_t)(r0 + c0 + r) * n + m] : 0.f;
      }
      if (tid < nr) {
        const float rd = rdiag[r0 + c0 + tid], rl = rloc[r0 + c0 + tid];
        sm[S::WR + tid] = rdiag_wloc ? 1.f / rd : rl / rd;
        sm[S::DR + tid] = dep[r0 + c0 + tid];
        sm[S::RL + tid] = rl;
      }
      __syncthreads();
      for (int t = tid; t < nr * NP; t += C::NT) sm[S::YW + t] = sm[S::Y + t] * sm[S::WR + t / NP];
      __syncthreads();
      gram_chunk<NP>(sm, nr, acc);
    }
    const double trace = gram_finish<NP>(sm, acc);
    if (minfl > 0.0 && infl < minfl) infl = minfl;
    const float c = (float)((double)(n - 1) / infl);
    for (int i = tid; i < NP; i += C::NT) sm[S::A + i * NP + i] += c;
    __syncthreads();
    if (try_ns && c > 0.f && trace < 1.0e6 * (double)c) {
      int its = 0;
      bool ok = false;
      const float s = ns_invsqrt<NP>(sm, c, 24, &its, 0.f, &ok);
      if (!ok) {
        try_ns = false;  // uniform over the CTA
        __syncthreads();
        goto gram_again;
      }
      const float* Z = sm + S::V;
      if (tid < NP) {
        float g = 0.f;
        for (int j = 0; j < NP; j++) g = fmaf(Z[j * NP + tid], sm[S::B + j], g);
        sm[S::G + tid] = g;
      }
      __syncthreads();
      if (tid < NP) {
        float w = 0.f;
        for (int j = 0; j < NP; j++) w = fmaf(Z[j * NP + tid], sm[S::G + j], w);
        sm[S::WB + tid] = w / s;
      }
      __syncthreads();
      const float coef = sqrtf((float)(n - 1) / s);
      const float* wb = sm + S::WB;
      const bool sep = transm != nullptr;
      for (int idx = tid; idx < n * n; idx += C::NT) {
        const int j = idx / n, i = idx - j * n;  // trans(i, j): background member i, analysis member j
        const float w = coef * Z[i * NP + j];
        T[idx] = sep ? w : w + wb[i];
      }
      if (sep)
        for (int i = tid; i < n; i += C::NT) transm[(size_t)p * n + i] = wb[i];
      if (tid == 0) {
        parm_infl[p] = infl_update(n, infl, acc.p1, trace, acc.p3);
        status[p] = LETKF_OK;
      }
      __syncthreads();
      continue;
    }
    jacobi_eig<NP>(sm, max_sweeps);
    const int st = eig_postprocess<NP>(sm, n);
    if (st != LETKF_OK) {
      for (int idx = tid; idx < n * n; idx += C::NT) T[idx] = NAN;
      if (tid == 0) status[p] = st;
      __syncthreads();
      continue;
    }
    const float* wb = sm + S::WB;
    const bool sep = transm != nullptr;
    form_w<NP>(sm, [&](int i, int j, float w) {
      if (i < n && j < n) T[(size_t)j * n + i] = sep ? w : w + wb[i];
    });
    if (sep)
      for (int i = tid; i < n; i += C::NT) transm[(size_t)p * n + i] = wb[i];
    if (tid == 0) {
      parm_infl[p] = infl_update(n, infl, acc.p1, trace, acc.p3);
      status[p] = LETKF_OK;
    }
    __syncthreads();
  }
}

template <int NP>
static int launch_mixed_np(int ne, int npts, const int64_t* offs, const float* rows, const float* rdiag,
                           const float* rloc, const float* dep, double* parm_infl, float* trans, float* transm,
                           int rdiag_wloc, double minfl, int* status, cudaStream_t stream) {
  // the Newton-Schulz product T sits after the Jacobi layout
  const size_t bytes = sizeof(float) * (size_t)NSSmem<NP>::TOTAL;
  auto kern = core_mixed_kernel<NP>;
  cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (err != cudaSuccess) return cuda_status(err);
  int dev = 0, nsm = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, MixedCfg<NP>::NT, bytes);
  if (per_sm < 1) per_sm = 1;
  int grid = nsm * per_sm;
  if (grid > npts) grid = npts;
  kern<<<grid, MixedCfg<NP>::NT, bytes, stream>>>(ne, npts, offs, rows, rdiag, rloc, dep, parm_infl, trans, transm,
                                                   rdiag_wloc, minfl, status, 12, 1);
  note_launch();
  return cuda_status(cudaGetLastError());
}

int launch_core_mixed(int ne, int npts, const int64_t* offs, const float* rows, const float* rdiag,
                      const float* rloc, const float* dep, double* parm_infl, float* trans, float* transm,
                      int rdiag_wloc, double minfl, int* status, cudaStream_t stream) {
  if (ne < 2 || npts < 0) return LETKF_ERR_ARG;
  if (ne > LETKF_MAX_NE) return LETKF_ERR_CAPACITY;
  if (npts == 0) return LETKF_OK;
  if (ne <= 32)
    return launch_mixed_np<32>(ne, npts, offs, rows, rdiag, rloc, dep, parm_infl, trans, transm, rdiag_wloc, minfl,
                               status, stream);
  if (ne <= 64)
    return launch_mixed_np<64>(ne, npts, offs, rows, rdiag, rloc, dep, parm_infl, trans, transm, rdiag_wloc, minfl,
                               status, stream);
  return launch_mixed_np<128>(ne, npts, offs, rows, rdiag, rloc, dep, parm_infl, trans, transm, rdiag_wloc, minfl,
                              status, stream);
}

}  // namespace letkf
