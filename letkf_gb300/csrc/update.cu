// update.cu -- ensemble update with the analysis weights (FP64 plain form).
//
//   mean(p,v) = (x(p,1,v) + ... + x(p,ne,v)) / ne      speedy/common/common_speedy.f90:335-370
//   xa(p,m,v) = mean + sum_k (x(p,k,v) - mean) * (trans(k,m) + transm(k))
//                                                     speedy/letkf/letkf_tools.f90:164-170,
//                                                     scale/letkf/letkf_tools.f90:237-251 (beta = 1)
// One CTA per point; the sum over k runs in the reference order.
#include "letkf_common.cuh"

namespace letkf {

constexpr int UPD_NT = 128;

// Points p0 .. p0+cnt-1 of arrays holding npts_total points; trans / transm
// are indexed from p0.
__global__ void __launch_bounds__(UPD_NT) update_f64_kernel(int n, int npts_total, int p0, int cnt, int nv,
                                                             const double* __restrict__ xb,
                                                             const double* __restrict__ trans,
                                                             const double* __restrict__ transm, double* xa) {
  extern __shared__ __align__(16) double su[];
  double* W = su;            // n*n
  double* tm = W + n * n;    // n
  double* xp = tm + n;       // nv*n
  double* mean = xp + nv * n;  // nv
  const int tid = threadIdx.x;
  for (int pl = blockIdx.x; pl < cnt; pl += gridDim.x) {
    const int p = p0 + pl;
    __syncthreads();
    for (int idx = tid; idx < n * n; idx += UPD_NT) W[idx] = trans[(size_t)pl * n * n + idx];
    for (int k = tid; k < n; k += UPD_NT) tm[k] = transm ? transm[(size_t)pl * n + k] : 0.0;
    for (int t = tid; t < nv * n; t += UPD_NT) {
      const int v = t / n, m = t - v * n;
      xp[t] = xb[((size_t)v * npts_total + p) * n + m];
    }
    __syncthreads();
    for (int v = tid; v < nv; v += UPD_NT) {
      double s = xp[v * n];
      for (int m = 1; m < n; m++) s = s + xp[v * n + m];
      mean[v] = s / (double)n;
    }
    __syncthreads();
    for (int t = tid; t < nv * n; t += UPD_NT) xp[t] = xp[t] - mean[t / n];
    __syncthreads();
    for (int t = tid; t < nv * n; t += UPD_NT) {
      const int v = t / n, m = t - v * n;
      double a = mean[v];
      if (transm) {
        for (int k = 0; k < n; k++) a = a + xp[v * n + k] * (W[(size_t)m * n + k] + tm[k]);
      } else {
        for (int k = 0; k < n; k++) a = a + xp[v * n + k] * W[(size_t)m * n + k];
      }
      xa[((size_t)v * npts_total + p) * n + m] = a;
    }
  }
}

int launch_update_f64_range(int ne, int npts_total, int p0, int cnt, int nv, const double* xb, const double* trans,
                            const double* transm, double* xa, cudaStream_t stream) {
  if (ne < 2 || npts_total < 0 || p0 < 0 || cnt < 0 || p0 + cnt > npts_total || nv < 1) return LETKF_ERR_ARG;
  if (ne > LETKF_MAX_NE) return LETKF_ERR_CAPACITY;
  if (cnt == 0) return LETKF_OK;
  const int npts = cnt;
  const size_t smem = sizeof(double) * ((size_t)ne * ne + ne + (size_t)nv * ne + nv);
  cudaError_t err = cudaFuncSetAttribute(update_f64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return cuda_status(err);
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  int grid = nsm * 8;
  if (grid > npts) grid = npts;
  update_f64_kernel<<<grid, UPD_NT, smem, stream>>>(ne, npts_total, p0, cnt, nv, xb, trans, transm, xa);
  note_launch();
  return cuda_status(cudaGetLastError());
}

int launch_update_f64(int ne, int npts, int nv, const double* xb, const double* trans, const double* transm,
                      double* xa, cudaStream_t stream) {
  return launch_update_f64_range(ne, npts, 0, npts, nv, xb, trans, transm, xa, stream);
}

}  // namespace letkf
