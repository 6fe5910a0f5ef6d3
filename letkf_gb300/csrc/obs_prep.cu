// obs_prep.cu -- observation-space departures and perturbations on the device
// (speedy/letkf/letkf_obs.f90:157-174; lorenz96/letkf/letkf.f90:196-212).
//
// Per observation n: mean = (hx(n,1) + ... + hx(n,ne)) / ne summed in member
// order in FP64, hdxf(n,:) = hx(n,:) - mean, dep(n) = y(n) - mean, and the
// gross-error check |dep| > gross_error * err rejects it (qc = 0).  A block
// stages 32 observations' member rows through shared memory so the row reads
// and writes are coalesced while each mean keeps the reference's order.
#include <cuda_runtime.h>
#include <stdint.h>

#include "letkf_gpu.h"

namespace letkf {

int cuda_status(cudaError_t e);
void note_launch();

constexpr int DEP_OBS = 32;
constexpr int DEP_NT = 128;

__global__ void __launch_bounds__(DEP_NT) obs_departure_kernel(int ne, int nobs, const double* __restrict__ hx,
                                                               const double* __restrict__ y,
                                                               const double* __restrict__ err, double gross,
                                                               const int* __restrict__ qc_in,
                                                               double* __restrict__ hdxf, double* __restrict__ dep,
                                                               int* __restrict__ qc_out) {
  extern __shared__ double rows[];  // [DEP_OBS][ne]
  __shared__ double mean[DEP_OBS];
  __shared__ int ok[DEP_OBS];
  const int o0 = blockIdx.x * DEP_OBS;
  const int nrow = min(DEP_OBS, nobs - o0);
  const size_t base = (size_t)o0 * ne;
  const int total = nrow * ne;
  for (int t = threadIdx.x; t < total; t += DEP_NT) rows[t] = hx[base + t];
  __syncthreads();
  if (threadIdx.x < nrow) {
    const int r = threadIdx.x, n = o0 + r;
    const int q = qc_in ? qc_in[n] : 1;
    ok[r] = q == 1;
    double s = rows[(size_t)r * ne];
    for (int m = 1; m < ne; m++) s = s + rows[(size_t)r * ne + m];
    s = s / (double)ne;
    mean[r] = s;
    if (q == 1) {
      const double d = y[n] - s;
      dep[n] = d;
      int qo = 1;
      if (gross > 0.0 && fabs(d) > gross * err[n]) qo = 0;
      if (qc_out) qc_out[n] = qo;
    } else {
      dep[n] = 0.0;  // not assimilated (the reference skips it)
      if (qc_out) qc_out[n] = 0;
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < total; t += DEP_NT) {
    const int r = t / ne;
    hdxf[base + t] = ok[r] ? rows[t] - mean[r] : rows[t];
  }
}

}  // namespace letkf

using namespace letkf;

extern "C" int letkf_obs_departure(int ne, int nobs, const double* hx, const double* y, const double* err,
                                   double gross_error, const int* qc_in, double* hdxf, double* dep, int* qc_out,
                                   void* stream) {
  if (ne < 1 || ne > 512 || nobs < 0) return LETKF_ERR_ARG;
  if (nobs > 0 && (!hx || !y || !hdxf || !dep || (gross_error > 0.0 && !err))) return LETKF_ERR_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return LETKF_ERR_NOGPU;
  }
  if (nobs == 0) return LETKF_OK;
  const size_t smem = sizeof(double) * DEP_OBS * (size_t)ne;
  if (smem > 48 * 1024) {
    if (cudaFuncSetAttribute(obs_departure_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
      return LETKF_ERR_CUDA;
  }
  obs_departure_kernel<<<(nobs + DEP_OBS - 1) / DEP_OBS, DEP_NT, smem, (cudaStream_t)stream>>>(
      ne, nobs, hx, y, err, gross_error, qc_in, hdxf, dep, qc_out);
  note_launch();
  return cuda_status(cudaGetLastError());
}
