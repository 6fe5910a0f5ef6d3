// obs_space.cu -- the obs-space clients of the batched core (GFS driver).
//
//  * letkf_obs_analysis: analysis ensemble at observation locations
//    (gfs/letkf/letkf_tools.f90:466-497): with trans the point's merged
//    transform (T + wbar 1^T, RTPP applied as weight_RTPP does, :959-970),
//    obsanal(n, m) = ybar(n) + sum_k obshdxf(n, k) trans(k, m), ybar =
//    obsdat - obsdep, the mean in member order, the q "no update" branch and
//    the relative-spread clip.
//  * letkf_efso: observation sensitivity (gfs/letkf/letkf_tools.f90:547-679)
//    over grid points with their local observation lists.
#include "letkf_common.cuh"

namespace letkf {

constexpr int OSA_NT = 128;
constexpr int EFSO_MAX_TERM = 8;
constexpr int EFSO_MAX_NV = 16;

__global__ void __launch_bounds__(OSA_NT) obs_analysis_kernel(int ne, int n, const double* __restrict__ trans,
                                                               const double* __restrict__ ybar,
                                                               const double* __restrict__ hdxf, double alpha,
                                                               const int* __restrict__ mode, double q_sprd_max,
                                                               double* anal, double* amean) {
  extern __shared__ double so[];
  double* h = so;         // [ne] obshdxf(n, :)
  double* a = so + ne;    // [ne] analysis members
  const int tid = threadIdx.x;
  for (int p = blockIdx.x; p < n; p += gridDim.x) {
    __syncthreads();
    for (int m = tid; m < ne; m += OSA_NT) h[m] = hdxf[(size_t)p * ne + m];
    __syncthreads();
    const int md = mode ? mode[p] : 0;
    const double yb = ybar[p];
    const double* tp = trans + (size_t)p * ne * ne;
    // thread per member m: it walks column m of trans (contiguous, stays in L1)
    for (int m = tid; m < ne; m += OSA_NT) {
      double v;
      if (md == 1) {
        v = yb + h[m];
      } else {
        v = yb;
        for (int k = 0; k < ne; k++) {
          double w = tp[(size_t)m * ne + k];
          if (alpha != 0.0) {
            w = (1.0 - alpha) * w;
            if (k == m) w = w + alpha;
          }
          v = v + h[k] * w;
        }
      }
      a[m] = v;
    }
    __syncthreads();
    if (tid == 0) {
      double s = 0.0;
      if (md == 1) {
        s = yb;
      } else {
        for (int m = 0; m < ne; m++) s = s + a[m];
        s = s / (double)ne;
        if (md == 2) {
          double sp = 0.0;
          for (int m = 0; m < ne; m++) sp = sp + (a[m] - s) * (a[m] - s);
          sp = sqrt(sp / (double)(ne - 1)) / s;
          if (sp > q_sprd_max)
            for (int m = 0; m < ne; m++) a[m] = s + (a[m] - s) * q_sprd_max / sp;
        }
      }
      if (amean) amean[p] = s;
    }
    __syncthreads();
    for (int m = tid; m < ne; m += OSA_NT) anal[(size_t)p * ne + m] = a[m];
  }
}

struct EfsoTerms {
  int term[EFSO_MAX_NV];
};

// one CTA per grid point: work1 in shared memory, one local observation per thread
__global__ void __launch_bounds__(OSA_NT) efso_djdy_kernel(int ne, int npts, int nv, int nterm, EfsoTerms tv,
                                                            const int64_t* __restrict__ offs,
                                                            const int* __restrict__ idx,
                                                            const double* __restrict__ rdiag,
                                                            const double* __restrict__ rloc,
                                                            const double* __restrict__ hdxa,
                                                            const double* __restrict__ fcst,
                                                            const double* __restrict__ fcer, double* djdy) {
  extern __shared__ double w1[];  // [nterm][ne]
  const int tid = threadIdx.x;
  for (int p = blockIdx.x; p < npts; p += gridDim.x) {
    const int64_t l0 = offs[p], l1 = offs[p + 1];
    if (l1 == l0) continue;
    __syncthreads();
    for (int i = tid; i < nterm * ne; i += OSA_NT) w1[i] = 0.0;
    __syncthreads();
    for (int m = tid; m < ne; m += OSA_NT)
      for (int v = 0; v < nv; v++) {
        const int t = tv.term[v];
        if (t < 0) continue;
        w1[t * ne + m] = w1[t * ne + m] + fcst[((size_t)v * npts + p) * ne + m] * fcer[(size_t)v * npts + p];
      }
    __syncthreads();
    for (int64_t l = l0 + tid; l < l1; l += OSA_NT) {
      const int ob = idx[l];
      const double rinv = 1.0 / rdiag[l], rl = rloc[l];  // one division per observation, not per member
      double acc[EFSO_MAX_TERM];
#pragma unroll
      for (int t = 0; t < EFSO_MAX_TERM; t++) acc[t] = 0.0;
      for (int m = 0; m < ne; m++) {
        const double hr = hdxa[(size_t)ob * ne + m] * rinv * rl;
#pragma unroll
        for (int t = 0; t < EFSO_MAX_TERM; t++)
          if (t < nterm) acc[t] = acc[t] + w1[t * ne + m] * hr;
      }
#pragma unroll
      for (int t = 0; t < EFSO_MAX_TERM; t++)
        if (t < nterm) atomicAdd(&djdy[(size_t)ob * nterm + t], acc[t]);
    }
  }
}

__global__ void efso_sense_kernel(int64_t n, int nterm, const double* __restrict__ djdy,
                                  const double* __restrict__ obsdep, double* obsense) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) obsense[i] = djdy[i] * obsdep[i / nterm];
}

static int grid_for(int n) {
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  return n < nsm * 8 ? n : nsm * 8;
}

static int have_device() {
  int nd = 0;
  if (cudaGetDeviceCount(&nd) != cudaSuccess || nd < 1) {
    cudaGetLastError();
    return 0;
  }
  return 1;
}

}  // namespace letkf

using namespace letkf;

extern "C" int letkf_obs_analysis(int ne, int n, const double* trans, const double* ybar, const double* hdxf,
                                  double relax_alpha, const int* mode, double q_sprd_max, double* anal,
                                  double* anal_mean, void* stream) {
  if (ne < 2 || ne > 4096 || n < 0 || (n > 0 && (!trans || !ybar || !hdxf || !anal))) return LETKF_ERR_ARG;
  if (!have_device()) return LETKF_ERR_NOGPU;
  if (n == 0) return LETKF_OK;
  const size_t smem = sizeof(double) * 2 * (size_t)ne;
  if (smem > 48 * 1024) {
    const cudaError_t e =
        cudaFuncSetAttribute(obs_analysis_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e);
  }
  obs_analysis_kernel<<<grid_for(n), OSA_NT, smem, (cudaStream_t)stream>>>(ne, n, trans, ybar, hdxf, relax_alpha,
                                                                            mode, q_sprd_max, anal, anal_mean);
  note_launch();
  return cuda_status(cudaGetLastError());
}

extern "C" int letkf_efso(int ne, int npts, int nv, int nterm, const int* term, const int64_t* offs, const int* idx,
                          const double* rdiag, const double* rloc, int nobs, const double* hdxa, const double* fcst,
                          const double* fcer, const double* obsdep, double* djdy, double* obsense, void* stream) {
  if (ne < 2 || npts < 0 || nv < 1 || nv > EFSO_MAX_NV || nterm < 1 || nterm > EFSO_MAX_TERM || nobs < 0 || !term)
    return LETKF_ERR_ARG;
  if (npts > 0 && (!offs || !fcst || !fcer)) return LETKF_ERR_ARG;
  if (nobs > 0 && (!hdxa || !obsdep || !djdy || !obsense)) return LETKF_ERR_ARG;
  EfsoTerms tv;
  for (int v = 0; v < EFSO_MAX_NV; v++) tv.term[v] = v < nv ? term[v] : -1;
  for (int v = 0; v < nv; v++)
    if (tv.term[v] >= nterm) return LETKF_ERR_ARG;
  if ((size_t)nterm * ne * sizeof(double) > 96 * 1024) return LETKF_ERR_CAPACITY;
  if (!have_device()) return LETKF_ERR_NOGPU;
  cudaStream_t s = (cudaStream_t)stream;
  if (nobs == 0) return LETKF_OK;
  int st = cuda_status(cudaMemsetAsync(djdy, 0, sizeof(double) * (size_t)nobs * nterm, s));
  if (st == LETKF_OK && npts > 0) {
    const size_t smem = sizeof(double) * (size_t)nterm * ne;
    if (smem > 48 * 1024) {
      const cudaError_t e =
          cudaFuncSetAttribute(efso_djdy_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return cuda_status(e);
    }
    efso_djdy_kernel<<<grid_for(npts), OSA_NT, smem, s>>>(ne, npts, nv, nterm, tv, offs, idx, rdiag, rloc, hdxa,
                                                          fcst, fcer, djdy);
    note_launch();
    st = cuda_status(cudaGetLastError());
  }
  if (st == LETKF_OK) {
    const int64_t tot = (int64_t)nobs * nterm;
    efso_sense_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(tot, nterm, djdy, obsdep, obsense);
    note_launch();
    st = cuda_status(cudaGetLastError());
  }
  return st;
}
