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

// ---------------------------------------------------------------------------
// Relaxed update of the SCALE driver (scale/letkf/letkf_tools.f90:215-268):
// per point and variable, W_rlx = RTPP (1-a) W + a I  (:1224-1237) or
// RTPS infl W with infl = a sqrt(var_g / (var_a (k-1))) - a + 1 (:1240-1268),
// T = (W_rlx + transm 1^T) beta + (1 - beta) I, xa = mean + xb' T; beta == 0
// leaves mean + xb'; optional clipping of the relative spread of one variable
// (Q_SPRD_MAX).  Each element is formed with the reference's operations in
// its order, so mode 0 with beta = 1 equals update_f64_kernel bit for bit.
namespace letkf {

struct RelaxArgs {
  int mode;           // 0 none, 1 RTPP, 2 RTPS
  double alpha;
  const double* beta; // [nv][npts] or NULL (1)
  int q_var;          // variable index of the spread clip, -1 none
  double q_sprd_max;  // <= 0: off
  double* rtps_infl;  // [nv][npts] or NULL
};

__global__ void __launch_bounds__(UPD_NT) update_relax_f64_kernel(int n, int npts, int nv, const double* __restrict__ xb,
                                                                   const double* __restrict__ trans,
                                                                   const double* __restrict__ transm,
                                                                   const double* __restrict__ pao, RelaxArgs r,
                                                                   double* xa) {
  extern __shared__ __align__(16) double su[];
  double* W = su;                  // n*n
  double* Pa = W + n * n;          // n*n (RTPS)
  double* tm = Pa + n * n;         // n
  double* xp = tm + n;             // nv*n
  double* mean = xp + nv * n;      // nv
  double* fac = mean + nv;         // nv: RTPS inflation
  double* bet = fac + nv;          // nv
  double* outv = bet + nv;         // nv*n analysis (for the spread clip)
  const int tid = threadIdx.x;
  for (int p = blockIdx.x; p < npts; p += gridDim.x) {
    __syncthreads();
    for (int idx = tid; idx < n * n; idx += UPD_NT) {
      W[idx] = trans[(size_t)p * n * n + idx];
      if (r.mode == 2) Pa[idx] = pao[(size_t)p * n * n + idx];
    }
    for (int k = tid; k < n; k += UPD_NT) tm[k] = transm ? transm[(size_t)p * n + k] : 0.0;
    for (int t = tid; t < nv * n; t += UPD_NT) {
      const int v = t / n, m = t - v * n;
      xp[t] = xb[((size_t)v * npts + p) * n + m];
    }
    __syncthreads();
    for (int v = tid; v < nv; v += UPD_NT) {
      double s = xp[v * n];
      for (int m = 1; m < n; m++) s = s + xp[v * n + m];
      mean[v] = s / (double)n;
      bet[v] = r.beta ? r.beta[(size_t)v * npts + p] : 1.0;
    }
    __syncthreads();
    for (int t = tid; t < nv * n; t += UPD_NT) xp[t] = xp[t] - mean[t / n];
    __syncthreads();
    // RTPS factor, one warp per variable: lanes split k so the Pa(k, m) reads of
    // a column are consecutive; beta == 0 skips weight_RTPS (factor 1)
    {
      const int lane = tid & 31;
      for (int v = tid >> 5; v < nv; v += UPD_NT / 32) {
        double f = 1.0;
        if (r.mode == 2 && bet[v] != 0.0) {
          const double* x = xp + v * n;
          double var_a = 0.0, var_g = 0.0;
          for (int m = 0; m < n; m++) {
            double part = 0.0;
            for (int k = lane; k < n; k += 32) part = part + x[k] * Pa[(size_t)m * n + k];
            var_a = var_a + part * x[m];
          }
          for (int m = lane; m < n; m += 32) var_g = var_g + x[m] * x[m];
          var_a = warp_sum(var_a);
          var_g = warp_sum(var_g);
          if (var_g > 0.0 && var_a > 0.0) f = r.alpha * sqrt(var_g / (var_a * (double)(n - 1))) - r.alpha + 1.0;
        }
        if (lane == 0) {
          if (r.mode == 2 && r.rtps_infl) r.rtps_infl[(size_t)v * npts + p] = f;
          fac[v] = f;
        }
      }
    }
    __syncthreads();
    for (int t = tid; t < nv * n; t += UPD_NT) {
      const int v = t / n, m = t - v * n;
      const double b = bet[v];
      double a = mean[v];
      if (b == 0.0) {
        a = a + xp[t];
      } else {
        for (int k = 0; k < n; k++) {
          double w = W[(size_t)m * n + k];
          if (r.mode == 1) {
            w = (1.0 - r.alpha) * w;
            if (k == m) w = w + r.alpha;
          } else if (r.mode == 2) {
            w = w * fac[v];
          }
          w = (w + tm[k]) * b;
          if (k == m) w = w + (1.0 - b);
          a = a + xp[v * n + k] * w;
        }
      }
      outv[t] = a;
    }
    __syncthreads();
    if (r.q_sprd_max > 0.0 && r.q_var >= 0 && r.q_var < nv && tid == 0) {
      double* q = outv + r.q_var * n;
      double qm = q[0];
      for (int m = 1; m < n; m++) qm = qm + q[m];
      qm = qm / (double)n;
      double sp = 0.0;
      for (int m = 0; m < n; m++) sp = sp + (q[m] - qm) * (q[m] - qm);
      sp = sqrt(sp / (double)(n - 1)) / qm;
      if (sp > r.q_sprd_max)
        for (int m = 0; m < n; m++) q[m] = qm + (q[m] - qm) * r.q_sprd_max / sp;
    }
    __syncthreads();
    for (int t = tid; t < nv * n; t += UPD_NT) {
      const int v = t / n, m = t - v * n;
      xa[((size_t)v * npts + p) * n + m] = outv[t];
    }
  }
}

// relax_beta (scale/letkf/letkf_tools.f90:1182-1220): 0 for the q variables
// above Q_UPDATE_TOP, the boundary-buffer ramp, else 1
__global__ void relax_beta_kernel(int npts, int nv, const double* __restrict__ ri, const double* __restrict__ rj,
                                  const double* __restrict__ rlev, int q_lo, int q_hi, double q_update_top,
                                  double bbw, double dx, double dy, int nlong, int nlatg, int ihalo, int jhalo,
                                  double* beta) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)npts * nv) return;
  const int v = (int)(t / npts), p = (int)(t - (int64_t)v * npts);
  double b = 1.0;
  if (rlev[p] < q_update_top && v >= q_lo && v <= q_hi) {
    beta[t] = 0.0;
    return;
  }
  if (bbw > 0.0) {
    const double d = fmin(fmin(ri[p] - ihalo, nlong + ihalo + 1 - ri[p]) * dx,
                          fmin(rj[p] - jhalo, nlatg + jhalo + 1 - rj[p]) * dy) / bbw;
    if (d < 1.0) b = fmax(d, 0.0);
  }
  beta[t] = b;
}

}  // namespace letkf

using namespace letkf;

extern "C" int letkf_update_relax_f64(int ne, int npts, int nv, const double* xb, const double* trans,
                                      const double* transm, const double* pao, const letkf_relax_desc* rd,
                                      double* xa, double* rtps_infl, void* stream) {
  if (ne < 2 || npts < 0 || nv < 1 || !xb || !trans || !xa || !rd) return LETKF_ERR_ARG;
  if (rd->mode < 0 || rd->mode > 2 || (rd->mode == 2 && !pao)) return LETKF_ERR_ARG;
  if (ne > LETKF_MAX_NE) return LETKF_ERR_CAPACITY;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return LETKF_ERR_NOGPU;
  }
  if (npts == 0) return LETKF_OK;
  RelaxArgs r;
  r.mode = rd->mode;
  r.alpha = rd->alpha;
  r.beta = rd->beta;
  r.q_var = rd->q_var;
  r.q_sprd_max = rd->q_sprd_max;
  r.rtps_infl = rtps_infl;
  const size_t smem = sizeof(double) * (2 * (size_t)ne * ne + ne + 2 * (size_t)nv * ne + 3 * (size_t)nv);
  cudaError_t err =
      cudaFuncSetAttribute(update_relax_f64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return cuda_status(err);
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int grid = npts < nsm * 8 ? npts : nsm * 8;
  update_relax_f64_kernel<<<grid, UPD_NT, smem, (cudaStream_t)stream>>>(ne, npts, nv, xb, trans, transm, pao, r, xa);
  note_launch();
  return cuda_status(cudaGetLastError());
}

extern "C" int letkf_relax_beta(int npts, int nv, const double* ri, const double* rj, const double* rlev, int q_lo,
                                int q_hi, double q_update_top, double boundary_buffer_width, double dx, double dy,
                                int nlong, int nlatg, int ihalo, int jhalo, double* beta, void* stream) {
  if (npts < 0 || nv < 1 || (npts > 0 && (!ri || !rj || !rlev || !beta))) return LETKF_ERR_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return LETKF_ERR_NOGPU;
  }
  const int64_t n = (int64_t)npts * nv;
  if (n == 0) return LETKF_OK;
  relax_beta_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      npts, nv, ri, rj, rlev, q_lo, q_hi, q_update_top, boundary_buffer_width, dx, dy, nlong, nlatg, ihalo, jhalo,
      beta);
  note_launch();
  return cuda_status(cudaGetLastError());
}
