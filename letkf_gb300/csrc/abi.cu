// abi.cu -- extern "C" entry points of libletkf_gpu.so (declared in include/letkf_gpu.h).
#include <atomic>
#include <cstring>
#include <vector>

#include "letkf_common.cuh"

namespace letkf {

static std::atomic<int64_t> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
int cuda_status(cudaError_t e) { return e == cudaSuccess ? LETKF_OK : LETKF_ERR_CUDA; }

int launch_core_f64(int, int, const int64_t*, const double*, const double*, const double*, const double*, double*,
                    double*, double*, double*, int, double, int*, cudaStream_t);
int launch_core_mixed(int, int, const int64_t*, const float*, const float*, const float*, const float*, double*,
                      float*, float*, int, double, int*, cudaStream_t);
int launch_update_f64(int, int, int, const double*, const double*, const double*, double*, cudaStream_t);
int launch_search_scale(int, int, const int*, int, const double*, const double*, const double*, const double*,
                        const double*, const int*, const int*, int, const double*, const double*, const double*,
                        const double*, const double*, const double*, const int64_t*, int*, int*, double*, double*,
                        cudaStream_t);
int launch_search_speedy(int, int, const double*, const double*, const int*, int, const double*, const double*,
                         const double*, const double*, const double*, const double*, int, const double*,
                         const double*, const double*, const int*, const double*, const double*, const double*,
                         const int64_t*, int*, int*, double*, double*, cudaStream_t);
int launch_search_gfs(int nlon, int nlat, const double* lon, const double* lat, const int* G, const double* elm,
                      const double* olon, const double* olat, const double* olev, const double* odat,
                      const double* oerr, int npts, const double* plon, const double* plat, const double* prlev,
                      const double* var_local, const double* params, const int64_t* offs, int* nobsl, int* idx,
                      double* rloc, double* rdiag, cudaStream_t stream);
int launch_exclusive_scan(int, const int*, int64_t*, int64_t*, cudaStream_t);
int launch_gather_rows(int, int64_t, const int*, const void*, const void*, int, void*, void*, cudaStream_t);

static int have_gpu() {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n < 1) {
    cudaGetLastError();
    return 0;
  }
  return 1;
}

}  // namespace letkf

using namespace letkf;

extern "C" {

const char* letkf_version(void) { return "letkf_gb300 0.1 (sm_103a)"; }

const char* letkf_status_string(int s) {
  switch (s) {
    case LETKF_OK: return "ok";
    case LETKF_ERR_ARG: return "bad argument";
    case LETKF_ERR_EIG: return "eigensolver failure (rs ierr /= 0 or no positive eigenvalue)";
    case LETKF_ERR_CUDA: return "CUDA runtime error";
    case LETKF_ERR_CAPACITY: return "size beyond the library's limits";
    case LETKF_ERR_NOGPU: return "no CUDA device";
    case LETKF_ERR_TIMEOUT: return "bounded device wait timed out";
    case LETKF_PENDING: return "job not finished";
    default: return "unknown status";
  }
}

int64_t letkf_launch_count(void) { return g_launches.load(); }

int letkf_device_sync(void) {
  if (!have_gpu()) return LETKF_ERR_NOGPU;
  return cuda_status(cudaDeviceSynchronize());
}

int letkf_core_c(int ne, int nobs, int nobsl, const double* hdxb, const double* rdiag, const double* rloc,
                 const double* dep, double* parm_infl, double* trans, double* transm, double* pao, int rdiag_wloc,
                 double minfl) {
  if (ne < 2 || nobsl < 0 || nobs < nobsl || !parm_infl || !trans) return LETKF_ERR_ARG;
  if (nobsl > 0 && (!hdxb || !rdiag || !rloc || !dep)) return LETKF_ERR_ARG;
  if (ne > LETKF_MAX_NE) return LETKF_ERR_CAPACITY;
  if (!have_gpu()) return LETKF_ERR_NOGPU;
  const size_t L = (size_t)nobsl, K = (size_t)ne;
  // host staging: hdxb(1:nobsl, :) column-major -> rows [nobsl][ne]
  std::vector<double> hrows(L * K + 1);
  for (size_t m = 0; m < K; m++)
    for (size_t i = 0; i < L; i++) hrows[i * K + m] = hdxb[m * (size_t)nobs + i];
  const size_t nbytes = sizeof(double) * (L * K + 3 * L + 2 * K * K + K + 1) + sizeof(int64_t) * 2 + sizeof(int);
  char* dbuf = nullptr;
  cudaStream_t s = cudaStreamPerThread;
  if (cudaMallocAsync((void**)&dbuf, nbytes, s) != cudaSuccess) return LETKF_ERR_CUDA;
  double* d_rows = (double*)dbuf;
  double* d_rdiag = d_rows + L * K;
  double* d_rloc = d_rdiag + L;
  double* d_dep = d_rloc + L;
  double* d_trans = d_dep + L;
  double* d_pao = d_trans + K * K;
  double* d_transm = d_pao + K * K;
  double* d_infl = d_transm + K;
  int64_t* d_offs = (int64_t*)(d_infl + 1);
  int* d_status = (int*)(d_offs + 2);
  int64_t hoffs[2] = {0, (int64_t)L};
  int st = LETKF_OK;
  if (L) {
    cudaMemcpyAsync(d_rows, hrows.data(), sizeof(double) * L * K, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_rdiag, rdiag, sizeof(double) * L, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_rloc, rloc, sizeof(double) * L, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_dep, dep, sizeof(double) * L, cudaMemcpyHostToDevice, s);
  }
  cudaMemcpyAsync(d_infl, parm_infl, sizeof(double), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(d_offs, hoffs, sizeof(hoffs), cudaMemcpyHostToDevice, s);
  st = launch_core_f64(ne, 1, d_offs, d_rows, d_rdiag, d_rloc, d_dep, d_infl, d_trans, transm ? d_transm : nullptr,
                       pao ? d_pao : nullptr, rdiag_wloc, minfl, d_status, s);
  int hstatus = LETKF_OK;
  if (st == LETKF_OK) {
    cudaMemcpyAsync(trans, d_trans, sizeof(double) * K * K, cudaMemcpyDeviceToHost, s);
    if (transm) cudaMemcpyAsync(transm, d_transm, sizeof(double) * K, cudaMemcpyDeviceToHost, s);
    if (pao) cudaMemcpyAsync(pao, d_pao, sizeof(double) * K * K, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(parm_infl, d_infl, sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&hstatus, d_status, sizeof(int), cudaMemcpyDeviceToHost, s);
  }
  cudaFreeAsync(dbuf, s);
  cudaError_t e = cudaStreamSynchronize(s);
  if (st != LETKF_OK) return st;
  if (e != cudaSuccess) return LETKF_ERR_CUDA;
  return hstatus;
}

int letkf_core_batch_f64(int ne, int npts, const int64_t* offs, const double* rows, const double* rdiag,
                         const double* rloc, const double* dep, double* parm_infl, double* trans, double* transm,
                         double* pao, int rdiag_wloc, double minfl, int* status, void* stream) {
  if (!offs || !parm_infl || !trans || !status) return LETKF_ERR_ARG;
  if (!have_gpu()) return LETKF_ERR_NOGPU;
  return launch_core_f64(ne, npts, offs, rows, rdiag, rloc, dep, parm_infl, trans, transm, pao, rdiag_wloc, minfl,
                         status, (cudaStream_t)stream);
}

int letkf_core_batch_mixed(int ne, int npts, const int64_t* offs, const float* rows, const float* rdiag,
                           const float* rloc, const float* dep, double* parm_infl, float* trans, float* transm,
                           int rdiag_wloc, double minfl, int* status, void* stream) {
  if (!offs || !parm_infl || !trans || !status) return LETKF_ERR_ARG;
  if (!have_gpu()) return LETKF_ERR_NOGPU;
  return launch_core_mixed(ne, npts, offs, rows, rdiag, rloc, dep, parm_infl, trans, transm, rdiag_wloc, minfl,
                           status, (cudaStream_t)stream);
}

int letkf_update_f64(int ne, int npts, int nv, const double* xb, const double* trans, const double* transm,
                     double* xa, void* stream) {
  if (!xb || !trans || !xa) return LETKF_ERR_ARG;
  if (!have_gpu()) return LETKF_ERR_NOGPU;
  return launch_update_f64(ne, npts, nv, xb, trans, transm, xa, (cudaStream_t)stream);
}

int letkf_search_scale(int nlon, int nlat, const int* nobsgrd, int nobs, const double* ori, const double* orj,
                       const double* olev, const double* odat, const double* oerr, const int* ocls,
                       const int* ovarloc, int npts, const double* pri, const double* prj, const double* prlev,
                       const double* prz, const double* var_local_row, const double* params, const int64_t* offs,
                       int* nobsl, int* idx, double* rloc, double* rdiag, void* stream) {
  if (nlon < 1 || nlat < 1 || nobs < 0 || npts < 0 || !nobsgrd || !params) return LETKF_ERR_ARG;
  if (!idx && !nobsl) return LETKF_ERR_ARG;
  if (idx && (!offs || !rloc || !rdiag)) return LETKF_ERR_ARG;
  if (!have_gpu()) return LETKF_ERR_NOGPU;
  double hp[16];
  if (cudaMemcpy(hp, params, sizeof(double) * 15, cudaMemcpyDefault) != cudaSuccess) {
    memcpy(hp, params, sizeof(double) * 15);
    cudaGetLastError();
  }
  return launch_search_scale(nlon, nlat, nobsgrd, nobs, ori, orj, olev, odat, oerr, ocls, ovarloc, npts, pri, prj,
                             prlev, prz, var_local_row, hp, offs, nobsl, idx, rloc, rdiag, (cudaStream_t)stream);
}

int letkf_search_speedy(int nlon, int nlat, const double* lon, const double* lat, const int* nobsgrd, int nobs,
                        const double* obselm, const double* obslon, const double* obslat, const double* obslev,
                        const double* obsdat, const double* obserr, int npts, const double* plon, const double* plat,
                        const double* pdlon_zero, const int* pilev, const double* plogpfm,
                        const double* var_local_row, const double* params, const int64_t* offs, int* nobsl,
                        int* idx, double* rloc, double* rdiag, void* stream) {
  if (nlon < 2 || nlat < 3 || nobs < 0 || npts < 0 || !nobsgrd || !params || !var_local_row) return LETKF_ERR_ARG;
  if (!idx && !nobsl) return LETKF_ERR_ARG;
  if (idx && (!offs || !rloc || !rdiag)) return LETKF_ERR_ARG;
  if (!have_gpu()) return LETKF_ERR_NOGPU;
  double hp[5];
  if (cudaMemcpy(hp, params, sizeof(double) * 5, cudaMemcpyDefault) != cudaSuccess) {
    memcpy(hp, params, sizeof(double) * 5);
    cudaGetLastError();
  }
  return launch_search_speedy(nlon, nlat, lon, lat, nobsgrd, nobs, obselm, obslon, obslat, obslev, obsdat, obserr,
                              npts, plon, plat, pdlon_zero, pilev, plogpfm, var_local_row, hp, offs, nobsl, idx, rloc,
                              rdiag, (cudaStream_t)stream);
}

int letkf_search_gfs(int nlon, int nlat, const double* lon, const double* lat, const int* nobsgrd, int nobs,
                     const double* obselm, const double* obslon, const double* obslat, const double* obslev,
                     const double* obsdat, const double* obserr, int npts, const double* plon, const double* plat,
                     const double* prlev, const double* var_local_row, const double* params, const int64_t* offs,
                     int* nobsl, int* idx, double* rloc, double* rdiag, void* stream) {
  if (nlon < 2 || nlat < 3 || nobs < 0 || npts < 0 || !nobsgrd || !params) return LETKF_ERR_ARG;
  if (npts > 0 && (!plon || !plat || !prlev)) return LETKF_ERR_ARG;
  if (!idx && !nobsl) return LETKF_ERR_ARG;
  if (idx && (!offs || !rloc || !rdiag)) return LETKF_ERR_ARG;
  if (!have_gpu()) return LETKF_ERR_NOGPU;
  double hp[8];
  if (cudaMemcpy(hp, params, sizeof(double) * 8, cudaMemcpyDefault) != cudaSuccess) {
    memcpy(hp, params, sizeof(double) * 8);
    cudaGetLastError();
  }
  return launch_search_gfs(nlon, nlat, lon, lat, nobsgrd, obselm, obslon, obslat, obslev, obsdat, obserr, npts, plon,
                           plat, prlev, var_local_row, hp, offs, nobsl, idx, rloc, rdiag, (cudaStream_t)stream);
}

int letkf_exclusive_scan(int n, const int* counts, int64_t* offs, void* stream) {
  if (n < 0 || !offs || (n > 0 && !counts)) return LETKF_ERR_ARG;
  if (!have_gpu()) return LETKF_ERR_NOGPU;
  cudaStream_t s = (cudaStream_t)stream;
  const int nb = n > 0 ? (n + 1023) / 1024 : 1;
  int64_t* scratch = nullptr;
  if (cudaMallocAsync((void**)&scratch, sizeof(int64_t) * nb, s) != cudaSuccess) return LETKF_ERR_CUDA;
  int st = launch_exclusive_scan(n, counts, offs, scratch, s);
  cudaFreeAsync(scratch, s);
  return st;
}

int letkf_gather_rows(int ne, int64_t nrows, const int* idx, const void* ens, const void* dep, int elem_bytes,
                      void* rows_out, void* dep_out, void* stream) {
  if (ne < 1 || nrows < 0 || (nrows > 0 && (!idx || !ens || !rows_out))) return LETKF_ERR_ARG;
  if (!have_gpu()) return LETKF_ERR_NOGPU;
  return launch_gather_rows(ne, nrows, idx, ens, dep, elem_bytes, rows_out, dep_out, (cudaStream_t)stream);
}

}  // extern "C"
