// search_limit.cu -- MAX_NOBS_PER_GRID selection of the SCALE search.
//
// scale/letkf/letkf_tools.f90:1041-1156: with MAX_NOBS_PER_GRID = M > 0 the
// SCALE obs_local keeps, per (element uid, obs type) group, the M accepted
// observations of smallest rdiag = err^2 / rloc, by an insertion sort into M
// slots, and emits them grouped by type then element, each group in slot order.
// The insertion rules make the kept set the M smallest keys (rdiag, arrival)
// of the group (ties keep the earlier observation), the first M arrivals take
// slots 1..M in order, and a later arrival that enters takes the slot of the
// element it evicts (the largest key).  Here one thread per point replays that
// with a max-heap keyed by (rdiag, arrival) whose entries carry their slot,
// over the point's unlimited list (the plain search's output, in candidate
// order); the heap lives in shared memory, one region of M entries per thread.
#include <climits>
#include <cstring>

#include "letkf_common.cuh"

namespace letkf {

int launch_exclusive_scan(int, const int*, int64_t*, int64_t*, cudaStream_t);

struct LimEntry {
  double r, rl;  // rdiag, rloc
  int t, slot, ob, pad;
};

__device__ __forceinline__ bool lim_gt(const LimEntry& a, const LimEntry& b) {
  return a.r > b.r || (a.r == b.r && a.t > b.t);
}

// Count pass (loffs == NULL): lcount[p] = sum over groups of min(n_g, M).
// Fill pass: the selected entries at loffs[p] .., grouped by ascending group
// key, each group in slot order.
__global__ void limit_select_kernel(int npts, const int64_t* __restrict__ uoffs, const int* __restrict__ uidx,
                                    const double* __restrict__ urloc, const double* __restrict__ urdiag,
                                    const int* __restrict__ ogrp, int M, const int64_t* __restrict__ loffs,
                                    int* lcount, int* lidx, double* lrloc, double* lrdiag) {
  extern __shared__ __align__(16) unsigned char lim_sm[];
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npts) return;
  LimEntry* H = reinterpret_cast<LimEntry*>(lim_sm) + (size_t)threadIdx.x * M;
  const int64_t u0 = uoffs[p], u1 = uoffs[p + 1];
  int64_t out = 0;
  const int64_t base = loffs ? loffs[p] : 0;
  int cur = INT_MIN;
  for (;;) {
    int nxt = INT_MAX;
    for (int64_t e = u0; e < u1; e++) {
      const int k = ogrp[uidx[e]];
      if (k > cur && k < nxt) nxt = k;
    }
    if (nxt == INT_MAX) break;
    if (!loffs) {
      int ng = 0;
      for (int64_t e = u0; e < u1; e++) ng += ogrp[uidx[e]] == nxt;
      out += ng < M ? ng : M;
    } else {
      int hn = 0, t = 0;
      for (int64_t e = u0; e < u1; e++) {
        const int ob = uidx[e];
        if (ogrp[ob] != nxt) continue;
        LimEntry x;
        x.r = urdiag[e];
        x.rl = urloc[e];
        x.t = t++;
        x.ob = ob;
        x.pad = 0;
        if (hn < M) {
          // letkf_tools.f90:1068-1106 with nobsl_t < M: slot nobsl_t + 1
          x.slot = hn;
          int i = hn++;
          while (i > 0) {
            const int up = (i - 1) >> 1;
            if (!lim_gt(x, H[up])) break;
            H[i] = H[up];
            i = up;
          }
          H[i] = x;
        } else if (x.r < H[0].r) {
          // :1108-1124: the largest key leaves, its slot is reused
          x.slot = H[0].slot;
          int i = 0;
          for (;;) {
            const int c0 = 2 * i + 1, c1 = c0 + 1;
            if (c0 >= hn) break;
            const int c = (c1 < hn && lim_gt(H[c1], H[c0])) ? c1 : c0;
            if (!lim_gt(H[c], x)) break;
            H[i] = H[c];
            i = c;
          }
          H[i] = x;
        }  // else :1063-1066, skipped (rdiag >= the largest kept)
      }
      for (int i = 0; i < hn; i++) {
        const int64_t at = base + out + H[i].slot;
        lidx[at] = H[i].ob;
        lrloc[at] = H[i].rl;
        lrdiag[at] = H[i].r;
      }
      out += hn;
    }
    cur = nxt;
  }
  if (!loffs) lcount[p] = (int)out;
}

static int limit_block(int M) {
  int bs = (int)(96 * 1024 / ((size_t)M * sizeof(LimEntry)));
  return bs < 1 ? 1 : (bs > 32 ? 32 : bs);
}

int launch_limit_select(int npts, const int64_t* uoffs, const int* uidx, const double* urloc, const double* urdiag,
                        const int* ogrp, int M, const int64_t* loffs, int* lcount, int* lidx, double* lrloc,
                        double* lrdiag, cudaStream_t s) {
  if (npts <= 0) return LETKF_OK;
  if (M < 1 || M > LETKF_MAX_NOBS_PER_GRID_LIMIT) return LETKF_ERR_CAPACITY;
  const int bs = limit_block(M);
  const size_t smem = (size_t)bs * M * sizeof(LimEntry);
  cudaError_t e = cudaFuncSetAttribute(limit_select_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_status(e);
  limit_select_kernel<<<(npts + bs - 1) / bs, bs, smem, s>>>(npts, uoffs, uidx, urloc, urdiag, ogrp, M, loffs, lcount,
                                                             lidx, lrloc, lrdiag);
  note_launch();
  return cuda_status(cudaGetLastError());
}

// ogrp[n] = (typ[n] - 1) * nid + (uid[n] - 1): the emission order of
// letkf_tools.f90:1141-1156 (types outer, elements inner)
__global__ void obs_group_kernel(int nobs, const int* __restrict__ uid, const int* __restrict__ typ, int nid,
                                 const int* __restrict__ perm, int* ogrp) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nobs) return;
  const int src = perm ? perm[n] : n;
  ogrp[n] = (typ[src] - 1) * nid + (uid[src] - 1);
}

int launch_obs_group(int nobs, const int* uid, const int* typ, int nid, const int* perm, int* ogrp, cudaStream_t s) {
  if (nobs <= 0) return LETKF_OK;
  obs_group_kernel<<<(nobs + 255) / 256, 256, 0, s>>>(nobs, uid, typ, nid, perm, ogrp);
  note_launch();
  return cuda_status(cudaGetLastError());
}

}  // namespace letkf

namespace letkf {
int launch_search_scale(int, int, const int*, int, const double*, const double*, const double*, const double*,
                        const double*, const int*, const int*, int, const double*, const double*, const double*,
                        const double*, const double*, const double*, const int64_t*, int*, int*, double*, double*,
                        cudaStream_t);

// The plain SCALE search of a point set (count, scan, fill) into stream-ordered
// scratch: per-point offsets uoffs[npts + 1] and the unlimited lists.
int unlimited_lists(int nlon, int nlat, const int* G, int nobs, const double* ori, const double* orj,
                    const double* olev, const double* odat, const double* oerr, const int* ocls, const int* ovarloc,
                    int npts, const double* pri, const double* prj, const double* prlev, const double* prz,
                    const double* var_local, const double* hp, cudaStream_t s, int64_t** uoffs, int** uidx,
                    double** urloc, double** urdiag) {
  *uoffs = nullptr;
  *uidx = nullptr;
  *urloc = *urdiag = nullptr;
  int* cnt = nullptr;
  int64_t* scr = nullptr;
  const size_t nb = (size_t)npts / 1024 + 2;
  if (cudaMallocAsync((void**)&cnt, sizeof(int) * ((size_t)npts + 1), s) != cudaSuccess ||
      cudaMallocAsync((void**)uoffs, sizeof(int64_t) * ((size_t)npts + 1), s) != cudaSuccess ||
      cudaMallocAsync((void**)&scr, sizeof(int64_t) * nb, s) != cudaSuccess) {
    if (cnt) cudaFreeAsync(cnt, s);
    if (scr) cudaFreeAsync(scr, s);
    return LETKF_ERR_CUDA;
  }
  int st = launch_search_scale(nlon, nlat, G, nobs, ori, orj, olev, odat, oerr, ocls, ovarloc, npts, pri, prj, prlev,
                               prz, var_local, hp, nullptr, cnt, nullptr, nullptr, nullptr, s);
  if (st == LETKF_OK) st = launch_exclusive_scan(npts, cnt, *uoffs, scr, s);
  int64_t total = 0;
  if (st == LETKF_OK) {
    cudaMemcpyAsync(&total, *uoffs + npts, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
    st = cuda_status(cudaStreamSynchronize(s));
  }
  const size_t m = (size_t)total + 1;
  if (st == LETKF_OK && (cudaMallocAsync((void**)uidx, sizeof(int) * m, s) != cudaSuccess ||
                         cudaMallocAsync((void**)urloc, sizeof(double) * m, s) != cudaSuccess ||
                         cudaMallocAsync((void**)urdiag, sizeof(double) * m, s) != cudaSuccess))
    st = LETKF_ERR_CUDA;
  if (st == LETKF_OK)
    st = launch_search_scale(nlon, nlat, G, nobs, ori, orj, olev, odat, oerr, ocls, ovarloc, npts, pri, prj, prlev,
                             prz, var_local, hp, *uoffs, cnt, *uidx, *urloc, *urdiag, s);
  cudaFreeAsync(cnt, s);
  cudaFreeAsync(scr, s);
  return st;
}

void free_unlimited(cudaStream_t s, int64_t* uoffs, int* uidx, double* urloc, double* urdiag) {
  void* p[] = {uoffs, uidx, urloc, urdiag};
  for (void* q : p)
    if (q) cudaFreeAsync(q, s);
}
}  // namespace letkf

using namespace letkf;

extern "C" int letkf_search_scale_limited(int nlon, int nlat, const int* nobsgrd, int nobs, const double* ori,
                                          const double* orj, const double* olev, const double* odat,
                                          const double* oerr, const int* ocls, const int* ovarloc, const int* ouid,
                                          const int* otyp, int nid, int max_nobs_per_grid, int npts,
                                          const double* pri, const double* prj, const double* prlev,
                                          const double* prz, const double* var_local_row, const double* params,
                                          const int64_t* offs, int* nobsl, int* idx, double* rloc, double* rdiag,
                                          void* stream) {
  if (nlon < 1 || nlat < 1 || nobs < 0 || npts < 0 || !nobsgrd || !params || nid < 1) return LETKF_ERR_ARG;
  if (max_nobs_per_grid < 1) return LETKF_ERR_ARG;
  if (max_nobs_per_grid > LETKF_MAX_NOBS_PER_GRID_LIMIT) return LETKF_ERR_CAPACITY;
  if (nobs > 0 && (!ouid || !otyp)) return LETKF_ERR_ARG;
  if (!idx && !nobsl) return LETKF_ERR_ARG;
  if (idx && (!offs || !rloc || !rdiag)) return LETKF_ERR_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return LETKF_ERR_NOGPU;
  }
  if (npts == 0) return LETKF_OK;
  cudaStream_t s = (cudaStream_t)stream;
  double hp[16];
  if (cudaMemcpy(hp, params, sizeof(double) * 15, cudaMemcpyDefault) != cudaSuccess) {
    memcpy(hp, params, sizeof(double) * 15);
    cudaGetLastError();
  }
  int* ogrp = nullptr;
  if (cudaMallocAsync((void**)&ogrp, sizeof(int) * ((size_t)nobs + 1), s) != cudaSuccess) return LETKF_ERR_CUDA;
  int st = launch_obs_group(nobs, ouid, otyp, nid, nullptr, ogrp, s);
  int64_t* uoffs = nullptr;
  int* uidx = nullptr;
  double *urloc = nullptr, *urdiag = nullptr;
  if (st == LETKF_OK)
    st = unlimited_lists(nlon, nlat, nobsgrd, nobs, ori, orj, olev, odat, oerr, ocls, ovarloc, npts, pri, prj, prlev,
                         prz, var_local_row, hp, s, &uoffs, &uidx, &urloc, &urdiag);
  if (st == LETKF_OK)
    st = launch_limit_select(npts, uoffs, uidx, urloc, urdiag, ogrp, max_nobs_per_grid, idx ? offs : nullptr,
                             idx ? nullptr : nobsl, idx, rloc, rdiag, s);
  free_unlimited(s, uoffs, uidx, urloc, urdiag);
  cudaFreeAsync(ogrp, s);
  const int st2 = cuda_status(cudaStreamSynchronize(s));
  return st != LETKF_OK ? st : st2;
}
