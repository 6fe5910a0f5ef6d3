// sweep.cu -- handle-based analysis sweep with the ensemble resident on the device.
//
// Replaces the das_letkf driver loop of the SCALE-style models
// (scale/letkf/letkf_tools.f90:38-476) for one GPU: observations are sorted
// into grid cells on the device (scale/letkf/letkf_obs.f90:735-830), every
// grid point is searched and analysed, and the ensemble is updated in place of
// the MPI scatter / gather (scale/common/common_mpi_scale.f90).  Two forms:
//   LETKF_PREC_F64    plain form: search -> packed local rows -> FP64 core ->
//                     FP64 update, in point chunks (scratch sized per chunk);
//   LETKF_PREC_MIXED  one fused persistent launch (sweep_mixed.cu).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "letkf_common.cuh"

namespace letkf {

struct SweepScaleParams;
struct SweepArgs;
// column cache: entries per CTA slot (32 bytes each) and slots per SM (the
// tensor-core sweep keeps at most four CTAs on an SM)
constexpr int LETKF_COL_CAP = 8192;
constexpr int LETKF_COL_SLOTS_PER_SM = 4;

int launch_sweep_mixed(const SweepArgs& a, cudaStream_t stream, int grid_cap);
int launch_sweep_tc(const SweepArgs& a, cudaStream_t stream, int grid_cap);
int prepare_sweep_mixed(int n);
int prepare_sweep_tc();
int launch_sweep_tc128(const SweepArgs& a, cudaStream_t stream, int grid_cap);
int prepare_sweep_tc128();
int launch_sweep_prep_obs(int, const double*, const double*, const double*, const double*, const double*,
                          const double*, const int*, const int*, const double*, const double*, float4*, float4*, int*,
                          cudaStream_t);
int launch_search_scale(int, int, const int*, int, const double*, const double*, const double*, const double*,
                        const double*, const int*, const int*, int, const double*, const double*, const double*,
                        const double*, const double*, const double*, const int64_t*, int*, int*, double*, double*,
                        cudaStream_t);
int launch_exclusive_scan(int, const int*, int64_t*, int64_t*, cudaStream_t);
int launch_core_f64(int, int, const int64_t*, const double*, const double*, const double*, const double*, double*,
                    double*, double*, double*, int, double, int*, cudaStream_t);
int launch_update_f64_range(int ne, int npts_total, int p0, int cnt, int nv, const double* xb, const double* trans,
                            const double* transm, double* xa, cudaStream_t stream);
int launch_gather_rows(int, int64_t, const int*, const void*, const void*, int, void*, void*, cudaStream_t);
int launch_limit_select(int, const int64_t*, const int*, const double*, const double*, const int*, int,
                        const int64_t*, int*, int*, double*, double*, cudaStream_t);
int launch_obs_group(int, const int*, const int*, int, const int*, int*, cudaStream_t);
int unlimited_lists(int, int, const int*, int, const double*, const double*, const double*, const double*,
                    const double*, const int*, const int*, int, const double*, const double*, const double*,
                    const double*, const double*, const double*, cudaStream_t, int64_t**, int**, double**, double**);
void free_unlimited(cudaStream_t, int64_t*, int*, double*, double*);

}  // namespace letkf

// full definitions needed here
#include "sweep_args.cuh"

namespace letkf {

// ---- device bucket sort of observations (stable) ----
__global__ void obs_cell_kernel(int nobs, int nlon, int nlat, int ihalo, int jhalo, const double* __restrict__ ri,
                                const double* __restrict__ rj, int* cell, int* counts) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nobs) return;
  int i = (int)ceil(ri[n] - 0.5) - ihalo, j = (int)ceil(rj[n] - 0.5) - jhalo;
  i = min(max(i, 1), nlon);
  j = min(max(j, 1), nlat);
  const int c = (j - 1) * nlon + (i - 1);
  cell[n] = c;
  atomicAdd(&counts[c], 1);
}

__global__ void obs_scatter_kernel(int nobs, const int* __restrict__ cell, const int64_t* __restrict__ start,
                                   int* cursor, int* perm) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nobs) return;
  const int c = cell[n];
  const int pos = (int)start[c] + atomicAdd(&cursor[c], 1);
  perm[pos] = n;
}

// restore input order inside each cell (insertion sort of a short segment)
__global__ void obs_stabilize_kernel(int ncell, const int64_t* __restrict__ start, int* perm) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncell) return;
  const int b = (int)start[c], e = (int)start[c + 1];
  for (int i = b + 1; i < e; i++) {
    const int v = perm[i];
    int k = i - 1;
    while (k >= b && perm[k] > v) {
      perm[k + 1] = perm[k];
      k--;
    }
    perm[k + 1] = v;
  }
}

// nobsgrd(0:nlon, 1:nlat) from the exclusive cell starts (letkf_obs.f90:765-774)
__global__ void obs_grd_kernel(int nlon, int nlat, const int64_t* __restrict__ start, int* G) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int ld = nlon + 1;
  if (t >= ld * nlat) return;
  const int j = t / ld, i = t - j * ld;  // j 0-based row, i = 0..nlon
  G[t] = (int)start[j * nlon + i];       // cumulative count before cell (i+1, j+1) == through cell (i, j+1)
}

// SPEEDY / GFS cell of an observation (speedy/letkf/letkf_obs.f90:243-313):
// band j with lat(j) <= y < lat(j+1) (j = 1..nlat-1), cell i with lon(i) <= x <
// lon(i+1) (i < nlon) or lon(nlon) <= x < 360 (i = nlon); key (j-1) nlon +
// (i-1), or -1 for an observation in no band or cell, or with qc /= 1
__global__ void latlon_cell_kernel(int nobs, int nlon, int nlat, const double* __restrict__ lon,
                                   const double* __restrict__ lat, const double* __restrict__ olon,
                                   const double* __restrict__ olat, const int* __restrict__ qc, int* cell,
                                   int* counts) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nobs) return;
  const double x = olon[n], y = olat[n];
  int c = -1;
  if ((!qc || qc[n] == 1) && y >= lat[0] && y < lat[nlat - 1]) {
    int lo = 0, hi = nlat - 2;  // the band j - 1 = lo with lat[lo] <= y < lat[lo + 1]
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (lat[mid] <= y) lo = mid;
      else hi = mid - 1;
    }
    const int jb = lo;
    if (x >= lon[0] && x < 360.0) {
      int a = 0, b = nlon - 1;  // the last cell runs to 360
      while (a < b) {
        const int mid = (a + b + 1) >> 1;
        if (lon[mid] <= x) a = mid;
        else b = mid - 1;
      }
      c = jb * nlon + a;
    }
  }
  cell[n] = c;
  if (c >= 0) atomicAdd(&counts[c], 1);
}

__global__ void latlon_scatter_kernel(int nobs, const int* __restrict__ cell, const int64_t* __restrict__ start,
                                      int* cursor, int* perm) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nobs) return;
  const int c = cell[n];
  if (c < 0) return;
  perm[(int)start[c] + atomicAdd(&cursor[c], 1)] = n;
}

// nobsgrd(i, j): cumulative count through cell (i, j) for the bands j < nlat;
// row nlat is not a band (the reference leaves it 0)
__global__ void latlon_grd_kernel(int nlon, int nlat, const int64_t* __restrict__ start, int* G) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nlon * nlat) return;
  G[t] = t < nlon * (nlat - 1) ? (int)start[t + 1] : 0;
}

template <typename T>
__global__ void permute_kernel(int n, int width, const int* __restrict__ perm, const T* __restrict__ src, T* dst) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n * width) return;
  const int64_t r = t / width;
  const int c = (int)(t - r * width);
  dst[t] = src[(int64_t)perm[r] * width + c];
}

template <typename T>
static void permute(int n, int width, const int* perm, const T* src, T* dst, cudaStream_t s) {
  if (n <= 0) return;
  const int64_t tot = (int64_t)n * width;
  permute_kernel<T><<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(n, width, perm, src, dst);
  note_launch();
}

__global__ void f64_to_f32_kernel(int64_t n, const double* __restrict__ a, float* b) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) b[t] = (float)a[t];
}

// coordinates of the points at processing positions order[0..n-1]
__global__ void gather_points_kernel(int n, const int* __restrict__ order, const double* __restrict__ ri,
                                     const double* __restrict__ rj, const double* __restrict__ rlev,
                                     const double* __restrict__ rz, double* ori, double* orj, double* orlev,
                                     double* orz) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int p = order[t];
  ori[t] = ri[p];
  orj[t] = rj[p];
  orlev[t] = rlev[p];
  orz[t] = rz[p];
}

}  // namespace letkf

using namespace letkf;

struct letkf_sweep_s {
  letkf_sweep_desc d;
  int nobs = 0;
  // points
  double *pri = nullptr, *prj = nullptr, *prlev = nullptr, *prz = nullptr, *plogr = nullptr;
  int* order = nullptr;
  std::vector<int> horder;     // the processing order, host copy
  std::vector<int64_t> hband;  // per order position: its band (tile row; the position itself without tiles)
  // sorted observations
  double *ori = nullptr, *orj = nullptr, *olev = nullptr, *odat = nullptr, *oerr = nullptr, *odep = nullptr;
  int *ocls = nullptr, *ovarloc = nullptr, *G = nullptr;
  double* var_local = nullptr;
  float4 *obsF = nullptr, *obsA = nullptr;
  int* meta = nullptr;
  float* ens32 = nullptr;
  double* ens64 = nullptr;
  int* operm = nullptr;  // sorted position -> input index of set_obs
  int* ogrp = nullptr;   // MAX_NOBS_PER_GRID group key per sorted observation (set_obs_groups)
  bool groups_set = false;
  size_t obs_cap = 0;  // observations the resident buffers hold (kept across set_obs calls)
  int max_nobs = 0;    // MAX_NOBS_PER_GRID (0: no limit)
  // column cache of the tensor-core search: enabled where most points of the
  // processing order share (ri, rj) with the point before them
  int4* col_ent = nullptr;
  int col_slots = 0;
  int col_unit = -1;  // order positions a CTA takes at a time (0: no cache; -1: the mean column length)
  int col_len = 1;     // mean length of the runs of equal (ri, rj) in the processing order
  bool columns = false;
  uint32_t fault_wait = 0;
  // selection probe
  int nprobe = 0, probe_cap = 0;
  int *probe_slot = nullptr, *probe_idx = nullptr, *probe_count = nullptr;
  float* probe_rloc = nullptr;
  // ensemble
  void *xb = nullptr, *xa = nullptr;
  double* infl = nullptr;
  int *status = nullptr, *nobsl = nullptr, *sweeps = nullptr, *counter = nullptr;
  int *defer_list = nullptr, *defer_count = nullptr, *defer_total = nullptr, *err_flag = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t ran = nullptr;  // recorded after a run issued on another stream
  int grid_cap = 0;
  int max_sweeps = 12;
  int use_ns = 1;
  int use_tc = 1;
  int tc_ns_max = 14;
  int tc_ns_scaled = 1;
  int tc_ns_tol_exp = 3;
  int polish_tol_exp = 7;
  int tc_polish = 0;
  int tc_scale_bound = 1;
  int polish_probe_exp = 9;
  int ns_cond_exp = 5;
  // CUDA graph of the mixed-form run: replayed while the kernel arguments,
  // launch choices and stream stay the same, captured again otherwise
  int use_graph = 1;
  cudaGraphExec_t gexec = nullptr;
  std::vector<unsigned char> gkey;
  int64_t glaunches = 0;  // kernels in the captured graph
  // run from host buffers: copy-in and copy-out streams, events (two per
  // chunk and two more), and the chunk plan
  cudaStream_t cs_in = nullptr, cs_out = nullptr;
  std::vector<cudaEvent_t> hev;
  int plan_n = 0;
  std::vector<int64_t> plan;   // per chunk: order range [o0, o1), its copies [c0, c1)
  std::vector<int64_t> pcopy;  // per copy: first row, rows, row stride, count (a strided block of point rows)
};

// Stream-ordered allocation: no call of a handle synchronises the whole
// device, so handles on other streams keep running (the serving slots).
static void dfree(void* p, cudaStream_t s) {
  if (p) cudaFreeAsync(p, s);
}

template <typename T>
static int dalloc(T** p, size_t n, cudaStream_t s) {
  *p = nullptr;
  if (n == 0) n = 1;
  return cudaMallocAsync((void**)p, n * sizeof(T), s) == cudaSuccess ? LETKF_OK : LETKF_ERR_CUDA;
}

static size_t elem(const letkf_sweep_s* h) { return h->d.precision == LETKF_PREC_F64 ? 8 : 4; }

extern "C" {

int letkf_sweep_create(letkf_sweep_t* out, const letkf_sweep_desc* d) {
  if (!out || !d) return LETKF_ERR_ARG;
  *out = nullptr;
  if (d->ne < 2 || d->nv < 1 || d->nv > 8 || d->nlon < 1 || d->nlat < 1 || d->npts < 0) return LETKF_ERR_ARG;
  if (d->precision != LETKF_PREC_F64 && d->precision != LETKF_PREC_MIXED) return LETKF_ERR_ARG;
  if (d->ne > LETKF_MAX_NE) return LETKF_ERR_CAPACITY;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return LETKF_ERR_NOGPU;
  }
  letkf_sweep_s* h = new letkf_sweep_s();
  h->d = *d;
  const size_t np = (size_t)d->npts;
  int st = LETKF_OK;
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->ran, cudaEventDisableTiming) != cudaSuccess) {
    letkf_sweep_destroy(h);
    return LETKF_ERR_CUDA;
  }
  cudaStream_t s = h->stream;
  st |= dalloc(&h->pri, np, s);
  st |= dalloc(&h->prj, np, s);
  st |= dalloc(&h->prlev, np, s);
  st |= dalloc(&h->prz, np, s);
  st |= dalloc(&h->plogr, np, s);
  st |= dalloc(&h->order, np, s);
  st |= dalloc((char**)&h->xb, np * d->nv * d->ne * elem(h), s);
  st |= dalloc((char**)&h->xa, np * d->nv * d->ne * elem(h), s);
  st |= dalloc(&h->infl, np, s);
  st |= dalloc(&h->status, np, s);
  st |= dalloc(&h->nobsl, np, s);
  st |= dalloc(&h->sweeps, np, s);
  st |= dalloc(&h->counter, 1, s);
  st |= dalloc(&h->defer_list, np, s);
  st |= dalloc(&h->defer_count, 1, s);
  st |= dalloc(&h->defer_total, 1, s);
  st |= dalloc(&h->err_flag, 1, s);
  st |= dalloc(&h->G, (size_t)(d->nlon + 1) * d->nlat, s);
  if (st != LETKF_OK) {
    letkf_sweep_destroy(h);
    return LETKF_ERR_CUDA;
  }
  cudaMemsetAsync(h->prz, 0, np * sizeof(double), s);
  cudaMemsetAsync(h->G, 0, sizeof(int) * (d->nlon + 1) * d->nlat, s);
  cudaMemsetAsync(h->err_flag, 0, sizeof(int), s);
  cudaMemsetAsync(h->defer_total, 0, sizeof(int), s);
  std::vector<double> one(np, 1.0);
  cudaMemcpyAsync(h->infl, one.data(), np * sizeof(double), cudaMemcpyHostToDevice, s);
  st = cuda_status(cudaStreamSynchronize(s));
  if (st != LETKF_OK) {
    letkf_sweep_destroy(h);
    return st;
  }
  *out = h;
  return LETKF_OK;
}

int letkf_sweep_destroy(letkf_sweep_t h) {
  if (!h) return LETKF_OK;
  void* ptrs[] = {h->pri,  h->prj,   h->prlev, h->prz,   h->plogr,   h->order, h->ori,     h->orj,    h->olev,
                  h->odat, h->oerr,  h->odep,  h->ocls,  h->ovarloc, h->G,     h->var_local, h->obsF,
                  h->obsA, h->meta,  h->ens32, h->ens64, h->xb,    h->xa,      h->infl,   h->status,
                  h->nobsl, h->sweeps, h->counter, h->defer_list, h->defer_count, h->defer_total, h->err_flag,
                  h->operm, h->ogrp, h->probe_slot, h->probe_idx, h->probe_count, h->probe_rloc,
                  h->col_ent};
  if (h->stream) {
    for (void* p : ptrs) dfree(p, h->stream);
    cudaStreamSynchronize(h->stream);
    cudaStreamDestroy(h->stream);
  }
  if (h->ran) cudaEventDestroy(h->ran);
  if (h->gexec) cudaGraphExecDestroy(h->gexec);
  for (cudaStream_t cs : {h->cs_in, h->cs_out})
    if (cs) {
      cudaStreamSynchronize(cs);
      cudaStreamDestroy(cs);
    }
  for (cudaEvent_t e : h->hev) cudaEventDestroy(e);
  delete h;
  return LETKF_OK;
}

int letkf_sweep_set_points(letkf_sweep_t h, const double* ri, const double* rj, const double* rlev, const double* rz,
                           int tile) {
  if (!h || !ri || !rj || !rlev) return LETKF_ERR_ARG;
  const int np = h->d.npts;
  for (int p = 0; p < np; p++)
    if (!(rlev[p] > 0.0)) return LETKF_ERR_ARG;
  // processing order: column tiles of tile x tile cells; inside a tile the
  // points of one column (equal ri, rj) follow each other in input order
  std::vector<int> order(np);
  std::iota(order.begin(), order.end(), 0);
  std::vector<int64_t> band(np);
  std::iota(band.begin(), band.end(), (int64_t)0);
  if (tile > 0) {
    std::vector<int64_t> key(np);
    const int64_t ntx = (h->d.nlon + tile - 1) / tile + 1;
    for (int p = 0; p < np; p++) {
      const int64_t ti = (int64_t)std::floor((ri[p] - 0.5) / tile), tj = (int64_t)std::floor((rj[p] - 0.5) / tile);
      key[p] = (tj + 1) * (ntx + 1) + (ti + 1);
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
      if (key[a] != key[b]) return key[a] < key[b];
      if (rj[a] != rj[b]) return rj[a] < rj[b];
      return ri[a] < ri[b];
    });
    for (int o = 0; o < np; o++) band[o] = key[order[o]] / (ntx + 1);
  }
  std::vector<double> lg(np);
  for (int p = 0; p < np; p++) lg[p] = std::log(rlev[p]);
  cudaStream_t s = h->stream;
  cudaMemcpyAsync(h->plogr, lg.data(), sizeof(double) * np, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(h->pri, ri, sizeof(double) * np, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(h->prj, rj, sizeof(double) * np, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(h->prlev, rlev, sizeof(double) * np, cudaMemcpyHostToDevice, s);
  if (rz) cudaMemcpyAsync(h->prz, rz, sizeof(double) * np, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(h->order, order.data(), sizeof(int) * np, cudaMemcpyHostToDevice, s);
  // columns: most positions share (ri, rj) with the one before them
  int64_t same = 0;
  for (int o = 1; o < np; o++) same += ri[order[o]] == ri[order[o - 1]] && rj[order[o]] == rj[order[o - 1]];
  h->columns = np > 1 && 2 * same >= (int64_t)np;
  h->col_len = np > 0 ? (int)std::min<int64_t>(4096, (np + (np - same) - 1) / (np - same)) : 1;
  if (h->columns && !h->col_ent) {
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    h->col_slots = nsm * LETKF_COL_SLOTS_PER_SM;
    if (dalloc(&h->col_ent, (size_t)h->col_slots * LETKF_COL_CAP * 2, s) != LETKF_OK) {
      h->col_ent = nullptr;
      h->col_slots = 0;
    }
  }
  const int st = cuda_status(cudaStreamSynchronize(s));
  h->horder.swap(order);
  h->hband.swap(band);
  h->plan_n = 0;
  return st;
}

int letkf_sweep_set_obs(letkf_sweep_t h, int nobs, const double* ri, const double* rj, const double* lev,
                        const double* dat, const double* err, const double* dep, const int* cls, const int* varloc,
                        const double* var_local_row, int nvarloc, const void* hdxf, int hdxf_f32) {
  if (!h || nobs < 0) return LETKF_ERR_ARG;
  if (nobs > 0 && (!ri || !rj || !lev || !dat || !err || !dep || !cls || !hdxf)) return LETKF_ERR_ARG;
  if (var_local_row && (!varloc || nvarloc < 1)) return LETKF_ERR_ARG;
  if (varloc)
    for (int i = 0; i < nobs; i++)
      if (varloc[i] < 0 || (var_local_row && varloc[i] >= nvarloc)) return LETKF_ERR_ARG;
  for (int i = 0; i < nobs; i++)
    if (cls[i] < 0 || cls[i] > 6) return LETKF_ERR_ARG;
  const int ne = h->d.ne, nlon = h->d.nlon, nlat = h->d.nlat;
  cudaStream_t s = h->stream;
  const size_t n = (size_t)nobs;
  int st = LETKF_OK;
  // resident sorted-observation buffers: kept while they are large enough, so
  // a cycle with no more observations than before keeps its device pointers
  // (and the captured run graph stays valid)
  if (n > h->obs_cap || h->ori == nullptr) {
    void* old[] = {h->ori, h->orj, h->olev, h->odat, h->oerr, h->odep, h->ocls, h->ovarloc,
                   h->obsF, h->obsA, h->meta, h->ens32, h->ens64, h->operm, h->ogrp};
    for (void* p : old) dfree(p, s);
    h->ori = h->orj = h->olev = h->odat = h->oerr = h->odep = nullptr;
    h->ocls = h->ovarloc = h->meta = h->operm = h->ogrp = nullptr;
    h->obsF = h->obsA = nullptr;
    h->ens32 = nullptr;
    h->ens64 = nullptr;
    h->obs_cap = 0;
    st |= dalloc(&h->ori, n, s);
    st |= dalloc(&h->orj, n, s);
    st |= dalloc(&h->olev, n, s);
    st |= dalloc(&h->odat, n, s);
    st |= dalloc(&h->oerr, n, s);
    st |= dalloc(&h->odep, n, s);
    st |= dalloc(&h->ocls, n, s);
    st |= dalloc(&h->ovarloc, n, s);
    st |= dalloc(&h->obsF, n, s);
    st |= dalloc(&h->obsA, n, s);
    st |= dalloc(&h->meta, n, s);
    st |= dalloc(&h->operm, n, s);
    st |= dalloc(&h->ogrp, n, s);
    if (h->d.precision == LETKF_PREC_MIXED) st |= dalloc(&h->ens32, n * ne, s);
    else st |= dalloc(&h->ens64, n * ne, s);
    if (st != LETKF_OK) return LETKF_ERR_CUDA;
    h->obs_cap = n;
  }
  h->nobs = nobs;
  h->groups_set = false;  // groups belong to an observation set
  dfree(h->var_local, s);  // variable localisation row (read by the record preparation and the plain form)
  h->var_local = nullptr;
  if (var_local_row && dalloc(&h->var_local, (size_t)nvarloc, s) != LETKF_OK) return LETKF_ERR_CUDA;
  if (var_local_row)
    cudaMemcpyAsync(h->var_local, var_local_row, sizeof(double) * nvarloc, cudaMemcpyHostToDevice, s);
  if (nobs == 0) {
    cudaMemsetAsync(h->G, 0, sizeof(int) * (nlon + 1) * nlat, s);
    return cuda_status(cudaStreamSynchronize(s));
  }
  // staging of the unsorted records
  double *t_ri, *t_rj, *t_lev, *t_dat, *t_err, *t_dep;
  int *t_cls, *t_vl, *cell, *counts, *cursor, *perm;
  int64_t *start, *scr;
  void* t_ens;
  const size_t es = hdxf_f32 ? 4 : 8;
  const int ncell = nlon * nlat;
  st |= dalloc(&t_ri, n, s);
  st |= dalloc(&t_rj, n, s);
  st |= dalloc(&t_lev, n, s);
  st |= dalloc(&t_dat, n, s);
  st |= dalloc(&t_err, n, s);
  st |= dalloc(&t_dep, n, s);
  st |= dalloc(&t_cls, n, s);
  st |= dalloc(&t_vl, n, s);
  st |= dalloc(&cell, n, s);
  st |= dalloc(&perm, n, s);
  st |= dalloc(&counts, (size_t)ncell, s);
  st |= dalloc(&cursor, (size_t)ncell, s);
  st |= dalloc(&start, (size_t)ncell + 1, s);
  st |= dalloc(&scr, (size_t)ncell / 1024 + 2, s);
  st |= dalloc((char**)&t_ens, n * ne * es, s);
  if (st != LETKF_OK) return LETKF_ERR_CUDA;
  cudaMemcpyAsync(t_ri, ri, 8 * n, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(t_rj, rj, 8 * n, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(t_lev, lev, 8 * n, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(t_dat, dat, 8 * n, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(t_err, err, 8 * n, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(t_dep, dep, 8 * n, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(t_cls, cls, 4 * n, cudaMemcpyHostToDevice, s);
  if (varloc) cudaMemcpyAsync(t_vl, varloc, 4 * n, cudaMemcpyHostToDevice, s);
  else cudaMemsetAsync(t_vl, 0, 4 * n, s);
  cudaMemcpyAsync(t_ens, hdxf, n * ne * es, cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(counts, 0, sizeof(int) * ncell, s);
  cudaMemsetAsync(cursor, 0, sizeof(int) * ncell, s);
  const unsigned gb = (unsigned)((n + 255) / 256);
  obs_cell_kernel<<<gb, 256, 0, s>>>(nobs, nlon, nlat, 0, 0, t_ri, t_rj, cell, counts);
  note_launch();
  launch_exclusive_scan(ncell, counts, start, scr, s);
  obs_scatter_kernel<<<gb, 256, 0, s>>>(nobs, cell, start, cursor, perm);
  obs_stabilize_kernel<<<(ncell + 255) / 256, 256, 0, s>>>(ncell, start, perm);
  obs_grd_kernel<<<((nlon + 1) * nlat + 255) / 256, 256, 0, s>>>(nlon, nlat, start, h->G);
  note_launch();
  note_launch();
  note_launch();
  cudaMemcpyAsync(h->operm, perm, sizeof(int) * n, cudaMemcpyDeviceToDevice, s);
  permute<double>(nobs, 1, perm, t_ri, h->ori, s);
  permute<double>(nobs, 1, perm, t_rj, h->orj, s);
  permute<double>(nobs, 1, perm, t_lev, h->olev, s);
  permute<double>(nobs, 1, perm, t_dat, h->odat, s);
  permute<double>(nobs, 1, perm, t_err, h->oerr, s);
  permute<double>(nobs, 1, perm, t_dep, h->odep, s);
  permute<int>(nobs, 1, perm, t_cls, h->ocls, s);
  permute<int>(nobs, 1, perm, t_vl, h->ovarloc, s);
  if (h->d.precision == LETKF_PREC_MIXED) {
    if (hdxf_f32) {
      permute<float>(nobs, ne, perm, (const float*)t_ens, h->ens32, s);
    } else {
      float* tmp;
      dalloc(&tmp, n * ne, s);
      f64_to_f32_kernel<<<(unsigned)((n * ne + 255) / 256), 256, 0, s>>>((int64_t)(n * ne), (const double*)t_ens,
                                                                         tmp);
      note_launch();
      permute<float>(nobs, ne, perm, tmp, h->ens32, s);
      dfree(tmp, s);
    }
  } else {
    if (hdxf_f32) return LETKF_ERR_ARG;
    permute<double>(nobs, ne, perm, (const double*)t_ens, h->ens64, s);
  }
  launch_sweep_prep_obs(nobs, h->ori, h->orj, h->olev, h->odat, h->oerr, h->odep, h->ocls, h->ovarloc, h->var_local,
                        h->d.params, h->obsF, h->obsA, h->meta, s);
  void* tmpb[] = {t_ri, t_rj, t_lev, t_dat, t_err, t_dep, t_cls, t_vl, cell, perm, counts, cursor, start, scr, t_ens};
  for (void* p : tmpb) dfree(p, s);
  return cuda_status(cudaStreamSynchronize(s));
}

// An input copied into the handle.  The handle's streams do not wait for the
// legacy default stream, so a device source (written there, or on any stream
// that synchronises with it) is copied on the legacy default stream, after the
// handle's own work has drained; a host source is copied on the handle's stream.
static int copy_in(letkf_sweep_t h, void* dst, const void* src, size_t bytes, int on_device) {
  int st = cuda_status(cudaStreamSynchronize(h->stream));
  if (st != LETKF_OK) return st;
  if (on_device) {
    cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, cudaStreamLegacy);
    return cuda_status(cudaStreamSynchronize(cudaStreamLegacy));
  }
  cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, h->stream);
  return cuda_status(cudaStreamSynchronize(h->stream));
}

int letkf_sweep_set_background(letkf_sweep_t h, const void* xb, int on_device) {
  if (!h || !xb) return LETKF_ERR_ARG;
  return copy_in(h, h->xb, xb, (size_t)h->d.npts * h->d.nv * h->d.ne * elem(h), on_device);
}

int letkf_sweep_set_inflation(letkf_sweep_t h, const double* infl, int on_device) {
  if (!h || !infl) return LETKF_ERR_ARG;
  return copy_in(h, h->infl, infl, sizeof(double) * h->d.npts, on_device);
}

int letkf_sweep_device_buffers(letkf_sweep_t h, void** xb, void** xa, double** infl, int** nobsl) {
  if (!h) return LETKF_ERR_ARG;
  if (xb) *xb = h->xb;
  if (xa) *xa = h->xa;
  if (infl) *infl = h->infl;
  if (nobsl) *nobsl = h->nobsl;
  return LETKF_OK;
}

int letkf_sweep_set_option(letkf_sweep_t h, int option, int value) {
  if (!h) return LETKF_ERR_ARG;
  switch (option) {
    case LETKF_OPT_GRID_CAP:
      if (value < 0) return LETKF_ERR_ARG;
      h->grid_cap = value;
      return LETKF_OK;
    case LETKF_OPT_GRID_SHARE:
      if (value < 1) return LETKF_ERR_ARG;
      h->grid_cap = value == 1 ? 0 : -value;  // the launchers read a negative cap as a share
      return LETKF_OK;
    case LETKF_OPT_MAX_SWEEPS:
      if (value < 1 || value > 64) return LETKF_ERR_ARG;
      h->max_sweeps = value;
      return LETKF_OK;
    case LETKF_OPT_TENSOR_CORES:
      if (value != 0 && value != 1) return LETKF_ERR_ARG;
      h->use_tc = value;
      return LETKF_OK;
    case LETKF_OPT_TC_NS_ITERS:
      if (value < 0 || value > 64) return LETKF_ERR_ARG;
      h->tc_ns_max = value;
      return LETKF_OK;
    case LETKF_OPT_TC_NS_SCALING:
      if (value != 0 && value != 1) return LETKF_ERR_ARG;
      h->tc_ns_scaled = value;
      return LETKF_OK;
    case LETKF_OPT_TC_NS_TOL:
      if (value < 1 || value > 7) return LETKF_ERR_ARG;
      h->tc_ns_tol_exp = value;
      return LETKF_OK;
    case LETKF_OPT_POLISH_TOL:
      if (value < 4 || value > 12) return LETKF_ERR_ARG;
      h->polish_tol_exp = value;
      return LETKF_OK;
    case LETKF_OPT_TC_POLISH:
      if (value != 0 && value != 1) return LETKF_ERR_ARG;
      h->tc_polish = value;
      return LETKF_OK;
    case LETKF_OPT_TC_SCALE_BOUND:
      if (value != 0 && value != 1) return LETKF_ERR_ARG;
      h->tc_scale_bound = value;
      return LETKF_OK;
    case LETKF_OPT_POLISH_PROBE:
      if (value < 0 || value > 14) return LETKF_ERR_ARG;
      h->polish_probe_exp = value;
      return LETKF_OK;
    case LETKF_OPT_NS_COND:
      if (value < 0 || value > 8) return LETKF_ERR_ARG;
      h->ns_cond_exp = value;
      return LETKF_OK;
    case LETKF_OPT_GRAPH:
      if (value != 0 && value != 1) return LETKF_ERR_ARG;
      h->use_graph = value;
      return LETKF_OK;
    case LETKF_OPT_MAX_NOBS_PER_GRID:
      if (value < 0) return LETKF_ERR_ARG;
      if (value > LETKF_MAX_NOBS_PER_GRID_LIMIT) return LETKF_ERR_CAPACITY;
      h->max_nobs = value;
      return LETKF_OK;
    case LETKF_OPT_FAULT_WAIT:
      if (value < 0) return LETKF_ERR_ARG;
      h->fault_wait = (uint32_t)value;
      return LETKF_OK;
    case LETKF_OPT_COLUMN_UNIT:
      if (value < -1 || value > 4096) return LETKF_ERR_ARG;
      h->col_unit = value;
      return LETKF_OK;
    case LETKF_OPT_EIGENSOLVER:
      if (value != LETKF_EIG_NEWTON_SCHULZ && value != LETKF_EIG_JACOBI) return LETKF_ERR_ARG;
      h->use_ns = value == LETKF_EIG_NEWTON_SCHULZ;
      return LETKF_OK;
    default: return LETKF_ERR_ARG;
  }
}

static int run_f64(letkf_sweep_t h, cudaStream_t s) {
  // plain form in chunks of points: search (count, scan, fill), gather, core, update
  const int ne = h->d.ne, nv = h->d.nv, np = h->d.npts, nobs = h->nobs;
  const int chunk = std::min(np, 16384);
  int *cnt, *idx = nullptr;
  int64_t *offs, *scr;
  double *rloc = nullptr, *rdiag = nullptr, *rows = nullptr, *dep = nullptr, *trans, *transm;
  int st = LETKF_OK;
  st |= dalloc(&cnt, (size_t)chunk, s);
  st |= dalloc(&offs, (size_t)chunk + 1, s);
  st |= dalloc(&scr, (size_t)chunk / 1024 + 2, s);
  st |= dalloc(&trans, (size_t)chunk * ne * ne, s);
  st |= dalloc(&transm, (size_t)chunk * ne, s);
  if (st != LETKF_OK) return LETKF_ERR_CUDA;
  size_t cap = 0;
  const bool limited = h->max_nobs > 0;
  if (limited && !h->groups_set && nobs > 0) st = LETKF_ERR_ARG;
  for (int p0 = 0; p0 < np && st == LETKF_OK; p0 += chunk) {
    const int c = std::min(chunk, np - p0);
    // MAX_NOBS_PER_GRID: the plain lists first, then the limited selection
    int64_t* uoffs = nullptr;
    int* uidx = nullptr;
    double *url = nullptr, *urd = nullptr;
    if (limited) {
      st = unlimited_lists(h->d.nlon, h->d.nlat, h->G, nobs, h->ori, h->orj, h->olev, h->odat, h->oerr, h->ocls,
                           h->ovarloc, c, h->pri + p0, h->prj + p0, h->prlev + p0, h->prz + p0, h->var_local,
                           h->d.params, s, &uoffs, &uidx, &url, &urd);
      if (st == LETKF_OK)
        st = launch_limit_select(c, uoffs, uidx, url, urd, h->ogrp, h->max_nobs, nullptr, cnt, nullptr, nullptr,
                                 nullptr, s);
    } else {
      st = launch_search_scale(h->d.nlon, h->d.nlat, h->G, nobs, h->ori, h->orj, h->olev, h->odat, h->oerr, h->ocls,
                               h->ovarloc, c, h->pri + p0, h->prj + p0, h->prlev + p0, h->prz + p0, h->var_local,
                               h->d.params, nullptr, cnt, nullptr, nullptr, nullptr, s);
    }
    if (st) {
      free_unlimited(s, uoffs, uidx, url, urd);
      break;
    }
    st = launch_exclusive_scan(c, cnt, offs, scr, s);
    int64_t total = 0;
    cudaMemcpyAsync(&total, offs + c, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    cudaMemcpyAsync(h->nobsl + p0, cnt, sizeof(int) * c, cudaMemcpyDeviceToDevice, s);
    if ((size_t)total > cap) {
      dfree(idx, s);
      dfree(rloc, s);
      dfree(rdiag, s);
      dfree(rows, s);
      dfree(dep, s);
      cap = (size_t)total + (size_t)total / 4 + 1024;
      st |= dalloc(&idx, cap, s);
      st |= dalloc(&rloc, cap, s);
      st |= dalloc(&rdiag, cap, s);
      st |= dalloc(&rows, cap * ne, s);
      st |= dalloc(&dep, cap, s);
      if (st) {
        free_unlimited(s, uoffs, uidx, url, urd);
        break;
      }
    }
    if (limited) {
      st = launch_limit_select(c, uoffs, uidx, url, urd, h->ogrp, h->max_nobs, offs, nullptr, idx, rloc, rdiag, s);
      free_unlimited(s, uoffs, uidx, url, urd);
    } else {
      st = launch_search_scale(h->d.nlon, h->d.nlat, h->G, nobs, h->ori, h->orj, h->olev, h->odat, h->oerr,
                               h->ocls, h->ovarloc, c, h->pri + p0, h->prj + p0, h->prlev + p0, h->prz + p0,
                               h->var_local, h->d.params, offs, cnt, idx, rloc, rdiag, s);
    }
    if (st) break;
    if (total > 0) {
      st = letkf::launch_gather_rows(ne, total, idx, h->ens64, h->odep, 8, rows, dep, s);
      if (st) break;
    }
    // SCALE convention: rdiag = err^2 / rloc with rdiag_wloc (letkf_tools.f90:199-206)
    st = launch_core_f64(ne, c, offs, rows, rdiag, rloc, dep, h->infl + p0, trans, transm, nullptr, 1, h->d.minfl,
                         h->status + p0, s);
    if (st) break;
    st = launch_update_f64_range(ne, np, p0, c, nv, (const double*)h->xb, trans, transm, (double*)h->xa, s);
  }
  void* fr[] = {cnt, idx, offs, scr, rloc, rdiag, rows, dep, trans, transm};
  for (void* p : fr) dfree(p, s);
  return st;
}

static int run_on(letkf_sweep_t h, cudaStream_t s);
static int check_err(letkf_sweep_t h);

int letkf_sweep_run(letkf_sweep_t h, void* stream) {
  if (!h) return LETKF_ERR_ARG;
  cudaStream_t s = stream ? (cudaStream_t)stream : h->stream;
  if (s != h->stream) {
    // the run reads what the handle's stream wrote; later calls on the
    // handle (copies out, frees) wait for the run
    cudaEventRecord(h->ran, h->stream);
    cudaStreamWaitEvent(s, h->ran, 0);
  }
  const int st = run_on(h, s);
  if (s != h->stream) {
    cudaEventRecord(h->ran, s);
    cudaStreamWaitEvent(h->stream, h->ran, 0);
  }
  return st;
}

static void build_args(letkf_sweep_t h, SweepArgs& a) {
  memset(&a, 0, sizeof(a));
  a.n = h->d.ne;
  a.nv = h->d.nv;
  a.npts = h->d.npts;
  a.nwork = h->d.npts;
  a.nlon = h->d.nlon;
  a.nlat = h->d.nlat;
  a.nobs = h->nobs;
  a.G = h->G;
  a.obsF = h->obsF;
  a.obsA = h->obsA;
  a.obsMeta = h->meta;
  a.ori = h->ori;
  a.orj = h->orj;
  a.olev = h->olev;
  a.odat = h->odat;
  a.ocls = h->ocls;
  double* f = &a.P.dx;
  for (int i = 0; i < 15; i++) f[i] = h->d.params[i];
  a.ens_obs = h->ens32;
  a.order = h->order;
  a.pri = h->pri;
  a.prj = h->prj;
  a.prlev = h->prlev;
  a.prz = h->prz;
  a.plogr = h->plogr;
  a.xb = (const float*)h->xb;
  a.xb_bulk = (h->d.ne % 4 == 0) && (reinterpret_cast<uintptr_t>(h->xb) % 16 == 0);
  a.xa = (float*)h->xa;
  a.infl = h->infl;
  a.nobsl_out = h->nobsl;
  a.sweeps_out = h->sweeps;
  a.status = h->status;
  a.counter = h->counter;
  a.minfl = h->d.minfl;
  a.max_sweeps = h->max_sweeps;
  a.max_ns_iter = 24;
  a.use_ns = h->use_ns;
  a.err_flag = h->err_flag;
  a.tc_ns_max = h->tc_ns_max;
  a.tc_ns_scaled = h->tc_ns_scaled;
  a.tc_ns_tol = (float)std::pow(10.0, -h->tc_ns_tol_exp);
  a.polish_tol = (float)std::pow(10.0, -h->polish_tol_exp);
  a.tc_polish = h->tc_polish;
  a.tc_scale_bound = h->tc_scale_bound;
  a.polish_probe = h->polish_probe_exp > 0 ? (float)std::pow(10.0, -h->polish_probe_exp) : 0.f;
  a.ns_cond_max = h->ns_cond_exp > 0 ? (float)std::pow(10.0, h->ns_cond_exp) : 0.f;
  a.defer_total = h->defer_total;
  a.defer_list = h->defer_list;  // read by the tensor-core sweep only
  a.defer_count = h->defer_count;
  a.probe_slot = h->nprobe > 0 ? h->probe_slot : nullptr;
  a.probe_cap = h->probe_cap;
  a.probe_idx = h->probe_idx;
  a.probe_rloc = h->probe_rloc;
  a.probe_count = h->probe_count;
  a.fault_wait_polls = h->fault_wait;
  // the column cache serves the tensor-core sweeps (ne <= 128)
  if (h->columns && h->col_ent && h->col_unit != 0 && h->d.ne <= 128) {
    a.col_ent = h->col_ent;
    a.col_cap = LETKF_COL_CAP;
    a.col_slots = h->col_slots;
    a.col_unit = h->col_unit > 0 ? h->col_unit : h->col_len;
  } else {
    a.col_unit = 1;
  }
}

// tensor-core sweeps: sweep_tc.cu for ne <= 64, sweep_tc128.cu for 64 < ne <= 128
static bool tc_path(letkf_sweep_t h) { return h->use_tc && h->use_ns && h->d.ne <= 128; }

static int launch_tc(letkf_sweep_t h, const SweepArgs& a, cudaStream_t s) {
  return h->d.ne <= 64 ? launch_sweep_tc(a, s, h->grid_cap) : launch_sweep_tc128(a, s, h->grid_cap);
}

static int prepare_tc(letkf_sweep_t h) { return h->d.ne <= 64 ? prepare_sweep_tc() : prepare_sweep_tc128(); }

static int launch_mixed_run(letkf_sweep_t h, const SweepArgs& a, cudaStream_t s) {
  cudaMemsetAsync(h->counter, 0, sizeof(int), s);
  const bool tc = tc_path(h);
  if (!tc && !a.use_ns) return launch_sweep_mixed(a, s, h->grid_cap);
  // Newton-Schulz sweep (tensor-core or SIMT), then the Jacobi pass over the
  // points it deferred
  cudaMemsetAsync(h->defer_count, 0, sizeof(int), s);
  int st = tc ? launch_tc(h, a, s) : launch_sweep_mixed(a, s, h->grid_cap);
  if (st != LETKF_OK) return st;
  SweepArgs b = a;
  if (a.list_offs) {
    b.qmap = h->defer_list;  // list mode: the deferred points are order positions
  } else {
    b.order = h->defer_list;
  }
  b.npts_dev = h->defer_count;
  b.use_ns = 0;
  cudaMemsetAsync(h->counter, 0, sizeof(int), s);
  return launch_sweep_mixed(b, s, h->grid_cap);
}

// The mixed-form run with the MAX_NOBS_PER_GRID limit: per piece of the
// processing order, the SCALE search of its points with the limit
// (letkf_search_scale_limited's two passes) into lists, then the sweep kernels
// analyse the piece from the lists.  Host synchronisation sizes the lists, so
// this run is not a CUDA graph.
static int run_limited(letkf_sweep_t h, const SweepArgs& a, cudaStream_t s) {
  const int np = h->d.npts;
  if (!h->groups_set && h->nobs > 0) return LETKF_ERR_ARG;
  const int chunk = std::min(np, 65536);
  double *cri = nullptr, *crj = nullptr, *crl = nullptr, *crz = nullptr;
  int* lcnt = nullptr;
  int64_t *lofs = nullptr, *scr = nullptr;
  int* lidx = nullptr;
  double *lrl = nullptr, *lrd = nullptr;
  size_t cap = 0;
  int st = LETKF_OK;
  st |= dalloc(&cri, (size_t)chunk, s);
  st |= dalloc(&crj, (size_t)chunk, s);
  st |= dalloc(&crl, (size_t)chunk, s);
  st |= dalloc(&crz, (size_t)chunk, s);
  st |= dalloc(&lcnt, (size_t)chunk, s);
  st |= dalloc(&lofs, (size_t)chunk + 1, s);
  st |= dalloc(&scr, (size_t)chunk / 1024 + 2, s);
  for (int o0 = 0; o0 < np && st == LETKF_OK; o0 += chunk) {
    const int c = std::min(chunk, np - o0);
    gather_points_kernel<<<(c + 255) / 256, 256, 0, s>>>(c, h->order + o0, h->pri, h->prj, h->prlev, h->prz, cri,
                                                         crj, crl, crz);
    note_launch();
    int64_t* uoffs = nullptr;
    int* uidx = nullptr;
    double *url = nullptr, *urd = nullptr;
    st = unlimited_lists(h->d.nlon, h->d.nlat, h->G, h->nobs, h->ori, h->orj, h->olev, h->odat, h->oerr, h->ocls,
                         h->ovarloc, c, cri, crj, crl, crz, h->var_local, h->d.params, s, &uoffs, &uidx, &url, &urd);
    if (st == LETKF_OK)
      st = launch_limit_select(c, uoffs, uidx, url, urd, h->ogrp, h->max_nobs, nullptr, lcnt, nullptr, nullptr,
                               nullptr, s);
    if (st == LETKF_OK) st = launch_exclusive_scan(c, lcnt, lofs, scr, s);
    int64_t total = 0;
    if (st == LETKF_OK) {
      cudaMemcpyAsync(&total, lofs + c, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
      st = cuda_status(cudaStreamSynchronize(s));
    }
    if (st == LETKF_OK && (size_t)total + 1 > cap) {
      dfree(lidx, s);
      dfree(lrl, s);
      dfree(lrd, s);
      cap = (size_t)total + (size_t)total / 4 + 1024;
      st |= dalloc(&lidx, cap, s);
      st |= dalloc(&lrl, cap, s);
      st |= dalloc(&lrd, cap, s);
    }
    if (st == LETKF_OK)
      st = launch_limit_select(c, uoffs, uidx, url, urd, h->ogrp, h->max_nobs, lofs, nullptr, lidx, lrl, lrd, s);
    free_unlimited(s, uoffs, uidx, url, urd);
    if (st != LETKF_OK) break;
    SweepArgs b = a;
    b.order = h->order + o0;
    b.nwork = c;
    b.list_offs = lofs;
    b.list_idx = lidx;
    b.list_rloc = lrl;
    st = launch_mixed_run(h, b, s);
    // the next piece's search reuses the point and list buffers
    if (st == LETKF_OK) st = cuda_status(cudaStreamSynchronize(s));
  }
  void* fr[] = {cri, crj, crl, crz, lcnt, lofs, scr, lidx, lrl, lrd};
  for (void* p : fr) dfree(p, s);
  return st;
}

static int run_on(letkf_sweep_t h, cudaStream_t s) {
  // a run reports only its own bounded-wait timeouts
  cudaMemsetAsync(h->err_flag, 0, sizeof(int), s);
  if (h->d.precision == LETKF_PREC_F64) return run_f64(h, s);
  SweepArgs a;
  build_args(h, a);
  cudaMemsetAsync(h->defer_total, 0, sizeof(int), s);
  if (h->max_nobs > 0) return run_limited(h, a, s);
  if (!h->use_graph) return launch_mixed_run(h, a, s);
  // key: kernel arguments, launch choices and stream
  std::vector<unsigned char> key(sizeof(a) + 3 * sizeof(int) + sizeof(s));
  unsigned char* k = key.data();
  memcpy(k, &a, sizeof(a));
  const int extra[3] = {h->grid_cap, h->use_tc, h->use_ns};
  memcpy(k + sizeof(a), extra, sizeof(extra));
  memcpy(k + sizeof(a) + sizeof(extra), &s, sizeof(s));
  if (!h->gexec || key != h->gkey) {
    if (h->gexec) {
      cudaGraphExecDestroy(h->gexec);
      h->gexec = nullptr;
    }
    // kernel attributes are set before the capture, not inside it
    int st = tc_path(h) ? prepare_tc(h) : LETKF_OK;
    if (st == LETKF_OK) st = prepare_sweep_mixed(h->d.ne);
    if (st != LETKF_OK) return st;
    const int64_t n0 = letkf_launch_count();
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_status(e);
    st = launch_mixed_run(h, a, s);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(s, &g);
    if (st == LETKF_OK && e != cudaSuccess) st = cuda_status(e);
    if (st == LETKF_OK) {
      e = cudaGraphInstantiate(&h->gexec, g, 0);
      if (e != cudaSuccess) {
        h->gexec = nullptr;
        st = cuda_status(e);
      }
    }
    if (g) cudaGraphDestroy(g);
    if (st != LETKF_OK) return st;
    h->gkey = key;
    h->glaunches = letkf_launch_count() - n0;
    const cudaError_t r = cudaGraphLaunch(h->gexec, s);
    return cuda_status(r);
  }
  const cudaError_t r = cudaGraphLaunch(h->gexec, s);
  for (int64_t i = 0; i < h->glaunches; i++) note_launch();
  return cuda_status(r);
}

// Chunk plan of the host-buffer run: about nchunks pieces of the processing
// order, cut where its band (tile row) changes.  A point's background row is
// read and its analysis row written by its own analysis only, so piece c
// copies exactly its points' rows in before it and out after it: the sorted
// rows form runs, and runs of equal length at a constant stride one strided
// copy (with level-major points and tile-row pieces: one copy per variable).
static void plan_host_run(letkf_sweep_t h, int nc) {
  const int64_t np = h->d.npts;
  std::vector<int64_t> cut{0};
  for (int c = 1; c < nc; c++) {
    int64_t o = np * c / nc;
    while (o < np && o > 0 && h->hband[(size_t)o] == h->hband[(size_t)o - 1]) o++;
    if (o > cut.back() && o < np) cut.push_back(o);
  }
  cut.push_back(np);
  h->plan.clear();
  h->pcopy.clear();
  std::vector<int> rows;
  for (size_t c = 0; c + 1 < cut.size(); c++) {
    const int64_t o0 = cut[c], o1 = cut[c + 1];
    rows.assign(h->horder.begin() + o0, h->horder.begin() + o1);
    std::sort(rows.begin(), rows.end());
    const int64_t c0 = (int64_t)h->pcopy.size() / 4;
    // runs of consecutive rows, merged into strided blocks
    int64_t bstart = -1, blen = 0, bstride = 0, bcount = 0;
    auto flush = [&]() {
      if (bcount > 0) h->pcopy.insert(h->pcopy.end(), {bstart, blen, bcount > 1 ? bstride : blen, bcount});
      bcount = 0;
    };
    size_t i = 0;
    while (i < rows.size()) {
      size_t j = i + 1;
      while (j < rows.size() && rows[j] == rows[j - 1] + 1) j++;
      const int64_t rs = rows[i], rl = (int64_t)(j - i);
      if (bcount == 1 && rl == blen) {
        bstride = rs - bstart;
        bcount = 2;
      } else if (bcount > 1 && rl == blen && rs == bstart + bcount * bstride) {
        bcount++;
      } else {
        flush();
        bstart = rs;
        blen = rl;
        bcount = 1;
      }
      i = j;
    }
    flush();
    h->plan.insert(h->plan.end(), {o0, o1, c0, (int64_t)h->pcopy.size() / 4});
  }
  h->plan_n = nc;
}

// the point rows of one strided block, for every variable, in one direction
static int copy_rows(const int64_t* cp, int nv, int64_t np, size_t row, void* dst, const void* src,
                     cudaMemcpyKind kind, cudaStream_t s) {
  for (int v = 0; v < nv; v++) {
    const size_t off = ((size_t)v * np + (size_t)cp[0]) * row;
    cudaError_t e;
    if (cp[3] == 1)
      e = cudaMemcpyAsync((char*)dst + off, (const char*)src + off, (size_t)cp[1] * row, kind, s);
    else
      e = cudaMemcpy2DAsync((char*)dst + off, (size_t)cp[2] * row, (const char*)src + off, (size_t)cp[2] * row,
                            (size_t)cp[1] * row, (size_t)cp[3], kind, s);
    if (e != cudaSuccess) return cuda_status(e);
  }
  return LETKF_OK;
}

int letkf_sweep_run_host(letkf_sweep_t h, const void* xb, void* xa, int nchunks, void* stream) {
  if (!h || !xb || !xa || nchunks < 1) return LETKF_ERR_ARG;
  const int np = h->d.npts;
  if (h->d.precision == LETKF_PREC_F64 || np == 0 || nchunks == 1 || h->max_nobs > 0) {
    int st = letkf_sweep_set_background(h, xb, 0);
    if (st == LETKF_OK) st = letkf_sweep_run(h, stream);
    if (st == LETKF_OK) st = letkf_sweep_get_analysis(h, xa, 0);
    return st;
  }
  if ((int)h->horder.size() != np) return LETKF_ERR_ARG;  // points not set
  if (nchunks > np) nchunks = np;
  if (nchunks > 1024) nchunks = 1024;
  cudaStream_t s = stream ? (cudaStream_t)stream : h->stream;
  for (cudaStream_t* cs : {&h->cs_in, &h->cs_out})
    if (!*cs && cudaStreamCreateWithFlags(cs, cudaStreamNonBlocking) != cudaSuccess) return LETKF_ERR_CUDA;
  while (h->hev.size() < (size_t)(2 * nchunks + 2)) {
    cudaEvent_t e = nullptr;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return LETKF_ERR_CUDA;
    h->hev.push_back(e);
  }
  if (h->plan_n != nchunks) plan_host_run(h, nchunks);
  const int npc = (int)(h->plan.size() / 4);
  cudaEvent_t* ev = h->hev.data();  // per piece: copied in, analysed; then entry and exit marks
  // work issued earlier on the handle's stream and on s comes first
  if (s != h->stream) {
    cudaEventRecord(h->ran, h->stream);
    cudaStreamWaitEvent(s, h->ran, 0);
  }
  cudaEventRecord(ev[2 * npc], s);
  cudaStreamWaitEvent(h->cs_in, ev[2 * npc], 0);
  cudaStreamWaitEvent(h->cs_out, ev[2 * npc], 0);
  SweepArgs a;
  build_args(h, a);
  cudaMemsetAsync(h->defer_total, 0, sizeof(int), s);
  cudaMemsetAsync(h->err_flag, 0, sizeof(int), s);
  const size_t row = (size_t)h->d.ne * elem(h);
  const int nv = h->d.nv;
  int st = LETKF_OK;
  for (int c = 0; c < npc && st == LETKF_OK; c++) {
    const int64_t* e = &h->plan[(size_t)c * 4];
    for (int64_t k = e[2]; k < e[3] && st == LETKF_OK; k++)
      st = copy_rows(&h->pcopy[(size_t)k * 4], nv, np, row, h->xb, xb, cudaMemcpyHostToDevice, h->cs_in);
    if (st != LETKF_OK) break;
    cudaEventRecord(ev[2 * c], h->cs_in);
    cudaStreamWaitEvent(s, ev[2 * c], 0);
    SweepArgs b = a;
    b.order = h->order + e[0];
    b.nwork = (int)(e[1] - e[0]);
    st = launch_mixed_run(h, b, s);
    if (st != LETKF_OK) break;
    cudaEventRecord(ev[2 * c + 1], s);
    cudaStreamWaitEvent(h->cs_out, ev[2 * c + 1], 0);
    for (int64_t k = e[2]; k < e[3] && st == LETKF_OK; k++)
      st = copy_rows(&h->pcopy[(size_t)k * 4], nv, np, row, xa, h->xa, cudaMemcpyDeviceToHost, h->cs_out);
  }
  // s and the handle's stream complete after the last copies
  cudaEventRecord(ev[2 * npc + 1], h->cs_out);
  cudaStreamWaitEvent(s, ev[2 * npc + 1], 0);
  cudaEventRecord(ev[2 * npc], h->cs_in);
  cudaStreamWaitEvent(s, ev[2 * npc], 0);
  if (s != h->stream) {
    cudaEventRecord(h->ran, s);
    cudaStreamWaitEvent(h->stream, h->ran, 0);
  }
  const int st2 = cuda_status(cudaStreamSynchronize(s));
  if (st == LETKF_OK) st = st2;
  return st != LETKF_OK ? st : check_err(h);
}

int letkf_sweep_autotune(letkf_sweep_t h, int sample_points, int* choice) {
  if (!h || sample_points < 1) return LETKF_ERR_ARG;
  if (h->d.precision == LETKF_PREC_F64 || h->d.npts == 0 || h->max_nobs > 0) {
    // nothing to tune (the plain form; the limited run keeps the handle's choice)
    if (choice) {
      choice[0] = 0;
      choice[1] = 0;
      choice[2] = 0;
      choice[3] = 0;
    }
    return LETKF_OK;
  }
  cudaStream_t s = h->stream;
  const size_t np = (size_t)h->d.npts;
  const int sample = sample_points < h->d.npts ? sample_points : h->d.npts;
  double* keep = nullptr;
  if (dalloc(&keep, np, s) != LETKF_OK) return LETKF_ERR_CUDA;
  cudaMemcpyAsync(keep, h->infl, np * sizeof(double), cudaMemcpyDeviceToDevice, s);
  struct Cand {
    int tc, ns, scaled;
  };
  std::vector<Cand> cands;
  if (h->d.ne <= 128) {
    cands.push_back({1, 1, 1});
    cands.push_back({1, 1, 0});
  }
  cands.push_back({0, 1, 1});
  cands.push_back({0, 0, 1});
  const Cand was = {h->use_tc, h->use_ns, h->tc_ns_scaled};
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int st = LETKF_OK, best = -1;
  float best_ms = 0.f;
  for (size_t c = 0; c < cands.size() && st == LETKF_OK; c++) {
    h->use_tc = cands[c].tc;
    h->use_ns = cands[c].ns;
    h->tc_ns_scaled = cands[c].scaled;
    SweepArgs a;
    build_args(h, a);
    a.nwork = sample;  // the first `sample` points of the processing order
    float ms = 0.f;
    for (int rep = 0; rep < 2 && st == LETKF_OK; rep++) {  // warm-up, then timed
      cudaMemcpyAsync(h->infl, keep, np * sizeof(double), cudaMemcpyDeviceToDevice, s);
      cudaEventRecord(e0, s);
      st = launch_mixed_run(h, a, s);
      cudaEventRecord(e1, s);
      if (st == LETKF_OK) st = cuda_status(cudaEventSynchronize(e1));
      if (st == LETKF_OK) st = cuda_status(cudaEventElapsedTime(&ms, e0, e1));
    }
    if (st == LETKF_OK && (best < 0 || ms < best_ms)) {
      best = (int)c;
      best_ms = ms;
    }
  }
  cudaMemcpyAsync(h->infl, keep, np * sizeof(double), cudaMemcpyDeviceToDevice, s);
  dfree(keep, s);
  const int st2 = cuda_status(cudaStreamSynchronize(s));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st == LETKF_OK) st = st2;
  if (st == LETKF_OK) st = check_err(h);
  const Cand pick = (st == LETKF_OK && best >= 0) ? cands[best] : was;
  h->use_tc = pick.tc;
  h->use_ns = pick.ns;
  h->tc_ns_scaled = pick.scaled;
  if (h->gexec) {
    cudaGraphExecDestroy(h->gexec);
    h->gexec = nullptr;
  }
  if (choice) {
    choice[0] = pick.tc;
    choice[1] = pick.ns;
    choice[2] = pick.scaled;
    choice[3] = best >= 0 ? (int)(1e3f * best_ms * 1000.f / (float)sample) : 0;
  }
  return st;
}

static int check_err(letkf_sweep_t h) {
  int f = 0;
  if (cudaMemcpy(&f, h->err_flag, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return LETKF_ERR_CUDA;
  return f ? LETKF_ERR_TIMEOUT : LETKF_OK;
}

int letkf_sweep_get_analysis(letkf_sweep_t h, void* xa, int on_device) {
  if (!h || !xa) return LETKF_ERR_ARG;
  const size_t bytes = (size_t)h->d.npts * h->d.nv * h->d.ne * elem(h);
  cudaMemcpyAsync(xa, h->xa, bytes, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, h->stream);
  const int st = cuda_status(cudaStreamSynchronize(h->stream));
  return st != LETKF_OK ? st : check_err(h);
}

int letkf_sweep_deferred(letkf_sweep_t h, int* count) {
  if (!h || !count) return LETKF_ERR_ARG;
  *count = 0;
  if (h->d.precision == LETKF_PREC_F64) return LETKF_OK;
  if (cudaMemcpyAsync(count, h->defer_total, sizeof(int), cudaMemcpyDeviceToHost, h->stream) != cudaSuccess)
    return LETKF_ERR_CUDA;
  return cuda_status(cudaStreamSynchronize(h->stream));
}

int letkf_sweep_get_diagnostics(letkf_sweep_t h, double* infl, int* nobsl, int* status, int* sweeps) {
  if (!h) return LETKF_ERR_ARG;
  const size_t np = (size_t)h->d.npts;
  cudaStreamSynchronize(h->stream);
  if (infl) cudaMemcpy(infl, h->infl, sizeof(double) * np, cudaMemcpyDeviceToHost);
  if (nobsl) cudaMemcpy(nobsl, h->nobsl, sizeof(int) * np, cudaMemcpyDeviceToHost);
  if (status) cudaMemcpy(status, h->status, sizeof(int) * np, cudaMemcpyDeviceToHost);
  if (sweeps) cudaMemcpy(sweeps, h->sweeps, sizeof(int) * np, cudaMemcpyDeviceToHost);
  const int st = cuda_status(cudaGetLastError());
  return st != LETKF_OK ? st : check_err(h);
}

int letkf_sweep_set_obs_groups(letkf_sweep_t h, const int* uid, const int* typ, int nid, int ntyp) {
  if (!h || nid < 1 || ntyp < 1 || (int64_t)nid * ntyp >= (int64_t)INT32_MAX) return LETKF_ERR_ARG;
  const int n = h->nobs;
  if (n > 0 && (!uid || !typ)) return LETKF_ERR_ARG;
  for (int i = 0; i < n; i++)
    if (uid[i] < 1 || uid[i] > nid || typ[i] < 1 || typ[i] > ntyp) return LETKF_ERR_ARG;
  h->groups_set = true;
  if (n == 0) return LETKF_OK;
  cudaStream_t s = h->stream;
  int *du = nullptr, *dt = nullptr;
  int st = dalloc(&du, (size_t)n, s);
  st |= dalloc(&dt, (size_t)n, s);
  if (st != LETKF_OK) return LETKF_ERR_CUDA;
  cudaMemcpyAsync(du, uid, sizeof(int) * n, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(dt, typ, sizeof(int) * n, cudaMemcpyHostToDevice, s);
  st = launch_obs_group(n, du, dt, nid, h->operm, h->ogrp, s);
  dfree(du, s);
  dfree(dt, s);
  const int st2 = cuda_status(cudaStreamSynchronize(s));
  if (st != LETKF_OK || st2 != LETKF_OK) h->groups_set = false;
  return st != LETKF_OK ? st : st2;
}

int letkf_sweep_set_probe(letkf_sweep_t h, int npts_probe, const int* points, int cap) {
  if (!h || npts_probe < 0 || (npts_probe > 0 && (!points || cap < 1))) return LETKF_ERR_ARG;
  if ((int64_t)npts_probe * cap > ((int64_t)1 << 31)) return LETKF_ERR_CAPACITY;
  const int np = h->d.npts;
  std::vector<int> slot(np, -1);
  for (int i = 0; i < npts_probe; i++) {
    const int p = points[i];
    if (p < 0 || p >= np || slot[p] >= 0) return LETKF_ERR_ARG;  // out of range or repeated
    slot[p] = i;
  }
  cudaStream_t s = h->stream;
  void* old[] = {h->probe_slot, h->probe_idx, h->probe_count, h->probe_rloc};
  for (void* p : old) dfree(p, s);
  h->probe_slot = h->probe_idx = h->probe_count = nullptr;
  h->probe_rloc = nullptr;
  h->nprobe = 0;
  h->probe_cap = 0;
  if (npts_probe == 0) return cuda_status(cudaStreamSynchronize(s));
  const size_t tot = (size_t)npts_probe * cap;
  int st = dalloc(&h->probe_slot, (size_t)np, s);
  st |= dalloc(&h->probe_idx, tot, s);
  st |= dalloc(&h->probe_rloc, tot, s);
  st |= dalloc(&h->probe_count, (size_t)npts_probe, s);
  if (st != LETKF_OK) return LETKF_ERR_CUDA;
  cudaMemcpyAsync(h->probe_slot, slot.data(), sizeof(int) * np, cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(h->probe_idx, 0xff, sizeof(int) * tot, s);
  cudaMemsetAsync(h->probe_count, 0xff, sizeof(int) * npts_probe, s);
  h->nprobe = npts_probe;
  h->probe_cap = cap;
  return cuda_status(cudaStreamSynchronize(s));
}

int letkf_sweep_get_probe(letkf_sweep_t h, int* count, int* obs, float* rloc) {
  if (!h || h->nprobe == 0) return LETKF_ERR_ARG;
  cudaStream_t s = h->stream;
  const size_t tot = (size_t)h->nprobe * h->probe_cap;
  std::vector<int> cnt(h->nprobe), idx(obs ? tot : 0), perm(obs ? (size_t)h->nobs : 0);
  cudaMemcpyAsync(cnt.data(), h->probe_count, sizeof(int) * h->nprobe, cudaMemcpyDeviceToHost, s);
  if (obs) {
    cudaMemcpyAsync(idx.data(), h->probe_idx, sizeof(int) * tot, cudaMemcpyDeviceToHost, s);
    if (h->nobs > 0) cudaMemcpyAsync(perm.data(), h->operm, sizeof(int) * h->nobs, cudaMemcpyDeviceToHost, s);
  }
  if (rloc) cudaMemcpyAsync(rloc, h->probe_rloc, sizeof(float) * tot, cudaMemcpyDeviceToHost, s);
  const int st = cuda_status(cudaStreamSynchronize(s));
  if (st != LETKF_OK) return st;
  if (count) memcpy(count, cnt.data(), sizeof(int) * h->nprobe);
  if (obs)
    for (size_t i = 0; i < tot; i++) obs[i] = (idx[i] >= 0 && idx[i] < h->nobs) ? perm[(size_t)idx[i]] : -1;
  return LETKF_OK;
}

int letkf_sweep_footprint(const letkf_sweep_desc* d, int nobs, size_t* bytes) {
  if (!d || !bytes || nobs < 0 || d->npts < 0 || d->ne < 1 || d->nv < 1) return LETKF_ERR_ARG;
  const size_t np = (size_t)d->npts, n = (size_t)nobs, ne = (size_t)d->ne;
  const size_t es = d->precision == LETKF_PREC_F64 ? 8 : 4;
  const size_t ncell = (size_t)d->nlon * d->nlat;
  // resident: points, ensembles, per-point outputs, bucket table, sorted observations
  size_t b = np * (6 * 8 + 4 * 5) + 2 * np * d->nv * ne * es + (ncell + d->nlat) * 4 + 64;
  b += n * (6 * 8 + 4 * 4 + 2 * 16 + 4 + ne * es);
  // set_obs staging (unsorted records, permutation, cell counts) while the above is live
  size_t stage = n * (6 * 8 + 4 * 4 + ne * 8) + ncell * 16 + 64;
  if (d->precision == LETKF_PREC_MIXED && d->ne <= 128 && np > 1) {
    // the tensor-core sweeps' column cache (allocated when the points come in
    // columns): slots per SM times the SMs of this device (152 when there is none)
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm < 1) {
      cudaGetLastError();
      nsm = 152;
    }
    b += (size_t)nsm * LETKF_COL_SLOTS_PER_SM * LETKF_COL_CAP * 32;
  }
  if (d->precision == LETKF_PREC_F64) {
    // run_f64 chunk buffers with the local lists of one chunk (L <= nobs per point)
    const size_t c = np < 16384 ? np : 16384;
    const size_t run = c * (4 + 8 + ne * ne * 8 + ne * 8) + 4096;
    stage = stage > run ? stage : run;
  }
  *bytes = b + stage;
  return LETKF_OK;
}

int letkf_sort_obs_latlon(int nlon, int nlat, const double* lon, const double* lat, int nobs, const double* olon,
                          const double* olat, const int* qc, int* perm, int* nsorted, int* nobsgrd, void* stream) {
  if (nlon < 2 || nlat < 3 || nobs < 0 || !lon || !lat || !perm || !nsorted || !nobsgrd) return LETKF_ERR_ARG;
  if (nobs > 0 && (!olon || !olat)) return LETKF_ERR_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return LETKF_ERR_NOGPU;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int ncell = nlon * nlat;
  int *cell = nullptr, *counts = nullptr, *cursor = nullptr;
  int64_t *start = nullptr, *scr = nullptr;
  int st = LETKF_OK;
  st |= dalloc(&cell, (size_t)nobs, s);
  st |= dalloc(&counts, (size_t)ncell, s);
  st |= dalloc(&cursor, (size_t)ncell, s);
  st |= dalloc(&start, (size_t)ncell + 1, s);
  st |= dalloc(&scr, (size_t)ncell / 1024 + 2, s);
  if (st == LETKF_OK) {
    cudaMemsetAsync(counts, 0, sizeof(int) * ncell, s);
    cudaMemsetAsync(cursor, 0, sizeof(int) * ncell, s);
    if (nobs > 0) {
      latlon_cell_kernel<<<(nobs + 255) / 256, 256, 0, s>>>(nobs, nlon, nlat, lon, lat, olon, olat, qc, cell, counts);
      note_launch();
    }
    st = launch_exclusive_scan(ncell, counts, start, scr, s);
  }
  if (st == LETKF_OK && nobs > 0) {
    latlon_scatter_kernel<<<(nobs + 255) / 256, 256, 0, s>>>(nobs, cell, start, cursor, perm);
    // input order inside each cell, as the reference's sequential loops give
    obs_stabilize_kernel<<<(ncell + 255) / 256, 256, 0, s>>>(ncell, start, perm);
    note_launch();
    note_launch();
  }
  if (st == LETKF_OK) {
    latlon_grd_kernel<<<(ncell + 255) / 256, 256, 0, s>>>(nlon, nlat, start, nobsgrd);
    note_launch();
    int64_t total = 0;
    cudaMemcpyAsync(&total, start + ncell, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
    st = cuda_status(cudaStreamSynchronize(s));
    *nsorted = (int)total;
  }
  void* fr[] = {cell, counts, cursor, start, scr};
  for (void* p : fr) dfree(p, s);
  const int st2 = cuda_status(cudaStreamSynchronize(s));
  return st != LETKF_OK ? st : st2;
}

int letkf_sweep_sorted_obs(letkf_sweep_t h, int* nobsgrd) {
  if (!h || !nobsgrd) return LETKF_ERR_ARG;
  cudaStreamSynchronize(h->stream);
  return cuda_status(
      cudaMemcpy(nobsgrd, h->G, sizeof(int) * (h->d.nlon + 1) * h->d.nlat, cudaMemcpyDeviceToHost));
}

}  // extern "C"
