// search_l96.cu -- Lorenz-96 observation selection (lorenz96/letkf/letkf.f90:220-254).
//
// The reference loops over all observations i = 1..ny for every grid point
// ix, takes the observation's grid index j as the first maximum of row i of H,
// keeps it when the cyclic distance min(|j - ix|, nx - |j - ix|) < xmaxloc
// (xmaxloc = xlocal * 2 * sqrt(10/3), :75) and drops it again when
// rloc = exp(-0.5 (dist/xlocal)^2) * exp(-0.5 (tdif/tlocal)^2) < 1e-4.
//
// The adaptive modes (msw_local 1, 2; :237-249) weight each candidate by the
// ensemble correlations between the observation's perturbations and the
// point's: wa^sa * wb^sb with wb = |cor(all members)| and wa = 1 - |cor(first
// ceil(k/2)) - cor(rest)| / 2, times the fixed weights in mode 2.
//
// Here the observations are bucketed by grid cell once per call, each point
// visits only the cells within the cut-off, and its list is then sorted by
// observation index, which is the reference's emission order.  Cost per point
// is O(L log L) instead of O(ny), so domains of 1e5 variables stay cheap.
#include <cuda_runtime.h>
#include <stdint.h>

#include "letkf_gpu.h"

namespace letkf {

int cuda_status(cudaError_t e);
void note_launch();
int launch_exclusive_scan(int n, const int* counts, int64_t* offs, int64_t* scratch, cudaStream_t stream);

// first maximum of row i of h (ny x nx, column-major), 1-based
__global__ void l96_cell_kernel(int nx, int ny, const double* __restrict__ h, int* __restrict__ cell) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ny) return;
  double mx = h[i];
  for (int j = 1; j < nx; j++) mx = fmax(mx, h[(size_t)j * ny + i]);
  int jj = nx + 1;
  for (int j = 0; j < nx; j++)
    if (h[(size_t)j * ny + i] == mx) {
      jj = j + 1;
      break;
    }
  cell[i] = jj;
}

__global__ void l96_bucket_count(int nx, int ny, const int* __restrict__ cell, int* __restrict__ cnt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ny) return;
  const int c = cell[i];
  if (c >= 1 && c <= nx) atomicAdd(&cnt[c - 1], 1);
}

__global__ void l96_bucket_fill(int nx, int ny, const int* __restrict__ cell, const int64_t* __restrict__ boff,
                                int* __restrict__ cursor, int* __restrict__ bobs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ny) return;
  const int c = cell[i];
  if (c >= 1 && c <= nx) bobs[boff[c - 1] + atomicAdd(&cursor[c - 1], 1)] = i;
}

struct L96Ctx {
  int nx, ny;
  const int64_t* boff;  // [nx + 1] bucket offsets
  const int* bobs;      // observation indices by bucket
  double xlocal, xmaxloc, tfac;
};

// rloc of an observation at cyclic distance dist, or -1 when not selected
__device__ __forceinline__ double l96_rloc(const L96Ctx& c, int dist) {
  const double d = (double)dist;
  if (!(d < c.xmaxloc)) return -1.0;
  const double q = d / c.xlocal;
  const double r = exp(-0.5 * (q * q)) * c.tfac;
  return r < 0.0001 ? -1.0 : r;
}

template <typename F>
__device__ __forceinline__ void l96_visit(const L96Ctx& c, int ix, F&& f) {
  const int nx = c.nx;
  int reach = (int)ceil(c.xmaxloc);  // dist < xmaxloc  =>  dist <= reach
  if (2 * reach + 1 >= nx) {
    for (int j = 1; j <= nx; j++) {
      const int a = abs(j - ix), dist = min(a, nx - a);
      f(j, dist);
    }
  } else {
    for (int off = -reach; off <= reach; off++) {
      int j = ix + off;
      if (j < 1) j += nx;
      if (j > nx) j -= nx;
      const int a = abs(j - ix), dist = min(a, nx - a);
      f(j, dist);
    }
  }
}

__global__ void l96_search_kernel(L96Ctx c, int npts, const int* __restrict__ pix, const int64_t* __restrict__ offs,
                                  int* __restrict__ nobsl, int* __restrict__ idx, double* __restrict__ rloc,
                                  double* __restrict__ rdiag, double rdiag_value) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npts) return;
  const int ix = pix[p];
  if (!idx) {
    int n = 0;
    l96_visit(c, ix, [&](int j, int dist) {
      if (l96_rloc(c, dist) >= 0.0) n += (int)(c.boff[j] - c.boff[j - 1]);
    });
    nobsl[p] = n;
    return;
  }
  const int64_t base = offs[p];
  int n = 0;
  l96_visit(c, ix, [&](int j, int dist) {
    const double r = l96_rloc(c, dist);
    if (r < 0.0) return;
    for (int64_t q = c.boff[j - 1]; q < c.boff[j]; q++) {
      // insertion into the list kept sorted by observation index
      const int ob = c.bobs[q];
      int t = n;
      while (t > 0 && idx[base + t - 1] > ob) {
        idx[base + t] = idx[base + t - 1];
        rloc[base + t] = rloc[base + t - 1];
        t--;
      }
      idx[base + t] = ob;
      rloc[base + t] = r;
      n++;
    }
  });
  if (rdiag)
    for (int t = 0; t < n; t++) rdiag[base + t] = rdiag_value;
}

// com_mean, com_stdev, com_covar, com_correl (common/common.f90:46-128) over
// n values read through v1(i), v2(i): sequential sums, every operation rounded
// on its own (no contraction), so a point's weights equal a CPU evaluation.
template <typename A, typename B>
__device__ double l96_correl(int n, A v1, B v2) {
  double m1 = 0.0, m2 = 0.0;
  for (int i = 0; i < n; i++) {
    m1 = __dadd_rn(m1, v1(i));
    m2 = __dadd_rn(m2, v2(i));
  }
  m1 = __ddiv_rn(m1, (double)n);
  m2 = __ddiv_rn(m2, (double)n);
  double s1 = 0.0, s2 = 0.0, cv = 0.0;
  for (int i = 0; i < n; i++) {
    const double d1 = __dsub_rn(v1(i), m1), d2 = __dsub_rn(v2(i), m2);
    s1 = __dadd_rn(s1, __dmul_rn(d1, d1));
    s2 = __dadd_rn(s2, __dmul_rn(d2, d2));
    cv = __dadd_rn(cv, __dmul_rn(d1, d2));
  }
  const double nm1 = (double)(n - 1);
  const double sd1 = __dsqrt_rn(__ddiv_rn(s1, nm1)), sd2 = __dsqrt_rn(__ddiv_rn(s2, nm1));
  return __ddiv_rn(__ddiv_rn(__ddiv_rn(cv, nm1), sd1), sd2);
}

// x^e; e == 1 returns x itself, as the exact power does
__device__ __forceinline__ double l96_pow(double x, double e) { return e == 1.0 ? x : pow(x, e); }

// Adaptive localisation inputs: msw_local (0 fixed, 1 adaptive, 2 both), the
// members split ne2 = ceil(ne/2), the exponents, the slot-stacked obs-space
// perturbations [nslot*ny][ne] and the analysis slot's first guess [nx][ne].
struct L96Adapt {
  int mode, ne, ne2;
  double sa, sb;
  const double* hdxf;
  const double* xf;
};

// rloc of observation row `ob` for the point whose first-guess row is xr with
// member mean xm (lorenz96/letkf/letkf.f90:237-249)
__device__ double l96_adapt_rloc(const L96Adapt& a, const double* __restrict__ xr, double xm, int ob, int dist,
                                 double xlocal, double tdif, double tlocal) {
  const double* hr = a.hdxf + (size_t)ob * a.ne;
  const int n2 = a.ne - a.ne2;
  const double c1 = l96_correl(a.ne2, [&](int i) { return hr[i]; }, [&](int i) { return __dsub_rn(xr[i], xm); });
  const double c2 = l96_correl(n2, [&](int i) { return hr[a.ne2 + i]; },
                               [&](int i) { return __dsub_rn(xr[a.ne2 + i], xm); });
  const double c3 = l96_correl(a.ne, [&](int i) { return hr[i]; }, [&](int i) { return __dsub_rn(xr[i], xm); });
  const double wb = fabs(c3);
  const double wa = __dsub_rn(1.0, __dmul_rn(0.5, fabs(__dsub_rn(c1, c2))));
  double r = __dmul_rn(l96_pow(wa, a.sa), l96_pow(wb, a.sb));
  if (a.mode == 2) {
    const double q = __ddiv_rn((double)dist, xlocal), tq = __ddiv_rn(tdif, tlocal);
    r = __dmul_rn(r, exp(-0.5 * __dmul_rn(q, q)));
    r = __dmul_rn(r, exp(-0.5 * __dmul_rn(tq, tq)));
  }
  return r;
}

// 4D-LETKF selection (lorenz96/letkf/letkf.f90:217-254): for analysis slot
// `slot` every observation slot n in order, tdif = |slot - n| (0 when tlocal <
// 0), the observation's row in the slot-stacked arrays being n*ny + i.  Buckets
// of slot n: boff + n*(nx+1), bobs + n*ny.  ADAPT selects the correlation
// weights; every candidate within xmaxloc is then weighted one by one and
// dropped below 1e-4, as the reference does.
struct L96Ctx4d {
  int nx, ny, nslot, slot;
  const int64_t* boff;
  const int* bobs;
  double xlocal, xmaxloc, tlocal;
};

template <bool ADAPT>
__global__ void l96_search4d_kernel(L96Ctx4d c, L96Adapt a, int npts, const int* __restrict__ pix,
                                    const int64_t* __restrict__ offs, int* __restrict__ nobsl, int* __restrict__ idx,
                                    double* __restrict__ rloc, double* __restrict__ rdiag, double rdiag_value) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npts) return;
  const int ix = pix[p];
  const int64_t base = idx ? offs[p] : 0;
  const double* xr = nullptr;
  double xm = 0.0;
  if (ADAPT) {
    xr = a.xf + (size_t)(ix - 1) * a.ne;
    for (int m = 0; m < a.ne; m++) xm = __dadd_rn(xm, xr[m]);
    xm = __ddiv_rn(xm, (double)a.ne);
  }
  int n = 0;
  for (int sl = 0; sl < c.nslot; sl++) {
    L96Ctx s1;
    s1.nx = c.nx;
    s1.ny = c.ny;
    s1.boff = c.boff + (size_t)sl * (c.nx + 1);
    s1.bobs = c.bobs + (size_t)sl * c.ny;
    s1.xlocal = c.xlocal;
    s1.xmaxloc = c.xmaxloc;
    const double tdif = c.tlocal < 0.0 ? 0.0 : (double)abs(c.slot - sl);
    const double tq = tdif / c.tlocal;
    s1.tfac = exp(-0.5 * (tq * tq));
    const int n0 = n;  // this slot's entries start here, sorted by observation index
    l96_visit(s1, ix, [&](int j, int dist) {
      double r0 = 0.0;
      if (ADAPT) {
        if (!((double)dist < c.xmaxloc)) return;
      } else {
        r0 = l96_rloc(s1, dist);
        if (r0 < 0.0) return;
        if (!idx) {
          n += (int)(s1.boff[j] - s1.boff[j - 1]);
          return;
        }
      }
      for (int64_t q = s1.boff[j - 1]; q < s1.boff[j]; q++) {
        const int ob = sl * c.ny + s1.bobs[q];
        double r = r0;
        if (ADAPT) {
          r = l96_adapt_rloc(a, xr, xm, ob, dist, c.xlocal, tdif, c.tlocal);
          if (r < 0.0001) continue;
          if (!idx) {
            n++;
            continue;
          }
        }
        int t = n;
        while (t > n0 && idx[base + t - 1] > ob) {
          idx[base + t] = idx[base + t - 1];
          rloc[base + t] = rloc[base + t - 1];
          t--;
        }
        idx[base + t] = ob;
        rloc[base + t] = r;
        n++;
      }
    });
  }
  if (!idx) {
    nobsl[p] = n;
    return;
  }
  if (rdiag)
    for (int t = 0; t < n; t++) rdiag[base + t] = rdiag_value;
}

}  // namespace letkf

using namespace letkf;

extern "C" {

int letkf_l96_obs_cell(int nx, int ny, const double* h, int* cell, void* stream) {
  if (nx < 1 || ny < 0 || (ny > 0 && (!h || !cell))) return LETKF_ERR_ARG;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n < 1) {
    cudaGetLastError();
    return LETKF_ERR_NOGPU;
  }
  if (ny == 0) return LETKF_OK;
  l96_cell_kernel<<<(ny + 127) / 128, 128, 0, (cudaStream_t)stream>>>(nx, ny, h, cell);
  note_launch();
  return cuda_status(cudaGetLastError());
}

int letkf_search_l96(int nx, int ny, const int* obs_cell, int npts, const int* pix, double xlocal, double tdif,
                     double tlocal, double obserr, const int64_t* offs, int* nobsl, int* idx, double* rloc,
                     double* rdiag, void* stream) {
  if (nx < 1 || ny < 0 || npts < 0 || !(xlocal > 0.0) || (ny > 0 && !obs_cell) || (npts > 0 && !pix))
    return LETKF_ERR_ARG;
  if (!idx && !nobsl) return LETKF_ERR_ARG;
  if (idx && (!offs || !rloc)) return LETKF_ERR_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return LETKF_ERR_NOGPU;
  }
  if (npts == 0) return LETKF_OK;
  cudaStream_t s = (cudaStream_t)stream;
  // buckets: counts [nx], offsets [nx+1], cursor [nx], observations [ny], scan scratch
  const int nb = (nx + 1023) / 1024 + 1;
  const size_t bytes = sizeof(int64_t) * ((size_t)nx + 1 + nb) + sizeof(int) * (2 * (size_t)nx + (size_t)ny + 1);
  unsigned char* buf = nullptr;
  if (cudaMallocAsync((void**)&buf, bytes, s) != cudaSuccess) return LETKF_ERR_CUDA;
  int64_t* boff = reinterpret_cast<int64_t*>(buf);
  int64_t* scr = boff + nx + 1;
  int* cnt = reinterpret_cast<int*>(scr + nb);
  int* cur = cnt + nx;
  int* bobs = cur + nx;
  int st = cuda_status(cudaMemsetAsync(cnt, 0, sizeof(int) * 2 * (size_t)nx, s));
  if (st == LETKF_OK && ny > 0) {
    l96_bucket_count<<<(ny + 255) / 256, 256, 0, s>>>(nx, ny, obs_cell, cnt);
    note_launch();
  }
  if (st == LETKF_OK) st = launch_exclusive_scan(nx, cnt, boff, scr, s);
  if (st == LETKF_OK && ny > 0) {
    l96_bucket_fill<<<(ny + 255) / 256, 256, 0, s>>>(nx, ny, obs_cell, boff, cur, bobs);
    note_launch();
  }
  if (st == LETKF_OK) {
    L96Ctx c;
    c.nx = nx;
    c.ny = ny;
    c.boff = boff;
    c.bobs = bobs;
    c.xlocal = xlocal;
    c.xmaxloc = xlocal * 2.0 * sqrt(10.0 / 3.0);
    const double tq = tlocal < 0.0 ? 0.0 : tdif / tlocal;
    c.tfac = tlocal < 0.0 ? 1.0 : exp(-0.5 * (tq * tq));
    l96_search_kernel<<<(npts + 127) / 128, 128, 0, s>>>(c, npts, pix, offs, nobsl, idx, rloc, rdiag,
                                                         obserr * obserr);
    note_launch();
    st = cuda_status(cudaGetLastError());
  }
  cudaFreeAsync(buf, s);
  return st;
}

}  // extern "C"

namespace {

// bucket every slot's observations by cell, then one selection launch
int search_l96_slots(int nx, int nslot, int ny, const int* obs_cell, int npts, const int* pix, int slot,
                     double xlocal, double tlocal, double obserr, const L96Adapt& a, const int64_t* offs,
                     int* nobsl, int* idx, double* rloc, double* rdiag, void* stream) {
  if (nx < 1 || nslot < 1 || ny < 0 || npts < 0 || slot < 0 || slot >= nslot || !(xlocal > 0.0) ||
      (ny > 0 && !obs_cell) || (npts > 0 && !pix))
    return LETKF_ERR_ARG;
  if (!idx && !nobsl) return LETKF_ERR_ARG;
  if (idx && (!offs || !rloc)) return LETKF_ERR_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return LETKF_ERR_NOGPU;
  }
  if (npts == 0) return LETKF_OK;
  cudaStream_t s = (cudaStream_t)stream;
  // per slot: bucket offsets [nx+1], counts and cursor [nx], observations [ny]; shared scan scratch
  const int nb = (nx + 1023) / 1024 + 1;
  const size_t ns = (size_t)nslot;
  const size_t bytes = sizeof(int64_t) * (ns * ((size_t)nx + 1) + nb) + sizeof(int) * (ns * (2 * (size_t)nx + ny) + 1);
  unsigned char* buf = nullptr;
  if (cudaMallocAsync((void**)&buf, bytes, s) != cudaSuccess) return LETKF_ERR_CUDA;
  int64_t* boff = reinterpret_cast<int64_t*>(buf);
  int64_t* scr = boff + ns * (nx + 1);
  int* cnt = reinterpret_cast<int*>(scr + nb);
  int* cur = cnt + ns * nx;
  int* bobs = cur + ns * nx;
  int st = cuda_status(cudaMemsetAsync(cnt, 0, sizeof(int) * 2 * ns * (size_t)nx, s));
  for (int sl = 0; sl < nslot && st == LETKF_OK; sl++) {
    const int* cell = obs_cell + (size_t)sl * ny;
    if (ny > 0) {
      l96_bucket_count<<<(ny + 255) / 256, 256, 0, s>>>(nx, ny, cell, cnt + (size_t)sl * nx);
      note_launch();
    }
    st = launch_exclusive_scan(nx, cnt + (size_t)sl * nx, boff + (size_t)sl * (nx + 1), scr, s);
    if (st == LETKF_OK && ny > 0) {
      l96_bucket_fill<<<(ny + 255) / 256, 256, 0, s>>>(nx, ny, cell, boff + (size_t)sl * (nx + 1),
                                                       cur + (size_t)sl * nx, bobs + (size_t)sl * ny);
      note_launch();
    }
  }
  if (st == LETKF_OK) {
    L96Ctx4d c;
    c.nx = nx;
    c.ny = ny;
    c.nslot = nslot;
    c.slot = slot;
    c.boff = boff;
    c.bobs = bobs;
    c.xlocal = xlocal;
    c.xmaxloc = xlocal * 2.0 * sqrt(10.0 / 3.0);
    c.tlocal = tlocal;
    const int grid = (npts + 127) / 128;
    if (a.mode == 0)
      l96_search4d_kernel<false><<<grid, 128, 0, s>>>(c, a, npts, pix, offs, nobsl, idx, rloc, rdiag, obserr * obserr);
    else
      l96_search4d_kernel<true><<<grid, 128, 0, s>>>(c, a, npts, pix, offs, nobsl, idx, rloc, rdiag, obserr * obserr);
    note_launch();
    st = cuda_status(cudaGetLastError());
  }
  cudaFreeAsync(buf, s);
  return st;
}

}  // namespace

extern "C" {

int letkf_search_l96_4d(int nx, int nslot, int ny, const int* obs_cell, int npts, const int* pix, int slot,
                        double xlocal, double tlocal, double obserr, const int64_t* offs, int* nobsl, int* idx,
                        double* rloc, double* rdiag, void* stream) {
  L96Adapt a = {};
  return search_l96_slots(nx, nslot, ny, obs_cell, npts, pix, slot, xlocal, tlocal, obserr, a, offs, nobsl, idx, rloc,
                          rdiag, stream);
}

int letkf_search_l96_adaptive(int nx, int nslot, int ny, const int* obs_cell, int npts, const int* pix, int slot,
                              double xlocal, double tlocal, double obserr, int msw_local, double sa, double sb,
                              int ne, const double* hdxf, const double* xf, const int64_t* offs, int* nobsl,
                              int* idx, double* rloc, double* rdiag, void* stream) {
  if (msw_local < 0 || msw_local > 2) return LETKF_ERR_ARG;
  L96Adapt a = {};
  a.mode = msw_local;
  if (msw_local != 0) {
    if (ne < 1 || (nslot > 0 && ny > 0 && !hdxf) || (npts > 0 && !xf)) return LETKF_ERR_ARG;
    a.ne = ne;
    a.ne2 = (ne + 1) / 2;  // CEILING(REAL(nbv)/2.0)
    a.sa = sa;
    a.sb = sb;
    a.hdxf = hdxf;
    a.xf = xf;
  }
  return search_l96_slots(nx, nslot, ny, obs_cell, npts, pix, slot, xlocal, tlocal, obserr, a, offs, nobsl, idx, rloc,
                          rdiag, stream);
}

}  // extern "C"
