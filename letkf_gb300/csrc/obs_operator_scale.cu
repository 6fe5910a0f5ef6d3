// obs_operator_scale.cu -- the SCALE observation operator H(x) for
// conventional observations on the device.
//
// For every (observation, member), obsope_cal's OBS_IN_FORMAT 1 path
// (scale/obs/obsope_tools.f90:340-380): phys2ijk (scale/common/
// common_obs_scale.f90:969-1075) turns the pressure of an upper-air
// observation into a fractional level rk against that member's full pressure
// (log p bilinear in (ri, rj) per level, from the lowest level valid in all
// four columns; too high, too low and outside the domain rejected with the
// reference's qc codes); surface observations (element > 9999) take rk = the
// observation's height.  Where that kept qc good, Trans_XtoY (:262-334)
// interpolates u, v (rotated by the map projection's coefficients, staggered
// on request), t, tv = t (1 + fvirt q), q, rh (trilinear, itpl_3d) or ps
// (bilinear, adjusted to the observation height by prsadj, :583-599, with qc
// iqc_ps_ter beyond PS_ADJUST_THRES).  hx = 0 where phys2ijk rejected (the
// obsda value's initial 0), undef with qc 90 for another element; qc(n) is the
// maximum over members (obsope_tools.f90:602-608).
//
// One warp per observation, members over the lanes; products and sums use the
// _rn intrinsics in the reference's expression order, so only log and pow
// differ (by an ulp) from a host build.  phys2ijk takes log of the full
// pressure at the four columns of each level it visits; where the
// observations would take more of those logs than the members' grids hold, a
// first kernel writes ln p for every grid point and member (the same device
// log of the same values, so the same bits) and phys2ijk reads it instead.
// Interpolation stencils keep their upper index in [2, n]: the value of the
// reference wherever its own stencil stays inside the arrays.
#include "letkf_common.cuh"

namespace letkf {

constexpr int SOPE_NT = 256;
constexpr int SC_U = 2819, SC_V = 2820, SC_T = 3073, SC_TV = 3074, SC_Q = 3330, SC_RH = 3331, SC_PS = 14593;
constexpr int IQC_PS_TER = 10, IQC_OUT_VHI = 20, IQC_OUT_VLO = 21, IQC_OUT_H = 22, IQC_OTYPE = 90;
constexpr double SC_UNDEF = -9.99e33;  // common/common.f90:38

struct ScaleFields {
  int nlonh, nlath, nlevh, nlev, khalo, ne;
  const double* lnp;  // [ne][nlath][nlonh][nlevh] ln p of every grid point, or NULL (computed on the way)
  const double* v3d;  // (k, i, j, n) of member m at v3d[m*mem3 + n*var3 + ((j-1)*nlonh + (i-1))*nlevh + (k-1)]
  int64_t mem3, var3;  // n = 0 u, 1 v, 2 t, 3 q, 4 rh, 5 p (full pressure)
  const double* v2d;  // (i, j, n) of member m at v2d[m*mem2 + n*var2 + (j-1)*nlonh + (i-1)]
  int64_t mem2, var2;  // n = 0 ps, 1 t2m, 2 q2m, 3 topo
};

__device__ __forceinline__ double smul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double sadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ssub(double a, double b) { return __dsub_rn(a, b); }

// upper stencil index of coordinate x over 1..n (CEILING, kept in [2, n]) and
// the weight x - (i - 1) of that index
__device__ __forceinline__ long long sc_stencil(double x, long long n, double* a) {
  long long i;
  if (x >= 1.0e15) i = 1000000000000000LL;
  else if (x <= -1.0e15) i = -1000000000000000LL;
  else i = (long long)ceil(x);
  if (i < 2) i = 2;
  if (i > n) i = n;
  *a = ssub(x, (double)(i - 1));
  return i;
}

__device__ __forceinline__ double sf3(const ScaleFields& f, int m, int n, long long k, long long i, long long j) {
  return f.v3d[(int64_t)m * f.mem3 + (int64_t)n * f.var3 + ((int64_t)(j - 1) * f.nlonh + (i - 1)) * f.nlevh + (k - 1)];
}
__device__ __forceinline__ double sf2(const ScaleFields& f, int m, int n, long long i, long long j) {
  return f.v2d[(int64_t)m * f.mem2 + (int64_t)n * f.var2 + (int64_t)(j - 1) * f.nlonh + (i - 1)];
}

// itpl_2d (:1254-1274)
__device__ double sc_itpl2(const ScaleFields& f, int m, int n, double ri, double rj) {
  double ai, aj;
  const long long i = sc_stencil(ri, f.nlonh, &ai), j = sc_stencil(rj, f.nlath, &aj);
  const double bi = ssub(1.0, ai), bj = ssub(1.0, aj);
  double s = smul(smul(sf2(f, m, n, i - 1, j - 1), bi), bj);
  s = sadd(s, smul(smul(sf2(f, m, n, i, j - 1), ai), bj));
  s = sadd(s, smul(smul(sf2(f, m, n, i - 1, j), bi), aj));
  return sadd(s, smul(smul(sf2(f, m, n, i, j), ai), aj));
}

// itpl_3d (:1298-1325) as Trans_XtoY calls it, itpl_3d(v3d(:,:,:,n), rk, ri,
// rj): its first coordinate runs over the levels
__device__ double sc_itpl3(const ScaleFields& f, int m, int n, double rk, double ri, double rj) {
  double aa, ab, ac;
  const long long a = sc_stencil(rk, f.nlevh, &aa), b = sc_stencil(ri, f.nlonh, &ab), c = sc_stencil(rj, f.nlath, &ac);
  const double ba = ssub(1.0, aa), bb = ssub(1.0, ab), bc = ssub(1.0, ac);
  double s = smul(smul(smul(sf3(f, m, n, a - 1, b - 1, c - 1), ba), bb), bc);
  s = sadd(s, smul(smul(smul(sf3(f, m, n, a, b - 1, c - 1), aa), bb), bc));
  s = sadd(s, smul(smul(smul(sf3(f, m, n, a - 1, b, c - 1), ba), ab), bc));
  s = sadd(s, smul(smul(smul(sf3(f, m, n, a, b, c - 1), aa), ab), bc));
  s = sadd(s, smul(smul(smul(sf3(f, m, n, a - 1, b - 1, c), ba), bb), ac));
  s = sadd(s, smul(smul(smul(sf3(f, m, n, a, b - 1, c), aa), bb), ac));
  s = sadd(s, smul(smul(smul(sf3(f, m, n, a - 1, b, c), ba), ab), ac));
  return sadd(s, smul(smul(smul(sf3(f, m, n, a, b, c), aa), ab), ac));
}

// LOG(p_full) at (k, i, j) of member m
__device__ __forceinline__ double sc_logp(const ScaleFields& f, int m, long long k, long long i, long long j) {
  if (f.lnp) return f.lnp[(((int64_t)m * f.nlath + (j - 1)) * f.nlonh + (i - 1)) * f.nlevh + (k - 1)];
  return log(sf3(f, m, 5, k, i, j));
}

// log p of level k bilinear in (ri, rj): itpl_2d_column of LOG(p_full) (:1019-1020)
__device__ __forceinline__ double sc_lnp(const ScaleFields& f, int m, long long k, long long i, long long j, double ai,
                                         double aj) {
  const double bi = ssub(1.0, ai), bj = ssub(1.0, aj);
  double s = smul(smul(sc_logp(f, m, k, i - 1, j - 1), bi), bj);
  s = sadd(s, smul(smul(sc_logp(f, m, k, i, j - 1), ai), bj));
  s = sadd(s, smul(smul(sc_logp(f, m, k, i - 1, j), bi), aj));
  return sadd(s, smul(smul(sc_logp(f, m, k, i, j), ai), aj));
}

// ln p of every grid point of every member
__global__ void scale_lnp_kernel(ScaleFields f, double* lnp) {
  const int64_t plane = (int64_t)f.nlath * f.nlonh * f.nlevh, n = plane * f.ne;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int m = (int)(t / plane);
    const int64_t r = t - (int64_t)m * plane;
    lnp[t] = log(f.v3d[(int64_t)m * f.mem3 + 5 * f.var3 + r]);
  }
}

// phys2ijk (:969-1075): qc, and rk where it is good
__device__ int sc_phys2ijk(const ScaleFields& f, int m, int elem, double ri, double rj, double rlev, double* rk) {
  if (ri < 1.0 || ri > f.nlonh || rj < 1.0 || rj > f.nlath) return IQC_OUT_H;
  if (elem > 9999) {  // surface observation
    *rk = rlev;
    return 0;
  }
  double ai, aj;
  const long long i = sc_stencil(ri, f.nlonh, &ai), j = sc_stencil(rj, f.nlath, &aj);
  const long long top = f.nlev + f.khalo;
  long long ks = 1 + f.khalo;
  for (long long jj = j - 1; jj <= j; jj++)
    for (long long ii = i - 1; ii <= i; ii++) {
      long long k;
      for (k = 1 + f.khalo; k <= top; k++)
        if (sf3(f, m, 5, k, ii, jj) >= 0.0) break;
      if (k > ks) ks = k;
    }
  const double lr = log(rlev);
  if (lr < sc_lnp(f, m, top, i, j, ai, aj)) return IQC_OUT_VHI;
  // ks = top + 1 (a column without a valid level): plev(ks) is a halo level, as in the reference
  if (lr > sc_lnp(f, m, ks, i, j, ai, aj)) return IQC_OUT_VLO;
  long long k;
  double pk = 0.0;
  for (k = ks + 1; k <= top; k++) {
    pk = sc_lnp(f, m, k, i, j, ai, aj);
    if (pk < lr) break;
  }
  if (k > top) pk = sc_lnp(f, m, k, i, j, ai, aj);  // the loop ran out (k = top + 1, or ks + 1 past it)
  const double pk1 = sc_lnp(f, m, k - 1, i, j, ai, aj);
  *rk = sadd((double)(k - 1), ssub(lr, pk1) / ssub(pk, pk1));
  return 0;
}

__global__ void __launch_bounds__(SOPE_NT) scale_obsope_kernel(ScaleFields f, int nobs, const int* __restrict__ elem,
                                                               const double* __restrict__ ri_,
                                                               const double* __restrict__ rj_,
                                                               const double* __restrict__ rlev_,
                                                               const double* __restrict__ rotc, int stggrd,
                                                               double ps_thres, double* hx, int* qc_member, int* qc) {
  const int lane = threadIdx.x & 31;
  const int nwarp = gridDim.x * (SOPE_NT / 32);
  const double fvirt = 461.50 / 287.05 - 1.0;            // common/common.f90:30-34
  const double ps_pow = 9.81 / (5.0e-3 * 287.05);        // gg / (gamma rd), prsadj
  for (int n = blockIdx.x * (SOPE_NT / 32) + (threadIdx.x >> 5); n < nobs; n += nwarp) {
    const int el = elem[n];
    const double ri = ri_[n], rj = rj_[n], lev = rlev_[n];
    const double rc1 = rotc ? rotc[2 * (size_t)n] : 1.0, rc2 = rotc ? rotc[2 * (size_t)n + 1] : 0.0;
    int qmax = 0;
    for (int m = lane; m < f.ne; m += 32) {
      double rk = 0.0, y = 0.0;
      int q = sc_phys2ijk(f, m, el, ri, rj, lev, &rk);
      if (q == 0) {  // Trans_XtoY
        y = SC_UNDEF;
        if (el == SC_U || el == SC_V) {
          double u, v;
          if (stggrd == 1) {
            u = sc_itpl3(f, m, 0, rk, ssub(ri, 0.5), rj);
            v = sc_itpl3(f, m, 1, rk, ri, ssub(rj, 0.5));
          } else {
            u = sc_itpl3(f, m, 0, rk, ri, rj);
            v = sc_itpl3(f, m, 1, rk, ri, rj);
          }
          y = el == SC_U ? ssub(smul(u, rc1), smul(v, rc2)) : sadd(smul(u, rc2), smul(v, rc1));
        } else if (el == SC_T) {
          y = sc_itpl3(f, m, 2, rk, ri, rj);
        } else if (el == SC_TV) {
          const double t = sc_itpl3(f, m, 2, rk, ri, rj), qv = sc_itpl3(f, m, 3, rk, ri, rj);
          y = smul(t, sadd(1.0, smul(fvirt, qv)));
        } else if (el == SC_Q) {
          y = sc_itpl3(f, m, 3, rk, ri, rj);
        } else if (el == SC_PS) {
          const double t = sc_itpl2(f, m, 1, ri, rj), qv = sc_itpl2(f, m, 2, ri, rj);
          const double topo = sc_itpl2(f, m, 3, ri, rj);
          y = sc_itpl2(f, m, 0, ri, rj);
          const double dz = ssub(rk, topo);
          if (dz != 0.0) {  // prsadj (:583-599)
            const double tv = smul(t, sadd(1.0, smul(0.608, qv)));
            y = smul(y, pow(sadd(smul(-5.0e-3, dz), tv) / tv, ps_pow));
          }
          if (fabs(dz) > ps_thres) q = IQC_PS_TER;
        } else if (el == SC_RH) {
          y = sc_itpl3(f, m, 4, rk, ri, rj);
        } else {
          q = IQC_OTYPE;
        }
      }
      hx[(size_t)n * f.ne + m] = y;
      if (qc_member) qc_member[(size_t)n * f.ne + m] = q;
      qmax = max(qmax, q);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) qmax = max(qmax, __shfl_xor_sync(0xffffffffu, qmax, o));
    if (qc && lane == 0) qc[n] = qmax;
  }
}

}  // namespace letkf

using namespace letkf;

extern "C" int letkf_scale_obsope(int nlonh, int nlath, int nlev, int khalo, int ne, const double* v3d,
                                  int64_t v3d_mem_stride, int64_t v3d_var_stride, const double* v2d,
                                  int64_t v2d_mem_stride, int64_t v2d_var_stride, int nobs, const int* elem,
                                  const double* ri, const double* rj, const double* rlev, const double* rotc,
                                  int stggrd, double ps_adjust_thres, double* hx, int* qc_member, int* qc,
                                  void* stream) {
  if (nlonh < 2 || nlath < 2 || nlev < 2 || khalo < 2 || ne < 1 || nobs < 0) return LETKF_ERR_ARG;
  const int64_t plane3 = (int64_t)nlonh * nlath * (nlev + 2 * khalo), plane2 = (int64_t)nlonh * nlath;
  if (!v3d || !v2d || v3d_var_stride < plane3 || v2d_var_stride < plane2 || v3d_mem_stride < 0 || v2d_mem_stride < 0)
    return LETKF_ERR_ARG;
  if (nobs > 0 && (!elem || !ri || !rj || !rlev || !hx)) return LETKF_ERR_ARG;
  int nd = 0;
  if (cudaGetDeviceCount(&nd) != cudaSuccess || nd < 1) {
    cudaGetLastError();
    return LETKF_ERR_NOGPU;
  }
  if (nobs == 0) return LETKF_OK;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int per = SOPE_NT / 32;
  const int need = (nobs + per - 1) / per;
  const int grid = need < nsm * 8 ? need : nsm * 8;
  ScaleFields f{nlonh, nlath, nlev + 2 * khalo, nlev, khalo, ne, nullptr, v3d, v3d_mem_stride, v3d_var_stride,
                v2d, v2d_mem_stride, v2d_var_stride};
  cudaStream_t s = (cudaStream_t)stream;
  // ln p once per grid point where the observations would visit more (four
  // columns, about half the levels each)
  const int64_t plane = (int64_t)nlath * nlonh * f.nlevh;
  double* lnp = nullptr;
  if ((int64_t)nobs * 4 * (nlev / 2 + 1) > plane && cudaMallocAsync((void**)&lnp, sizeof(double) * plane * ne, s) ==
                                                        cudaSuccess) {
    const int64_t n = plane * ne;
    const int64_t blocks = (n + 255) / 256;
    scale_lnp_kernel<<<(unsigned)(blocks < (int64_t)nsm * 16 ? blocks : (int64_t)nsm * 16), 256, 0, s>>>(f, lnp);
    note_launch();
    f.lnp = lnp;
  } else {
    cudaGetLastError();  // an allocation that failed leaves the on-the-way logs
  }
  scale_obsope_kernel<<<grid, SOPE_NT, 0, s>>>(f, nobs, elem, ri, rj, rlev, rotc, stggrd, ps_adjust_thres, hx,
                                               qc_member, qc);
  note_launch();
  const int st = cuda_status(cudaGetLastError());
  if (lnp) cudaFreeAsync(lnp, s);
  return st;
}
