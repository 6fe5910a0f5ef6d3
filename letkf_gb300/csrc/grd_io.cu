// grd_io.cu -- SPEEDY grid-file records on the device.
//
// A grd file (speedy/common/common_speedy.f90:163-287, read_grd / read_grd4 /
// write_grd / write_grd4) is nrec direct-access records of nlon*nlat REAL(4)
// values, lon fastest: u(k = 1..nlev), v, t, q, then ps, rain.  The reference
// builds with byte-swapped I/O (speedy/letkf/make_letkf.sh:6, -byteswapio),
// so the files are big-endian.  The host reads the members' files back to back
// into one pinned buffer and copies it once; these kernels swap, widen to FP64
// and scatter into the analysis layout (or the reverse for writing), so
// read_ens_mpi / write_ens_mpi (speedy/common/common_mpi_speedy.f90:354-414)
// cost one H2D / D2H copy of the file bytes.  letkf_ens_mean_spread is
// ensmean_grd (common_speedy.f90:335-370) plus the spread of
// write_ensmspr_mpi (common_mpi_speedy.f90:461-515), summed in member order.
#include "letkf_common.cuh"

namespace letkf {

constexpr int GIO_NT = 256;

__device__ __forceinline__ uint32_t bswap32(uint32_t x) { return __byte_perm(x, 0u, 0x0123); }

// raw element (m, r0 + r, ij) -> out[m*ms + r*rs + ij]
template <bool F64>
__global__ void __launch_bounds__(GIO_NT) grd_decode_kernel(int64_t nij, int nrec, int ne, const uint32_t* __restrict__ raw,
                                                         int swap, int r0, int nr, void* out, int64_t ms, int64_t rs) {
  const int64_t total = (int64_t)ne * nr * nij;
  for (int64_t t = (int64_t)blockIdx.x * GIO_NT + threadIdx.x; t < total; t += (int64_t)gridDim.x * GIO_NT) {
    const int64_t q = t / nij, ij = t - q * nij;
    const int m = (int)(q / nr), r = (int)(q - (int64_t)m * nr);
    uint32_t u = raw[((int64_t)m * nrec + r0 + r) * nij + ij];
    if (swap) u = bswap32(u);
    const float v = __uint_as_float(u);
    const int64_t o = (int64_t)m * ms + (int64_t)r * rs + ij;
    if (F64) static_cast<double*>(out)[o] = (double)v;
    else static_cast<float*>(out)[o] = v;
  }
}

template <bool F64>
__global__ void __launch_bounds__(GIO_NT) grd_encode_kernel(int64_t nij, int nrec, int ne, const void* in, int64_t ms,
                                                         int64_t rs, int r0, int nr, int swap, uint32_t* raw) {
  const int64_t total = (int64_t)ne * nr * nij;
  for (int64_t t = (int64_t)blockIdx.x * GIO_NT + threadIdx.x; t < total; t += (int64_t)gridDim.x * GIO_NT) {
    const int64_t q = t / nij, ij = t - q * nij;
    const int m = (int)(q / nr), r = (int)(q - (int64_t)m * nr);
    const int64_t i = (int64_t)m * ms + (int64_t)r * rs + ij;
    const float v = F64 ? __double2float_rn(static_cast<const double*>(in)[i]) : static_cast<const float*>(in)[i];
    uint32_t u = __float_as_uint(v);
    if (swap) u = bswap32(u);
    raw[((int64_t)m * nrec + r0 + r) * nij + ij] = u;
  }
}

// 16-byte path: 4 values per thread (uint4 of file words, two double2 / one
// float4 of field values); one (member, record) row per blockIdx.y
__device__ __forceinline__ uint4 bswap4(uint4 u) {
  return make_uint4(bswap32(u.x), bswap32(u.y), bswap32(u.z), bswap32(u.w));
}

template <bool F64>
__global__ void __launch_bounds__(GIO_NT) grd_decode_vec_kernel(int64_t nij4, int nrec, int ne,
                                                             const uint4* __restrict__ raw, int swap, int r0, int nr,
                                                             void* out, int64_t ms, int64_t rs) {
  const int64_t nq = (int64_t)ne * nr;
  for (int64_t q = blockIdx.y; q < nq; q += gridDim.y) {
    const int m = (int)(q / nr), r = (int)(q - (int64_t)m * nr);
    const uint4* src = raw + ((int64_t)m * nrec + r0 + r) * nij4;
    const int64_t o = (int64_t)m * ms + (int64_t)r * rs;
    for (int64_t i = (int64_t)blockIdx.x * GIO_NT + threadIdx.x; i < nij4; i += (int64_t)gridDim.x * GIO_NT) {
      uint4 u = src[i];
      if (swap) u = bswap4(u);
      const float4 f = make_float4(__uint_as_float(u.x), __uint_as_float(u.y), __uint_as_float(u.z),
                                   __uint_as_float(u.w));
      if (F64) {
        double2* d = reinterpret_cast<double2*>(static_cast<double*>(out) + o) + 2 * i;
        d[0] = make_double2((double)f.x, (double)f.y);
        d[1] = make_double2((double)f.z, (double)f.w);
      } else {
        reinterpret_cast<float4*>(static_cast<float*>(out) + o)[i] = f;
      }
    }
  }
}

template <bool F64>
__global__ void __launch_bounds__(GIO_NT) grd_encode_vec_kernel(int64_t nij4, int nrec, int ne, const void* in,
                                                             int64_t ms, int64_t rs, int r0, int nr, int swap,
                                                             uint4* raw) {
  const int64_t nq = (int64_t)ne * nr;
  for (int64_t q = blockIdx.y; q < nq; q += gridDim.y) {
    const int m = (int)(q / nr), r = (int)(q - (int64_t)m * nr);
    uint4* dst = raw + ((int64_t)m * nrec + r0 + r) * nij4;
    const int64_t o = (int64_t)m * ms + (int64_t)r * rs;
    for (int64_t i = (int64_t)blockIdx.x * GIO_NT + threadIdx.x; i < nij4; i += (int64_t)gridDim.x * GIO_NT) {
      float4 f;
      if (F64) {
        const double2* d = reinterpret_cast<const double2*>(static_cast<const double*>(in) + o) + 2 * i;
        const double2 a = d[0], b = d[1];
        f = make_float4(__double2float_rn(a.x), __double2float_rn(a.y), __double2float_rn(b.x),
                        __double2float_rn(b.y));
      } else {
        f = reinterpret_cast<const float4*>(static_cast<const float*>(in) + o)[i];
      }
      uint4 u = make_uint4(__float_as_uint(f.x), __float_as_uint(f.y), __float_as_uint(f.z), __float_as_uint(f.w));
      if (swap) u = bswap4(u);
      dst[i] = u;
    }
  }
}

static bool vec_ok(int64_t nij, const void* raw, const void* field, int64_t ms, int64_t rs) {
  return nij % 4 == 0 && ms % 4 == 0 && rs % 4 == 0 && reinterpret_cast<uintptr_t>(raw) % 16 == 0 &&
         reinterpret_cast<uintptr_t>(field) % 16 == 0;
}

static dim3 vec_grid(int64_t nij4, int64_t nq) {
  const int64_t gx = (nij4 + GIO_NT - 1) / GIO_NT;
  return dim3((unsigned)(gx < 4096 ? gx : 4096), (unsigned)(nq < 65535 ? nq : 65535));
}

__global__ void __launch_bounds__(GIO_NT) ens_mean_spread_kernel(int64_t nij, int nrec, int ne,
                                                                 const double* __restrict__ x, int64_t ms, int64_t rs,
                                                                 double* mean, double* sprd) {
  const int64_t total = (int64_t)nrec * nij;
  for (int64_t t = (int64_t)blockIdx.x * GIO_NT + threadIdx.x; t < total; t += (int64_t)gridDim.x * GIO_NT) {
    const int64_t r = t / nij, ij = t - r * nij;
    const double* p = x + r * rs + ij;
    double s = p[0];
    for (int m = 1; m < ne; m++) s = __dadd_rn(s, p[(int64_t)m * ms]);
    s = s / (double)ne;
    if (mean) mean[t] = s;
    if (sprd) {
      double d = __dsub_rn(p[0], s);
      double v = __dmul_rn(d, d);
      for (int m = 1; m < ne; m++) {
        d = __dsub_rn(p[(int64_t)m * ms], s);
        v = __dadd_rn(v, __dmul_rn(d, d));
      }
      sprd[t] = sqrt(v / (double)(ne - 1));
    }
  }
}

static int gio_grid(int64_t total) {
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int64_t need = (total + GIO_NT - 1) / GIO_NT;
  const int64_t cap = (int64_t)nsm * 8;
  return (int)(need < cap ? need : cap);
}

static int gio_device() {
  int nd = 0;
  if (cudaGetDeviceCount(&nd) != cudaSuccess || nd < 1) {
    cudaGetLastError();
    return LETKF_ERR_NOGPU;
  }
  return LETKF_OK;
}

}  // namespace letkf

using namespace letkf;

extern "C" int letkf_grd_decode(int64_t nij, int nrec, int ne, const void* raw, int byteswap, int r0, int nr,
                                int out_f64, void* out, int64_t out_mem_stride, int64_t out_rec_stride,
                                void* stream) {
  if (nij < 1 || nrec < 1 || ne < 1 || r0 < 0 || nr < 0 || r0 + nr > nrec || !raw || !out || out_mem_stride < 0 ||
      out_rec_stride < 0)
    return LETKF_ERR_ARG;
  if (reinterpret_cast<uintptr_t>(raw) % 4) return LETKF_ERR_ARG;
  const int st = gio_device();
  if (st != LETKF_OK) return st;
  const int64_t total = (int64_t)ne * nr * nij;
  if (total == 0) return LETKF_OK;
  cudaStream_t s = (cudaStream_t)stream;
  if (vec_ok(nij, raw, out, out_mem_stride, out_rec_stride)) {
    const dim3 g = vec_grid(nij / 4, (int64_t)ne * nr);
    const uint4* r4 = static_cast<const uint4*>(raw);
    if (out_f64)
      grd_decode_vec_kernel<true><<<g, GIO_NT, 0, s>>>(nij / 4, nrec, ne, r4, byteswap, r0, nr, out, out_mem_stride,
                                                       out_rec_stride);
    else
      grd_decode_vec_kernel<false><<<g, GIO_NT, 0, s>>>(nij / 4, nrec, ne, r4, byteswap, r0, nr, out, out_mem_stride,
                                                        out_rec_stride);
    note_launch();
    return cuda_status(cudaGetLastError());
  }
  const uint32_t* r = static_cast<const uint32_t*>(raw);
  if (out_f64)
    grd_decode_kernel<true><<<gio_grid(total), GIO_NT, 0, s>>>(nij, nrec, ne, r, byteswap, r0, nr, out,
                                                                out_mem_stride, out_rec_stride);
  else
    grd_decode_kernel<false><<<gio_grid(total), GIO_NT, 0, s>>>(nij, nrec, ne, r, byteswap, r0, nr, out,
                                                                 out_mem_stride, out_rec_stride);
  note_launch();
  return cuda_status(cudaGetLastError());
}

extern "C" int letkf_grd_encode(int64_t nij, int nrec, int ne, const void* in, int in_f64, int64_t in_mem_stride,
                                int64_t in_rec_stride, int r0, int nr, int byteswap, void* raw, void* stream) {
  if (nij < 1 || nrec < 1 || ne < 1 || r0 < 0 || nr < 0 || r0 + nr > nrec || !raw || !in || in_mem_stride < 0 ||
      in_rec_stride < 0)
    return LETKF_ERR_ARG;
  if (reinterpret_cast<uintptr_t>(raw) % 4) return LETKF_ERR_ARG;
  const int st = gio_device();
  if (st != LETKF_OK) return st;
  const int64_t total = (int64_t)ne * nr * nij;
  if (total == 0) return LETKF_OK;
  cudaStream_t s = (cudaStream_t)stream;
  if (vec_ok(nij, raw, in, in_mem_stride, in_rec_stride)) {
    const dim3 g = vec_grid(nij / 4, (int64_t)ne * nr);
    uint4* r4 = static_cast<uint4*>(raw);
    if (in_f64)
      grd_encode_vec_kernel<true><<<g, GIO_NT, 0, s>>>(nij / 4, nrec, ne, in, in_mem_stride, in_rec_stride, r0, nr,
                                                       byteswap, r4);
    else
      grd_encode_vec_kernel<false><<<g, GIO_NT, 0, s>>>(nij / 4, nrec, ne, in, in_mem_stride, in_rec_stride, r0, nr,
                                                        byteswap, r4);
    note_launch();
    return cuda_status(cudaGetLastError());
  }
  uint32_t* r = static_cast<uint32_t*>(raw);
  if (in_f64)
    grd_encode_kernel<true><<<gio_grid(total), GIO_NT, 0, s>>>(nij, nrec, ne, in, in_mem_stride, in_rec_stride, r0,
                                                                nr, byteswap, r);
  else
    grd_encode_kernel<false><<<gio_grid(total), GIO_NT, 0, s>>>(nij, nrec, ne, in, in_mem_stride, in_rec_stride, r0,
                                                                 nr, byteswap, r);
  note_launch();
  return cuda_status(cudaGetLastError());
}

extern "C" int letkf_ens_mean_spread(int64_t nij, int nrec, int ne, const double* x, int64_t mem_stride,
                                     int64_t rec_stride, double* mean, double* sprd, void* stream) {
  if (nij < 1 || nrec < 1 || ne < 1 || !x || (!mean && !sprd) || mem_stride < 0 || rec_stride < 0)
    return LETKF_ERR_ARG;
  const int st = gio_device();
  if (st != LETKF_OK) return st;
  const int64_t total = (int64_t)nrec * nij;
  ens_mean_spread_kernel<<<gio_grid(total), GIO_NT, 0, (cudaStream_t)stream>>>(nij, nrec, ne, x, mem_stride,
                                                                               rec_stride, mean, sprd);
  note_launch();
  return cuda_status(cudaGetLastError());
}
