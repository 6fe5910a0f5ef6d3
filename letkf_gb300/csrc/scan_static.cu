// scan_static.cu -- exclusive scan whose scratch lives in a fixed device array.
//
// letkf_exclusive_scan obtains its block-sum scratch from the stream-ordered
// allocator.  Some callers cannot allocate device memory at the point where
// they need offsets: a Fortran driver whose device memory is handed out once
// by its own pool, code that runs while an allocation would break a
// real-time or memory-capped budget, or a host thread that must not touch the
// allocator (its device heap is reserved by another framework).  This entry
// point serves them: it performs no allocation of any kind and uses a
// file-scope device array instead.
#include <mutex>

#include "letkf_common.cuh"

namespace letkf {

int launch_exclusive_scan(int, const int*, int64_t*, int64_t*, cudaStream_t);

// One block sum per 1024 counts: n <= LETKF_SCAN_STATIC_MAX_N.  128 KiB that
// every device which loads this library keeps until the process exits.
static __device__ __align__(256) int64_t g_scan_block_sums[LETKF_SCAN_STATIC_MAX_N / 1024];

constexpr int kMaxDevices = 64;
static std::mutex g_scan_mu;
static int64_t* g_scan_ptr[kMaxDevices] = {nullptr};

// Device address of g_scan_block_sums on the current device.  The array's
// name in host code only stands for the symbol; the address that kernels may
// use has to be asked for once per device, with that device current.  The
// address belongs to the device's primary context: it is cached per device for
// the life of the process, so it is not valid across cudaDeviceReset (a
// process that resets a device must not call this entry point afterwards).
static int scan_scratch_address(int64_t** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return LETKF_ERR_CUDA;
  }
  std::lock_guard<std::mutex> lk(g_scan_mu);
  if (!g_scan_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_scan_block_sums);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return LETKF_ERR_CUDA;
    }
    g_scan_ptr[dev] = static_cast<int64_t*>(p);
  }
  *out = g_scan_ptr[dev];
  return LETKF_OK;
}

}  // namespace letkf

extern "C" int letkf_exclusive_scan_static(int n, const int* counts, int64_t* offs, void* stream) {
  using namespace letkf;
  if (n < 0 || !offs || (n > 0 && !counts)) return LETKF_ERR_ARG;
  if (n > LETKF_SCAN_STATIC_MAX_N) return LETKF_ERR_CAPACITY;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return LETKF_ERR_NOGPU;
  }
  int64_t* scratch = nullptr;
  const int st = scan_scratch_address(&scratch);
  if (st != LETKF_OK) return st;
  // every block-sum slot a call reads is written by that call first, so no
  // clearing is needed between calls
  return launch_exclusive_scan(n, counts, offs, scratch, (cudaStream_t)stream);
}
