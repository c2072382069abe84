// noalloc.cu — the mixed-precision product engine for callers that cannot
// allocate device memory.
//
// Some callers of this library cannot call cudaMalloc at the point where
// they need a product: a host application whose device memory is owned by its
// own pool or framework (an embedding that forbids allocation inside its time
// loop), or a plugin whose host grants it no allocation rights.  dqmc_product_device_noalloc serves
// them: the caller passes device buffers for A, B and C, and the BF16 slice
// scratch lives in the file-scope array below, a fixed 1.75 MB reserved in
// every GPU that loads the library until the process exits.
//
// The array is shared by all calls on a device and keeps the last call's
// contents.  Nothing in it has to start at zero: every call rewrites all the
// slices and exponents it reads (the slicing kernel also writes the zero
// padding of each row).  Calls that overlap on the GPU (concurrent streams,
// or several host threads) race on it; the caller serialises them.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/dqmc_gb300.h"
#include "dqmc_device.cuh"
#include "ozaki.cuh"

namespace dqmc {
cudaError_t configure_ozaki_kernels();
void oz_selftest(const double* A, const double* B, double* C, unsigned short* sa, int* ea, unsigned short* sb, int* eb,
                 int N, cudaStream_t st);
int set_last_error(int code, const char* msg);
}  // namespace dqmc

namespace {

constexpr int kNoAllocMaxN = 256;                        // 7-bit x 7 slices, ldk = N
constexpr size_t kSliceElems = 7ull * kNoAllocMaxN * kNoAllocMaxN;
// the slicing kernel writes cfg_for_k(n).slices slices of n x ldk(n) elements per
// operand; both grow with n, so the largest n bounds every call
static_assert((size_t)dqmc::ozaki::cfg_for_k(kNoAllocMaxN).slices * kNoAllocMaxN * ((kNoAllocMaxN + 15) / 16 * 16) <=
                  kSliceElems,
              "no-alloc scratch too small for the slice configuration of its largest n");
constexpr size_t kScratchBytes = 2 * kSliceElems * sizeof(unsigned short)  // A and B slices
                                 + 2 * kNoAllocMaxN * sizeof(int);          // row / column exponents

// the scratch: host code must not take this name as a device address
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_addr[kMaxDevices] = {nullptr};
bool g_ready[kMaxDevices] = {false};

}  // namespace

extern "C" int dqmc_product_device_noalloc(int n, const double* a, const double* b, double* c, void* stream) {
  if (n < 1 || n > kNoAllocMaxN)
    return dqmc::set_last_error(DQMC_ERR_ARG,
                                "dqmc_product_device_noalloc: n must be in [1, 256] (fixed 1.75 MB scratch)");
  if (!a || !b || !c) return dqmc::set_last_error(DQMC_ERR_ARG, "dqmc_product_device_noalloc: null pointer");
  // an error left pending by the caller's own earlier work is theirs, not this call's:
  // report it as such and launch nothing
  cudaError_t e = cudaPeekAtLastError();
  if (e != cudaSuccess) {
    cudaGetLastError();
    return dqmc::set_last_error(DQMC_ERR_CUDA, "dqmc_product_device_noalloc: a CUDA error was pending before the call");
  }
  int dev = 0;
  e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return dqmc::set_last_error(DQMC_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return dqmc::set_last_error(DQMC_ERR_CUDA, "device ordinal out of range");
  void* base = nullptr;
  {
    // first call on this device: resolve the array's device address (with the
    // device current) and set the kernels' shared-memory limits.  Make that
    // first call before any stream capture.
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_ready[dev]) {
      e = cudaGetSymbolAddress(&g_addr[dev], g_noalloc_scratch);
      if (e != cudaSuccess) return dqmc::set_last_error(DQMC_ERR_CUDA, cudaGetErrorString(e));
      e = dqmc::configure_ozaki_kernels();
      if (e != cudaSuccess) return dqmc::set_last_error(DQMC_ERR_CUDA, cudaGetErrorString(e));
      g_ready[dev] = true;
    }
    base = g_addr[dev];
  }
  auto* sa = static_cast<unsigned short*>(base);
  auto* sb = sa + kSliceElems;
  int* ea = reinterpret_cast<int*>(sb + kSliceElems);
  int* eb = ea + kNoAllocMaxN;
  dqmc::oz_selftest(a, b, c, sa, ea, sb, eb, n, static_cast<cudaStream_t>(stream));
  e = cudaGetLastError();
  if (e != cudaSuccess) return dqmc::set_last_error(DQMC_ERR_CUDA, cudaGetErrorString(e));
  return DQMC_OK;
}
