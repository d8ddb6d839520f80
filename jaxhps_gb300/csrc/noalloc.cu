// Batched inverse that allocates nothing: hps_inverse_batched_static.
//
// Some callers cannot hand the library a workspace: code that runs where
// cudaMalloc is forbidden or unavailable (inside another allocator's
// callbacks, in a process whose device memory is owned by a pool that hands
// out only the caller's input/output buffers, or in a plugin host that does
// not expose an allocator at all).  For them this file provides one entry
// point whose scratch memory is a file-scope __device__ array, reserved when
// the module is loaded on a device and held by that device until the process
// exits.  The caller still passes the matrices and the output buffers.
//
// Limits and behaviour:
//  * The scratch holds HPS_STATIC_SCRATCH_BYTES (64 MiB).  Requests whose
//    blocked-inverse workspace would exceed it are rejected with
//    HPS_ERR_WORKSPACE before anything is launched.
//  * The scratch is shared by every call on a device and keeps the previous
//    call's contents.  Each call overwrites every scratch region before
//    reading it (the pivot-used flags are cleared by the copy-in kernel), so
//    stale contents never leak into a result; but two calls whose kernels
//    overlap on the GPU (different streams, or different host threads on the
//    same device) race on the scratch and must be serialised by the caller.
//  * The device address of the array is looked up once per device, on the
//    first call made with that device current (cudaGetSymbolAddress).  That
//    first call should therefore come before any stream capture begins.  The
//    address is cached per device index, which holds while the process keeps
//    the runtime's primary context (a cudaDeviceReset would invalidate it).
//  * The size check uses hps_inverse_workspace_size, which adds 256 bytes of
//    alignment slack; the usable limit is therefore 256 bytes below the
//    array's size.

#include <cuda_runtime.h>

#include <mutex>

#include "hps_common.cuh"
#include "hps_internal.h"
#include "../../include/jaxhps_gb300.h"

namespace hps {

constexpr size_t kStaticScratchBytes = HPS_STATIC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

// In host code this name is only a handle for the runtime's symbol lookup,
// never a device address: the address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

static std::mutex g_scratch_mu;
static void* g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of g_static_scratch on the current device (looked up once).
static cudaError_t static_scratch(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (g_scratch_ptr[dev] == nullptr) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return cudaSuccess;
}

template <class T>
static int inverse_static_entry(int n, const void* A, long long lda, long long sA, void* X, long long ldx,
                                long long sX, int batch, int* info, void* stream) {
  void* ws = nullptr;
  cudaError_t e = static_scratch(&ws);
  if (e != cudaSuccess) {
    set_error("hps_inverse_batched_static: looking up the static scratch failed: %s", cudaGetErrorString(e));
    return HPS_ERR_CUDA;
  }
  e = inverse_batched<T>(n, (const T*)A, lda, sA, (T*)X, ldx, sX, batch, info, ws, kStaticScratchBytes,
                         (cudaStream_t)stream);
  if (e != cudaSuccess) {
    set_error("hps_inverse_batched_static: %s", cudaGetErrorString(e));
    return HPS_ERR_CUDA;
  }
  return HPS_OK;
}

}  // namespace hps

using namespace hps;

extern "C" {

int hps_inverse_batched_static(int dtype, int n, const void* A, long long lda, long long strideA, void* X,
                               long long ldx, long long strideX, int batch, int* info, void* stream) {
  if (n < 0 || batch < 0 || !A || !X || dtype < HPS_F64 || dtype > HPS_C64) {
    set_error("hps_inverse_batched_static: invalid arguments");
    return HPS_ERR_ARG;
  }
  const size_t need = inverse_workspace_bytes(dtype, n, batch);
  if (need > kStaticScratchBytes) {
    set_error("hps_inverse_batched_static: n=%d, batch=%d needs %zu scratch bytes, above the fixed %zu-byte "
              "static scratch; use hps_inverse_batched with a workspace or split the batch",
              n, batch, need, kStaticScratchBytes);
    return HPS_ERR_WORKSPACE;
  }
  switch (dtype) {
    case HPS_F64: return inverse_static_entry<double>(n, A, lda, strideA, X, ldx, strideX, batch, info, stream);
    case HPS_F32: return inverse_static_entry<float>(n, A, lda, strideA, X, ldx, strideX, batch, info, stream);
    case HPS_C128: return inverse_static_entry<c128>(n, A, lda, strideA, X, ldx, strideX, batch, info, stream);
    default: return inverse_static_entry<c64>(n, A, lda, strideA, X, ldx, strideX, batch, info, stream);
  }
}

}  // extern "C"
