// Internal (C++) interfaces shared between the translation units of the
// native library.  The public boundary is the C ABI in include/jaxhps_gb300.h.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

#include "hps_common.cuh"

namespace hps {

// D = alpha*A@B + beta*C over a strided batch (row-major).  C may be null
// (then beta is ignored) and may alias D.
template <class T>
cudaError_t gemm_batched(int M, int N, int K, T alpha, const T* A, long long lda, long long sA,
                         const T* B, long long ldb, long long sB, T beta, const T* C, long long ldc,
                         long long sC, T* D, long long ldd, long long sD, int batch, cudaStream_t st);

// Batched inverse by Gauss-Jordan elimination with partial (row) pivoting.
// X may alias A.  info[b] = 0 on success, k+1 if the k-th pivot was zero.
// flags: INV_TENSOR_MEMORY lets FP32 blocks of 64 < n <= 224 use the
// tensor-memory kernel (while inverse_tc_policy() is 1); INV_BLOCK_RECURSIVE
// lets FP32 matrices of n >= 224 use the recursive 2 x 2 block inversion
// (pivots within its smallest blocks only; while inverse_rec_policy() is 1).
enum InverseFlags : int { INV_TENSOR_MEMORY = 1, INV_BLOCK_RECURSIVE = 2 };
size_t inverse_workspace_bytes(int dtype, int n, int batch);
template <class T>
cudaError_t inverse_batched(int n, const T* A, long long lda, long long sA, T* X, long long ldx,
                            long long sX, int batch, int* info, void* ws, size_t ws_bytes,
                            cudaStream_t st, int flags = 0);
int inverse_rec_policy();
int set_inverse_rec_policy(int policy);

// FP32 GEMM on the tensor cores (TF32 split into hi + lo, three products);
// gemm_tc_error() reports whether a CTA's bounded wait ever ran out.
cudaError_t gemm_tf32x3(int M, int N, int K, float alpha, const float* A, long long lda, long long sA,
                        const float* B, long long ldb, long long sB, float beta, const float* C, long long ldc,
                        long long sC, float* D, long long ldd, long long sD, int batch, cudaStream_t st);
cudaError_t gemm_tf32x3_c64(int M, int N, int K, float alpha, const c64* A, long long lda, long long sA,
                            const c64* B, long long ldb, long long sB, float beta, const c64* C, long long ldc,
                            long long sC, c64* D, long long ldd, long long sD, int batch, cudaStream_t st);
// Warp-specialised TMA + tcgen05 3xTF32 kernel for N <= 64 (gemm_tc.cu):
// cudaErrorNotSupported for layouts it does not take (gemm_tma_supported).
bool gemm_tma_supported(int M, int N, int K, const float* A, long long lda, long long sA, const float* B,
                        long long ldb, long long sB, int batch);
cudaError_t gemm_tma_f32(int M, int N, int K, float alpha, const float* A, long long lda, long long sA,
                         const float* B, long long ldb, long long sB, float beta, const float* C, long long ldc,
                         long long sC, float* D, long long ldd, long long sD, int batch, cudaStream_t st);
int gemm_tc_error();
// Reads the flag and clears it (both synchronise with the device).
int gemm_tc_error_reset();
// Spin limits of the bounded waits on the current device (polls < 0: keep);
// the previous value is returned through `previous` when it is not null.
cudaError_t set_tc_spin_limit(long long polls, long long* previous);
cudaError_t set_panel_spin_limit(long long polls, long long* previous);
cudaError_t set_itc_spin_limit(long long polls, long long* previous);

// FP32 batched inverse with the tableau in tensor memory (inverse_tc.cu),
// for 64 < n <= 224; used by inverse_batched<float> for the calls that pass
// tensor_memory = true while inverse_tc_policy() is 1, for every call at 2.
bool inverse_tc_supported(int n);
cudaError_t inverse_tc_f32(int n, const float* A, long long lda, long long sA, float* X, long long ldx,
                           long long sX, int batch, int* info, cudaStream_t st);
int inverse_tc_policy();
int set_inverse_tc_policy(int policy);

// Autotuning table of the FP32 products (gemm.cu): per-shape kernel variant,
// a forced variant for timing, and the shape recorder.
int gemm_tune_set(int M, int N, int K, int batch, int variant);
void gemm_tune_clear();
int gemm_force_variant(int variant);
long long gemm_shapes(int mode, long long* out, long long cap);
// Sets the tensor-core policy of gemm_batched (0, 1, 2); returns the old one.
int set_gemm_policy(int p);

// Largest n served by the register-resident single-CTA kernel.
int inverse_small_nmax(int dtype);

// Number of kernels this library has launched (process-wide), reported by
// hps_launch_count().  Every launch site calls note_launch().
void note_launch();

// Kernel classes for the live profiler (hps_profile_begin/end).
// 5-7 single out the kernels that carry most of a mixed-precision step: the
// TMA GEMM (work in algorithmic bytes), the FP32-pair residual update (bytes)
// and the tensor-memory leaf inverse (flops).
enum KernelClass : int {
  KC_GEMM = 1,
  KC_INVERSE = 2,
  KC_MOVE = 3,
  KC_RESIDUAL = 4,
  KC_GEMM_TMA = 5,
  KC_RESIDUAL_DF = 6,
  KC_INVERSE_TC = 7
};

// RAII scope placed around one kernel launch (or a sequence of them): when
// the profiler is armed for `cls`, records a CUDA event pair on `st` around
// it and adds its algorithmic flop (or byte) count.  Scopes opened inside
// another scope record nothing; the outermost one owns the time.
struct ProfScope {
  bool on;
  cudaStream_t st;
  int slot;
  ProfScope(int cls, cudaStream_t st, double work);
  ~ProfScope();
};

// Records an error message for hps_last_error().
void set_error(const char* fmt, ...);

}  // namespace hps
