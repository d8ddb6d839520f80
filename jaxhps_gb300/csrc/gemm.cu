// Strided-batched GEMM on CUDA cores:  D = alpha * A @ B + beta * C
// (row-major, every operand with its own leading dimension and batch
// stride; a batch stride of 0 broadcasts one operand to the whole batch).
//
// This is the workhorse of every HPS stage: leaf operator products
// (Y = A_ii^-1 (-A_ie P), T = Q Y), the Schur-complement products of the
// merges (S = -D^-1 C, T = A + B S) and the down pass (g = S g + g~,
// u = Y g + v).  Register-tiled, double-buffered through shared memory,
// templated over the element type so the same code serves f64 / f32 /
// complex128 / complex64.
#include <stdlib.h>

#include <atomic>
#include <map>
#include <mutex>
#include <tuple>
#include <type_traits>
#include <vector>

#include <cooperative_groups.h>

#include "hps_common.cuh"

#include "hps_internal.h"

namespace hps {

template <class T, int BM, int BN, int BK, int TM, int TN>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
gemm_kernel(int M, int N, int K, T alpha, const T* __restrict__ A, long long lda, long long sA,
            const T* __restrict__ B, long long ldb, long long sB, T beta, const T* C,
            long long ldc, long long sC, T* D, long long ldd, long long sD, int use_c) {
  constexpr int NTX = BN / TN;
  constexpr int NTY = BM / TM;
  constexpr int NT = NTX * NTY;
  constexpr int LA = (BM * BK + NT - 1) / NT;
  constexpr int LB = (BK * BN + NT - 1) / NT;
  __shared__ T As[2][BK][BM + 1];
  __shared__ T Bs[2][BK][BN];

  const long long bz = blockIdx.z;
  A += bz * sA;
  B += bz * sB;
  D += bz * sD;
  if (use_c) C += bz * sC;
  const int m0 = blockIdx.y * BM;
  const int n0 = blockIdx.x * BN;
  const int tid = threadIdx.x;
  const int tx = tid % NTX;
  const int ty = tid / NTX;

  T ra[LA], rb[LB];
  auto load_tiles = [&](int k0) {
#pragma unroll
    for (int l = 0; l < LA; ++l) {
      int e = tid + l * NT;
      T v = zero<T>();
      if (e < BM * BK) {
        int r = e / BK, c = e % BK;
        int gm = m0 + r, gk = k0 + c;
        if (gm < M && gk < K) v = A[(long long)gm * lda + gk];
      }
      ra[l] = v;
    }
#pragma unroll
    for (int l = 0; l < LB; ++l) {
      int e = tid + l * NT;
      T v = zero<T>();
      if (e < BK * BN) {
        int r = e / BN, c = e % BN;
        int gk = k0 + r, gn = n0 + c;
        if (gk < K && gn < N) v = B[(long long)gk * ldb + gn];
      }
      rb[l] = v;
    }
  };
  auto store_tiles = [&](int buf) {
#pragma unroll
    for (int l = 0; l < LA; ++l) {
      int e = tid + l * NT;
      if (e < BM * BK) As[buf][e % BK][e / BK] = ra[l];
    }
#pragma unroll
    for (int l = 0; l < LB; ++l) {
      int e = tid + l * NT;
      if (e < BK * BN) Bs[buf][e / BN][e % BN] = rb[l];
    }
  };

  T acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = zero<T>();

  const int ktiles = (K + BK - 1) / BK;
  if (ktiles > 0) {
    load_tiles(0);
    store_tiles(0);
    __syncthreads();
  }
  for (int kt = 0; kt < ktiles; ++kt) {
    const int buf = kt & 1;
    if (kt + 1 < ktiles) load_tiles((kt + 1) * BK);
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      T a[TM], b[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = As[buf][kk][ty + i * NTY];
#pragma unroll
      for (int j = 0; j < TN; ++j) b[j] = Bs[buf][kk][tx + j * NTX];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = fma_(a[i], b[j], acc[i][j]);
    }
    if (kt + 1 < ktiles) {
      store_tiles(buf ^ 1);
      __syncthreads();
    }
  }

#pragma unroll
  for (int i = 0; i < TM; ++i) {
    const int gm = m0 + ty + i * NTY;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int gn = n0 + tx + j * NTX;
      if (gn >= N) continue;
      T v = mul(alpha, acc[i][j]);
      if (use_c) v = fma_(beta, C[(long long)gm * ldc + gn], v);
      D[(long long)gm * ldd + gn] = v;
    }
  }
}

// FP32 8x8 register tiles with 16-byte shared-memory loads.  Thread (tx, ty)
// owns rows {4ty .. 4ty+3} and {BM/2 + 4ty ..} and columns {4tx .. 4tx+3}
// and {BN/2 + 4tx ..}: each k step reads its 8 A and 8 B values with four
// 16-byte loads (a warp's loads from one row of As or Bs cover one
// contiguous 64- or 128-byte span), where gemm_kernel<float, .., 8, 8> uses
// sixteen 4-byte loads.  A is stored transposed with a row pitch of BM + 4
// floats, which makes the transposing stores conflict-free.  Global tiles
// move as float4 where the rows allow it (vec_* flags, checked on the host).
// The k order of every output's FMA chain is that of gemm_kernel, so the two
// kernels give identical results.
//
// SPLIT: split-K for products with few output tiles and a long K (the
// correction's products at the top merge levels: a few tall N = 64 tiles,
// K in the thousands).  The `splits` CTAs of a thread-block cluster share one
// output tile, CTA r accumulating the K-slice r; each stores its partial tile
// in shared memory and, after a cluster barrier, sums its BM / splits rows
// of the tile over the partials of ranks 0, 1, ... in that order (reads
// through distributed shared memory), so the result is deterministic and no
// global workspace is needed.
template <int BM, int BN, bool SPLIT = false>
__global__ void __launch_bounds__((BM / 8) * (BN / 8), 65536 / ((BM / 8) * (BN / 8) * 128))   // <= 128 registers
gemm_f32_v4_kernel(int M, int N, int K, float alpha, const float* __restrict__ A, long long lda, long long sA,
                   const float* __restrict__ B, long long ldb, long long sB, float beta, const float* C,
                   long long ldc, long long sC, float* D, long long ldd, long long sD, int use_c, int vec_a,
                   int vec_b, int vec_cd, int splits) {
  constexpr int BK = 8;
  constexpr int NTX = BN / 8, NTY = BM / 8, NT = NTX * NTY;
  constexpr int PA = BM + 4;
  constexpr int A4 = BM * BK / 4 / NT;   // float4 chunks of the A tile per thread
  constexpr int B4 = BK * BN / 4 / NT;
  static_assert(A4 >= 1 && B4 >= 1 && A4 * 4 * NT == BM * BK && B4 * 4 * NT == BK * BN, "tile split");
  __shared__ __align__(16) float As[2][BK][PA];
  __shared__ __align__(16) float Bs[2][BK][BN];

  const long long bz = blockIdx.z;
  A += bz * sA;
  B += bz * sB;
  D += bz * sD;
  if (use_c) C += bz * sC;
  const int m0 = blockIdx.y * BM;
  int tile_x = blockIdx.x, kbeg = 0, kend = K;
  if constexpr (SPLIT) {
    // cluster dims (splits, 1, 1): the CTAs of a cluster are consecutive in x
    const int r = (int)(blockIdx.x % (unsigned)splits);
    tile_x = (int)(blockIdx.x / (unsigned)splits);
    const int kc = ((K + splits - 1) / splits + BK - 1) / BK * BK;   // multiple of BK: float4 loads stay aligned
    kbeg = min(K, r * kc);
    kend = min(K, kbeg + kc);
  }
  const int n0 = tile_x * BN;
  const int tid = threadIdx.x;
  const int tx = tid % NTX;
  const int ty = tid / NTX;

  float4 ra[A4], rb[B4];
  auto load_tiles = [&](int k0) {
#pragma unroll
    for (int l = 0; l < A4; ++l) {
      const int f = tid + l * NT;
      const int r = f / (BK / 4), c = (f % (BK / 4)) * 4;
      const int gm = m0 + r, gk = k0 + c;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (gm < M) {
        const float* src = A + (long long)gm * lda + gk;
        if (vec_a && gk + 3 < kend) {
          v = *reinterpret_cast<const float4*>(src);
        } else {
          if (gk < kend) v.x = src[0];
          if (gk + 1 < kend) v.y = src[1];
          if (gk + 2 < kend) v.z = src[2];
          if (gk + 3 < kend) v.w = src[3];
        }
      }
      ra[l] = v;
    }
#pragma unroll
    for (int l = 0; l < B4; ++l) {
      const int f = tid + l * NT;
      const int r = f / (BN / 4), c = (f % (BN / 4)) * 4;
      const int gk = k0 + r, gn = n0 + c;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (gk < kend) {
        const float* src = B + (long long)gk * ldb + gn;
        if (vec_b && gn + 3 < N) {
          v = *reinterpret_cast<const float4*>(src);
        } else {
          if (gn < N) v.x = src[0];
          if (gn + 1 < N) v.y = src[1];
          if (gn + 2 < N) v.z = src[2];
          if (gn + 3 < N) v.w = src[3];
        }
      }
      rb[l] = v;
    }
  };
  auto store_tiles = [&](int buf) {
#pragma unroll
    for (int l = 0; l < A4; ++l) {
      const int f = tid + l * NT;
      const int r = f / (BK / 4), c = (f % (BK / 4)) * 4;
      As[buf][c + 0][r] = ra[l].x;
      As[buf][c + 1][r] = ra[l].y;
      As[buf][c + 2][r] = ra[l].z;
      As[buf][c + 3][r] = ra[l].w;
    }
#pragma unroll
    for (int l = 0; l < B4; ++l) {
      const int f = tid + l * NT;
      const int r = f / (BN / 4), c = (f % (BN / 4)) * 4;
      *reinterpret_cast<float4*>(&Bs[buf][r][c]) = rb[l];
    }
  };

  float acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;

  const int ktiles = (kend - kbeg + BK - 1) / BK;
  if (ktiles > 0) {
    load_tiles(kbeg);
    store_tiles(0);
    __syncthreads();
  }
  for (int kt = 0; kt < ktiles; ++kt) {
    const int buf = kt & 1;
    if (kt + 1 < ktiles) load_tiles(kbeg + (kt + 1) * BK);
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      const float4 a0 = *reinterpret_cast<const float4*>(&As[buf][kk][4 * ty]);
      const float4 a1 = *reinterpret_cast<const float4*>(&As[buf][kk][BM / 2 + 4 * ty]);
      const float4 b0 = *reinterpret_cast<const float4*>(&Bs[buf][kk][4 * tx]);
      const float4 b1 = *reinterpret_cast<const float4*>(&Bs[buf][kk][BN / 2 + 4 * tx]);
      const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float b[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    if (kt + 1 < ktiles) {
      store_tiles(buf ^ 1);
      __syncthreads();
    }
  }

  if constexpr (SPLIT) {
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    __shared__ __align__(16) float part[BM * BN];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int row = i < 4 ? 4 * ty + i : BM / 2 + 4 * ty + i - 4;
#pragma unroll
      for (int h = 0; h < 2; ++h)
        *reinterpret_cast<float4*>(&part[row * BN + h * (BN / 2) + 4 * tx]) =
            make_float4(acc[i][4 * h], acc[i][4 * h + 1], acc[i][4 * h + 2], acc[i][4 * h + 3]);
    }
    cluster.sync();
    const int rank = (int)cluster.block_rank();
    const int rows = BM / splits;
    for (int e = tid; e < rows * BN; e += NT) {
      const int row = rank * rows + e / BN, col = e % BN;
      float sum = 0.f;
      for (int q = 0; q < splits; ++q) sum += *cluster.map_shared_rank(&part[row * BN + col], q);
      const int gm = m0 + row, gn = n0 + col;
      if (gm < M && gn < N) {
        float x = alpha * sum;
        if (use_c) x = fmaf(beta, C[(long long)gm * ldc + gn], x);
        D[(long long)gm * ldd + gn] = x;
      }
    }
    cluster.sync();   // the partial tiles stay alive until every CTA has read them
    return;
  }

#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int gm = m0 + (i < 4 ? 4 * ty + i : BM / 2 + 4 * ty + i - 4);
    if (gm >= M) continue;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int gn = n0 + h * (BN / 2) + 4 * tx;
      float v[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) v[j] = alpha * acc[i][4 * h + j];
      if (vec_cd && gn + 3 < N) {
        if (use_c) {
          const float4 c = *reinterpret_cast<const float4*>(C + (long long)gm * ldc + gn);
          v[0] = fmaf(beta, c.x, v[0]);
          v[1] = fmaf(beta, c.y, v[1]);
          v[2] = fmaf(beta, c.z, v[2]);
          v[3] = fmaf(beta, c.w, v[3]);
        }
        *reinterpret_cast<float4*>(D + (long long)gm * ldd + gn) = make_float4(v[0], v[1], v[2], v[3]);
      } else {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          if (gn + j >= N) continue;
          float x = v[j];
          if (use_c) x = fmaf(beta, C[(long long)gm * ldc + gn + j], x);
          D[(long long)gm * ldd + gn + j] = x;
        }
      }
    }
  }
}

static inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

template <int BM, int BN>
static cudaError_t launch_gemm_f32_v4(int M, int N, int K, float alpha, const float* A, long long lda, long long sA,
                                      const float* B, long long ldb, long long sB, float beta, const float* C,
                                      long long ldc, long long sC, float* D, long long ldd, long long sD, int batch,
                                      cudaStream_t st) {
  const int use_c = (C != nullptr);
  constexpr int NT = (BM / 8) * (BN / 8);
  // float4 rows: leading dimensions and batch strides multiples of 4 floats,
  // base addresses 16-byte aligned (then every row start and k or n offset
  // that is a multiple of 4 is 16-byte aligned too)
  const int vec_a = (lda % 4 == 0) && (sA % 4 == 0) && aligned16(A);
  const int vec_b = (ldb % 4 == 0) && (sB % 4 == 0) && aligned16(B);
  const int vec_cd = (ldd % 4 == 0) && (sD % 4 == 0) && aligned16(D) &&
                     (!use_c || ((ldc % 4 == 0) && (sC % 4 == 0) && aligned16(C)));
  for (int b0 = 0; b0 < batch; b0 += 65535) {
    const int nb = batch - b0 < 65535 ? batch - b0 : 65535;
    dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM, nb);
    ProfScope ps(KC_GEMM, st, 2.0 * M * (double)N * K * nb);
    note_launch();
    // batch offsets keep the alignment: sA, sB, sC, sD are multiples of 4 when the flags are set
    gemm_f32_v4_kernel<BM, BN><<<grid, NT, 0, st>>>(M, N, K, alpha, A + b0 * sA, lda, sA, B + b0 * sB, ldb, sB, beta,
                                                    use_c ? C + b0 * sC : nullptr, ldc, sC, D + b0 * sD, ldd, sD,
                                                    use_c, vec_a, vec_b, vec_cd, 1);
  }
  return cudaGetLastError();
}

// Split-K launch of gemm_f32_v4_kernel<BM, BN, true>: clusters of `splits`
// CTAs (2, 4 or 8, dividing BM) along x, one cluster per output tile.
template <int BM, int BN>
static cudaError_t launch_gemm_f32_v4_split(int M, int N, int K, float alpha, const float* A, long long lda,
                                            long long sA, const float* B, long long ldb, long long sB, float beta,
                                            const float* C, long long ldc, long long sC, float* D, long long ldd,
                                            long long sD, int batch, int splits, cudaStream_t st) {
  if (splits < 2 || splits > 8 || BM % splits != 0) return cudaErrorInvalidValue;
  const int use_c = (C != nullptr);
  constexpr int NT = (BM / 8) * (BN / 8);
  const int vec_a = (lda % 4 == 0) && (sA % 4 == 0) && aligned16(A);
  const int vec_b = (ldb % 4 == 0) && (sB % 4 == 0) && aligned16(B);
  const int vec_cd = (ldd % 4 == 0) && (sD % 4 == 0) && aligned16(D) &&
                     (!use_c || ((ldc % 4 == 0) && (sC % 4 == 0) && aligned16(C)));
  const int tiles_n = (N + BN - 1) / BN;
  for (int b0 = 0; b0 < batch; b0 += 65535) {
    const int nb = batch - b0 < 65535 ? batch - b0 : 65535;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(tiles_n * splits), (unsigned)((M + BM - 1) / BM), (unsigned)nb);
    cfg.blockDim = dim3(NT);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)splits;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    ProfScope ps(KC_GEMM, st, 2.0 * M * (double)N * K * nb);
    note_launch();
    const cudaError_t e = cudaLaunchKernelEx(&cfg, gemm_f32_v4_kernel<BM, BN, true>, M, N, K, alpha, A + b0 * sA,
                                             lda, sA, B + b0 * sB, ldb, sB, beta, use_c ? C + b0 * sC : nullptr,
                                             ldc, sC, D + b0 * sD, ldd, sD, use_c, vec_a, vec_b, vec_cd, splits);
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

template <class T, int BM, int BN, int BK, int TM, int TN>
static cudaError_t launch_gemm_cfg(int M, int N, int K, T alpha, const T* A, long long lda, long long sA,
                                   const T* B, long long ldb, long long sB, T beta, const T* C,
                                   long long ldc, long long sC, T* D, long long ldd, long long sD,
                                   int batch, cudaStream_t st) {
  const int use_c = (C != nullptr);
  constexpr int NT = (BM / TM) * (BN / TN);
  for (int b0 = 0; b0 < batch; b0 += 65535) {
    int nb = batch - b0 < 65535 ? batch - b0 : 65535;
    dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM, nb);
    const double cplx = (sizeof(T) == 16 || (sizeof(T) == 8 && DTypeOf<T>::value == C64)) ? 4.0 : 1.0;
    ProfScope ps(KC_GEMM, st, 2.0 * cplx * M * (double)N * K * nb);
    note_launch();
    gemm_kernel<T, BM, BN, BK, TM, TN><<<grid, NT, 0, st>>>(
        M, N, K, alpha, A + b0 * sA, lda, sA, B + b0 * sB, ldb, sB, beta,
        use_c ? C + b0 * sC : nullptr, ldc, sC, D + b0 * sD, ldd, sD, use_c);
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Skinny products (N <= 8 columns: one or a few right-hand sides).  A tiled
// kernel would spend most of a 64-wide N tile on padding; here one warp owns
// one row of A, its lanes stride over K (coalesced reads of A, the dominant
// traffic) and the N partial sums are reduced with shuffles.  The kernel is
// bound by reading A once.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float shfl_xor_(float v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
__device__ __forceinline__ double shfl_xor_(double v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
__device__ __forceinline__ c64 shfl_xor_(c64 v, int m) {
  return c64{__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m)};
}
__device__ __forceinline__ c128 shfl_xor_(c128 v, int m) {
  return c128{__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m)};
}

constexpr int SK_WARPS = 8;

template <class T, int NB>
__global__ void __launch_bounds__(SK_WARPS * 32)
gemm_skinny_kernel(int M, int N, int K, T alpha, const T* __restrict__ A, long long lda, long long sA,
                   const T* __restrict__ B, long long ldb, long long sB, T beta, const T* C, long long ldc,
                   long long sC, T* D, long long ldd, long long sD, int use_c) {
  const int lane = threadIdx.x & 31;
  const int row = blockIdx.x * SK_WARPS + (threadIdx.x >> 5);
  if (row >= M) return;  // uniform across the warp
  const long long bz = blockIdx.y;
  const T* a = A + bz * sA + (long long)row * lda;
  const T* b = B + bz * sB;
  T acc[NB];
#pragma unroll
  for (int n = 0; n < NB; ++n) acc[n] = zero<T>();
#pragma unroll 4
  for (int k = lane; k < K; k += 32) {
    const T av = a[k];
    const T* br = b + (long long)k * ldb;
#pragma unroll
    for (int n = 0; n < NB; ++n)
      if (n < N) acc[n] = fma_(av, br[n], acc[n]);
  }
#pragma unroll
  for (int n = 0; n < NB; ++n)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc[n] = add(acc[n], shfl_xor_(acc[n], o));
  if (lane < N) {
    T v = acc[0];
#pragma unroll
    for (int n = 1; n < NB; ++n)
      if (lane == n) v = acc[n];
    T out = mul(alpha, v);
    if (use_c) out = fma_(beta, C[bz * sC + (long long)row * ldc + lane], out);
    D[bz * sD + (long long)row * ldd + lane] = out;
  }
}

template <class T, int NB>
static cudaError_t launch_skinny(int M, int N, int K, T alpha, const T* A, long long lda, long long sA, const T* B,
                                 long long ldb, long long sB, T beta, const T* C, long long ldc, long long sC, T* D,
                                 long long ldd, long long sD, int batch, cudaStream_t st) {
  const int use_c = (C != nullptr);
  for (int b0 = 0; b0 < batch; b0 += 65535) {
    const int nb = batch - b0 < 65535 ? batch - b0 : 65535;
    dim3 grid((M + SK_WARPS - 1) / SK_WARPS, nb);
    const double cplx = (sizeof(T) == 16 || (sizeof(T) == 8 && DTypeOf<T>::value == C64)) ? 4.0 : 1.0;
    ProfScope ps(KC_GEMM, st, 2.0 * cplx * M * (double)N * K * nb);
    note_launch();
    gemm_skinny_kernel<T, NB><<<grid, SK_WARPS * 32, 0, st>>>(
        M, N, K, alpha, A + b0 * sA, lda, sA, B + b0 * sB, ldb, sB, beta, use_c ? C + b0 * sC : nullptr, ldc, sC,
        D + b0 * sD, ldd, sD, use_c);
  }
  return cudaGetLastError();
}

// Which products run on the tensor cores (gemm_tc.cu): 0 none, 1 the shapes
// where they were measured faster (default), 2 every FP32 / complex64 product,
// 3 none and the FP32 8x8 tiles with 4-byte shared loads (gemm_kernel) in
// place of gemm_f32_v4_kernel, for comparisons.  HPS_GEMM_TC=0 in the
// environment starts the process at 0; hps_gemm_policy() changes it.
static std::atomic<int> g_policy{-1};

static int gemm_policy() {
  int p = g_policy.load(std::memory_order_relaxed);
  if (p < 0) {
    const char* e = getenv("HPS_GEMM_TC");
    p = (e && e[0] == '0') ? 0 : 1;
    g_policy.store(p, std::memory_order_relaxed);
  }
  return p;
}

int set_gemm_policy(int p) {
  if (p < 0 || p > 3) return -1;
  const int old = gemm_policy();
  g_policy.store(p, std::memory_order_relaxed);
  return old;
}

// ---------------------------------------------------------------------------
// Autotuning of the FP32 products.  A tuner (jaxhps_gb300/autotune.py) records
// the shapes a build + solve issues (hps_gemm_shapes), times every kernel
// variant below on each shape (hps_gemm_force_variant) and stores the fastest
// per (M, N, K, batch) (hps_gemm_tune_set); gemm_batched<float> then runs the
// stored variant and falls back to the measured rules below for other shapes.
// ---------------------------------------------------------------------------
enum GemmVariant {
  GV_TC = 0,          // tcgen05 3xTF32 (gemm_tc.cu)
  GV_V4_128x128 = 1,  // SIMT 8x8 register tiles, 128 x 128 CTA tile
  GV_V4_128x64 = 2,
  GV_V4_64x64 = 3,
  GV_SPLIT2 = 4,      // 64 x 64 tiles, K split over a 2-CTA cluster
  GV_SPLIT4 = 5,
  GV_SPLIT8 = 6,
  GV_GENERIC = 7,     // SIMT 4x4 register tiles, 64 x 64
  GV_TMA = 8,         // warp-specialised TMA + tcgen05 3xTF32, N <= 64 (gemm_tc.cu)
  GV_COUNT = 9
};

static std::mutex g_tune_mu;
static std::map<std::tuple<int, int, int, int>, int> g_tune;
static std::atomic<int> g_tune_size{0};
static std::atomic<int> g_force_variant{-1};
static std::atomic<int> g_shape_log{0};
static std::vector<std::vector<long long>> g_shapes;

int gemm_tune_set(int M, int N, int K, int batch, int variant) {
  if (variant >= GV_COUNT) return -1;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  const auto key = std::make_tuple(M, N, K, batch);
  if (variant < 0) g_tune.erase(key);
  else g_tune[key] = variant;
  g_tune_size.store((int)g_tune.size());
  return 0;
}

void gemm_tune_clear() {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune.clear();
  g_tune_size.store(0);
}

int gemm_force_variant(int variant) {
  if (variant >= GV_COUNT) return -2;
  return g_force_variant.exchange(variant < 0 ? -1 : variant);
}

long long gemm_shapes(int mode, long long* out, long long cap) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  if (mode == 1) {
    g_shapes.clear();
    g_shape_log.store(1);
  } else if (mode == 0) {
    g_shape_log.store(0);
  }
  if (out)
    for (long long i = 0; i < (long long)g_shapes.size() && i < cap; ++i)
      for (int j = 0; j < 13; ++j) out[i * 13 + j] = g_shapes[(size_t)i][(size_t)j];
  return (long long)g_shapes.size();
}

static void log_shape(int M, int N, int K, int batch, long long lda, long long sA, long long ldb, long long sB,
                      long long ldc, long long sC, long long ldd, long long sD, bool has_c) {
  std::vector<long long> e{M, N, K, batch, lda, sA, ldb, sB, ldc, sC, ldd, sD, has_c ? 1 : 0};
  std::lock_guard<std::mutex> lk(g_tune_mu);
  for (const auto& x : g_shapes)
    if (x == e) return;
  g_shapes.push_back(e);
}

static int tuned_variant(int M, int N, int K, int batch) {
  const int f = g_force_variant.load(std::memory_order_relaxed);
  if (f >= 0) return f;
  if (g_tune_size.load(std::memory_order_relaxed) == 0) return -1;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  const auto it = g_tune.find(std::make_tuple(M, N, K, batch));
  return it == g_tune.end() ? -1 : it->second;
}

static cudaError_t run_variant_f32(int v, int M, int N, int K, float alpha, const float* A, long long lda,
                                   long long sA, const float* B, long long ldb, long long sB, float beta,
                                   const float* C, long long ldc, long long sC, float* D, long long ldd,
                                   long long sD, int batch, cudaStream_t st) {
  if (v == GV_TMA) {
    // layouts the TMA kernel does not take run the 64 x 64 SIMT tiles
    const cudaError_t e = gemm_tma_f32(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, D, ldd, sD, batch, st);
    if (e != cudaErrorNotSupported) return e;
    v = GV_V4_64x64;
  }
  switch (v) {
    case GV_TC:
      return gemm_tf32x3(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, D, ldd, sD, batch, st);
    case GV_V4_128x128:
      return launch_gemm_f32_v4<128, 128>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, D, ldd, sD,
                                          batch, st);
    case GV_V4_128x64:
      return launch_gemm_f32_v4<128, 64>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, D, ldd, sD,
                                         batch, st);
    case GV_V4_64x64:
      return launch_gemm_f32_v4<64, 64>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, D, ldd, sD,
                                        batch, st);
    case GV_SPLIT2:
    case GV_SPLIT4:
    case GV_SPLIT8:
      return launch_gemm_f32_v4_split<64, 64>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, D, ldd, sD,
                                              batch, 2 << (v - GV_SPLIT2), st);
    default:
      return launch_gemm_cfg<float, 64, 64, 8, 4, 4>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, D,
                                                     ldd, sD, batch, st);
  }
}

template <class T>
cudaError_t gemm_batched(int M, int N, int K, T alpha, const T* A, long long lda, long long sA,
                         const T* B, long long ldb, long long sB, T beta, const T* C, long long ldc,
                         long long sC, T* D, long long ldd, long long sD, int batch, cudaStream_t st) {
  if (M <= 0 || N <= 0 || batch <= 0) return cudaSuccess;
  if constexpr (std::is_same<T, float>::value) {
    if (!(N <= 8 && K >= 32)) {
      if (g_shape_log.load(std::memory_order_relaxed))
        log_shape(M, N, K, batch, lda, sA, ldb, sB, ldc, sC, ldd, sD, C != nullptr);
      const int v = tuned_variant(M, N, K, batch);
      if (v >= 0)
        return run_variant_f32(v, M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, D, ldd, sD, batch, st);
    }
  }
  if (N <= 8 && K >= 32) {
    if (N == 1)
      return launch_skinny<T, 1>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, D, ldd, sD, batch, st);
    if (N <= 2)
      return launch_skinny<T, 2>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, D, ldd, sD, batch, st);
    if (N <= 4)
      return launch_skinny<T, 4>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, D, ldd, sD, batch, st);
    return launch_skinny<T, 8>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, D, ldd, sD, batch, st);
  }
  const int pol = gemm_policy();
  if constexpr (std::is_same<T, float>::value) {
    // products with few right-hand-side columns (the leaf solves, the
    // refinement's corrections at every level): the streaming TMA kernel, one
    // persistent CTA per SM.  Measured against the autotuner's timings of the
    // 2D workloads: it wins from M, K >= 128 and about 48 row tiles on; with
    // K <= 64 or M < 128 (half-empty 128-row tiles) the SIMT tiles are faster,
    // and with fewer row tiles K split over a cluster (below)
    if (pol == 1 && N > 8 && N <= 64 && M >= 128 && K >= 128 && (long long)((M + 127) / 128) * batch >= 48) {
      const cudaError_t e = gemm_tma_f32(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, D, ldd, sD, batch,
                                         st);
      if (e != cudaErrorNotSupported) return e;
    }
    // a wide product with fewer 64 x 64 output tiles than SMs (the top merge
    // levels and the recursive inversion's blocks, one to four matrices):
    // K split over the CTAs of a cluster fills the GPU where the tensor-core
    // kernel's 128 x 128 tiles would leave most SMs idle (measured 2-3x)
    if (pol == 1 && N > 64 && K >= 128) {
      const long long t64 = (long long)((M + 63) / 64) * ((N + 63) / 64) * batch;
      if (t64 < 152) {
        int S = 8;
        while (S > 2 && (t64 * S > 4 * 152 || K / S < 16)) S >>= 1;
        return launch_gemm_f32_v4_split<64, 64>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, D, ldd,
                                                sD, batch, S, st);
      }
    }
    // measured: the tensor-core kernel wins once tiles are wide (N >= 128)
    // and have enough K-steps to amortise its pipeline prologue and epilogue;
    // below that the 8x8-register SIMT tiles are as fast or faster
    if (pol == 2 || (pol == 1 && M >= 128 && N >= 128 && K >= 128))
      return gemm_tf32x3(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, D, ldd, sD, batch, st);
  }
  if constexpr (std::is_same<T, c64>::value) {
    // complex64 as one real product of size (M, 2N, 2K) on the tensor cores
    if (alpha.y == 0.f && beta.y == 0.f && (pol == 2 || (pol == 1 && M >= 128 && N >= 128 && K >= 128)))
      return gemm_tf32x3_c64(M, N, K, alpha.x, A, lda, sA, B, ldb, sB, beta.x, C, ldc, sC, D, ldd, sD, batch, st);
  }
  if constexpr (std::is_same<T, float>::value) {
    const bool v4 = (pol != 3);
    const long long tiles128 = (long long)((M + 127) / 128) * ((N + 127) / 128) * batch;
    if (M >= 96 && N >= 96 && tiles128 >= 120)
      return v4 ? launch_gemm_f32_v4<128, 128>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, D, ldd,
                                               sD, batch, st)
                : launch_gemm_cfg<T, 128, 128, 8, 8, 8>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, D,
                                                        ldd, sD, batch, st);
    // N <= 64 (many right-hand sides, leaf and merge blocks): 8x8 register
    // tiles (4 16-byte shared loads per 64 FMAs where 4x4 tiles need 8 4-byte
    // loads per 16)
    const long long tiles_m128 = (long long)((M + 127) / 128) * batch;
    if (N > 32 && N <= 64 && M >= 96 && tiles_m128 >= 152)
      return v4 ? launch_gemm_f32_v4<128, 64>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, D, ldd, sD,
                                              batch, st)
                : launch_gemm_cfg<T, 128, 64, 8, 8, 8>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, D,
                                                       ldd, sD, batch, st);
    const long long tiles_m64 = (long long)((M + 63) / 64) * batch;
    if (N > 32 && N <= 64 && M >= 32 && tiles_m64 >= 304)
      return v4 ? launch_gemm_f32_v4<64, 64>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, D, ldd, sD,
                                             batch, st)
                : launch_gemm_cfg<T, 64, 64, 8, 8, 8>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, D,
                                                      ldd, sD, batch, st);
    // fewer 64 x 64 output tiles than two per SM and a long K: split K over
    // the CTAs of a cluster, up to about four CTAs per SM, K-slices of at
    // least 128
    const long long tiles64 = tiles_m64 * ((N + 63) / 64);
    if (v4 && N > 8 && K >= 512 && tiles64 < 2 * 152) {
      int S = 8;
      while (S > 2 && (tiles64 * S > 4 * 152 || K / S < 128)) S >>= 1;
      return launch_gemm_f32_v4_split<64, 64>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, D, ldd, sD,
                                              batch, S, st);
    }
    return launch_gemm_cfg<T, 64, 64, 8, 4, 4>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc,
                                               sC, D, ldd, sD, batch, st);
  }
  if (sizeof(T) == 16 && M <= 32 && N <= 32)
    return launch_gemm_cfg<T, 32, 32, 8, 2, 2>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc,
                                               sC, D, ldd, sD, batch, st);
  return launch_gemm_cfg<T, 64, 64, 8, 4, 4>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc,
                                             sC, D, ldd, sD, batch, st);
}

#define HPS_INST_GEMM(T)                                                                          \
  template cudaError_t gemm_batched<T>(int, int, int, T, const T*, long long, long long, const T*, \
                                       long long, long long, T, const T*, long long, long long,    \
                                       T*, long long, long long, int, cudaStream_t);
HPS_INST_GEMM(float)
HPS_INST_GEMM(double)
HPS_INST_GEMM(c64)
HPS_INST_GEMM(c128)

}  // namespace hps
