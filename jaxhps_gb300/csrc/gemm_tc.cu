// FP32 batched GEMM on the 5th-generation tensor cores (tcgen05, TMEM).
//
// D[b] = alpha A[b] B[b] + beta C[b], row-major FP32, with FP32-level
// accuracy from TF32 products by the split-operand method of Ootomo & Yokota
// ("Recovering single precision accuracy from Tensor Cores while surpassing
// the FP32 theoretical peak performance", 2022): x = x_hi + x_lo with x_hi
// the TF32 rounding of x, and A B ~ A_hi B_hi + A_hi B_lo + A_lo B_hi, all
// three products accumulated in one FP32 TMEM accumulator.
//
// One CTA of 256 threads computes a 128 x BN tile of D.  Per K-tile of 32:
// all threads load the A (128 x 32) and B (32 x BN) tiles, split them and
// store them K-major in shared memory in the 128-byte swizzled layout the
// tensor core reads (row r of a tile occupies bytes [128 r, 128 r + 128),
// its 16-byte chunk c stored at chunk c ^ (r mod 8)); thread 0 issues
// 3 x 4 tcgen05.mma (K = 8 each) and commits them to the stage's mbarrier.
// Two stages: the loads of tile t+1 overlap the MMAs of tile t.  All waits
// are bounded (thread 0 waits, the CTA follows its verdict); a timeout sets
// a device error flag (gemm_tc_error) and the CTA winds down.  The accumulator
// is read back with tcgen05.ld (warp w owns TMEM lanes 32w..32w+31, i.e.
// tile rows 32w..32w+31).
#include <cuda.h>
#include <cudaTypedefs.h>

#include "hps_common.cuh"
#include "hps_internal.h"
#include "tc_common.cuh"

namespace hps {

constexpr int TC_BM = 128;
constexpr int TC_BK = 32;
constexpr int TC_NT = 256;
// try_wait polls before an mbarrier wait gives up (default 2^22: well under
// a second).  A device variable so that hps_set_spin_limits can change it;
// TC_SPIN_FLOOR bounds it from below, because a CTA that gives up waits a
// second time, with the same limit, for its MMAs in flight before it frees
// the tensor memory they write.
static __device__ long long g_tc_spin_limit = 1ll << 22;
constexpr long long TC_SPIN_FLOOR = 1ll << 20;

// Set by a CTA whose mbarrier wait ran out (a static device flag: the
// library allocates no device memory).
static __device__ int g_tc_err = 0;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// x = hi + lo with hi the TF32 value nearest to x (ties away from zero: add
// half a TF32 unit to the bit pattern, clear the 13 dropped bits; two integer
// operations on the full-rate pipes) and lo = x - hi, exact (at most 13
// significant bits; the tensor core reads its leading 11).
__device__ __forceinline__ void split_tf32(float x, uint32_t& h, uint32_t& l) {
  h = (__float_as_uint(x) + 0x1000u) & 0xFFFFE000u;
  l = __float_as_uint(x - __uint_as_float(h));
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (stride byte offset), leading byte offset unused (1),
// descriptor version bits 46-48 = 0b001.
__device__ __forceinline__ uint64_t make_desc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);          // start address
  d |= (uint64_t)1 << 16;                            // leading byte offset (unused for this layout)
  d |= (uint64_t)(1024 >> 4) << 32;                  // stride byte offset
  d |= (uint64_t)1 << 46;                            // fixed 0b001
  d |= (uint64_t)2 << 61;                            // 128-byte swizzle
  return d;
}

// Instruction descriptor: D F32 (bits 4-5 = 1), A and B TF32 (bits 7-9, 10-12
// = 2), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t make_idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Bounded wait for the completion of the phase with the given parity.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  const long long limit = *(volatile long long*)&g_tc_spin_limit;
  for (long long it = 0; it < limit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// Byte offset of element (row r, k) in a K-major 128-byte-swizzled tile.
__device__ __forceinline__ uint32_t sw128_off(int r, int k) {
  const int byte = k * 4;
  return (uint32_t)(r * 128 + ((((byte >> 4) ^ (r & 7)) & 7) << 4) + (byte & 15));
}

// Splits 4 consecutive K values of one row into TF32 hi / lo and stores them
// as one 16-byte chunk each (4 consecutive k never straddle a swizzle chunk).
__device__ __forceinline__ void store_split4(unsigned char* hi_base, unsigned char* lo_base, int r, int k,
                                             float4 x) {
  uint4 h, l;
  split_tf32(x.x, h.x, l.x);
  split_tf32(x.y, h.y, l.y);
  split_tf32(x.z, h.z, l.z);
  split_tf32(x.w, h.w, l.w);
  const uint32_t o = sw128_off(r, k);
  *reinterpret_cast<uint4*>(hi_base + o) = h;
  *reinterpret_cast<uint4*>(lo_base + o) = l;
}

// Asynchronous global -> shared copies of `bytes` (zero-filled up to `size`).
__device__ __forceinline__ void cp_async16(void* dst, const void* src, int src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(src_bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src, int src_bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(src_bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

template <int BN>
struct TcCfg {
  static constexpr int NS = (BN >= 128) ? 2 : 4;                // K-tiles in flight (stage ring)
  static constexpr int A_BYTES = TC_BM * TC_BK * 4;             // one operand tile (16 KB)
  static constexpr int B_BYTES = BN * TC_BK * 4;
  // stage: A_hi (cp.async target, swizzled) | A_lo | B_hi | B_lo | B_raw (32 x BN row-major)
  static constexpr int OFF_ALO = A_BYTES;
  static constexpr int OFF_BHI = 2 * A_BYTES;
  static constexpr int OFF_BLO = 2 * A_BYTES + B_BYTES;
  static constexpr int OFF_BRAW = 2 * A_BYTES + 2 * B_BYTES;
  static constexpr int STAGE = 2 * A_BYTES + 3 * B_BYTES;
  static constexpr size_t SMEM = NS * (size_t)STAGE + 1024;
};

// Persistent: each CTA loops over (batch, m-tile, n-tile) work items; TMEM
// and the barriers are set up once per CTA and the barrier phases carry over.
//
// CPLX: complex64 operands as one real product.  With A (M x K complex,
// interleaved re/im) read as a real M x 2K matrix and B (K x N complex)
// expanded to the real 2K x 2N matrix with 2x2 blocks [[Br, Bi], [-Bi, Br]],
// the real product is C (M x N complex, interleaved) itself:
//   C[m][2n]   = sum_k Ar Br - Ai Bi,   C[m][2n+1] = sum_k Ar Bi + Ai Br.
// The kernel then runs on the real dimensions (M, 2N, 2K); only the B
// staging differs: a K-tile of 32 real rows is 16 complex rows, copied raw
// and expanded while it is split into TF32 hi / lo.
template <int BN, bool CPLX>
__global__ void __launch_bounds__(TC_NT)
gemm_tf32x3_kernel(int M, int N, int K, float alpha, const float* __restrict__ A, long long lda, long long sA,
                   const float* __restrict__ B, long long ldb, long long sB, float beta, const float* C,
                   long long ldc, long long sC, float* D, long long ldd, long long sD, int batch, int vecA,
                   int vecB) {
  using Cfg = TcCfg<BN>;
  constexpr int A_BYTES = Cfg::A_BYTES;
  constexpr int B_BYTES = Cfg::B_BYTES;
  constexpr int STAGE = Cfg::STAGE;
  constexpr int NS = Cfg::NS;
  constexpr int A_F4 = TC_BM * TC_BK / 4 / TC_NT;   // 16-byte chunks per thread, A tile (4)
  constexpr int B_F4 = TC_BK * BN / 4 / TC_NT;      // 16-byte chunks per thread, B tile (2 or 4)
  constexpr int B_ROWS = CPLX ? TC_BK / 2 : TC_BK;  // rows of B copied per K-tile
  constexpr int B_F4L = B_ROWS * BN / 4 / TC_NT;    // 16-byte copies per thread, B tile
  const int KB = CPLX ? K / 2 : K;                  // rows of B in global memory
  constexpr int OUT_LD = BN + 1;                     // epilogue staging stride (odd: conflict-free)
  extern __shared__ unsigned char tc_smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023) & ~uintptr_t(1023));
  __shared__ uint64_t bars[4];
  __shared__ uint32_t tmem_base_s;
  __shared__ int fail_s;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int i = 0; i < NS; ++i) mbar_init(&bars[i], 1);
    fail_s = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_s)),
                 "r"(BN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base_s;
  constexpr uint32_t idesc = make_idesc_tf32(TC_BM, BN);

  const int tiles_m = (M + TC_BM - 1) / TC_BM, tiles_n = (N + BN - 1) / BN;
  const long long n_tiles = (long long)batch * tiles_m * tiles_n;
  const int nk = (K + TC_BK - 1) / TC_BK;
  uint32_t uses[4] = {0, 0, 0, 0};   // commits issued on each stage barrier
  bool pending[4] = {false, false, false, false};
  float* out_s = reinterpret_cast<float*>(smem);

  for (long long tile = blockIdx.x; tile < n_tiles && !fail_s; tile += gridDim.x) {
    const long long b = tile / ((long long)tiles_m * tiles_n);
    const int rem = (int)(tile % ((long long)tiles_m * tiles_n));
    const int m0 = (rem / tiles_n) * TC_BM, n0 = (rem % tiles_n) * BN;
    const float* Ab = A + b * sA;
    const float* Bb = B + b * sB;
    int s_last = 0;
    // K-tiles arrive by cp.async into a ring of NS stages: A straight into the
    // swizzled K-major layout, B row-major into B_raw.  Each iteration rounds
    // A to its TF32 part in place (A_hi) with the remainder in A_lo, builds the
    // transposed B_hi / B_lo of its stage, issues the stage's MMAs, then refills
    // the stage whose MMAs finished with the tile NS-1 ahead.
    auto issue_tile = [&](int kt) {
      unsigned char* sb = smem + (kt % NS) * STAGE;
      const int k0 = kt * TC_BK;
#pragma unroll
      for (int i = 0; i < A_F4; ++i) {
        const int f = tid + TC_NT * i;
        const int r = f >> 3, c = f & 7;
        const int gm = m0 + r, gk = k0 + c * 4;
        unsigned char* dst = sb + sw128_off(r, c * 4);
        const float* src = Ab + (long long)(gm < M ? gm : 0) * lda + (gk < K ? gk : 0);
        const int avail = (gm < M) ? max(0, min(4, K - gk)) : 0;
        if (vecA) {
          cp_async16(dst, src, avail * 4);
        } else {
#pragma unroll
          for (int j = 0; j < 4; ++j) cp_async4(dst + 4 * j, (j < avail) ? src + j : src, (j < avail) ? 4 : 0);
        }
      }
#pragma unroll
      for (int i = 0; i < B_F4L; ++i) {
        const int f = tid + TC_NT * i;
        const int kr = f / (BN / 4), nn = (f % (BN / 4)) * 4;
        const int gk = (CPLX ? k0 / 2 : k0) + kr, gn = n0 + nn;
        unsigned char* dst = sb + Cfg::OFF_BRAW + kr * (BN * 4) + nn * 4;
        const float* src = Bb + (long long)(gk < KB ? gk : 0) * ldb + (gn < N ? gn : 0);
        const int avail = (gk < KB) ? max(0, min(4, N - gn)) : 0;
        if (vecB) {
          cp_async16(dst, src, avail * 4);
        } else {
#pragma unroll
          for (int j = 0; j < 4; ++j) cp_async4(dst + 4 * j, (j < avail) ? src + j : src, (j < avail) ? 4 : 0);
        }
      }
    };
#pragma unroll
    for (int p0 = 0; p0 < NS - 1; ++p0) {
      if (p0 < nk) issue_tile(p0);
      cp_async_commit();
    }
    for (int t = 0; t < nk; ++t) {
      const int s = t % NS;
      unsigned char* st_base = smem + s * STAGE;
      cp_async_wait<NS - 2>();           // tile t has landed (this thread's copies)
      __syncthreads();                   // ... and everyone's
#pragma unroll
      for (int i = 0; i < A_F4; ++i) {
        const int f = tid + TC_NT * i;
        const uint32_t o = sw128_off(f >> 3, (f & 7) * 4);
        // round A_hi to TF32 in place, A_lo = A - A_hi
        const float4 x = *reinterpret_cast<const float4*>(st_base + o);
        store_split4(st_base, st_base + Cfg::OFF_ALO, f >> 3, (f & 7) * 4, x);
      }
      // B: item f takes column n = f % BN and k = 4 (f / BN) .. +3 (lanes on consecutive n)
      const float* rb = reinterpret_cast<const float*>(st_base + Cfg::OFF_BRAW);
#pragma unroll
      for (int i = 0; i < B_F4; ++i) {
        const int f = tid + TC_NT * i;
        const int nn = f % BN, kq = (f / BN) * 4;
        float4 x;
        if (CPLX) {
          // real rows kq..kq+3 are complex rows kq/2, kq/2+1; an odd real row
          // holds (-Bi, Br) where an even one holds (Br, Bi)
          const int r0 = (kq >> 1) * BN, r1 = r0 + BN, nx = nn ^ 1;
          const float sg = (nn & 1) ? 1.0f : -1.0f;
          x = make_float4(rb[r0 + nn], sg * rb[r0 + nx], rb[r1 + nn], sg * rb[r1 + nx]);
        } else {
          x = make_float4(rb[(kq + 0) * BN + nn], rb[(kq + 1) * BN + nn], rb[(kq + 2) * BN + nn],
                          rb[(kq + 3) * BN + nn]);
        }
        store_split4(st_base + Cfg::OFF_BHI, st_base + Cfg::OFF_BLO, nn, kq, x);
      }
      // make the generic-proxy stores visible to the tensor core (async proxy)
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncthreads();
      if (tid == 0) {
        tc_fence_after();
        const uint32_t a_hi = smem_u32(st_base), a_lo = a_hi + Cfg::OFF_ALO;
        const uint32_t b_hi = a_hi + Cfg::OFF_BHI, b_lo = a_hi + Cfg::OFF_BLO;
#pragma unroll
        for (int kk = 0; kk < TC_BK / 8; ++kk) {
          const uint32_t off = kk * 32;   // 8 TF32 = 32 bytes along K inside the swizzle row
          const uint32_t acc = (t > 0 || kk > 0) ? 1u : 0u;
          mma_tf32(tmem, make_desc_sw128(a_hi + off), make_desc_sw128(b_hi + off), idesc, acc);
          mma_tf32(tmem, make_desc_sw128(a_hi + off), make_desc_sw128(b_lo + off), idesc, 1u);
          mma_tf32(tmem, make_desc_sw128(a_lo + off), make_desc_sw128(b_hi + off), idesc, 1u);
        }
        mma_commit(&bars[s]);
      }
      uses[s] += 1;
      pending[s] = true;
      s_last = s;
      // refill the stage of tile t-1 (tile t+NS-1) once its MMAs are done
      const int tn = t + NS - 1;
      if (tn < nk) {
        const int sr = tn % NS;
        if (pending[sr]) {
          if (tid == 0 && !mbar_wait(&bars[sr], (uses[sr] - 1) & 1)) fail_s = 1;
          pending[sr] = false;
          __syncthreads();
          if (fail_s) break;
        }
        issue_tile(tn);
      }
      cp_async_commit();
    }
    cp_async_wait<0>();
    if (fail_s) break;
    // all of this tile's MMAs: the last commit covers the earlier ones; the other
    // stages' pending phases have completed too and are consumed here
    if (tid == 0 && nk > 0 && !mbar_wait(&bars[s_last], (uses[s_last] - 1) & 1)) fail_s = 1;
    for (int i = 0; i < NS; ++i) {
      if (i != s_last && pending[i] && tid == 0 && !mbar_wait(&bars[i], (uses[i] - 1) & 1)) fail_s = 1;
      pending[i] = false;
    }
    __syncthreads();
    if (fail_s) break;
    tc_fence_after();
    // accumulator -> shared memory (row = warp*32 + lane), then coalesced rows to D
    // warp w reads TMEM lanes 32 (w % 4) .. +31 (its lane group) and half w / 4 of the columns
    const int wq = warp & 3, wh = warp >> 2;
    const int rl = wq * 32 + lane;
#pragma unroll 1
    for (int c0 = wh * (BN / 2); c0 < (wh + 1) * (BN / 2); c0 += 16) {
      uint32_t v[16];
      const uint32_t taddr = tmem + ((uint32_t)(wq * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
          : "r"(taddr)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
      for (int j = 0; j < 16; ++j) out_s[rl * OUT_LD + c0 + j] = __uint_as_float(v[j]);
    }
    tc_fence_before();
    __syncthreads();
    const float* Cb = C ? C + b * sC : nullptr;
    float* Db = D + b * sD;
    for (int e = tid; e < TC_BM * BN; e += TC_NT) {
      const int r = e / BN, c = e % BN;
      const int row = m0 + r, col = n0 + c;
      if (row < M && col < N) {
        float x = alpha * out_s[r * OUT_LD + c];
        if (Cb) x = fmaf(beta, Cb[(long long)row * ldc + col], x);
        Db[(long long)row * ldd + col] = x;
      }
    }
    __syncthreads();   // the staging area is the next tile's stage 0
  }
  if (fail_s && tid == 0) {
    atomicExch(&g_tc_err, 1);
    // give in-flight MMAs a second bounded chance to drain before TMEM is freed
    for (int s = 0; s < NS; ++s)
      if (uses[s]) mbar_wait(&bars[s], (uses[s] - 1) & 1);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN) : "memory");
  }
}

template <int BN>
static size_t tc_smem_bytes() {
  return TcCfg<BN>::SMEM;
}

int gemm_tc_error() {
  int h = 0;
  cudaMemcpyFromSymbol(&h, g_tc_err, sizeof(int));
  return h;
}

int gemm_tc_error_reset() {
  int h = 0;
  cudaMemcpyFromSymbol(&h, g_tc_err, sizeof(int));
  const int zero_flag = 0;
  cudaMemcpyToSymbol(g_tc_err, &zero_flag, sizeof(int));
  return h;
}

cudaError_t set_tc_spin_limit(long long polls, long long* previous) {
  long long old = 0;
  cudaError_t e = cudaMemcpyFromSymbol(&old, g_tc_spin_limit, sizeof(old));
  if (e != cudaSuccess) return e;
  if (previous) *previous = old;
  if (polls >= 0) {
    if (polls < TC_SPIN_FLOOR) polls = TC_SPIN_FLOOR;
    e = cudaMemcpyToSymbol(g_tc_spin_limit, &polls, sizeof(polls));
  }
  return e;
}

template <int BN, bool CPLX>
static cudaError_t launch_tc(int M, int N, int K, float alpha, const float* A, long long lda, long long sA,
                             const float* B, long long ldb, long long sB, float beta, const float* C, long long ldc,
                             long long sC, float* D, long long ldd, long long sD, int batch, cudaStream_t st) {
  const size_t smem = tc_smem_bytes<BN>();
  cudaFuncSetAttribute(gemm_tf32x3_kernel<BN, CPLX>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 148;
  }
  int per_sm = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gemm_tf32x3_kernel<BN, CPLX>, TC_NT, smem);
  if (per_sm < 1) per_sm = 1;
  const long long n_tiles = (long long)batch * ((M + TC_BM - 1) / TC_BM) * ((N + BN - 1) / BN);
  const long long grid = n_tiles < (long long)sms * per_sm ? n_tiles : (long long)sms * per_sm;
  // float4 loads need 16-byte aligned rows and batch offsets
  const int vecA = (lda % 4 == 0) && (sA % 4 == 0) && ((reinterpret_cast<uintptr_t>(A) & 15) == 0);
  const int vecB = (ldb % 4 == 0) && (sB % 4 == 0) && ((reinterpret_cast<uintptr_t>(B) & 15) == 0);
  ProfScope ps(KC_GEMM, st, 2.0 * (double)M * N * K * batch);
  note_launch();
  gemm_tf32x3_kernel<BN, CPLX><<<(unsigned)grid, TC_NT, smem, st>>>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C,
                                                                    ldc, sC, D, ldd, sD, batch, vecA, vecB);
  return cudaGetLastError();
}

cudaError_t gemm_tf32x3(int M, int N, int K, float alpha, const float* A, long long lda, long long sA,
                        const float* B, long long ldb, long long sB, float beta, const float* C, long long ldc,
                        long long sC, float* D, long long ldd, long long sD, int batch, cudaStream_t st) {
  if (M <= 0 || N <= 0 || batch <= 0) return cudaSuccess;
  if (K <= 0) return cudaErrorInvalidValue;   // callers keep K = 0 on the SIMT path
  if (N >= 128)
    return launch_tc<128, false>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, D, ldd, sD, batch, st);
  return launch_tc<64, false>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, D, ldd, sD, batch, st);
}

// complex64 with real alpha, beta: the real product of the interleaved views
// on dimensions (M, 2N, 2K), strides in floats.
cudaError_t gemm_tf32x3_c64(int M, int N, int K, float alpha, const c64* A, long long lda, long long sA,
                            const c64* B, long long ldb, long long sB, float beta, const c64* C, long long ldc,
                            long long sC, c64* D, long long ldd, long long sD, int batch, cudaStream_t st) {
  if (M <= 0 || N <= 0 || batch <= 0) return cudaSuccess;
  if (K <= 0) return cudaErrorInvalidValue;
  const float* Af = reinterpret_cast<const float*>(A);
  const float* Bf = reinterpret_cast<const float*>(B);
  const float* Cf = reinterpret_cast<const float*>(C);
  float* Df = reinterpret_cast<float*>(D);
  if (2 * N >= 128)
    return launch_tc<128, true>(M, 2 * N, 2 * K, alpha, Af, 2 * lda, 2 * sA, Bf, 2 * ldb, 2 * sB, beta, Cf, 2 * ldc,
                                2 * sC, Df, 2 * ldd, 2 * sD, batch, st);
  return launch_tc<64, true>(M, 2 * N, 2 * K, alpha, Af, 2 * lda, 2 * sA, Bf, 2 * ldb, 2 * sB, beta, Cf, 2 * ldc,
                             2 * sC, Df, 2 * ldd, 2 * sD, batch, st);
}

// ---------------------------------------------------------------------------
// Warp-specialised TMA + tcgen05 kernel for the batched products with few
// right-hand-side columns (N <= 64): the leaf solves v = inv(A_ii) r, the
// leaf operators Y = inv(A_ii) W, du = Y g + v, h = Q v.  These are
// HBM-bound (each leaf's A is read once, ~20 flops per byte), so the kernel is
// built to stream: a persistent CTA per SM, a ring of LT_NS stages filled by
// the tensor memory accelerator (cp.async.bulk.tensor; A tiles land directly
// in the 128-byte-swizzled K-major layout, B tiles row-major), and five
// roles that never meet at a CTA barrier:
//   warp 0     producer: one lane issues the TMA loads of each K-tile (A box
//              32 x 128, B box 64 x 32) against the stage's `full` barrier;
//   warp 1     MMA: one lane issues, per K-tile, the three TF32 products
//              A_hi B_hi + A_hi B_lo + A_lo B_hi (the split-operand method of
//              Ootomo & Yokota, as gemm_tf32x3_kernel) as 4 x (one
//              tcgen05.mma 128 x 128 x 8 of A_hi against [B_hi | B_lo] and one
//              128 x 64 x 8 of A_lo against B_hi) into a TMEM accumulator of
//              128 columns, commits the stage back to the producer (`empty`)
//              and, after the last K-tile, the accumulator to the epilogue
//              (`accf`);
//   warps 2-9  converters: split the landed A tile into TF32 hi (in place)
//              and lo, transpose B into K-major hi / lo, then release the
//              stage to the MMA warp (`conv`);
//   warps 10-13 epilogue: read the accumulator with tcgen05.ld (warp w owns
//              TMEM lanes 32 (w % 4) ..), add its two halves, hand it back
//              (`acce`), and write alpha acc + beta C row by row.
// Two accumulators (256 TMEM columns) let the MMAs of the next 128-row tile
// start while the epilogue drains the previous one.  M and K tails come from
// the TMA's zero fill; N < 64 from the zero-filled B columns.  Every wait is
// bounded (g_tc_spin_limit polls); a wait that runs out sets g_tc_err, every
// role winds down, the CTA waits (bounded) for its loads and MMAs in flight
// and frees its tensor memory.
// ---------------------------------------------------------------------------
constexpr int LT_BM = 128, LT_BN = 64, LT_BK = 32, LT_NS = 4;
constexpr int LT_CW = 8;                           // converter warps
constexpr int LT_CT = LT_CW * 32;
constexpr int LT_NT = (2 + LT_CW + 4) * 32;           // 448
constexpr int LT_A_BYTES = LT_BM * LT_BK * 4;         // 16 KB
constexpr int LT_B_BYTES = LT_BN * LT_BK * 4;         // 8 KB
constexpr int LT_OFF_ALO = LT_A_BYTES;
constexpr int LT_OFF_BHI = 2 * LT_A_BYTES;
constexpr int LT_OFF_BLO = LT_OFF_BHI + LT_B_BYTES;
constexpr int LT_OFF_BRAW = LT_OFF_BLO + LT_B_BYTES;  // B as loaded: 32 rows (k) of 64 floats (n)
constexpr int LT_STAGE = LT_OFF_BRAW + LT_B_BYTES;    // 56 KB, a multiple of 1024 (four stages: 224 KB)
constexpr size_t LT_SMEM = LT_NS * (size_t)LT_STAGE + 1024;

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// 3D tiled TMA load of one box into shared memory, completing on `bar`
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// The CTA's failure flag read once per lane and agreed across the warp, so
// that a warp leaves its loop as a whole.
__device__ __forceinline__ bool warp_flag(volatile int* f) { return __any_sync(0xffffffffu, *f != 0); }

// Bounded wait by a whole warp: every lane polls (its own acquire), then the
// warp agrees (a lane that gave up makes the wait fail for all).
__device__ __forceinline__ bool warp_wait(uint64_t* bar, uint32_t parity) {
  const bool ok = mbar_wait(bar, parity);
  return __all_sync(0xffffffffu, ok);
}

__global__ void __launch_bounds__(LT_NT, 1)
gemm_tma_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int M, int N, int K,
                float alpha, float beta, const float* C, long long ldc, long long sC, float* D, long long ldd,
                long long sD, int batch, int a_batched, int b_batched, int vec_out) {
  extern __shared__ unsigned char lt_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(lt_raw) + 1023) & ~uintptr_t(1023));
  __shared__ uint64_t full[LT_NS], conv[LT_NS], empty[LT_NS], accf[2], acce[2];
  __shared__ uint32_t armed[LT_NS], committed[LT_NS], acc_committed[2];
  __shared__ uint32_t tmem_s;
  __shared__ int fail_s;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int i = 0; i < LT_NS; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&conv[i], LT_CW);
      mbar_init(&empty[i], 1);
      armed[i] = committed[i] = 0;
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&accf[i], 1);
      mbar_init(&acce[i], 4);
      acc_committed[i] = 0;
    }
    fail_s = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_s)),
                 "r"(4 * LT_BN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_s;
  const int tiles_m = (M + LT_BM - 1) / LT_BM;
  const long long n_units = (long long)batch * tiles_m;
  const int nk = (K + LT_BK - 1) / LT_BK;
  volatile int* fail = &fail_s;

  // Each role runs its loop with the whole warp converged: every lane polls
  // the barrier (each its own acquire), the warp agrees on the outcome, and
  // one lane issues the TMA loads, MMAs and commits.
  if (warp == 0) {
    // ---------------- producer ----------------
    if (lane == 0) {
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmA)) : "memory");
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmB)) : "memory");
    }
    uint32_t it = 0;
    for (long long u = blockIdx.x; u < n_units && !warp_flag(fail); u += gridDim.x) {
      const int b = (int)(u / tiles_m), m0 = (int)(u % tiles_m) * LT_BM;
      for (int kt = 0; kt < nk; ++kt, ++it) {
        const int s = it % LT_NS;
        const uint32_t use = it / LT_NS;
        if (use > 0 && !warp_wait(&empty[s], (use - 1) & 1)) {
          *fail = 1;
          break;
        }
        if (lane == 0) {
          unsigned char* sb = smem + s * LT_STAGE;
          mbar_expect_tx(&full[s], LT_A_BYTES + LT_B_BYTES);
          armed[s] += 1;
          tma_load_3d(sb, &tmA, kt * LT_BK, m0, a_batched ? b : 0, &full[s]);
          tma_load_3d(sb + LT_OFF_BRAW, &tmB, 0, kt * LT_BK, b_batched ? b : 0, &full[s]);
        }
        __syncwarp();
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    // per 8-deep K step: A_hi [B_hi | B_lo] as one N = 128 product (B_lo is
    // stored right after B_hi: 64 more K-major rows) into columns 0..127 of the
    // accumulator, then A_lo B_hi into columns 0..63; the epilogue adds the halves
    constexpr uint32_t idesc_hb = make_idesc_tf32(LT_BM, 2 * LT_BN);
    constexpr uint32_t idesc_lb = make_idesc_tf32(LT_BM, LT_BN);
    uint32_t it = 0, acc_it = 0;
    for (long long u = blockIdx.x; u < n_units && !warp_flag(fail); u += gridDim.x, ++acc_it) {
      const int a = acc_it & 1;
      const uint32_t ause = acc_it >> 1;
      if (ause > 0 && !warp_wait(&acce[a], (ause - 1) & 1)) {
        *fail = 1;
        break;
      }
      tc_fence_after();
      const uint32_t dt = tmem + (uint32_t)(a * 2 * LT_BN);
      bool ok = true;
      for (int kt = 0; kt < nk; ++kt, ++it) {
        const int s = it % LT_NS;
        if (!warp_wait(&conv[s], (it / LT_NS) & 1)) {
          ok = false;
          break;
        }
        tc_fence_after();
        if (lane == 0) {
          const uint32_t a_hi = smem_u32(smem + s * LT_STAGE), a_lo = a_hi + LT_OFF_ALO;
          const uint32_t b_hi = a_hi + LT_OFF_BHI, b_lo = a_hi + LT_OFF_BLO;
#pragma unroll
          for (int kk = 0; kk < LT_BK / 8; ++kk) {
            const uint32_t off = kk * 32;   // 8 TF32 = 32 bytes along K inside the swizzle row
            mma_tf32(dt, make_desc_sw128(a_hi + off), make_desc_sw128(b_hi + off), idesc_hb,
                     (kt > 0 || kk > 0) ? 1u : 0u);
            mma_tf32(dt, make_desc_sw128(a_lo + off), make_desc_sw128(b_hi + off), idesc_lb, 1u);
          }
          mma_commit(&empty[s]);
          committed[s] += 1;
        }
        __syncwarp();
      }
      if (!ok) {
        *fail = 1;
        break;
      }
      if (lane == 0) {
        mma_commit(&accf[a]);
        acc_committed[a] += 1;
      }
      __syncwarp();
    }
  } else if (warp < 2 + LT_CW) {
    // ---------------- converters (LT_CT threads) ----------------
    const int ct = tid - 64;
    uint32_t it = 0;
    for (long long u = blockIdx.x; u < n_units && !warp_flag(fail); u += gridDim.x) {
      bool ok = true;
      for (int kt = 0; kt < nk; ++kt, ++it) {
        const int s = it % LT_NS;
        if (!warp_wait(&full[s], (it / LT_NS) & 1)) {
          ok = false;
          break;
        }
        unsigned char* sb = smem + s * LT_STAGE;
        // A: TF32 hi in place (the swizzle is a permutation of 16-byte chunks,
        // so the split is layout-free), lo into A_lo at the same offsets
#pragma unroll
        for (int i = 0; i < LT_A_BYTES / 16 / LT_CT; ++i) {
          const int off = (ct + LT_CT * i) * 16;
          const float4 x = *reinterpret_cast<const float4*>(sb + off);
          uint4 h, l;
          split_tf32(x.x, h.x, l.x);
          split_tf32(x.y, h.y, l.y);
          split_tf32(x.z, h.z, l.z);
          split_tf32(x.w, h.w, l.w);
          *reinterpret_cast<uint4*>(sb + off) = h;
          *reinterpret_cast<uint4*>(sb + LT_OFF_ALO + off) = l;
        }
        // B: row-major 32 x 64 -> K-major (row n, 32 k) swizzled hi / lo;
        // item f takes column n = f % 64 and k = 4 (f / 64) .. +3
        const float* rb = reinterpret_cast<const float*>(sb + LT_OFF_BRAW);
#pragma unroll
        for (int i = 0; i < LT_BN * LT_BK / 4 / LT_CT; ++i) {
          const int f = ct + LT_CT * i;
          const int nn = f % LT_BN, kq = (f / LT_BN) * 4;
          const float4 x = make_float4(rb[(kq + 0) * LT_BN + nn], rb[(kq + 1) * LT_BN + nn], rb[(kq + 2) * LT_BN + nn],
                                       rb[(kq + 3) * LT_BN + nn]);
          store_split4(sb + LT_OFF_BHI, sb + LT_OFF_BLO, nn, kq, x);
        }
        // generic-proxy stores -> visible to the tensor core (async proxy)
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive(&conv[s]);
        __syncwarp();
      }
      if (!ok) {
        *fail = 1;
        break;
      }
    }
  } else {
    // ---------------- epilogue (128 threads) ----------------
    const int q = warp & 3;
    uint32_t acc_it = 0;
    for (long long u = blockIdx.x; u < n_units && !warp_flag(fail); u += gridDim.x, ++acc_it) {
      const int a = acc_it & 1;
      if (!warp_wait(&accf[a], (acc_it >> 1) & 1)) {
        *fail = 1;
        break;
      }
      tc_fence_after();
      const long long b = u / tiles_m;
      const int row = (int)(u % tiles_m) * LT_BM + q * 32 + lane;
      float v0[32], v1[32], w[32];
      const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(a * 2 * LT_BN);
      tc::tmem_ld32(taddr, v0);
      tc::tmem_ld32(taddr + 2 * 32, w);
#pragma unroll
      for (int j = 0; j < 32; ++j) v0[j] += w[j];
      tc::tmem_ld32(taddr + 32, v1);
      tc::tmem_ld32(taddr + 3 * 32, w);
#pragma unroll
      for (int j = 0; j < 32; ++j) v1[j] += w[j];
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&acce[a]);
      __syncwarp();
      if (row < M) {
        const float* Cr = C ? C + b * sC + (long long)row * ldc : nullptr;
        float* Dr = D + b * sD + (long long)row * ldd;
        if (vec_out) {
#pragma unroll
          for (int c = 0; c < LT_BN; c += 4) {
            if (c < N) {
              float4 x = make_float4(c < 32 ? v0[c] : v1[c - 32], c < 32 ? v0[c + 1] : v1[c - 31],
                                     c < 32 ? v0[c + 2] : v1[c - 30], c < 32 ? v0[c + 3] : v1[c - 29]);
              x.x *= alpha;
              x.y *= alpha;
              x.z *= alpha;
              x.w *= alpha;
              if (Cr) {
                const float4 y = *reinterpret_cast<const float4*>(Cr + c);
                x.x = fmaf(beta, y.x, x.x);
                x.y = fmaf(beta, y.y, x.y);
                x.z = fmaf(beta, y.z, x.z);
                x.w = fmaf(beta, y.w, x.w);
              }
              *reinterpret_cast<float4*>(Dr + c) = x;
            }
          }
        } else {
#pragma unroll
          for (int c = 0; c < LT_BN; ++c) {
            if (c < N) {
              float x = alpha * (c < 32 ? v0[c] : v1[c - 32]);
              if (Cr) x = fmaf(beta, Cr[c], x);
              Dr[c] = x;
            }
          }
        }
      }
    }
  }
  __syncthreads();
  if (fail_s && tid == 0) {
    atomicExch(&g_tc_err, 1);
    // give the loads and MMAs in flight a second bounded chance to finish
    // before the CTA leaves and frees the tensor memory they write
    for (int s = 0; s < LT_NS; ++s) {
      if (armed[s]) mbar_wait(&full[s], (armed[s] - 1) & 1);
      if (committed[s]) mbar_wait(&empty[s], (committed[s] - 1) & 1);
    }
    for (int a = 0; a < 2; ++a)
      if (acc_committed[a]) mbar_wait(&accf[a], (acc_committed[a] - 1) & 1);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(4 * LT_BN) : "memory");
  }
}

// The layouts the TMA kernel takes: 16-byte aligned bases, row strides and
// batch strides (or a broadcast operand), N <= 64.
bool gemm_tma_supported(int M, int N, int K, const float* A, long long lda, long long sA, const float* B,
                        long long ldb, long long sB, int batch) {
  auto al16 = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; };
  if (M <= 0 || N <= 0 || N > LT_BN || K <= 0 || batch <= 0) return false;
  if (!al16(A) || !al16(B) || lda % 4 || ldb % 4 || lda < K || ldb < N) return false;
  if (batch > 1 && ((sA != 0 && sA % 4) || (sB != 0 && sB % 4))) return false;
  return true;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point: the
// library does not link the driver library, so it still loads (to report its
// symbols and errors) on a machine without a GPU driver.
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    cudaGetLastError();
  }
  return fn;
}

static bool encode_map(CUtensorMap* map, const float* base, long long d0, long long d1, long long d2, long long ld,
                       long long sb, int box0, int box1, bool swizzle) {
  const PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
  if (!encode) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)d0, (cuuint64_t)d1, (cuuint64_t)d2};
  // the batch stride of a single-entry (or broadcast) third dimension is never
  // used; any valid multiple of 16 bytes will do
  const long long sbb = (d2 > 1) ? sb * 4 : ((ld * 4 * d1 + 15) / 16) * 16;
  const cuuint64_t strides[2] = {(cuuint64_t)(ld * 4), (cuuint64_t)sbb};
  const cuuint32_t box[3] = {(cuuint32_t)box0, (cuuint32_t)box1, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims,
                                            strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                            swizzle ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                                            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

cudaError_t gemm_tma_f32(int M, int N, int K, float alpha, const float* A, long long lda, long long sA,
                         const float* B, long long ldb, long long sB, float beta, const float* C, long long ldc,
                         long long sC, float* D, long long ldd, long long sD, int batch, cudaStream_t st) {
  if (M <= 0 || N <= 0 || batch <= 0) return cudaSuccess;
  if (!gemm_tma_supported(M, N, K, A, lda, sA, B, ldb, sB, batch)) return cudaErrorNotSupported;
  const int a_batched = (batch > 1 && sA != 0) ? 1 : 0, b_batched = (batch > 1 && sB != 0) ? 1 : 0;
  CUtensorMap tmA, tmB;
  if (!encode_map(&tmA, A, K, M, a_batched ? batch : 1, lda, sA, LT_BK, LT_BM, true) ||
      !encode_map(&tmB, B, N, K, b_batched ? batch : 1, ldb, sB, LT_BN, LT_BK, false))
    return cudaErrorNotSupported;
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 148;
  }
  cudaError_t e = cudaFuncSetAttribute(gemm_tma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)LT_SMEM);
  if (e != cudaSuccess) return e;
  const long long units = (long long)batch * ((M + LT_BM - 1) / LT_BM);
  const unsigned grid = (unsigned)(units < sms ? units : sms);
  auto al16 = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; };
  const int vec_out = al16(D) && ldd % 4 == 0 && (batch == 1 || sD % 4 == 0) && N % 4 == 0 &&
                      (!C || (al16(C) && ldc % 4 == 0 && (batch == 1 || sC % 4 == 0)));
  // algorithmic bytes: A and B once (a broadcast operand once in all), C, D
  const double bytes = 4.0 * ((double)M * K * (a_batched ? batch : 1) + (double)K * N * (b_batched ? batch : 1) +
                              (double)M * N * batch * (C ? 2.0 : 1.0));
  ProfScope ps(KC_GEMM_TMA, st, bytes);
  note_launch();
  gemm_tma_kernel<<<grid, LT_NT, LT_SMEM, st>>>(tmA, tmB, M, N, K, alpha, beta, C, ldc, sC, D, ldd, sD, batch,
                                               a_batched, b_batched, vec_out);
  return cudaGetLastError();
}

}  // namespace hps
