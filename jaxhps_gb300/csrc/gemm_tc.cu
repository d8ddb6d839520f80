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
#include "hps_common.cuh"
#include "hps_internal.h"

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

__device__ __forceinline__ uint32_t f32_to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
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
  h.x = f32_to_tf32(x.x); l.x = f32_to_tf32(x.x - __uint_as_float(h.x));
  h.y = f32_to_tf32(x.y); l.y = f32_to_tf32(x.y - __uint_as_float(h.y));
  h.z = f32_to_tf32(x.z); l.z = f32_to_tf32(x.z - __uint_as_float(h.z));
  h.w = f32_to_tf32(x.w); l.w = f32_to_tf32(x.w - __uint_as_float(h.w));
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

}  // namespace hps
