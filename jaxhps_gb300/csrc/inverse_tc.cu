// Batched FP32 inverse with the Gauss-Jordan tableau resident in tensor
// memory and its trailing updates on the tcgen05 tensor cores.
//
// Replaces the explicit inverses jnp.linalg.inv of the reference's leaf
// stage (local_solve/_uniform_2D_DtN.py:257) for the FP32 builds: FP32,
// 64 < n <= 256 (the 2D leaves' n = (p-2)^2, 196 at p = 16).
//
// One persistent CTA of 256 threads per SM works through the matrices.  The
// n x n tableau M lives in TMEM as FP32: rows 0..127 in columns [0, 256),
// rows 128..255 in columns [256, 512) (one 128-lane half each); thread t owns
// row t (warp w reads and writes TMEM lanes 32 (w mod 4) .. +31 of half w/4).
//
// In-place Gauss-Jordan with partial pivoting, without row exchanges, in
// panels of 32 columns k0 .. k0+31:
//  * panel: every thread loads its row's 32 panel values from TMEM into
//    registers; per column one block barrier: each warp proposes its largest
//    unused |value| (smallest row on ties) together with that row's panel
//    values, every thread picks the same pivot row r from the 8 proposals and
//    applies the Gauss-Jordan step to its 32 values (pivot row scaled, the
//    others reduced, the column replaced by the transformed unit vector).
//  * the same row operations on the other columns are one rank-32 product:
//    M <- M + U' G', with U' (n x 32) the final panel values minus 1 at
//    (r_k, k) and G' (32 x n) the pivot rows r_k of M before the panel, zero
//    in the panel columns.  U' and G' are split into TF32 hi + lo (Ootomo &
//    Yokota 2022: U'G' ~ hi hi + hi lo + lo hi) and staged K-major in the
//    128-byte-swizzled layout; one thread issues 3 x 4 tcgen05.mma.kind::tf32
//    (K = 8 each) per 128-row half with the tableau itself as the FP32
//    accumulator.  The panel columns (zero in G') are written back with
//    tcgen05.st before the MMAs.
//  * at the end inv(A)[k][j] = M[piv[k]][col(j)], piv[k] the pivot row of
//    column k and col(j) the column where row j was the pivot, staged through
//    shared memory for coalesced stores.
// An exactly zero pivot sets info[b] = column + 1 (the matrix is singular);
// an MMA completion wait that runs out of polls sets info[b] = -1 for that
// matrix and the CTA, after a second bounded wait for its MMAs in flight,
// frees its tensor memory and returns.
#include <cuda_runtime.h>

#include "hps_common.cuh"
#include "hps_internal.h"
#include "tc_common.cuh"

namespace hps {

constexpr int ITC_NT = 256;
constexpr int ITC_BW = 32;
constexpr int ITC_NMAX = 256;

// Polls of the MMA completion wait (see hps_set_spin_limits); never below
// ITC_SPIN_FLOOR, because a CTA that gives up waits once more, with the same
// limit, before it frees the tensor memory its MMAs write.
static __device__ long long g_itc_spin_limit = 1ll << 22;
constexpr long long ITC_SPIN_FLOOR = 1ll << 20;

// Shared-memory layout (bytes from the 1024-aligned base).  The input and
// output staging (128 rows x XS floats) reuses the operand tiles.
struct ItcLayout {
  int NH, NP, NC, GS, XS;
  size_t a_off, b_off, g_off, end;
};

__host__ __device__ inline ItcLayout itc_layout(int n) {
  ItcLayout L;
  L.NH = n > 128 ? 2 : 1;
  L.NP = (n + 15) & ~15;           // MMA N: columns updated per half
  L.NC = (n + 31) / 32;            // 32-column chunks of a row
  L.GS = L.NC * 32;                // pivot-row staging stride (floats)
  L.XS = L.NC * 32 + 1;            // odd: conflict-free per-row access
  L.a_off = 0;                                             // NH x (hi 16 KB | lo 16 KB)
  L.b_off = L.a_off + (size_t)L.NH * 2 * 128 * 128;        // hi NP x 128 B | lo NP x 128 B
  L.g_off = L.b_off + (size_t)2 * L.NP * 128;              // 32 x GS floats
  size_t e = L.g_off + (size_t)32 * L.GS * 4;
  const size_t x = (size_t)128 * L.XS * 4;
  L.end = e > x ? e : x;
  return L;
}

__global__ void __launch_bounds__(ITC_NT, 1)
inv_tc_kernel(int n, const float* __restrict__ A, long long lda, long long sA, float* __restrict__ X, long long ldx,
              long long sX, int batch, int* info) {
  const ItcLayout L = itc_layout(n);
  extern __shared__ unsigned char itc_smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(itc_smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* a_tiles = smem + L.a_off;
  unsigned char* b_hi = smem + L.b_off;
  unsigned char* b_lo = b_hi + (size_t)L.NP * 128;
  float* gst = reinterpret_cast<float*>(smem + L.g_off);
  float* xs = reinterpret_cast<float*>(smem);

  __shared__ __align__(16) float slot_v[2][8][ITC_BW];
  __shared__ float slot_m[2][8];
  __shared__ int slot_i[2][8];
  __shared__ int colpiv[ITC_NMAX];
  __shared__ int cof[ITC_NMAX];
  __shared__ uint64_t bar;
  __shared__ uint32_t tmem_s;
  __shared__ int fail_s;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int half = warp >> 2, rl = tid & 127;
  const uint32_t ncols = L.NH == 2 ? 512u : 256u;
  if (tid == 0) {
    tc::mbar_init(&bar, 1);
    fail_s = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc::smem_u32(&tmem_s)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = tmem_s;
  // this thread's TMEM row: lane quadrant of the warp, column base of its half
  const uint32_t trow = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(half * 256);
  // warps whose 32 rows are all padding (or beyond the allocated halves)
  // never touch TMEM; their rows read as zero
  const bool tm_rows = half < L.NH && 32 * warp < n;
  const uint32_t idesc = tc::idesc_tf32(128, L.NP);
  long long limit = *(volatile long long*)&g_itc_spin_limit;
  if (limit < ITC_SPIN_FLOOR) limit = ITC_SPIN_FLOOR;
  uint32_t phase = 0;
  bool in_flight = false;

  for (int b = blockIdx.x; b < batch; b += gridDim.x) {
    const float* Ab = A + (long long)b * sA;
    // ---- A -> TMEM, one half at a time through shared memory ----
    for (int h = 0; h < L.NH; ++h) {
      __syncthreads();
      const int w = L.NC * 32;
      for (int e = tid; e < 128 * w; e += ITC_NT) {
        const int r = e / w, c = e - r * w, row = 128 * h + r;
        xs[r * L.XS + c] = (row < n && c < n) ? __ldg(Ab + (long long)row * lda + c) : 0.0f;
      }
      __syncthreads();
      if (half == h && tm_rows) {
        for (int ch = 0; ch < L.NC; ++ch) {
          float v[32];
#pragma unroll
          for (int j = 0; j < 32; ++j) v[j] = xs[rl * L.XS + ch * 32 + j];
          tc::tmem_st32(trow + ch * 32, v);
        }
        tc::tmem_wait_st();
      }
    }
    int used = tid >= n;   // padding rows never pivot
    int myk = -1;          // the column where this row was the pivot

    for (int k0 = 0; k0 < n; k0 += ITC_BW) {
      const int bw = min(ITC_BW, n - k0);
      tc::fence_before();
      __syncthreads();
      tc::fence_after();
      float p[32];
      if (tm_rows) tc::tmem_ld32(trow + k0, p);
      if (tid >= n) {
#pragma unroll
        for (int j = 0; j < 32; ++j) p[j] = 0.0f;
      }
      // ---- panel: Gauss-Jordan restricted to the 32 panel columns ----
#pragma unroll
      for (int c = 0; c < ITC_BW; ++c) {
        if (c < bw) {
          const int buf = c & 1;
          float m = used ? -1.0f : fabsf(p[c]);
          int idx = tid;
#pragma unroll
          for (int off = 16; off; off >>= 1) {
            const float om = __shfl_xor_sync(0xffffffffu, m, off);
            const int oi = __shfl_xor_sync(0xffffffffu, idx, off);
            if (om > m || (om == m && oi < idx)) {
              m = om;
              idx = oi;
            }
          }
          if (tid == idx) {
            float4* d = reinterpret_cast<float4*>(slot_v[buf][warp]);
#pragma unroll
            for (int q = 0; q < 8; ++q) d[q] = make_float4(p[4 * q], p[4 * q + 1], p[4 * q + 2], p[4 * q + 3]);
          }
          if (lane == 0) {
            slot_m[buf][warp] = m;
            slot_i[buf][warp] = idx;
          }
          __syncthreads();
          float bm = slot_m[buf][0];
          int bi = slot_i[buf][0], bwp = 0;
#pragma unroll
          for (int w = 1; w < 8; ++w) {
            const float mw = slot_m[buf][w];
            const int iw = slot_i[buf][w];
            if (mw > bm || (mw == bm && iw < bi)) {
              bm = mw;
              bi = iw;
              bwp = w;
            }
          }
          float v[32];
          const float4* s = reinterpret_cast<const float4*>(slot_v[buf][bwp]);
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const float4 x = s[q];
            v[4 * q] = x.x;
            v[4 * q + 1] = x.y;
            v[4 * q + 2] = x.z;
            v[4 * q + 3] = x.w;
          }
          const bool ok = bm > 0.0f;
          if (!ok && tid == 0 && info && info[b] == 0) info[b] = k0 + c + 1;
          const float pinv = ok ? 1.0f / v[c] : 0.0f;
          if (tid == bi) {
            used = 1;
            myk = k0 + c;
            colpiv[k0 + c] = tid;
#pragma unroll
            for (int j = 0; j < 32; ++j) p[j] = (j == c) ? pinv : v[j] * pinv;
          } else {
            const float f = p[c];
#pragma unroll
            for (int j = 0; j < 32; ++j) p[j] = (j == c) ? -f * pinv : fmaf(-f, v[j] * pinv, p[j]);
          }
        }
      }
      // ---- U' = final panel values - 1 at (pivot row, its column), into the A tile of this half ----
      if (half < L.NH) {
        unsigned char* ah = a_tiles + (size_t)half * 2 * 16384;
        unsigned char* al = ah + 16384;
        const int kme = myk - k0;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          float u[4];
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int j = 4 * q + i;
            u[i] = (j < bw) ? (p[j] - ((j == kme) ? 1.0f : 0.0f)) : 0.0f;
          }
          tc::store_split4(ah, al, rl, 4 * q, u[0], u[1], u[2], u[3]);
        }
      }
      // ---- pivot rows before the update -> staging (G' rows) ----
      const bool piv_here = myk >= k0 && myk < k0 + bw;
      for (int ch = 0; ch < L.NC && tm_rows; ++ch) {
        float w32[32];
        tc::tmem_ld32(trow + ch * 32, w32);
        if (piv_here) {
          float4* d = reinterpret_cast<float4*>(gst + (size_t)(myk - k0) * L.GS + ch * 32);
#pragma unroll
          for (int q = 0; q < 8; ++q)
            d[q] = make_float4(w32[4 * q], w32[4 * q + 1], w32[4 * q + 2], w32[4 * q + 3]);
        }
      }
      // ---- panel columns back into TMEM (the MMA adds zero to them) ----
      if (tm_rows) {
        tc::tmem_st32(trow + k0, p);
        tc::tmem_wait_st();
      }
      __syncthreads();
      // ---- G'^T into the B tile: row j (tableau column), K = pivot index ----
      for (int e = tid; e < 8 * L.NP; e += ITC_NT) {
        const int kq = (e / L.NP) * 4, j = e - (e / L.NP) * L.NP;
        const bool z = j >= n || (j >= k0 && j < k0 + ITC_BW);
        float g4[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) g4[i] = (z || kq + i >= bw) ? 0.0f : gst[(size_t)(kq + i) * L.GS + j];
        tc::store_split4(b_hi, b_lo, j, kq, g4[0], g4[1], g4[2], g4[3]);
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      tc::fence_before();
      __syncthreads();
      if (tid == 0) {
        tc::fence_after();
        const uint32_t bh = tc::smem_u32(b_hi), bl = tc::smem_u32(b_lo);
        for (int h = 0; h < L.NH; ++h) {
          const uint32_t ah = tc::smem_u32(a_tiles + (size_t)h * 2 * 16384), al = ah + 16384;
          const uint32_t d = tmem + (uint32_t)(h * 256);
#pragma unroll
          for (int kk = 0; kk < ITC_BW / 8; ++kk) {
            const uint32_t off = kk * 32;
            tc::mma_tf32(d, tc::desc_sw128(ah + off), tc::desc_sw128(bh + off), idesc, 1u);
            tc::mma_tf32(d, tc::desc_sw128(ah + off), tc::desc_sw128(bl + off), idesc, 1u);
            tc::mma_tf32(d, tc::desc_sw128(al + off), tc::desc_sw128(bh + off), idesc, 1u);
          }
        }
        tc::mma_commit(&bar);
        in_flight = true;
        if (!tc::mbar_wait(&bar, phase, limit)) fail_s = 1;
        else in_flight = false;
        phase ^= 1u;
      }
      __syncthreads();
      if (fail_s) break;
    }
    if (fail_s) {
      if (tid == 0 && info) info[b] = -1;
      break;
    }
    // ---- output: inv(A)[k][j] = M[colpiv[k]][cof[j]] ----
    if (tid < n) cof[tid] = myk;
    tc::fence_before();
    for (int h = 0; h < L.NH; ++h) {
      __syncthreads();
      tc::fence_after();
      if (half == h && tm_rows) {
        for (int ch = 0; ch < L.NC; ++ch) {
          float w32[32];
          tc::tmem_ld32(trow + ch * 32, w32);
#pragma unroll
          for (int j = 0; j < 32; ++j) xs[rl * L.XS + ch * 32 + j] = w32[j];
        }
      }
      __syncthreads();
      float* Xb = X + (long long)b * sX;
      for (int k = warp; k < n; k += ITC_NT / 32) {
        const int r = colpiv[k];
        if ((r >> 7) != h) continue;
        const float* src = xs + (size_t)(r & 127) * L.XS;
        for (int j = lane; j < n; j += 32) Xb[(long long)k * ldx + j] = src[cof[j]];
      }
    }
  }
  if (tid == 0 && in_flight) tc::mbar_wait(&bar, phase ^ 1u, limit);   // drain MMAs of a failed wait
  tc::fence_before();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
  }
}

bool inverse_tc_supported(int n) { return n > 64 && n <= ITC_NMAX; }

cudaError_t inverse_tc_f32(int n, const float* A, long long lda, long long sA, float* X, long long ldx,
                           long long sX, int batch, int* info, cudaStream_t st) {
  if (!inverse_tc_supported(n)) return cudaErrorInvalidValue;
  const ItcLayout L = itc_layout(n);
  const size_t smem = L.end + 1024;
  cudaError_t e = cudaFuncSetAttribute(inv_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  const int grid = batch < sms ? batch : sms;
  note_launch();
  inv_tc_kernel<<<grid, ITC_NT, smem, st>>>(n, A, lda, sA, X, ldx, sX, batch, info);
  return cudaGetLastError();
}

cudaError_t set_itc_spin_limit(long long polls, long long* previous) {
  long long old = 0;
  cudaError_t e = cudaMemcpyFromSymbol(&old, g_itc_spin_limit, sizeof(old));
  if (e != cudaSuccess) return e;
  if (previous) *previous = old;
  if (polls >= 0) {
    if (polls < ITC_SPIN_FLOOR) polls = ITC_SPIN_FLOOR;
    e = cudaMemcpyToSymbol(g_itc_spin_limit, &polls, sizeof(polls));
  }
  return e;
}

}  // namespace hps
