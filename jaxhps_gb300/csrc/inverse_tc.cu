// Batched FP32 inverse with the Gauss-Jordan tableau resident in tensor
// memory and its trailing updates on the tcgen05 tensor cores.
//
// Replaces the explicit inverses jnp.linalg.inv of the reference's leaf
// stage (local_solve/_uniform_2D_DtN.py:257) for the FP32 builds: FP32,
// 64 < n <= 224 (2D leaves: n = (p-2)^2, 196 at p = 16).  The leaf stage uses
// it by default; the merges' inverses (merge/_schur_complement.py:146) keep
// the SIMT kernels, whose FP32 rounding of the update the mixed-precision
// solve converges better with (hps_inverse_policy).
//
// One persistent CTA of 256 threads per SM works through the matrices.  The
// n x n tableau M lives in TMEM as FP32: rows 0..127 in columns [0, 256),
// rows 128..255 in columns [256, 512) (one 128-lane half each); thread t owns
// row t (warp w reads and writes TMEM lanes 32 (w mod 4) .. +31 of half w/4).
//
// In-place Gauss-Jordan with partial pivoting, without row exchanges, in
// panels of 32 columns k0 .. k0+31:
//  * panel: every thread loads its row's 32 panel values from TMEM into
//    registers.  Per column one block barrier: each warp finds its largest
//    unused |value| (smallest row on ties) with two redux.sync and posts it
//    with that row's 32 panel values; every warp reduces the 8 posts the same
//    way, so every thread picks the same pivot row r, and applies the
//    Gauss-Jordan step to its values (the pivot row scaled, the other rows
//    reduced, the column replaced by the transformed unit vector).  Columns
//    go in steps of four (registers 0..3) and the registers rotate by four
//    positions after each step, so the column loop's body is the same for
//    every step.
//  * the same row operations on the other columns are one rank-32 product.
//    With G' (32 x n) the pivot rows r_k of M before the panel (zero in the
//    panel columns) and U' (n x 32) the final panel values, the pivot rows of
//    M are zeroed and M <- M + U' G': the panel column of pivot k holds the
//    row operations applied to the unit vector e_{r_k}, so the other rows get
//    M + X G' and the pivot rows the inverted pivot block times G' (zeroing
//    them first keeps M from being cancelled against itself in the tensor
//    core).  U' and G' are split into three TF32 parts each, x = x0 + x1 + x2
//    (x0 the TF32 rounding of x, x1 of the remainder, x2 of what is left),
//    and the six products x0y0, x0y1, x1y0, x1y1, x0y2, x2y0 are accumulated
//    in FP32 in the tableau itself: the omitted terms are below 2^-32 of the
//    product (the published TF32 emulation method of Ootomo & Yokota 2022,
//    extended to three parts).  The operands are staged K-major in the
//    128-byte-swizzled layout; one thread issues 6 x 4 tcgen05.mma.kind::tf32
//    (K = 8 each) per 128-row half.  The panel columns (zero in G') are
//    written back with tcgen05.st before the MMAs.
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
constexpr int ITC_NMAX = 224;
constexpr int ITC_TILE = 128 * 128;   // one 128-row operand tile of 32 FP32 (bytes)

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
  L.GS = L.NC * 32 + 4;            // pivot-row staging stride (floats; +4: rows on different banks)
  L.XS = L.NC * 32 + 1;            // odd: conflict-free per-row access
  L.a_off = 0;                                             // NH x 3 parts x 16 KB
  L.b_off = L.a_off + (size_t)L.NH * 3 * ITC_TILE;         // 3 parts x NP x 128 B
  L.g_off = L.b_off + (size_t)3 * L.NP * 128;              // 32 x GS floats
  size_t e = L.g_off + (size_t)32 * L.GS * 4;
  const size_t x = (size_t)128 * L.XS * 4;
  L.end = e > x ? e : x;
  return L;
}

// x = x0 + x1 + x2 in TF32 parts (FP32 bit patterns) for 4 consecutive K
// values of one row, stored as one 16-byte chunk per part.
__device__ __forceinline__ void store_split4x3(unsigned char* p0, unsigned char* p1, unsigned char* p2, int r,
                                               int k, const float (&x)[4]) {
  uint32_t a[4], b[4], c[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    a[i] = tc::f32_to_tf32(x[i]);
    const float r1 = x[i] - __uint_as_float(a[i]);
    b[i] = tc::f32_to_tf32(r1);
    c[i] = tc::f32_to_tf32(r1 - __uint_as_float(b[i]));
  }
  const uint32_t o = tc::sw128_off(r, k);
  *reinterpret_cast<uint4*>(p0 + o) = make_uint4(a[0], a[1], a[2], a[3]);
  *reinterpret_cast<uint4*>(p1 + o) = make_uint4(b[0], b[1], b[2], b[3]);
  *reinterpret_cast<uint4*>(p2 + o) = make_uint4(c[0], c[1], c[2], c[3]);
}

// Rotates the 32 registers left by R (v[32 - R + i] <- v[i]).
template <int R>
__device__ __forceinline__ void rotate32(float (&v)[32]) {
  float t[R];
#pragma unroll
  for (int i = 0; i < R; ++i) t[i] = v[i];
#pragma unroll
  for (int j = 0; j < 32 - R; ++j) v[j] = v[j + R];
#pragma unroll
  for (int i = 0; i < R; ++i) v[32 - R + i] = t[i];
}

// Posts of the 8 warps for one panel column (double-buffered by column parity).
struct ItcSlots {
  float v[2][8][ITC_BW];
  unsigned m[2][8];
  unsigned i[2][8];
};

// One Gauss-Jordan step on panel register CC (column k of the matrix):
// pivot choice over the unused rows of the whole CTA (largest |value|,
// smallest row on ties), then the row update of this thread's 32 values.
template <int CC>
__device__ __forceinline__ void gj_step(float (&p)[32], int k, int buf, int tid, int warp, int lane, int& used,
                                        int& myk, ItcSlots& S, int* colpiv, int* info_b) {
  const unsigned full = 0xffffffffu;
  // warp choice: key 0 for used rows, |value| bits + 1 for the others (an
  // unused zero still outranks a used row)
  const unsigned mb = used ? 0u : __float_as_uint(fabsf(p[CC])) + 1u;
  const unsigned wmax = __reduce_max_sync(full, mb);
  const unsigned widx = __reduce_min_sync(full, mb == wmax ? (unsigned)tid : 0xffffffffu);
  if ((unsigned)tid == widx) {
    float4* d = reinterpret_cast<float4*>(S.v[buf][warp]);
#pragma unroll
    for (int q = 0; q < 8; ++q) d[q] = make_float4(p[4 * q], p[4 * q + 1], p[4 * q + 2], p[4 * q + 3]);
  }
  if (lane == 0) {
    S.m[buf][warp] = wmax;
    S.i[buf][warp] = widx;
  }
  __syncthreads();
  // CTA choice: every warp reduces the 8 posts (lane l reads post l mod 8)
  const unsigned m8 = S.m[buf][lane & 7], i8 = S.i[buf][lane & 7];
  const unsigned bm = __reduce_max_sync(full, m8);
  const int bi = (int)__reduce_min_sync(full, m8 == bm ? i8 : 0xffffffffu);
  const bool ok = bm > 1u;
  float v[32];
  {
    const float4* s = reinterpret_cast<const float4*>(S.v[buf][bi >> 5]);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const float4 x = s[q];
      v[4 * q] = x.x;
      v[4 * q + 1] = x.y;
      v[4 * q + 2] = x.z;
      v[4 * q + 3] = x.w;
    }
  }
  if (!ok && tid == 0 && info_b && *info_b == 0) *info_b = k + 1;
  const float pinv = ok ? __frcp_rn(v[CC]) : 0.0f;
  // other rows: p - (p[CC] pinv) v, the column itself -(p[CC] pinv)
  const float w = -(p[CC] * pinv);
#pragma unroll
  for (int j = 0; j < 32; ++j)
    if (j != CC) p[j] = fmaf(w, v[j], p[j]);
  p[CC] = w;
  if (tid == bi) {   // the pivot row: pinv v, the column pinv
#pragma unroll
    for (int j = 0; j < 32; ++j)
      if (j != CC) p[j] = v[j] * pinv;
    p[CC] = pinv;
    used = 1;
    myk = k;
    colpiv[k] = tid;
  }
}

__global__ void __launch_bounds__(ITC_NT, 1)
inv_tc_kernel(int n, const float* __restrict__ A, long long lda, long long sA, float* __restrict__ X, long long ldx,
              long long sX, int batch, int* info) {
  const ItcLayout L = itc_layout(n);
  extern __shared__ unsigned char itc_smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(itc_smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* a_tiles = smem + L.a_off;
  unsigned char* b_tiles = smem + L.b_off;
  const size_t b_part = (size_t)L.NP * 128;
  float* gst = reinterpret_cast<float*>(smem + L.g_off);
  float* xs = reinterpret_cast<float*>(smem);

  __shared__ __align__(16) ItcSlots slots;
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
    // ---- A -> TMEM, one half at a time through shared memory; the loads are
    // asynchronous copies (all of a half in flight at once, zero-filled
    // outside the matrix) ----
    for (int h = 0; h < L.NH; ++h) {
      __syncthreads();
      const int w = L.NC * 32;
      for (int e = tid; e < 128 * w; e += ITC_NT) {
        const int r = e / w, c = e - r * w, row = 128 * h + r;
        const bool in = row < n && c < n;
        const float* src = in ? Ab + (long long)row * lda + c : Ab;
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(tc::smem_u32(xs + r * L.XS + c)),
                     "l"(src), "r"(in ? 4 : 0)
                     : "memory");
      }
      asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
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
    int* info_b = info ? info + b : nullptr;

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
      // ---- panel: Gauss-Jordan restricted to the 32 panel columns; the
      // current column is p[0] (steps of four: p[0..3]), the registers
      // rotate after each step ----
      int c = 0;
#pragma unroll 1
      for (; c + 4 <= bw; c += 4) {
        gj_step<0>(p, k0 + c, 0, tid, warp, lane, used, myk, slots, colpiv, info_b);
        gj_step<1>(p, k0 + c + 1, 1, tid, warp, lane, used, myk, slots, colpiv, info_b);
        gj_step<2>(p, k0 + c + 2, 0, tid, warp, lane, used, myk, slots, colpiv, info_b);
        gj_step<3>(p, k0 + c + 3, 1, tid, warp, lane, used, myk, slots, colpiv, info_b);
        rotate32<4>(p);
      }
#pragma unroll 1
      for (; c < bw; ++c) {
        gj_step<0>(p, k0 + c, c & 1, tid, warp, lane, used, myk, slots, colpiv, info_b);
        rotate32<1>(p);
      }
      // back to natural column order after a short last panel
#pragma unroll 1
      for (; c < ITC_BW; ++c) rotate32<1>(p);
      // ---- U' = final panel values, into the A tiles of this half ----
      if (half < L.NH) {
        unsigned char* a0 = a_tiles + (size_t)half * 3 * ITC_TILE;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          float u[4];
#pragma unroll
          for (int i = 0; i < 4; ++i) u[i] = (4 * q + i < bw) ? p[4 * q + i] : 0.0f;
          store_split4x3(a0, a0 + ITC_TILE, a0 + 2 * ITC_TILE, rl, 4 * q, u);
        }
      }
      // ---- pivot rows before the update -> staging (G' rows); then zeroed in TMEM ----
      const bool piv_here = myk >= k0 && myk < k0 + bw;
      const bool warp_piv = __any_sync(0xffffffffu, piv_here);
      for (int ch = 0; ch < L.NC && tm_rows; ++ch) {
        float w32[32];
        tc::tmem_ld32(trow + ch * 32, w32);
        if (piv_here) {
          float4* d = reinterpret_cast<float4*>(gst + (size_t)(myk - k0) * L.GS + ch * 32);
#pragma unroll
          for (int q = 0; q < 8; ++q)
            d[q] = make_float4(w32[4 * q], w32[4 * q + 1], w32[4 * q + 2], w32[4 * q + 3]);
#pragma unroll
          for (int j = 0; j < 32; ++j) w32[j] = 0.0f;
        }
        if (warp_piv) tc::tmem_st32(trow + ch * 32, w32);
      }
      if (tm_rows && warp_piv) tc::tmem_wait_st();   // before the panel columns are stored over them
      // ---- panel columns back into TMEM (the MMA adds zero to them) ----
      if (tm_rows) {
        tc::tmem_st32(trow + k0, p);
        tc::tmem_wait_st();
      }
      __syncthreads();
      // ---- G'^T into the B tiles: row j (tableau column), K = pivot index ----
      for (int e = tid; e < 8 * L.NP; e += ITC_NT) {
        const int kq = (e / L.NP) * 4, j = e - (e / L.NP) * L.NP;
        const bool z = j >= n || (j >= k0 && j < k0 + ITC_BW);
        float g4[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) g4[i] = (z || kq + i >= bw) ? 0.0f : gst[(size_t)(kq + i) * L.GS + j];
        store_split4x3(b_tiles, b_tiles + b_part, b_tiles + 2 * b_part, j, kq, g4);
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      tc::fence_before();
      __syncthreads();
      if (tid == 0) {
        tc::fence_after();
        const uint32_t b0 = tc::smem_u32(b_tiles);
        const uint32_t bp = (uint32_t)b_part;
        for (int h = 0; h < L.NH; ++h) {
          const uint32_t a0 = tc::smem_u32(a_tiles + (size_t)h * 3 * ITC_TILE);
          const uint32_t d = tmem + (uint32_t)(h * 256);
#pragma unroll
          for (int kk = 0; kk < ITC_BW / 8; ++kk) {
            const uint32_t off = kk * 32;
            // (A part, B part): x0y0, x0y1, x1y0, x1y1, x0y2, x2y0
            tc::mma_tf32(d, tc::desc_sw128(a0 + off), tc::desc_sw128(b0 + off), idesc, 1u);
            tc::mma_tf32(d, tc::desc_sw128(a0 + off), tc::desc_sw128(b0 + bp + off), idesc, 1u);
            tc::mma_tf32(d, tc::desc_sw128(a0 + ITC_TILE + off), tc::desc_sw128(b0 + off), idesc, 1u);
            tc::mma_tf32(d, tc::desc_sw128(a0 + ITC_TILE + off), tc::desc_sw128(b0 + bp + off), idesc, 1u);
            tc::mma_tf32(d, tc::desc_sw128(a0 + off), tc::desc_sw128(b0 + 2 * bp + off), idesc, 1u);
            tc::mma_tf32(d, tc::desc_sw128(a0 + 2 * ITC_TILE + off), tc::desc_sw128(b0 + off), idesc, 1u);
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
