// Batched matrix inverse by Gauss-Jordan elimination with partial pivoting.
//
// The reference forms every leaf and merge operator through explicit
// inverses (jnp.linalg.inv at local_solve/_uniform_2D_DtN.py:257,
// local_solve/_uniform_2D_ItI.py:167, merge/_schur_complement.py:107,146);
// this file is the GPU replacement for those calls.
//
// Pivoting is "implicit": rows are never moved.  Column k is eliminated
// with the largest-magnitude entry among rows not yet used as pivots; the
// in-place tableau then holds inv(A) up to a row/column relabelling that is
// undone on write-out:  inv(A)[k][j] = M[piv[k]][rinv[j]].
//
// Two implementations:
//  * inv_reg_kernel  - one 512-thread CTA per matrix, the whole matrix held
//    in registers (block-cyclic over a 32x16 thread grid).  Two barriers
//    per pivot; the rank-1 update reads one column and one scaled row from
//    shared memory.  Serves n <= 208 (f32), 128 (f64, c64), 64 (c128).
//  * blocked GJE     - panels of BP columns: one CTA per matrix selects the
//    pivots of the panel (tableau restricted to the panel columns), then
//    the block sweep is applied to the rest of the matrix by two batched
//    GEMMs and a row scatter:
//        M[Rbar,Cbar] += U G,   M[R,Cbar] = E G,
//    with U = new panel (pivot rows zeroed), G = pivot rows (panel columns
//    zeroed), E = inv(A[R,C]) (the panel's pivot rows after elimination).
#include <stdio.h>

#include <stdlib.h>

#include <cooperative_groups.h>

#include "hps_common.cuh"
#include "hps_internal.h"

namespace hps {

// --------------------------------------------------------------------------
// Register-resident single-CTA kernel
// --------------------------------------------------------------------------
template <class T, int NMAX>
__global__ void __launch_bounds__(512, 1)
inv_reg_kernel(int n, const T* __restrict__ A, long long lda, long long sA, T* X, long long ldx,
               long long sX, int* info) {
  constexpr int TY = 32, TX = 16;
  constexpr int RM = (NMAX + TY - 1) / TY;
  constexpr int RN = (NMAX + TX - 1) / TX;
  __shared__ T colbuf[2][NMAX];
  __shared__ T rowbuf[2][NMAX];
  __shared__ int piv[NMAX];
  __shared__ int colof[NMAX];
  __shared__ unsigned char used[NMAX];
  __shared__ int s_info;

  const long long bb = blockIdx.x;
  const T* Ab = A + bb * sA;
  const int tid = threadIdx.x;
  const int ty = tid / TX, tx = tid % TX, lane = tid & 31;

  T m[RM][RN];
#pragma unroll
  for (int a = 0; a < RM; ++a)
#pragma unroll
    for (int c = 0; c < RN; ++c) {
      const int i = ty + TY * a, j = tx + TX * c;
      m[a][c] = (i < n && j < n) ? Ab[(long long)i * lda + j] : zero<T>();
    }
  for (int i = tid; i < NMAX; i += blockDim.x) used[i] = (i < n) ? 0 : 1;
  if (tid == 0) s_info = 0;
  __syncthreads();

  for (int k = 0; k < n; ++k) {
    const int buf = k & 1;
    const int kx = k % TX, kc = k / TX;
    // (1) publish column k
    if (tx == kx) {
#pragma unroll
      for (int a = 0; a < RM; ++a) {
        const int i = ty + TY * a;
        T v = zero<T>();
#pragma unroll
        for (int c = 0; c < RN; ++c)
          if (c == kc) v = m[a][c];
        if (i < n) colbuf[buf][i] = v;
      }
    }
    __syncthreads();
    // (2) pivot row: every warp computes the same argmax redundantly
    using MagT = typename MagOf<T>::type;
    MagT best = -1;
    int bi = n;
    for (int i = lane; i < n; i += 32) {
      if (!used[i]) {
        const MagT mg = nan_to_inf(pivmag(colbuf[buf][i]));
        if (mg > best) {
          best = mg;
          bi = i;
        }
      }
    }
#pragma unroll
    for (int off = 16; off; off >>= 1) {
      const MagT ob = __shfl_xor_sync(0xffffffffu, best, off);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
      if (ob > best || (ob == best && oi < bi)) {
        best = ob;
        bi = oi;
      }
    }
    const int r = bi;
    T pinv = zero<T>();
    if (best > 0) {
      pinv = rcp_(colbuf[buf][r]);
    } else if (tid == 0 && s_info == 0) {
      s_info = k + 1;
    }
    // (3) publish the scaled pivot row
    const int ry = r % TY, ra = r / TY;
    if (ty == ry) {
#pragma unroll
      for (int a = 0; a < RM; ++a) {
        if (a != ra) continue;
#pragma unroll
        for (int c = 0; c < RN; ++c) {
          const int j = tx + TX * c;
          if (j < n) rowbuf[buf][j] = mul(m[a][c], pinv);
        }
      }
    }
    __syncthreads();
    // (4) rank-1 update of the register tile, then row r / column k fix-ups
    T rj[RN];
#pragma unroll
    for (int c = 0; c < RN; ++c) {
      const int j = tx + TX * c;
      rj[c] = (j < n) ? rowbuf[buf][j] : zero<T>();
    }
#pragma unroll
    for (int a = 0; a < RM; ++a) {
      const int i = ty + TY * a;
      const T ci = (i < n) ? colbuf[buf][i] : zero<T>();
#pragma unroll
      for (int c = 0; c < RN; ++c) m[a][c] = fms_(ci, rj[c], m[a][c]);
    }
    if (ty == ry) {
#pragma unroll
      for (int a = 0; a < RM; ++a)
        if (a == ra) {
#pragma unroll
          for (int c = 0; c < RN; ++c) m[a][c] = rj[c];
        }
    }
    if (tx == kx) {
#pragma unroll
      for (int a = 0; a < RM; ++a) {
        const int i = ty + TY * a;
        T nv = (i < n) ? neg(mul(colbuf[buf][i], pinv)) : zero<T>();
        if (i == r) nv = pinv;
#pragma unroll
        for (int c = 0; c < RN; ++c)
          if (c == kc) m[a][c] = nv;
      }
    }
    if (tid == 0) {
      used[r] = 1;
      piv[k] = r;
      colof[r] = k;
    }
  }
  __syncthreads();
  if (tid == 0 && info) info[bb] = s_info;
  T* Xb = X + bb * sX;
#pragma unroll
  for (int a = 0; a < RM; ++a)
#pragma unroll
    for (int c = 0; c < RN; ++c) {
      const int i = ty + TY * a, j = tx + TX * c;
      if (i < n && j < n) Xb[(long long)colof[i] * ldx + piv[j]] = m[a][c];
    }
}

// --------------------------------------------------------------------------
// Shared-memory blocked kernel: one 512-thread CTA per matrix, the tableau
// in shared memory.  Panels of KB columns: the panel's pivots are chosen by
// Gauss-Jordan restricted to the panel columns (three barriers per column),
// then one rank-KB block-sweep update of the other columns with register
// tiles (RA rows x RN columns per thread, KB-long dot products):
//     M[i][j] = (i in R ? 0 : M[i][j]) + sum_k Z[i][k] G[k][j]
// where Z = the panel after elimination and G = the pivot rows before it.
// --------------------------------------------------------------------------
constexpr int SB_NT = 512;
constexpr int SB_TY = 16, SB_TX = 32;

template <class T>
size_t inv_sblock_smem(int n, int KB) {
  const int ldm = n + 1;
  // M | G (KB x n, the sweep) sharing storage with the panel's two row
  // buffers (2 x n x KB) | piv | colof | used
  return sizeof(T) * ((size_t)n * ldm + 2 * (size_t)KB * n) + sizeof(int) * 2 * (size_t)n + (size_t)n + 16;
}

template <class T, int KB, int RN>
__global__ void __launch_bounds__(SB_NT, 1)
inv_sblock_kernel(int n, const T* __restrict__ A, long long lda, long long sA, T* X, long long ldx, long long sX,
                  int* info) {
  using MagT = typename MagOf<T>::type;
  constexpr int RA = 4;
  constexpr int NW = SB_NT / 32;
  extern __shared__ __align__(16) unsigned char sbraw[];
  const int ldm = n + 1;
  T* M = reinterpret_cast<T*>(sbraw);
  T* G = M + (size_t)n * ldm;        // sweep: pivot rows (KB x n)
  T* PB = G;                         // panel: 2 buffers of every row's panel segment, [c2][row] (KB x n each)
  int* piv = reinterpret_cast<int*>(G + 2 * (size_t)KB * n);
  int* colof = piv + n;
  unsigned char* used = reinterpret_cast<unsigned char*>(colof + n);
  __shared__ int Rs[KB];
  __shared__ MagT cand_m[2][NW];
  __shared__ int cand_i[2][NW];
  __shared__ int s_info;

  const long long bb = blockIdx.x;
  const T* Ab = A + bb * sA;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int ty = tid / SB_TX, tx = tid % SB_TX;
  const bool has_row = tid < n;   // thread tid owns row tid during the panels (n <= SB_NT)

  for (int e = tid; e < n * n; e += SB_NT) {
    const int i = e / n, j = e % n;
    M[i * ldm + j] = Ab[(long long)i * lda + j];
  }
  for (int i = tid; i < n; i += SB_NT) used[i] = 0;
  if (tid == 0) s_info = 0;
  __syncthreads();

  // warp-level arg-max of (magnitude, row), ties to the smaller row; lane 0
  // publishes the warp's candidate
  auto publish_candidate = [&](int buf, MagT mg, int bi) {
#pragma unroll
    for (int off = 16; off; off >>= 1) {
      const MagT ob = __shfl_xor_sync(0xffffffffu, mg, off);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
      if (ob > mg || (ob == mg && oi < bi)) {
        mg = ob;
        bi = oi;
      }
    }
    if (lane == 0) {
      cand_m[buf][warp] = mg;
      cand_i[buf][warp] = bi;
    }
  };

  for (int k0 = 0; k0 < n; k0 += KB) {
    const int bw = min(KB, n - k0);
    // ---- panel: Gauss-Jordan restricted to columns k0 .. k0+bw-1, one
    // barrier per column.  Each thread keeps its row's panel segment in
    // registers and publishes it (double-buffered) so that every thread can
    // form the scaled pivot row itself after the barrier.
    T rv[KB];
    int ust = has_row ? used[tid] : 1;   // 0 free, 1 pivot of an earlier block, 2 of this block
#pragma unroll
    for (int c2 = 0; c2 < KB; ++c2) rv[c2] = (has_row && c2 < bw) ? M[tid * ldm + k0 + c2] : zero<T>();
    if (has_row) {
#pragma unroll
      for (int c2 = 0; c2 < KB; ++c2) PB[c2 * n + tid] = rv[c2];   // consecutive rows: conflict-free
    }
    publish_candidate(0, (has_row && !ust) ? nan_to_inf(pivmag(rv[0])) : (MagT)-1, (has_row && !ust) ? tid : n);
    __syncthreads();
    // unrolled over the block: c is a constant in each copy, so rv[c] and the
    // (c2 == c) choices below are plain register accesses
#pragma unroll
    for (int c = 0; c < KB; ++c) {
      if (c >= bw) break;
      const int pb = c & 1;
      MagT best = -1;
      int r = n;
#pragma unroll
      for (int w = 0; w < NW; ++w) {
        const MagT ob = cand_m[pb][w];
        const int oi = cand_i[pb][w];
        if (ob > best || (ob == best && oi < r)) {
          best = ob;
          r = oi;
        }
      }
      // r < n: rows not yet pivots remain (n - k0 - c of them), each a candidate
      if (r >= n) r = 0;
      const T* prow = PB + (size_t)pb * n * KB + r;
      T rr[KB];
#pragma unroll
      for (int c2 = 0; c2 < KB; ++c2) rr[c2] = prow[c2 * n];   // one address per load: broadcast
      T pinv = zero<T>();
#pragma unroll
      for (int c2 = 0; c2 < KB; ++c2)
        if (c2 == c) pinv = (best > 0) ? rcp_(rr[c2]) : zero<T>();
#pragma unroll
      for (int c2 = 0; c2 < KB; ++c2) rr[c2] = mul(rr[c2], pinv);
      if (tid == 0) {
        Rs[c] = r;
        piv[k0 + c] = r;
        colof[r] = k0 + c;
        if (!(best > 0) && s_info == 0) s_info = k0 + c + 1;
      }
      if (has_row) {
        if (tid == r) {
#pragma unroll
          for (int c2 = 0; c2 < KB; ++c2) rv[c2] = (c2 == c) ? pinv : rr[c2];
          ust = 2;
        } else {
          T f = zero<T>();
#pragma unroll
          for (int c2 = 0; c2 < KB; ++c2)
            if (c2 == c) f = rv[c2];
#pragma unroll
          for (int c2 = 0; c2 < KB; ++c2) rv[c2] = (c2 == c) ? neg(mul(f, pinv)) : fms_(f, rr[c2], rv[c2]);
        }
      }
      if (c + 1 < bw) {
        if (has_row) {
          T* dst = PB + (size_t)(pb ^ 1) * n * KB + tid;
#pragma unroll
          for (int c2 = 0; c2 < KB; ++c2) dst[c2 * n] = rv[c2];
        }
        T nxt = zero<T>();
#pragma unroll
        for (int c2 = 0; c2 < KB; ++c2)
          if (c2 == c + 1) nxt = rv[c2];
        publish_candidate(pb ^ 1, (has_row && !ust) ? nan_to_inf(pivmag(nxt)) : (MagT)-1,
                          (has_row && !ust) ? tid : n);
        __syncthreads();
      }
    }
    __syncthreads();   // every thread has read the last pivot row before G overwrites the buffers
    if (has_row) {
#pragma unroll
      for (int c2 = 0; c2 < KB; ++c2)
        if (c2 < bw) M[tid * ldm + k0 + c2] = rv[c2];
      used[tid] = (unsigned char)ust;
    }
    __syncthreads();
    // ---- pivot rows outside the panel, before the sweep
    for (int e = tid; e < bw * n; e += SB_NT) {
      const int k = e / n, j = e % n;
      G[k * n + j] = (j >= k0 && j < k0 + bw) ? zero<T>() : M[Rs[k] * ldm + j];
    }
    __syncthreads();
    // ---- rank-bw block sweep of the non-panel columns
    for (int a0 = ty * RA; a0 < n; a0 += SB_TY * RA) {
      T acc[RA][RN];
      bool isR[RA];
#pragma unroll
      for (int a = 0; a < RA; ++a) {
        const int i = a0 + a;
        isR[a] = (i < n) && used[i] == 2;
#pragma unroll
        for (int b = 0; b < RN; ++b) {
          const int j = tx + SB_TX * b;
          acc[a][b] = (i < n && j < n && !isR[a]) ? M[i * ldm + j] : zero<T>();
        }
      }
#pragma unroll 4
      for (int k = 0; k < bw; ++k) {
        T z[RA], gk[RN];
#pragma unroll
        for (int a = 0; a < RA; ++a) z[a] = (a0 + a < n) ? M[(a0 + a) * ldm + k0 + k] : zero<T>();
#pragma unroll
        for (int b = 0; b < RN; ++b) {
          const int j = tx + SB_TX * b;
          gk[b] = (j < n) ? G[k * n + j] : zero<T>();
        }
#pragma unroll
        for (int a = 0; a < RA; ++a)
#pragma unroll
          for (int b = 0; b < RN; ++b) acc[a][b] = fma_(z[a], gk[b], acc[a][b]);
      }
#pragma unroll
      for (int a = 0; a < RA; ++a) {
        const int i = a0 + a;
        if (i >= n) continue;
#pragma unroll
        for (int b = 0; b < RN; ++b) {
          const int j = tx + SB_TX * b;
          if (j < n && (j < k0 || j >= k0 + bw)) M[i * ldm + j] = acc[a][b];
        }
      }
    }
    __syncthreads();
    if (tid < bw) used[Rs[tid]] = 1;
    __syncthreads();
  }
  if (tid == 0 && info) info[bb] = s_info;
  // inv(A)[k][j] = M[piv[k]][rinv[j]], written row by row (coalesced);
  // colof is rinv: colof[piv[j]] = j
  T* Xb = X + bb * sX;
  for (int e = tid; e < n * n; e += SB_NT) {
    const int k = e / n, j = e % n;
    Xb[(long long)k * ldx + j] = M[piv[k] * ldm + colof[j]];
  }
}

// --------------------------------------------------------------------------
// Blocked Gauss-Jordan (global-memory tableau)
// --------------------------------------------------------------------------
constexpr int BP = 32;       // panel width
constexpr int PANEL_NT = 1024;
constexpr int PANEL_SMEM_ROWS = 4096;   // used flags kept in shared memory up to this n

struct GjeWs {
  // per-matrix region sizes (bytes), each 256-byte aligned; sync = the
  // multi-CTA panel's barrier and proposal slots
  size_t mat, pan, u, g, h, e, piv, rinv, used, sync, per;
};

// Multi-CTA panels run as thread-block clusters unless HPS_CLUSTER_PANELS=0.
static bool cluster_panels_enabled() {
  static const bool on = [] {
    const char* e = getenv("HPS_CLUSTER_PANELS");
    return !(e && e[0] == '0');
  }();
  return on;
}

// Upper bound on the CTAs that share one matrix's panel.
static int coop_nct_cap(int n) { return n / 16 < 1 ? 1 : (n / 16 > 1024 ? 1024 : n / 16); }

static size_t al256(size_t x) { return (x + 255) & ~size_t(255); }

static GjeWs gje_layout(size_t es, int n) {
  GjeWs w;
  w.mat = al256(es * (size_t)n * n);
  w.pan = al256(es * (size_t)n * BP);
  w.u = al256(es * (size_t)n * BP);
  w.g = al256(es * (size_t)BP * n);
  w.h = al256(es * (size_t)BP * n);
  w.e = al256(es * (size_t)BP * BP);
  w.piv = al256(4 * (size_t)n);
  w.rinv = al256(4 * (size_t)n);
  w.used = al256((size_t)n);
  {
    // as coop_layout() below with 8-byte magnitudes (an upper bound for every
    // type), for the larger of the cooperative cap and a 16-CTA cluster
    const size_t cap = (size_t)(coop_nct_cap(n) > 16 ? coop_nct_cap(n) : 16);
    w.sync = 256 + al256(2 * cap * 8) + al256(2 * cap * sizeof(int)) + al256(2 * cap * BP * es);
  }
  w.per = w.mat + w.pan + w.u + w.g + w.h + w.e + w.piv + w.rinv + w.used + w.sync;
  return w;
}

// Copies A into the tableau, clears the used flags and sets piv and rinv to
// the identity permutation: a panel that gives up after a barrier timeout
// leaves its piv entries unwritten, and the later kernels index rows and
// columns through piv / rinv, which therefore always hold indices below n.
template <class T>
__global__ void gje_copy_in_kernel(int n, const T* __restrict__ A, long long lda, long long sA, T* Mat,
                                   unsigned char* used, int* piv, int* rinv) {
  const long long b = blockIdx.y;
  const long long nn = (long long)n * n;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nn;
       e += (long long)gridDim.x * blockDim.x) {
    const long long i = e / n, j = e % n;
    Mat[b * nn + e] = A[b * sA + i * lda + j];
  }
  if (blockIdx.x == 0)
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      used[b * n + i] = 0;
      piv[b * n + i] = i;
      rinv[b * n + i] = i;
    }
}

// Panel pivot selection: Gauss-Jordan restricted to the bw panel columns
// k0..k0+bw-1 over all n rows, rows already used as pivots excluded.
// One CTA per matrix.  The panel lives in shared memory column-major
// (P[c*ldp + i], consecutive threads on consecutive rows: conflict-free)
// when it fits, otherwise in a global workspace with the same layout.
// Outputs: the new panel written back into Mat, U (panel with this block's
// pivot rows zeroed), E (the block's pivot rows = inv(A[R,C])), G (pivot
// rows of Mat outside the panel columns), piv[k0..k0+bw-1].
template <class T>
__global__ void __launch_bounds__(PANEL_NT)
gje_panel_kernel(int n, int k0, int bw, T* Mat, T* Pw, int use_smem, T* U, T* G, T* E, int* piv,
                 unsigned char* used, int* info) {
  // blockDim.x threads (a multiple of 32, <= PANEL_NT); thread t owns rows
  // t, t + blockDim.x, ...  Two CTA barriers per column: B1 after every row
  // update (which also forms the next column's pivot candidates), B2 after
  // threads 0..bw-1 have formed the scaled pivot row while P is unchanged.
  using MagT = typename MagOf<T>::type;
  const long long b = blockIdx.x;
  const long long nn = (long long)n * n;
  T* M = Mat + b * nn;
  int* pv = piv + b * n;
  unsigned char* us = used + b * n;
  extern __shared__ unsigned char smraw[];
  const int ldp = n;
  const int NT = blockDim.x;
  T* P = use_smem ? reinterpret_cast<T*>(smraw) : Pw + b * (long long)n * BP;
  __shared__ T rowr[BP];
  __shared__ int Rs[BP];
  __shared__ MagT wbest[2][PANEL_NT / 32];
  __shared__ int widx[2][PANEL_NT / 32];
  __shared__ unsigned char ul_s[PANEL_SMEM_ROWS];
  __shared__ T s_pinv_p;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = NT >> 5;
  // used flags: shared when they fit, else the global array itself
  unsigned char* ul = n <= PANEL_SMEM_ROWS ? ul_s : us;

  for (int e = tid; e < n * bw; e += NT) {
    const int i = e / bw, c = e % bw;
    P[c * ldp + i] = M[(long long)i * n + k0 + c];
  }
  if (n <= PANEL_SMEM_ROWS)
    for (int i = tid; i < n; i += NT) ul_s[i] = us[i];
  __syncthreads();

  auto better = [](MagT m, int i, MagT bm, int bi) { return m > bm || (m == bm && i < bi); };
  auto publish = [&](int buf, MagT best, int bi) {
#pragma unroll
    for (int off = 16; off; off >>= 1) {
      const MagT ob = __shfl_xor_sync(0xffffffffu, best, off);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
      if (better(ob, oi, best, bi)) {
        best = ob;
        bi = oi;
      }
    }
    if (lane == 0) {
      wbest[buf][warp] = best;
      widx[buf][warp] = bi;
    }
  };
  {
    MagT best = -1;
    int bi = n;
    for (int i = tid; i < n; i += NT)
      if (!ul[i]) {
        const MagT mg = nan_to_inf(pivmag(P[i]));
        if (better(mg, i, best, bi)) {
          best = mg;
          bi = i;
        }
      }
    publish(0, best, bi);
  }
  __syncthreads();   // B1 of column 0

  for (int c = 0; c < bw; ++c) {
    const int buf = c & 1;
    // every thread picks the same pivot from the warp candidates
    MagT best = -1;
    int r = n;
    for (int w = 0; w < nw; ++w) {
      const MagT m = wbest[buf][w];
      const int ix = widx[buf][w];
      if (better(m, ix, best, r)) {
        best = m;
        r = ix;
      }
    }
    if (r >= n) r = 0;   // unreachable: n - k0 - c rows are still free
    if (tid < bw) {
      const T pinv = (best > 0) ? rcp_(P[c * ldp + r]) : zero<T>();
      rowr[tid] = mul(P[tid * ldp + r], pinv);
      if (tid == 0) s_pinv_p = pinv;
    }
    if (tid == 0) {
      pv[k0 + c] = r;
      Rs[c] = r;
      if (!(best > 0) && info && info[b] == 0) info[b] = k0 + c + 1;
    }
    __syncthreads();   // B2: rowr and the pivot's reciprocal ready, every thread has read the candidates
    // (row r is rewritten by its owner below: nobody reads it after B2)
    const T pinv = s_pinv_p;
    MagT nb = -1;
    int ni = n;
    for (int i = tid; i < n; i += NT) {
      if (i == r) continue;
      const T f = P[c * ldp + i];
      for (int c2 = 0; c2 < bw; ++c2) {
        T& x = P[c2 * ldp + i];
        x = (c2 == c) ? neg(mul(f, pinv)) : fms_(f, rowr[c2], x);
      }
      if (c + 1 < bw && !ul[i]) {
        const MagT mg = nan_to_inf(pivmag(P[(c + 1) * ldp + i]));
        if (better(mg, i, nb, ni)) {
          nb = mg;
          ni = i;
        }
      }
    }
    // the pivot row last: its column c value was the pivot every thread read
    if (r % NT == tid) {
      for (int c2 = 0; c2 < bw; ++c2) P[c2 * ldp + r] = (c2 == c) ? pinv : rowr[c2];
      ul[r] = 2;
    }
    if (c + 1 < bw) publish(buf ^ 1, nb, ni);
    __syncthreads();   // B1 of column c + 1
  }

  // outputs: new panel back into M, U (pivot rows zeroed), E, G
  T* Ub = U + b * (long long)n * BP;
  T* Gb = G + b * (long long)BP * n;
  T* Eb = E + b * (long long)BP * BP;
  for (int e = tid; e < n * bw; e += NT) {
    const int i = e / bw, c = e % bw;
    const T v = P[c * ldp + i];
    M[(long long)i * n + k0 + c] = v;
    Ub[(long long)i * BP + c] = (ul[i] == 2) ? zero<T>() : v;
  }
  for (int e = tid; e < bw * bw; e += NT) {
    const int c1 = e / bw, c2 = e % bw;
    Eb[c1 * BP + c2] = P[c2 * ldp + Rs[c1]];
  }
  for (long long e = tid; e < (long long)bw * n; e += NT) {
    const int c1 = (int)(e / n), j = (int)(e % n);
    Gb[(long long)c1 * n + j] = (j >= k0 && j < k0 + bw) ? zero<T>() : M[(long long)Rs[c1] * n + j];
  }
  __syncthreads();
  if (n <= PANEL_SMEM_ROWS)
    for (int i = tid; i < n; i += NT) us[i] = ul_s[i] == 2 ? 1 : ul_s[i];
  else
    for (int c = tid; c < bw; c += NT) us[Rs[c]] = 1;
}

// --------------------------------------------------------------------------
// Multi-CTA panel selection (few large matrices).
//
// Same result as gje_panel_kernel, but the panel's rows are split over
// gridDim.x CTAs (a cooperative launch, so all of them are resident).  Per
// panel column every CTA proposes its best unused row; the proposals (the
// magnitude, the row index and the row's bw panel values) go to slots in
// global memory, double-buffered by column parity, and one bounded grid
// barrier per column makes them visible.  Every CTA then picks the same
// pivot (largest magnitude, smallest index on ties) and updates its rows.
// A barrier that does not complete within its spin limit sets the matrix's
// error flag; the CTAs return and info[b] is set to -1.
// --------------------------------------------------------------------------
constexpr int CP_NT = 256;
// Polls of the grid barrier before it gives up (each poll sleeps >= 100 ns:
// the default 2^24 is a second or more).  A device variable so that
// hps_set_spin_limits can change it; read once per barrier.
static __device__ long long g_cp_spin_limit = 1ll << 24;

struct CoopHdr {
  unsigned count;
  unsigned gen;
  int err;
  int pad;
};

__device__ __forceinline__ float ld_cg(const float* p) { return __ldcg(p); }
__device__ __forceinline__ double ld_cg(const double* p) { return __ldcg(p); }
__device__ __forceinline__ int ld_cg(const int* p) { return __ldcg(p); }
__device__ __forceinline__ c64 ld_cg(const c64* p) {
  const float2 v = __ldcg(reinterpret_cast<const float2*>(p));
  return c64{v.x, v.y};
}
__device__ __forceinline__ c128 ld_cg(const c128* p) {
  const double2 v = __ldcg(reinterpret_cast<const double2*>(p));
  return c128{v.x, v.y};
}

__device__ __forceinline__ float shfl_T(float v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ double shfl_T(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ c64 shfl_T(c64 v, int src) {
  return c64{__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src)};
}
__device__ __forceinline__ c128 shfl_T(c128 v, int src) {
  return c128{__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src)};
}

// Barrier over the nct CTAs of one matrix; false on timeout or on an
// earlier failure of this matrix.
__device__ __forceinline__ bool coop_barrier(CoopHdr* hdr, unsigned nct) {
  __shared__ int s_ok;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile CoopHdr* vh = hdr;
    int ok = vh->err == 0;
    if (ok) {
      const unsigned g = vh->gen;
      __threadfence();
      const unsigned arrived = atomicAdd(&hdr->count, 1u) + 1u;
      if (arrived == nct) {
        atomicExch(&hdr->count, 0u);
        __threadfence();
        atomicAdd(&hdr->gen, 1u);
      } else {
        long long it = 0;
        const long long limit = *(volatile long long*)&g_cp_spin_limit;
        while (vh->gen == g) {
          if (vh->err != 0 || ++it > limit) {
            ok = 0;
            atomicExch(&hdr->err, 1);
            break;
          }
          __nanosleep(100);
        }
      }
      __threadfence();
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Byte offsets inside one matrix's synchronisation block.
struct CoopLayout {
  size_t mag, idx, cand, per;
};

__host__ __device__ inline CoopLayout coop_layout(size_t es, size_t mag_size, int nct) {
  auto a = [](size_t x) { return (x + 255) & ~size_t(255); };
  CoopLayout c;
  c.mag = 256;
  c.idx = c.mag + a(2 * (size_t)nct * mag_size);
  c.cand = c.idx + a(2 * (size_t)nct * sizeof(int));
  c.per = c.cand + a(2 * (size_t)nct * BP * es);
  return c;
}

// Hardware barrier over the CTAs of a thread-block cluster, with
// release / acquire ordering at cluster scope for the global-memory exchange
// of pivot candidates.  A cluster is co-scheduled by construction and every
// CTA reaches every barrier, so it needs no timeout.
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

template <class T>
__global__ void __launch_bounds__(CP_NT)
gje_panel_coop_kernel(int n, int k0, int bw, int rows_per, T* Mat, T* U, T* G, T* E, int* piv,
                      unsigned char* used, int* info, unsigned char* sync, CoopLayout lay) {
  using MagT = typename MagOf<T>::type;
  const int b = blockIdx.y, cta = blockIdx.x, nct = gridDim.x;
  const long long nn = (long long)n * n;
  T* M = Mat + (long long)b * nn;
  int* pv = piv + (long long)b * n;
  unsigned char* us = used + (long long)b * n;
  unsigned char* sb = sync + (size_t)b * lay.per;
  CoopHdr* hdr = reinterpret_cast<CoopHdr*>(sb);
  MagT* smag = reinterpret_cast<MagT*>(sb + lay.mag);
  int* sidx = reinterpret_cast<int*>(sb + lay.idx);
  T* scand = reinterpret_cast<T*>(sb + lay.cand);

  extern __shared__ __align__(16) unsigned char smraw[];
  T* P = reinterpret_cast<T*>(smraw);   // P[c * rows_per + i], i local row
  T* fcol = P + (size_t)BP * rows_per;
  unsigned char* ul = reinterpret_cast<unsigned char*>(fcol + rows_per);
  __shared__ T rowr[BP];
  __shared__ int Rs[BP];
  __shared__ MagT wbest[CP_NT / 32];
  __shared__ int widx[CP_NT / 32];
  __shared__ int s_r, s_cta;
  __shared__ MagT s_best;
  __shared__ T s_pinv;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int r0 = cta * rows_per;
  const int nr = max(0, min(n - r0, rows_per));

  for (int e = tid; e < nr * bw; e += CP_NT) {
    const int i = e / bw, c = e % bw;
    P[c * rows_per + i] = M[(long long)(r0 + i) * n + k0 + c];
  }
  for (int i = tid; i < nr; i += CP_NT) ul[i] = us[r0 + i];
  __syncthreads();

  for (int c = 0; c < bw; ++c) {
    const int buf = c & 1;
    // this CTA's candidate
    MagT best = -1;
    int bi = n;
    for (int i = tid; i < nr; i += CP_NT) {
      if (!ul[i]) {
        const MagT mg = nan_to_inf(pivmag(P[c * rows_per + i]));
        if (mg > best) {
          best = mg;
          bi = r0 + i;
        }
      }
    }
#pragma unroll
    for (int off = 16; off; off >>= 1) {
      const MagT ob = __shfl_xor_sync(0xffffffffu, best, off);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
      if (ob > best || (ob == best && oi < bi)) {
        best = ob;
        bi = oi;
      }
    }
    if (lane == 0) {
      wbest[warp] = best;
      widx[warp] = bi;
    }
    __syncthreads();
    if (warp == 0) {
      best = lane < CP_NT / 32 ? wbest[lane] : (MagT)-1;
      bi = lane < CP_NT / 32 ? widx[lane] : n;
#pragma unroll
      for (int off = 16; off; off >>= 1) {
        const MagT ob = __shfl_xor_sync(0xffffffffu, best, off);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
        if (ob > best || (ob == best && oi < bi)) {
          best = ob;
          bi = oi;
        }
      }
      if (lane == 0) {
        smag[buf * nct + cta] = best;
        sidx[buf * nct + cta] = bi;
        s_r = bi;
      }
    }
    __syncthreads();
    {
      const int lbi = s_r;
      if (tid < BP)
        scand[((size_t)buf * nct + cta) * BP + tid] =
            (lbi < n && tid < bw) ? P[tid * rows_per + (lbi - r0)] : zero<T>();
    }
    if (!coop_barrier(hdr, (unsigned)nct)) {
      if (cta == 0 && tid == 0 && info) info[b] = -1;
      return;
    }
    // the pivot: same choice in every CTA
    if (warp == 0) {
      best = -1;
      bi = n;
      int bc = 0;
      for (int k = lane; k < nct; k += 32) {
        const MagT m = ld_cg(smag + buf * nct + k);
        const int ix = ld_cg(sidx + buf * nct + k);
        if (m > best || (m == best && ix < bi)) {
          best = m;
          bi = ix;
          bc = k;
        }
      }
#pragma unroll
      for (int off = 16; off; off >>= 1) {
        const MagT ob = __shfl_xor_sync(0xffffffffu, best, off);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
        const int oc = __shfl_xor_sync(0xffffffffu, bc, off);
        if (ob > best || (ob == best && oi < bi)) {
          best = ob;
          bi = oi;
          bc = oc;
        }
      }
      if (lane == 0) {
        s_r = bi;
        s_best = best;
        s_cta = bc;
        Rs[c] = bi;
        if (cta == 0) {
          pv[k0 + c] = bi;
          if (!(best > 0) && info && info[b] == 0) info[b] = k0 + c + 1;
        }
      }
    }
    __syncthreads();
    const int r = s_r;
    if (tid == 0) {
      const T pc = ld_cg(scand + ((size_t)buf * nct + s_cta) * BP + c);
      s_pinv = (s_best > 0) ? rcp_(pc) : zero<T>();
    }
    __syncthreads();
    const T pinv = s_pinv;
    if (tid < bw) rowr[tid] = mul(ld_cg(scand + ((size_t)buf * nct + s_cta) * BP + tid), pinv);
    for (int i = tid; i < nr; i += CP_NT) fcol[i] = P[c * rows_per + i];
    if (tid == 0 && r >= r0 && r < r0 + nr) ul[r - r0] = 2;
    __syncthreads();
    for (int e = tid; e < nr * bw; e += CP_NT) {
      const int i = e % nr, c2 = e / nr;
      T& x = P[c2 * rows_per + i];
      if (r0 + i == r) {
        x = (c2 == c) ? pinv : rowr[c2];
      } else {
        const T f = fcol[i];
        x = (c2 == c) ? neg(mul(f, pinv)) : fms_(f, rowr[c2], x);
      }
    }
    __syncthreads();
  }

  // outputs, as gje_panel_kernel: panel back into M, U, E (pivot rows this CTA owns), G, used flags
  T* Ub = U + (long long)b * n * BP;
  T* Gb = G + (long long)b * BP * n;
  T* Eb = E + (long long)b * BP * BP;
  for (int e = tid; e < nr * bw; e += CP_NT) {
    const int i = e / bw, c = e % bw;
    const T v = P[c * rows_per + i];
    M[(long long)(r0 + i) * n + k0 + c] = v;
    Ub[(long long)(r0 + i) * BP + c] = (ul[i] == 2) ? zero<T>() : v;
  }
  for (int e = tid; e < bw * bw; e += CP_NT) {
    const int c1 = e / bw, c2 = e % bw;
    const int rr = Rs[c1];
    if (rr >= r0 && rr < r0 + nr) Eb[c1 * BP + c2] = P[c2 * rows_per + (rr - r0)];
  }
  for (long long e = (long long)cta * CP_NT + tid; e < (long long)bw * n; e += (long long)nct * CP_NT) {
    const int c1 = (int)(e / n), j = (int)(e % n);
    Gb[(long long)c1 * n + j] = (j >= k0 && j < k0 + bw) ? zero<T>() : M[(long long)Rs[c1] * n + j];
  }
  for (int i = tid; i < nr; i += CP_NT) us[r0 + i] = (ul[i] == 2) ? 1 : ul[i];
}

// Panel of one matrix on the nct CTAs of a thread-block cluster, pivot
// candidates exchanged through distributed shared memory.  Per column: each
// CTA publishes (magnitude, row, the row's panel values) in its own shared
// memory (double-buffered); after the cluster barrier warp 0 of every CTA
// reads the nct candidates in one round of remote loads, picks the pivot and
// reads the pivot row in a second round; every thread then updates whole rows
// of its CTA's slice (no read/write hazard inside a row) and computes the
// next column's candidate on the way.  Two CTA barriers and one cluster
// barrier per column.  Outputs as gje_panel_coop_kernel.
template <class T>
struct PanelPub {
  typename MagOf<T>::type mag;
  int idx;
  T row[BP];
};

template <class T>
__global__ void __launch_bounds__(CP_NT)
gje_panel_cluster_kernel(int n, int k0, int bw, int rows_per, T* Mat, T* U, T* G, T* E, int* piv,
                         unsigned char* used, int* info) {
  namespace cg = cooperative_groups;
  using MagT = typename MagOf<T>::type;
  cg::cluster_group cluster = cg::this_cluster();
  const int b = blockIdx.y, cta = (int)cluster.block_rank(), nct = (int)cluster.num_blocks();
  const long long nn = (long long)n * n;
  T* M = Mat + (long long)b * nn;
  int* pv = piv + (long long)b * n;
  unsigned char* us = used + (long long)b * n;

  extern __shared__ __align__(16) unsigned char smraw[];
  T* P = reinterpret_cast<T*>(smraw);   // P[c * rows_per + i], i local row
  unsigned char* ul = reinterpret_cast<unsigned char*>(P + (size_t)BP * rows_per);
  __shared__ PanelPub<T> pub[2];
  __shared__ T rowr[BP];
  __shared__ int Rs[BP];
  __shared__ MagT wbest[CP_NT / 32];
  __shared__ int widx[CP_NT / 32];
  __shared__ int s_r;
  __shared__ T s_pinv;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int r0 = cta * rows_per;
  const int nr = max(0, min(n - r0, rows_per));

  for (int e = tid; e < nr * bw; e += CP_NT) {
    const int i = e / bw, c = e % bw;
    P[c * rows_per + i] = M[(long long)(r0 + i) * n + k0 + c];
  }
  for (int i = tid; i < nr; i += CP_NT) ul[i] = us[r0 + i];
  __syncthreads();

  auto better = [](MagT m, int i, MagT bm, int bi) { return m > bm || (m == bm && i < bi); };
  // candidate of column 0 over this thread's rows
  MagT best = -1;
  int bi = n;
  for (int i = tid; i < nr; i += CP_NT)
    if (!ul[i]) {
      const MagT mg = nan_to_inf(pivmag(P[i]));
      if (better(mg, r0 + i, best, bi)) {
        best = mg;
        bi = r0 + i;
      }
    }

  for (int c = 0; c < bw; ++c) {
    const int buf = c & 1;
    // CTA candidate -> pub[buf]
#pragma unroll
    for (int off = 16; off; off >>= 1) {
      const MagT ob = __shfl_xor_sync(0xffffffffu, best, off);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
      if (better(ob, oi, best, bi)) {
        best = ob;
        bi = oi;
      }
    }
    if (lane == 0) {
      wbest[warp] = best;
      widx[warp] = bi;
    }
    __syncthreads();
    if (warp == 0) {
      MagT m = lane < CP_NT / 32 ? wbest[lane] : (MagT)-1;
      int ix = lane < CP_NT / 32 ? widx[lane] : n;
#pragma unroll
      for (int off = 16; off; off >>= 1) {
        const MagT ob = __shfl_xor_sync(0xffffffffu, m, off);
        const int oi = __shfl_xor_sync(0xffffffffu, ix, off);
        if (better(ob, oi, m, ix)) {
          m = ob;
          ix = oi;
        }
      }
      if (lane == 0) {
        pub[buf].mag = m;
        pub[buf].idx = ix;
      }
      if (lane < BP) pub[buf].row[lane] = (ix < n && lane < bw) ? P[lane * rows_per + (ix - r0)] : zero<T>();
    }
    cluster_sync_all();
    // the pivot: the same choice in every CTA
    if (warp == 0) {
      MagT m = -1;
      int ix = n, wc = 0;
      if (lane < nct) {
        const PanelPub<T>* rp = cluster.map_shared_rank(&pub[buf], lane);
        m = rp->mag;
        ix = rp->idx;
        wc = lane;
      }
#pragma unroll
      for (int off = 16; off; off >>= 1) {
        const MagT ob = __shfl_xor_sync(0xffffffffu, m, off);
        const int oi = __shfl_xor_sync(0xffffffffu, ix, off);
        const int oc = __shfl_xor_sync(0xffffffffu, wc, off);
        if (better(ob, oi, m, ix)) {
          m = ob;
          ix = oi;
          wc = oc;
        }
      }
      const PanelPub<T>* wp = cluster.map_shared_rank(&pub[buf], wc);
      const T rv = lane < BP ? wp->row[lane] : zero<T>();
      const T pc = shfl_T(rv, c);   // lane c holds the pivot element
      const T pinv = (m > 0) ? rcp_(pc) : zero<T>();
      if (lane < BP) rowr[lane] = mul(rv, pinv);
      if (lane == 0) {
        s_r = ix;
        s_pinv = pinv;
        Rs[c] = ix;
        if (cta == 0) {
          pv[k0 + c] = ix;
          if (!(m > 0) && info && info[b] == 0) info[b] = k0 + c + 1;
        }
      }
    }
    __syncthreads();
    const int r = s_r;
    const T pinv = s_pinv;
    // whole-row updates; the next column's candidate on the way
    best = -1;
    bi = n;
    for (int i = tid; i < nr; i += CP_NT) {
      if (r0 + i == r) {
        for (int c2 = 0; c2 < bw; ++c2) P[c2 * rows_per + i] = (c2 == c) ? pinv : rowr[c2];
        ul[i] = 2;
      } else {
        const T f = P[c * rows_per + i];
        for (int c2 = 0; c2 < bw; ++c2) {
          T& x = P[c2 * rows_per + i];
          x = (c2 == c) ? neg(mul(f, pinv)) : fms_(f, rowr[c2], x);
        }
        if (c + 1 < bw && !ul[i]) {
          const MagT mg = nan_to_inf(pivmag(P[(c + 1) * rows_per + i]));
          if (better(mg, r0 + i, best, bi)) {
            best = mg;
            bi = r0 + i;
          }
        }
      }
    }
  }
  // no CTA leaves while another may still read its published candidates
  cluster_sync_all();

  T* Ub = U + (long long)b * n * BP;
  T* Gb = G + (long long)b * BP * n;
  T* Eb = E + (long long)b * BP * BP;
  for (int e = tid; e < nr * bw; e += CP_NT) {
    const int i = e / bw, c = e % bw;
    const T v = P[c * rows_per + i];
    M[(long long)(r0 + i) * n + k0 + c] = v;
    Ub[(long long)(r0 + i) * BP + c] = (ul[i] == 2) ? zero<T>() : v;
  }
  for (int e = tid; e < bw * bw; e += CP_NT) {
    const int c1 = e / bw, c2 = e % bw;
    const int rr = Rs[c1];
    if (rr >= r0 && rr < r0 + nr) Eb[c1 * BP + c2] = P[c2 * rows_per + (rr - r0)];
  }
  for (long long e = (long long)cta * CP_NT + tid; e < (long long)bw * n; e += (long long)nct * CP_NT) {
    const int c1 = (int)(e / n), j = (int)(e % n);
    Gb[(long long)c1 * n + j] = (j >= k0 && j < k0 + bw) ? zero<T>() : M[(long long)Rs[c1] * n + j];
  }
  for (int i = tid; i < nr; i += CP_NT) us[r0 + i] = (ul[i] == 2) ? 1 : ul[i];
}

template <class T>
__global__ void gje_scatter_rows_kernel(int n, int k0, int bw, T* Mat, const T* H, const int* piv) {
  const long long b = blockIdx.y;
  const long long nn = (long long)n * n;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)bw * n;
       e += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(e / n), j = (int)(e % n);
    if (j >= k0 && j < k0 + bw) continue;
    const int r = piv[b * n + k0 + c];
    Mat[b * nn + (long long)r * n + j] = H[b * (long long)BP * n + (long long)c * n + j];
  }
}

__global__ void gje_rinv_kernel(int n, const int* piv, int* rinv) {
  const long long b = blockIdx.y;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    rinv[b * n + piv[b * n + k]] = k;
}

template <class T>
__global__ void gje_permute_out_kernel(int n, const T* Mat, const int* piv, const int* rinv, T* X,
                                       long long ldx, long long sX) {
  const long long b = blockIdx.y;
  const long long nn = (long long)n * n;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nn;
       e += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(e / n), j = (int)(e % n);
    X[b * sX + (long long)k * ldx + j] =
        Mat[b * nn + (long long)piv[b * n + k] * n + rinv[b * n + j]];
  }
}

// --------------------------------------------------------------------------
// Dispatch
// --------------------------------------------------------------------------
// Shared-memory blocked kernel: chooses RN (= columns per thread / 32) and
// launches when the tableau fits in shared memory.
constexpr size_t SB_SMEM_MAX = 220 * 1024;

// Panel width: 16 columns of 4-byte elements, 8 of 8-byte ones (the panel
// keeps two rows of it in registers, fully unrolled).
template <class T>
constexpr int sb_kb() {
  return sizeof(T) <= 4 ? 16 : 8;
}

template <class T>
static bool sblock_fits(int n) {
  return n > 64 && n <= 256 && inv_sblock_smem<T>(n, sb_kb<T>()) <= SB_SMEM_MAX;
}

template <class T, int RN>
static cudaError_t launch_sblock_rn(int n, const T* A, long long lda, long long sA, T* X, long long ldx, long long sX,
                                    int batch, int* info, cudaStream_t st) {
  const size_t smem = inv_sblock_smem<T>(n, sb_kb<T>());
  cudaFuncSetAttribute(inv_sblock_kernel<T, sb_kb<T>(), RN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const double cplx = (DTypeOf<T>::value == C64 || DTypeOf<T>::value == C128) ? 4.0 : 1.0;
  ProfScope ps(KC_INVERSE, st, 2.0 * cplx * (double)n * n * n * batch);
  note_launch();
  inv_sblock_kernel<T, sb_kb<T>(), RN><<<batch, SB_NT, smem, st>>>(n, A, lda, sA, X, ldx, sX, info);
  return cudaGetLastError();
}

template <class T>
static cudaError_t launch_sblock(int n, const T* A, long long lda, long long sA, T* X, long long ldx, long long sX,
                                 int batch, int* info, cudaStream_t st) {
  if (n <= 128) return launch_sblock_rn<T, 4>(n, A, lda, sA, X, ldx, sX, batch, info, st);
  if (n <= 192) return launch_sblock_rn<T, 6>(n, A, lda, sA, X, ldx, sX, batch, info, st);
  return launch_sblock_rn<T, 8>(n, A, lda, sA, X, ldx, sX, batch, info, st);
}

int inverse_small_nmax(int dtype) {
  switch (dtype) {
    case F32: return 208;
    case F64: return 128;
    case C64: return 128;
    case C128: return 64;
  }
  return 0;
}

// Which inversions of FP32 matrices of 64 < n <= 224 run on the
// tensor-memory Gauss-Jordan kernel (inverse_tc.cu): 0 none, 1 (default) the
// leaf stage's (the callers that pass tensor_memory = true), 2 every one
// (hps_inverse_batched and the merges too; for tests and measurements: the
// tensor core accumulates the update in FP32 with its own rounding, which on
// the merges' interface matrices costs the mixed-precision solve one or two
// refinement steps).  HPS_INVERSE_TC=0 in the environment starts a process
// at 0.
static int g_inverse_tc_policy = -1;

int inverse_tc_policy() {
  if (g_inverse_tc_policy < 0) {
    const char* e = getenv("HPS_INVERSE_TC");
    g_inverse_tc_policy = (e && e[0] == '0') ? 0 : 1;
  }
  return g_inverse_tc_policy;
}

int set_inverse_tc_policy(int policy) {
  const int old = inverse_tc_policy();
  if (policy < 0 || policy > 2) return -1;
  g_inverse_tc_policy = policy;
  return old;
}

static bool inverse_tc_takes(int n, bool tensor_memory) {
  const int p = inverse_tc_policy();
  return inverse_tc_supported(n) && (p == 2 || (p == 1 && tensor_memory));
}

static size_t flat_workspace_bytes(int dtype, int n, int batch) {
  if (n <= inverse_small_nmax(dtype)) return 0;
  if ((dtype == F32 && sblock_fits<float>(n)) || (dtype == F64 && sblock_fits<double>(n)) ||
      (dtype == C64 && sblock_fits<c64>(n)))
    return 0;
  const size_t es = dtype_size(dtype);
  return gje_layout(es, n).per * (size_t)batch + 256;
}

// ---------------------------------------------------------------------------
// Recursive 2 x 2 block inversion (FP32, n >= REC_MIN).  With A split at h1
// into [[A11, A12], [A21, A22]] and the Schur complement S = A22 - A21 W,
// W = A11^-1 A12, V = A21 A11^-1:
//     A^-1 = [[A11^-1 + W S^-1 V, -W S^-1], [-S^-1 V, S^-1]],
// i.e. two half-size inversions (recursively) and six half-size products, all
// batched over the matrices of the call: 2 n^3 flops as Gauss-Jordan, but
// carried by the GEMM kernels instead of n dependent pivot columns.  Pivots
// are searched within the blocks the recursion ends at (n < REC_MIN, the
// Gauss-Jordan kernels), not across them, which suits the interface matrices
// of the DtN merges (their leading blocks are themselves interface operators
// of the same kind); a zero pivot in a block is reported through info with
// the block's column offset.  Used for FP32 while inverse_rec_policy() is 1.
// ---------------------------------------------------------------------------
template <class T>
static cudaError_t inverse_batched_flat(int n, const T* A, long long lda, long long sA, T* X, long long ldx,
                                        long long sX, int batch, int* info, void* ws, size_t ws_bytes,
                                        cudaStream_t st, bool tensor_memory);

// ---------------------------------------------------------------------------
// Block Gauss-Jordan inversion of one FP32 matrix per CTA, n <= 128, for the
// interface blocks the recursive inversion ends at (and the n <= 128 merge
// interfaces).  The matrix lives in registers (thread (ty, tx) of a 16 x 32
// grid owns rows ty + 16 a, columns tx + 32 c); each of the n / 16 steps
// publishes the 16-wide column and row blocks to shared memory, one warp
// inverts the 16 x 16 diagonal block in registers (Gauss-Jordan with partial
// pivoting inside the block, a column of [M_kk | I] per lane), the CTA forms
// the new row block R = P M_k. and every thread updates its elements as an
// outer product:
//     M_ij -= M_ik R_kj,  M_kj = R_kj,  M_ik = -M_ik P,  M_kk = P.
// Pivots are searched within the 16 x 16 blocks only (as in the recursion
// above); a zero pivot sets info to its column (1-based).  Six barriers per
// 16 columns where the per-column kernels need one or two per column.
// ---------------------------------------------------------------------------
constexpr int B16_NT = 512, B16_TY = 16, B16_TX = 32, B16_B = 16, B16_NMAX = 128;
constexpr int B16_RM = B16_NMAX / B16_TY, B16_RN = B16_NMAX / B16_TX;   // 8 x 4 elements per thread

__global__ void __launch_bounds__(B16_NT, 1)
inv_block16_kernel(int n, const float* __restrict__ A, long long lda, long long sA, float* X, long long ldx,
                   long long sX, int* info) {
  __shared__ float Cb[B16_NMAX][B16_B + 1];   // the step's column block (old values)
  __shared__ float Rk[B16_B][B16_NMAX + 1];   // the step's row block, then R = P M_k.
  __shared__ float Pk[B16_B][B16_B + 1];      // inverse of the diagonal block
  __shared__ float Ag[1][B16_B][2 * B16_B + 1];   // [M_kk | I] after elimination
  __shared__ int rowof_s[B16_B];
  __shared__ int s_info;
  const long long bb = blockIdx.x;
  const float* Ab = A + bb * sA;
  const int tid = threadIdx.x, ty = tid / B16_TX, tx = tid % B16_TX, lane = tid & 31, warp = tid >> 5;
  float m[B16_RM][B16_RN];
#pragma unroll
  for (int a = 0; a < B16_RM; ++a)
#pragma unroll
    for (int c = 0; c < B16_RN; ++c) {
      const int i = ty + B16_TY * a, j = tx + B16_TX * c;
      m[a][c] = (i < n && j < n) ? Ab[(long long)i * lda + j] : 0.f;
    }
  if (tid == 0) s_info = 0;
  for (int k0 = 0; k0 < n; k0 += B16_B) {
    const int bs = min(B16_B, n - k0);
    // (1) publish the column block and the row block
#pragma unroll
    for (int a = 0; a < B16_RM; ++a)
#pragma unroll
      for (int c = 0; c < B16_RN; ++c) {
        const int i = ty + B16_TY * a, j = tx + B16_TX * c;
        if (i < n && j >= k0 && j < k0 + bs) Cb[i][j - k0] = m[a][c];
        if (j < n && i >= k0 && i < k0 + bs) Rk[i - k0][j] = m[a][c];
      }
    __syncthreads();
    // (2) the diagonal block by Gauss-Jordan on [M_kk | I] in warp 0: lane c
    // holds column c of the 16 x 32 tableau in registers.  Per pivot, lane k
    // scans its column for the largest unused row (the lowest such row on
    // ties, a NaN taken as the largest) and every lane takes the pivot, the
    // column-k factors and the pivot's reciprocal from lane k by shuffles,
    // then eliminates its own column: no block barrier inside the 16 pivots.
    if (warp == 0) {
      float t[B16_B];
#pragma unroll
      for (int r = 0; r < B16_B; ++r) {
        if (lane < B16_B) t[r] = (r < bs && lane < bs) ? Cb[k0 + r][lane] : (r == lane ? 1.f : 0.f);
        else t[r] = (lane - B16_B == r) ? 1.f : 0.f;
      }
      unsigned used = 0;
      unsigned long long rows = 0;   // pivot row of step k in bits 4k .. 4k+3
      int first_zero = -1;
#pragma unroll 1
      for (int k = 0; k < B16_B; ++k) {
        // largest unused |t| of the column, the lowest row on ties, as a
        // tree (each merge keeps its lower half unless the upper is larger)
        float bv[B16_B];
        int bi[B16_B];
#pragma unroll
        for (int r = 0; r < B16_B; ++r) {
          float v = ((used >> r) & 1u) ? -1.f : fabsf(t[r]);
          if (v != v) v = INFINITY;   // a NaN pivot is taken (and poisons the result) rather than skipped
          bv[r] = v;
          bi[r] = r;
        }
#pragma unroll
        for (int w = 1; w < B16_B; w <<= 1)
#pragma unroll
          for (int r = 0; r < B16_B; r += 2 * w)
            if (bv[r + w] > bv[r]) {
              bv[r] = bv[r + w];
              bi[r] = bi[r + w];
            }
        const float best = __shfl_sync(0xffffffffu, bv[0], k);
        const int who = __shfl_sync(0xffffffffu, bi[0], k);
        float f[B16_B];
#pragma unroll
        for (int r = 0; r < B16_B; ++r) f[r] = __shfl_sync(0xffffffffu, t[r], k);
        // t[who] and f[who] by a multiplexer tree on the bits of who
        float mt[B16_B / 2], mf[B16_B / 2];
#pragma unroll
        for (int r = 0; r < B16_B / 2; ++r) {
          mt[r] = (who & 1) ? t[2 * r + 1] : t[2 * r];
          mf[r] = (who & 1) ? f[2 * r + 1] : f[2 * r];
        }
#pragma unroll
        for (int w = 2, bit = 2; w <= B16_B / 2; w <<= 1, bit <<= 1)
#pragma unroll
          for (int r = 0; r < B16_B / 2; r += w) {
            mt[r] = (who & bit) ? mt[r + w / 2] : mt[r];
            mf[r] = (who & bit) ? mf[r + w / 2] : mf[r];
          }
        const float prow = mt[0], fk = mf[0];   // this column's entry in the pivot row; column k's
        const float pinv = (best > 0.f) ? __frcp_rn(fk) : 0.f;
        const float pv = prow * pinv;
#pragma unroll
        for (int r = 0; r < B16_B; ++r) t[r] = (r == who) ? pv : fmaf(-f[r], pv, t[r]);
        used |= 1u << who;
        rows |= (unsigned long long)who << (4 * k);
        if (first_zero < 0 && !(best > 0.f) && k < bs) first_zero = k;
      }
      if (lane < B16_B) rowof_s[lane] = (int)((rows >> (4 * lane)) & 15ull);
      if (lane == 0 && first_zero >= 0 && s_info == 0) s_info = k0 + first_zero + 1;
#pragma unroll
      for (int r = 0; r < B16_B; ++r) Ag[0][r][lane] = t[r];
    }
    __syncthreads();
    {
      // the pivot row of column k holds row k of the inverse
      const int r = tid >> 5, c = tid & 31;
      if (r < bs && c < bs) Pk[r][c] = Ag[0][rowof_s[r]][B16_B + c];
    }
    __syncthreads();
    // (3) R = P M_k. into registers of the threads that own those columns:
    // thread (ty, tx) forms R[ty][j] for its columns j (bs <= 16 rows)
    float r_new[B16_RN];
    {
      float prow[B16_B];
#pragma unroll
      for (int d = 0; d < B16_B; ++d) prow[d] = (ty < bs && d < bs) ? Pk[ty][d] : 0.f;
#pragma unroll
      for (int c = 0; c < B16_RN; ++c) {
        const int j = tx + B16_TX * c;
        float acc = 0.f;
        if (ty < bs && j < n) {
#pragma unroll
          for (int d = 0; d < B16_B; ++d)
            if (d < bs) acc = fmaf(prow[d], Rk[d][j], acc);
        }
        r_new[c] = acc;
      }
    }
    __syncthreads();
#pragma unroll
    for (int c = 0; c < B16_RN; ++c) {
      const int j = tx + B16_TX * c;
      if (ty < bs && j < n) Rk[ty][j] = r_new[c];
    }
    __syncthreads();
    // (4) every element as an outer-product update from the snapshots in
    // shared memory: per d, the 8 column-block values of this thread's rows
    // and the 4 values of the new row block (or of P, in the block's own
    // columns) of its columns, each loaded once:
    //     rows outside the block:  M_ij = [j outside] M_ij - sum_d C_id R'_dj
    //     rows inside the block:   M_ij = R'_(i-k0) j
    // with R' = R outside the block's columns and P inside them.
#pragma unroll
    for (int a = 0; a < B16_RM; ++a) {
      const int i = ty + B16_TY * a;
      const bool ib = i >= k0 && i < k0 + bs;
#pragma unroll
      for (int c = 0; c < B16_RN; ++c) {
        const int j = tx + B16_TX * c;
        if (ib || (j >= k0 && j < k0 + bs)) m[a][c] = 0.f;
      }
    }
#pragma unroll
    for (int d = 0; d < B16_B; ++d) {
      if (d >= bs) break;
      float cv[B16_RM], rv[B16_RN];
#pragma unroll
      for (int a = 0; a < B16_RM; ++a) {
        const int i = ty + B16_TY * a;
        cv[a] = (i < n && !(i >= k0 && i < k0 + bs)) ? Cb[i][d] : 0.f;
      }
#pragma unroll
      for (int c = 0; c < B16_RN; ++c) {
        const int j = tx + B16_TX * c;
        rv[c] = (j >= n) ? 0.f : (j >= k0 && j < k0 + bs) ? Pk[d][j - k0] : Rk[d][j];
      }
#pragma unroll
      for (int a = 0; a < B16_RM; ++a)
#pragma unroll
        for (int c = 0; c < B16_RN; ++c) m[a][c] = fmaf(-cv[a], rv[c], m[a][c]);
    }
#pragma unroll
    for (int a = 0; a < B16_RM; ++a) {
      const int i = ty + B16_TY * a;
      if (!(i >= k0 && i < k0 + bs)) continue;
#pragma unroll
      for (int c = 0; c < B16_RN; ++c) {
        const int j = tx + B16_TX * c;
        if (j < n) m[a][c] = (j >= k0 && j < k0 + bs) ? Pk[i - k0][j - k0] : Rk[i - k0][j];
      }
    }
    __syncthreads();   // the next step overwrites Cb, Rk and Pk
  }
  if (tid == 0 && info) info[bb] = s_info;
  float* Xb = X + bb * sX;
#pragma unroll
  for (int a = 0; a < B16_RM; ++a)
#pragma unroll
    for (int c = 0; c < B16_RN; ++c) {
      const int i = ty + B16_TY * a, j = tx + B16_TX * c;
      if (i < n && j < n) Xb[(long long)i * ldx + j] = m[a][c];
    }
}

static cudaError_t launch_block16(int n, const float* A, long long lda, long long sA, float* X, long long ldx,
                                  long long sX, int batch, int* info, cudaStream_t st) {
  for (int b0 = 0; b0 < batch; b0 += 1 << 30) {
    const int nb = batch - b0;
    ProfScope ps(KC_INVERSE, st, 2.0 * (double)n * n * n * nb);
    note_launch();
    inv_block16_kernel<<<nb, B16_NT, 0, st>>>(n, A + (long long)b0 * sA, lda, sA, X + (long long)b0 * sX, ldx, sX,
                                              info ? info + b0 : nullptr);
  }
  return cudaGetLastError();
}

constexpr int REC_MIN = 224;
static int g_inverse_rec_policy = -1;

int inverse_rec_policy() {
  if (g_inverse_rec_policy < 0) {
    const char* e = getenv("HPS_INVERSE_RECURSIVE");
    g_inverse_rec_policy = (e && e[0] == '0') ? 0 : 1;
  }
  return g_inverse_rec_policy;
}

int set_inverse_rec_policy(int policy) {
  const int old = inverse_rec_policy();
  if (policy == 0 || policy == 1) g_inverse_rec_policy = policy;
  return old;
}

static int rec_split(int n) { return (n / 2) & ~3; }

// FP32 workspace of the recursion below for (n, batch): W, S, V of this level,
// the block info scratch, then the larger of the two half-size sub-problems.
static size_t rec_workspace_bytes(int n, int batch) {
  if (n < REC_MIN) return al256(sizeof(int) * (size_t)batch) + flat_workspace_bytes(F32, n, batch);
  const int h1 = rec_split(n), h2 = n - h1;
  const size_t lvl = al256(sizeof(float) * (size_t)batch * ((size_t)h1 * h2 + (size_t)h2 * h2 + (size_t)h2 * h1)) +
                     al256(sizeof(int) * (size_t)batch);
  const size_t a = rec_workspace_bytes(h1, batch), b = rec_workspace_bytes(h2, batch);
  return lvl + (a > b ? a : b) + 256;
}

size_t inverse_workspace_bytes(int dtype, int n, int batch) {
  const size_t flat = flat_workspace_bytes(dtype, n, batch);
  if (dtype != F32 || n < REC_MIN) return flat;
  const size_t rec = rec_workspace_bytes(n, batch);
  return rec > flat ? rec : flat;
}

// info[b] = tmp[b] (+ column offset for a zero pivot) where info[b] is still 0
__global__ void info_merge_kernel(int batch, const int* __restrict__ tmp, int* info, int offset) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < batch && info[b] == 0 && tmp[b] != 0) info[b] = tmp[b] > 0 ? tmp[b] + offset : tmp[b];
}

static cudaError_t info_merge(int batch, const int* tmp, int* info, int offset, cudaStream_t st) {
  note_launch();
  info_merge_kernel<<<(batch + 255) / 256, 256, 0, st>>>(batch, tmp, info, offset);
  return cudaGetLastError();
}

// X = A^-1 for a batch of FP32 matrices (X may alias A with ldx == lda, sX == sA);
// info[b] receives the first zero pivot (1-based, in A's columns) or -1.
static cudaError_t inverse_rec_f32(int n, const float* A, long long lda, long long sA, float* X, long long ldx,
                                   long long sX, int batch, int* info, unsigned char* ws, size_t ws_bytes,
                                   int col0, cudaStream_t st) {
  if (n < REC_MIN) {
    // a block the recursion ends at: block Gauss-Jordan (n <= 128) or the
    // pivoted per-column kernels; info via scratch
    int* tinfo = reinterpret_cast<int*>(ws);
    const size_t ib = al256(sizeof(int) * (size_t)batch);
    cudaError_t e = (n <= B16_NMAX)
                        ? launch_block16(n, A, lda, sA, X, ldx, sX, batch, info ? tinfo : nullptr, st)
                        : inverse_batched_flat<float>(n, A, lda, sA, X, ldx, sX, batch, info ? tinfo : nullptr,
                                                      ws + ib, ws_bytes - ib, st, false);
    if (e != cudaSuccess || !info) return e;
    return info_merge(batch, tinfo, info, col0, st);
  }
  const int h1 = rec_split(n), h2 = n - h1;
  const long long sW = (long long)h1 * h2, sS = (long long)h2 * h2, sV = (long long)h2 * h1;
  float* W = reinterpret_cast<float*>(ws);
  float* S = W + sW * batch;
  float* V = S + sS * batch;
  const size_t lvl = al256(sizeof(float) * (size_t)batch * (size_t)(sW + sS + sV)) + al256(sizeof(int) * (size_t)batch);
  unsigned char* sub = ws + lvl;
  const size_t sub_bytes = ws_bytes - lvl;
  const float* A12 = A + h1;
  const float* A21 = A + (long long)h1 * lda;
  const float* A22 = A21 + h1;
  float* X11 = X;
  float* X12 = X + h1;
  float* X21 = X + (long long)h1 * ldx;
  float* X22 = X21 + h1;
  cudaError_t e;
  // X11 = A11^-1
  if ((e = inverse_rec_f32(h1, A, lda, sA, X11, ldx, sX, batch, info, sub, sub_bytes, col0, st)) != cudaSuccess) return e;
  // W = X11 A12;  S = A22 - A21 W
  if ((e = gemm_batched<float>(h1, h2, h1, 1.f, X11, ldx, sX, A12, lda, sA, 0.f, nullptr, 0, 0, W, h2, sW, batch,
                               st)) != cudaSuccess) return e;
  if ((e = gemm_batched<float>(h2, h2, h1, -1.f, A21, lda, sA, W, h2, sW, 1.f, A22, lda, sA, S, h2, sS, batch,
                               st)) != cudaSuccess) return e;
  // V = A21 X11 (before X21 overwrites A21 when X aliases A)
  if ((e = gemm_batched<float>(h2, h1, h1, 1.f, A21, lda, sA, X11, ldx, sX, 0.f, nullptr, 0, 0, V, h1, sV, batch,
                               st)) != cudaSuccess) return e;
  // X22 = S^-1
  if ((e = inverse_rec_f32(h2, S, h2, sS, X22, ldx, sX, batch, info, sub, sub_bytes, col0 + h1, st)) != cudaSuccess)
    return e;
  // X12 = -W X22;  X21 = -X22 V;  X11 -= X12 V
  if ((e = gemm_batched<float>(h1, h2, h2, -1.f, W, h2, sW, X22, ldx, sX, 0.f, nullptr, 0, 0, X12, ldx, sX, batch,
                               st)) != cudaSuccess) return e;
  if ((e = gemm_batched<float>(h2, h1, h2, -1.f, X22, ldx, sX, V, h1, sV, 0.f, nullptr, 0, 0, X21, ldx, sX, batch,
                               st)) != cudaSuccess) return e;
  return gemm_batched<float>(h1, h1, h2, -1.f, X12, ldx, sX, V, h1, sV, 1.f, X11, ldx, sX, X11, ldx, sX, batch, st);
}

template <class T>
cudaError_t inverse_batched(int n, const T* A, long long lda, long long sA, T* X, long long ldx,
                            long long sX, int batch, int* info, void* ws, size_t ws_bytes,
                            cudaStream_t st, int flags) {
  const bool tensor_memory = (flags & INV_TENSOR_MEMORY) != 0;
  if constexpr (DTypeOf<T>::value == F32) {
    // interface matrices of 64 < n <= 128: one block Gauss-Jordan CTA each
    // (measured: below 64 the per-column register kernel is as fast)
    if ((flags & INV_BLOCK_RECURSIVE) && n > 64 && n <= B16_NMAX && batch > 0 && inverse_rec_policy() == 1 &&
        !inverse_tc_takes(n, tensor_memory)) {
      ProfScope whole(KC_INVERSE, st, 2.0 * (double)n * n * n * batch);
      return launch_block16(n, (const float*)A, lda, sA, (float*)X, ldx, sX, batch, info, st);
    }
    if ((flags & INV_BLOCK_RECURSIVE) && n >= REC_MIN && batch > 0 && inverse_rec_policy() == 1 &&
        !inverse_tc_takes(n, tensor_memory)) {
      const size_t need = rec_workspace_bytes(n, batch);
      if (ws == nullptr || ws_bytes < need) {
        set_error("inverse: workspace too small (%zu < %zu)", ws_bytes, need);
        return cudaErrorInvalidValue;
      }
      ProfScope whole(KC_INVERSE, st, 2.0 * (double)n * n * n * batch);
      if (info) cudaMemsetAsync(info, 0, sizeof(int) * (size_t)batch, st);
      unsigned char* base = reinterpret_cast<unsigned char*>(
          (reinterpret_cast<uintptr_t>(ws) + 255) & ~uintptr_t(255));
      return inverse_rec_f32(n, (const float*)A, lda, sA, (float*)X, ldx, sX, batch, info, base,
                             ws_bytes - (size_t)(base - reinterpret_cast<unsigned char*>(ws)), 0, st);
    }
  }
  return inverse_batched_flat<T>(n, A, lda, sA, X, ldx, sX, batch, info, ws, ws_bytes, st, tensor_memory);
}

template <class T, int NMAX>
static cudaError_t launch_reg(int n, const T* A, long long lda, long long sA, T* X, long long ldx,
                             long long sX, int batch, int* info, cudaStream_t st) {
  for (int b0 = 0; b0 < batch; b0 += 1 << 30) {
    const int nb = batch - b0;
    const double cplx = (DTypeOf<T>::value == C64 || DTypeOf<T>::value == C128) ? 4.0 : 1.0;
    ProfScope ps(KC_INVERSE, st, 2.0 * cplx * (double)n * n * n * nb);
    note_launch();
    inv_reg_kernel<T, NMAX><<<nb, 512, 0, st>>>(n, A + (long long)b0 * sA, lda, sA,
                                                X + (long long)b0 * sX, ldx, sX,
                                                info ? info + b0 : nullptr);
  }
  return cudaGetLastError();
}

template <class T>
static cudaError_t inverse_small(int n, const T* A, long long lda, long long sA, T* X, long long ldx,
                                 long long sX, int batch, int* info, cudaStream_t st);

template <>
cudaError_t inverse_small<float>(int n, const float* A, long long lda, long long sA, float* X,
                                 long long ldx, long long sX, int batch, int* info, cudaStream_t st) {
  if (n <= 32) return launch_reg<float, 32>(n, A, lda, sA, X, ldx, sX, batch, info, st);
  if (n <= 64) return launch_reg<float, 64>(n, A, lda, sA, X, ldx, sX, batch, info, st);
  if (n <= 128) return launch_reg<float, 128>(n, A, lda, sA, X, ldx, sX, batch, info, st);
  return launch_reg<float, 208>(n, A, lda, sA, X, ldx, sX, batch, info, st);
}
template <>
cudaError_t inverse_small<double>(int n, const double* A, long long lda, long long sA, double* X,
                                  long long ldx, long long sX, int batch, int* info, cudaStream_t st) {
  if (n <= 32) return launch_reg<double, 32>(n, A, lda, sA, X, ldx, sX, batch, info, st);
  if (n <= 64) return launch_reg<double, 64>(n, A, lda, sA, X, ldx, sX, batch, info, st);
  return launch_reg<double, 128>(n, A, lda, sA, X, ldx, sX, batch, info, st);
}
template <>
cudaError_t inverse_small<c64>(int n, const c64* A, long long lda, long long sA, c64* X,
                               long long ldx, long long sX, int batch, int* info, cudaStream_t st) {
  if (n <= 32) return launch_reg<c64, 32>(n, A, lda, sA, X, ldx, sX, batch, info, st);
  if (n <= 64) return launch_reg<c64, 64>(n, A, lda, sA, X, ldx, sX, batch, info, st);
  return launch_reg<c64, 128>(n, A, lda, sA, X, ldx, sX, batch, info, st);
}
template <>
cudaError_t inverse_small<c128>(int n, const c128* A, long long lda, long long sA, c128* X,
                                long long ldx, long long sX, int batch, int* info, cudaStream_t st) {
  if (n <= 32) return launch_reg<c128, 32>(n, A, lda, sA, X, ldx, sX, batch, info, st);
  return launch_reg<c128, 64>(n, A, lda, sA, X, ldx, sX, batch, info, st);
}

template <class T>
static cudaError_t inverse_batched_flat(int n, const T* A, long long lda, long long sA, T* X, long long ldx,
                                        long long sX, int batch, int* info, void* ws, size_t ws_bytes,
                                        cudaStream_t st, bool tensor_memory) {
  if (n <= 0 || batch <= 0) return cudaSuccess;
  // one profiler record for the whole inversion (its panel kernels and the
  // GEMM updates nested below): 2 n^3 flops per matrix, x4 for complex
  const double cplx = (sizeof(T) == 16 || DTypeOf<T>::value == C64) ? 4.0 : 1.0;
  const bool on_tc = DTypeOf<T>::value == F32 && inverse_tc_takes(n, tensor_memory);
  ProfScope whole(on_tc ? KC_INVERSE_TC : KC_INVERSE, st, 2.0 * cplx * (double)n * n * n * batch);
  if (info) cudaMemsetAsync(info, 0, sizeof(int) * (size_t)batch, st);
  const int dtype = DTypeOf<T>::value;
  if constexpr (DTypeOf<T>::value == F32) {
    if (on_tc)
      return inverse_tc_f32(n, (const float*)A, lda, sA, (float*)X, ldx, sX, batch, info, st);
  }
  if constexpr (sizeof(T) <= 8) {
    if (sblock_fits<T>(n)) return launch_sblock<T>(n, A, lda, sA, X, ldx, sX, batch, info, st);
  }
  if (n <= inverse_small_nmax(dtype)) return inverse_small<T>(n, A, lda, sA, X, ldx, sX, batch, info, st);

  const size_t es = sizeof(T);
  const GjeWs L = gje_layout(es, n);
  if (ws == nullptr || ws_bytes < L.per * (size_t)batch) {
    set_error("inverse: workspace too small (%zu < %zu)", ws_bytes, L.per * (size_t)batch);
    return cudaErrorInvalidValue;
  }
  unsigned char* base = reinterpret_cast<unsigned char*>(ws);
  base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(base) + 255) & ~uintptr_t(255));
  T* Mat = reinterpret_cast<T*>(base);
  base += L.mat * batch;
  T* Pw = reinterpret_cast<T*>(base);
  base += L.pan * batch;
  T* U = reinterpret_cast<T*>(base);
  base += L.u * batch;
  T* G = reinterpret_cast<T*>(base);
  base += L.g * batch;
  T* H = reinterpret_cast<T*>(base);
  base += L.h * batch;
  T* E = reinterpret_cast<T*>(base);
  base += L.e * batch;
  int* piv = reinterpret_cast<int*>(base);
  base += L.piv * batch;
  int* rinv = reinterpret_cast<int*>(base);
  base += L.rinv * batch;
  unsigned char* used = base;
  base += L.used * batch;
  unsigned char* syncb = base;

  // Few matrices: split each panel over several CTAs (cooperative launch).
  int nct = 0, rows_per = 0;
  size_t csmem = 0;
  {
    int dev = 0, sms = 0, coop_ok = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&coop_ok, cudaDevAttrCooperativeLaunch, dev);
    if (coop_ok && sms > 0 && batch < sms && n > 64) {
      nct = 2 * sms / batch;
      if (nct > coop_nct_cap(n)) nct = coop_nct_cap(n);
      bool fits = false;
      for (int iter = 0; iter < 6 && nct >= 2; ++iter) {
        rows_per = (n + nct - 1) / nct;
        nct = (n + rows_per - 1) / rows_per;
        csmem = es * ((size_t)BP * rows_per + rows_per) + (size_t)rows_per + 16;
        if (csmem > 200 * 1024) break;
        cudaFuncSetAttribute(gje_panel_coop_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)csmem);
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gje_panel_coop_kernel<T>, CP_NT, csmem);
        if ((long long)per_sm * sms >= (long long)nct * batch) {
          fits = true;
          break;
        }
        nct = per_sm * sms / batch;
      }
      if (!fits || nct < 2) nct = 0;
      cudaGetLastError();   // a refused attribute or occupancy query only disables this path
    }
  }
  // Prefer one thread-block cluster per matrix (hardware barrier): up to 16
  // CTAs, each holding rows_per rows of the panel in shared memory.
  int ncl = 0, rows_cl = 0;
  size_t clsmem = 0;
  if (nct > 0 && cluster_panels_enabled()) {
    for (int want : {16, 8}) {
      if (want > (coop_nct_cap(n) > 16 ? coop_nct_cap(n) : 16)) continue;
      const int rp = (n + want - 1) / want;
      const int nc = (n + rp - 1) / rp;
      const size_t sm = es * (size_t)BP * rp + (size_t)rp + 16;
      if (sm > 200 * 1024 || nc < 2) continue;
      auto kern = gje_panel_cluster_kernel<T>;
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      if (nc > 8) cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(nc, batch);
      cfg.blockDim = dim3(CP_NT);
      cfg.dynamicSmemBytes = sm;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = nc;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      int max_cl = 0;
      if (cudaOccupancyMaxActiveClusters(&max_cl, kern, &cfg) == cudaSuccess && max_cl >= 1) {
        ncl = nc;
        rows_cl = rp;
        clsmem = sm;
        break;
      }
    }
    cudaGetLastError();   // a refused attribute or occupancy query only disables this path
  }
  if (ncl > 0) {
    nct = ncl;
    rows_per = rows_cl;
    csmem = clsmem;
  }
  const CoopLayout clay = coop_layout(es, sizeof(typename MagOf<T>::type), nct > 0 ? nct : 1);
  if (nct > 0) {
    cudaError_t e = cudaMemsetAsync(syncb, 0, clay.per * (size_t)batch, st);
    if (e != cudaSuccess) return e;
  }

  const long long nn = (long long)n * n;
  for (int b0 = 0; b0 < batch; b0 += 65535) {
    const int nb = (batch - b0) < 65535 ? (batch - b0) : 65535;
    int gx = (int)((nn + 255) / 256);
    if (gx > 1024) gx = 1024;
    note_launch();
    gje_copy_in_kernel<T><<<dim3(gx, nb), 256, 0, st>>>(n, A + (long long)b0 * sA, lda, sA,
                                                        Mat + (long long)b0 * nn, used + (long long)b0 * n,
                                                        piv + (long long)b0 * n, rinv + (long long)b0 * n);
  }
  // Panel width: the widest of 32/16/8/4 whose panel fits in shared memory;
  // wider panels mean fewer (rank-bw) trailing GEMM updates.
  int bwmax = BP;
  int use_smem = 0;
  size_t pan_smem = 0;
  if (nct == 0) {
    while (bwmax > 4 && es * (size_t)n * bwmax > 200 * 1024) bwmax /= 2;
    pan_smem = es * (size_t)n * bwmax;
    use_smem = pan_smem <= 200 * 1024;
    if (!use_smem) bwmax = BP;
    if (use_smem)
      cudaFuncSetAttribute(gje_panel_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pan_smem);
  }
  const T one_ = one<T>();
  for (int k0 = 0; k0 < n; k0 += bwmax) {
    int bw = (n - k0) < bwmax ? (n - k0) : bwmax;
    ProfScope ps(KC_INVERSE, st, 2.0 * (double)n * bw * bw * batch);
    note_launch();
    cudaError_t e;
    if (nct > 0) {
      int n_ = n, k0_ = k0, rp = rows_per;
      T *Mat_ = Mat, *U_ = U, *G_ = G, *E_ = E;
      int* piv_ = piv;
      unsigned char* used_ = used;
      int* info_ = info;
      unsigned char* sync_ = syncb;
      CoopLayout lay_ = clay;
      if (ncl > 0) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(nct, batch);
        cfg.blockDim = dim3(CP_NT);
        cfg.dynamicSmemBytes = csmem;
        cfg.stream = st;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = nct;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        e = cudaLaunchKernelEx(&cfg, gje_panel_cluster_kernel<T>, n_, k0_, bw, rp, Mat_, U_, G_, E_, piv_, used_,
                               info_);
      } else {
        void* args[] = {&n_, &k0_, &bw, &rp, &Mat_, &U_, &G_, &E_, &piv_, &used_, &info_, &sync_, &lay_};
        e = cudaLaunchCooperativeKernel((void*)gje_panel_coop_kernel<T>, dim3(nct, batch), dim3(CP_NT), args,
                                        csmem, st);
      }
    } else {
      const int pnt = n >= PANEL_NT ? PANEL_NT : ((n + 31) / 32) * 32;
      gje_panel_kernel<T><<<batch, pnt, use_smem ? pan_smem : 0, st>>>(n, k0, bw, Mat, Pw, use_smem, U, G, E, piv,
                                                                       used, info);
      e = cudaGetLastError();
    }
    if (e != cudaSuccess) return e;
    // H = E G
    e = gemm_batched<T>(bw, n, bw, one_, E, BP, BP * BP, G, n, (long long)BP * n, zero<T>(), nullptr, 0,
                        0, H, n, (long long)BP * n, batch, st);
    if (e != cudaSuccess) return e;
    // Mat += U G
    e = gemm_batched<T>(n, n, bw, one_, U, BP, (long long)n * BP, G, n, (long long)BP * n, one_, Mat, n,
                        nn, Mat, n, nn, batch, st);
    if (e != cudaSuccess) return e;
    for (int b0 = 0; b0 < batch; b0 += 65535) {
      const int nb = (batch - b0) < 65535 ? (batch - b0) : 65535;
      int gx = (bw * n + 255) / 256;
      note_launch();
      gje_scatter_rows_kernel<T><<<dim3(gx, nb), 256, 0, st>>>(
          n, k0, bw, Mat + (long long)b0 * nn, H + (long long)b0 * BP * n, piv + (long long)b0 * n);
    }
  }
  for (int b0 = 0; b0 < batch; b0 += 65535) {
    const int nb = (batch - b0) < 65535 ? (batch - b0) : 65535;
    note_launch();
    gje_rinv_kernel<<<dim3((n + 255) / 256, nb), 256, 0, st>>>(n, piv + (long long)b0 * n,
                                                               rinv + (long long)b0 * n);
    int gx = (int)((nn + 255) / 256);
    if (gx > 2048) gx = 2048;
    note_launch();
    gje_permute_out_kernel<T><<<dim3(gx, nb), 256, 0, st>>>(
        n, Mat + (long long)b0 * nn, piv + (long long)b0 * n, rinv + (long long)b0 * n,
        X + (long long)b0 * sX, ldx, sX);
  }
  return cudaGetLastError();
}

cudaError_t set_panel_spin_limit(long long polls, long long* previous) {
  long long old = 0;
  cudaError_t e = cudaMemcpyFromSymbol(&old, g_cp_spin_limit, sizeof(old));
  if (e != cudaSuccess) return e;
  if (previous) *previous = old;
  if (polls >= 0) e = cudaMemcpyToSymbol(g_cp_spin_limit, &polls, sizeof(polls));
  return e;
}

#define HPS_INST_INV(T)                                                                       \
  template cudaError_t inverse_batched<T>(int, const T*, long long, long long, T*, long long, \
                                          long long, int, int*, void*, size_t, cudaStream_t, int);
HPS_INST_INV(float)
HPS_INST_INV(double)
HPS_INST_INV(c64)
HPS_INST_INV(c128)

}  // namespace hps
