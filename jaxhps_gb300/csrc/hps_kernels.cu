// HPS data-movement kernels: leaf operator assembly, merge block gather
// and down-pass scatter.  The index bookkeeping of the reference (child
// side orderings, interface flips, the exterior roll after a merge) is
// precomputed on the host as small integer maps and applied here, so one
// kernel serves 2D quad merges and 3D oct merges alike.
#include <type_traits>

#include "hps_common.cuh"
#include "hps_internal.h"
#include "../../include/jaxhps_gb300.h"

namespace hps {

// ---------------------------------------------------------------------------
// Leaf operator assembly  (reference: local_solve/_uniform_2D_DtN.py:182-225)
//
// For interior row i (global row row0+i) of every leaf l:
//   A[l][row0+i][j] = sum_o coeff[o][l][row0+i] * ops[o][row0+i][j]
// Columns j < col_split go to out_lo[l][i][j], the rest to
// out_hi[l][i][j-col_split].  One CTA per (row, leaf group); the operator
// rows are staged in shared memory once and reused for the whole group.
//
// FP32 / complex64 output with real FP64 coefficients (the mixed-precision
// builds): the sum is formed in double-float arithmetic on the FP32 pipe
// (operands split into FP32 pairs once, while staging; TwoProd by FMA and
// TwoSum per term, relative error below 2^-44) and rounded to FP32, which is
// the FP64 sum rounded to FP32 except within 2^-44 of a rounding tie.  GB300
// runs FP64 at 1/64 of the FP32 rate, so the FP64 form of this kernel was
// bound by its 4 FP64 operations per element, not by its stores.
// ---------------------------------------------------------------------------
template <class T, class CT>
__host__ __device__ constexpr bool assemble_in_pairs() {
  return (std::is_same<T, float>::value || std::is_same<T, c64>::value) && std::is_same<CT, double>::value;
}

__device__ __forceinline__ float2 split_pair(double x) {
  const float h = __double2float_rn(x);
  return make_float2(h, __double2float_rn(x - (double)h));
}

template <class T, class CT>
__global__ void leaf_assemble_kernel(int n_leaves, int n_pts, int row0, int col_split, int n_ops,
                                     const double* __restrict__ ops, const CT* __restrict__ coeffs,
                                     T* out_lo, long long ld_lo, long long s_lo, T* out_hi,
                                     long long ld_hi, long long s_hi, int leaves_per_cta, int l_base,
                                     int staged) {
  extern __shared__ double ds_smem[];  // [n_ops][n_pts] when staged
  const int i = blockIdx.x;
  const int row = row0 + i;
  if constexpr (assemble_in_pairs<T, CT>()) {
    if (staged) {
      float2* dp = reinterpret_cast<float2*>(ds_smem);   // operator rows as pairs, [n_ops][n_pts]
      float2* cp = dp + (size_t)n_ops * n_pts;            // coefficient pairs, [leaf in group][n_ops]
      int* nzc = reinterpret_cast<int*>(cp + (size_t)leaves_per_cta * n_ops);   // nonzero columns
      unsigned char* nzf = reinterpret_cast<unsigned char*>(nzc + n_pts);        // column flags
      __shared__ int nnz_s;
      const int l0 = l_base + blockIdx.y * leaves_per_cta;
      const int l1 = min(n_leaves, l0 + leaves_per_cta);
      if (threadIdx.x == 0) nnz_s = 0;
      for (int e = threadIdx.x; e < n_ops * n_pts; e += blockDim.x) {
        const int o = e / n_pts, j = e % n_pts;
        dp[e] = split_pair(ops[((long long)o * n_pts + row) * n_pts + j]);
      }
      for (int e = threadIdx.x; e < (l1 - l0) * n_ops; e += blockDim.x) {
        const int ll = e / n_ops, o = e % n_ops;
        cp[e] = split_pair(coeffs[((long long)o * n_leaves + l0 + ll) * n_pts + row]);
      }
      __syncthreads();
      // The operators are differentiation matrices on a tensor grid: a row of
      // D_xx or D_yy is nonzero only on the row's own grid lines, so most
      // entries of the sum are exact zeros.  Those are stored directly; the
      // nonzero columns (a zero FP32 head means a zero pair) are listed once
      // and their sums spread over all threads of the CTA.
      for (int j = threadIdx.x; j < n_pts; j += blockDim.x) {
        bool nz = false;
        for (int o = 0; o < n_ops; ++o) nz |= dp[o * n_pts + j].x != 0.f;
        nzf[j] = nz;
        if (nz) nzc[atomicAdd(&nnz_s, 1)] = j;
      }
      __syncthreads();
      const int nnz = nnz_s;
      auto store = [&](int l, int j, float r) {
        T v;
        if constexpr (std::is_same<T, float>::value) v = r;
        else v = c64{r, 0.f};
        if (j < col_split) out_lo[l * s_lo + (long long)i * ld_lo + j] = v;
        else out_hi[l * s_hi + (long long)i * ld_hi + (j - col_split)] = v;
      };
      for (int l = l0; l < l1; ++l)
        for (int j = threadIdx.x; j < n_pts; j += blockDim.x)
          if (!nzf[j]) store(l, j, 0.f);
      for (int w = threadIdx.x; w < (l1 - l0) * nnz; w += blockDim.x) {
        const int ll = w / nnz, j = nzc[w - ll * nnz];
        const float2* cl = cp + (size_t)ll * n_ops;
        float sh = 0.f, se = 0.f;
        for (int o = 0; o < n_ops; ++o) {
          const float2 c = cl[o], d = dp[o * n_pts + j];
          const float pr = c.x * d.x;
          float pe = fmaf(c.x, d.x, -pr);
          pe = fmaf(c.x, d.y, pe);
          pe = fmaf(c.y, d.x, pe);
          const float t = sh + pr;
          const float bb = t - sh;
          const float err = (sh - (t - bb)) + (pr - bb);
          sh = t;
          se += err + pe;
        }
        store(l0 + ll, j, sh + se);
      }
      return;
    }
  }
  const double* ds;
  long long ds_ld;   // stride between operators
  if (staged) {
    for (int e = threadIdx.x; e < n_ops * n_pts; e += blockDim.x) {
      const int o = e / n_pts, j = e % n_pts;
      ds_smem[e] = ops[((long long)o * n_pts + row) * n_pts + j];
    }
    __syncthreads();
    ds = ds_smem;
    ds_ld = n_pts;
  } else {
    // rows too long for shared memory (large 3D leaves): read them from L2
    ds = ops + (long long)row * n_pts;
    ds_ld = (long long)n_pts * n_pts;
  }
  const int l0 = l_base + blockIdx.y * leaves_per_cta;
  const int l1 = min(n_leaves, l0 + leaves_per_cta);
  for (int l = l0; l < l1; ++l) {
    for (int j = threadIdx.x; j < n_pts; j += blockDim.x) {
      CT acc;
      if constexpr (sizeof(CT) == 8) {
        acc = 0.0;
        for (int o = 0; o < n_ops; ++o)
          acc = fma(coeffs[((long long)o * n_leaves + l) * n_pts + row], ds[o * ds_ld + j], acc);
      } else {
        acc = c128{0.0, 0.0};
        for (int o = 0; o < n_ops; ++o) {
          const CT c = coeffs[((long long)o * n_leaves + l) * n_pts + row];
          const double d = ds[o * ds_ld + j];
          acc.x = fma(c.x, d, acc.x);
          acc.y = fma(c.y, d, acc.y);
        }
      }
      T v;
      if constexpr (sizeof(CT) == 8) v = from_real<T>(acc);
      else v = from_c128<T>(acc);
      if (j < col_split) out_lo[l * s_lo + (long long)i * ld_lo + j] = v;
      else out_hi[l * s_hi + (long long)i * ld_hi + (j - col_split)] = v;
    }
  }
}

template <class T, class CT>
cudaError_t leaf_assemble(int n_leaves, int n_pts, int row0, int n_rows, int col_split, int n_ops,
                          const double* ops, const CT* coeffs, T* out_lo, long long ld_lo, long long s_lo,
                          T* out_hi, long long ld_hi, long long s_hi, cudaStream_t st) {
  const int lpc = 32;
  size_t smem = sizeof(double) * (size_t)n_ops * n_pts;
  // coefficient pairs, the nonzero-column list and the column flags
  if (assemble_in_pairs<T, CT>()) smem += sizeof(float2) * (size_t)lpc * n_ops + (sizeof(int) + 1) * (size_t)n_pts;
  const int staged = smem <= 200 * 1024;
  if (!staged) smem = 0;
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(leaf_assemble_kernel<T, CT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
  const int gy = (n_leaves + lpc - 1) / lpc;
  for (int y0 = 0; y0 < gy; y0 += 65535) {
    const int ny = gy - y0 < 65535 ? gy - y0 : 65535;
    dim3 grid(n_rows, ny);
    ProfScope ps(KC_MOVE, st, (double)sizeof(T) * n_rows * (double)n_pts * (ny * lpc < n_leaves - y0 * lpc ? ny * lpc : n_leaves - y0 * lpc));
    note_launch();
    leaf_assemble_kernel<T, CT><<<grid, 256, smem, st>>>(n_leaves, n_pts, row0, col_split, n_ops, ops, coeffs,
                                                         out_lo, ld_lo, s_lo, out_hi, ld_hi, s_hi, lpc,
                                                         y0 * lpc, staged);
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// dst[b][r][c] = src[r][c] (or 0 when src is null) for r < rows, c < cols.
// Used for the Chebyshev-boundary rows of Y (= P) and of v (= 0).
// ---------------------------------------------------------------------------
template <class T>
__global__ void set_rows_kernel(int rows, int cols, const T* src, long long lds, T* dst, long long ldd,
                                long long sd) {
  const long long b = blockIdx.y;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < rows * cols; e += gridDim.x * blockDim.x) {
    const int r = e / cols, c = e % cols;
    dst[b * sd + (long long)r * ldd + c] = src ? src[(long long)r * lds + c] : zero<T>();
  }
}

template <class T>
cudaError_t set_rows(int batch, int rows, int cols, const T* src, long long lds, T* dst, long long ldd,
                     long long sd, cudaStream_t st) {
  if (batch <= 0 || rows <= 0 || cols <= 0) return cudaSuccess;
  int gx = (rows * cols + 255) / 256;
  if (gx > 64) gx = 64;
  for (int b0 = 0; b0 < batch; b0 += 65535) {
    const int nb = batch - b0 < 65535 ? batch - b0 : 65535;
    note_launch();
    set_rows_kernel<T><<<dim3(gx, nb), 256, 0, st>>>(rows, cols, src, lds, dst + b0 * sd, ldd, sd);
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Row equilibration of a batch of square matrices by powers of two.
//   s[b][r] = 2^-e with max_c |A[b][r][c]| = f 2^e, f in [0.5, 1);  A[b][r][:] *= s[b][r]
// and the matching column scaling of the inverse, X[b][:][c] *= s[b][c],
// which turns inv(diag(s) A) into inv(A).  Scaling by powers of two is exact,
// so only the pivot order of the elimination changes: rows whose magnitudes
// differ by orders (the ItI leaf matrix stacks impedance rows ~p^2/h over
// PDE rows ~p^4/h^2) no longer lose the small rows' digits to the large.
// One warp per row.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float scale_by(float v, double s) { return v * (float)s; }
__device__ __forceinline__ double scale_by(double v, double s) { return v * s; }
__device__ __forceinline__ c64 scale_by(c64 v, double s) { return c64{v.x * (float)s, v.y * (float)s}; }
__device__ __forceinline__ c128 scale_by(c128 v, double s) { return c128{v.x * s, v.y * s}; }
__device__ __forceinline__ double absmag(float v) { return fabs((double)v); }
__device__ __forceinline__ double absmag(double v) { return fabs(v); }
__device__ __forceinline__ double absmag(c64 v) { return fmax(fabs((double)v.x), fabs((double)v.y)); }
__device__ __forceinline__ double absmag(c128 v) { return fmax(fabs(v.x), fabs(v.y)); }

template <class T>
__global__ void row_equilibrate_kernel(long long rows_total, int n, T* A, long long lda, long long sA, double* s) {
  const long long row = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= rows_total) return;
  const long long b = row / n;
  const int r = (int)(row % n);
  T* a = A + b * sA + (long long)r * lda;
  double m = 0.0;
  for (int c = lane; c < n; c += 32) m = fmax(m, absmag(a[c]));
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  int e = 0;
  if (m > 0.0 && m <= 1.7e308) frexp(m, &e);
  const double sc = ldexp(1.0, -e);
  for (int c = lane; c < n; c += 32) a[c] = scale_by(a[c], sc);
  if (lane == 0) s[row] = sc;
}

template <class T>
__global__ void col_scale_kernel(int batch, int n, T* X, long long ldx, long long sX, const double* __restrict__ s) {
  const long long total = (long long)batch * n * n;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long b = e / ((long long)n * n);
    const int rc = (int)(e % ((long long)n * n));
    const int r = rc / n, c = rc % n;
    T* x = X + b * sX + (long long)r * ldx + c;
    *x = scale_by(*x, s[b * n + c]);
  }
}

template <class T>
cudaError_t row_equilibrate(int batch, int n, T* A, long long lda, long long sA, double* s, cudaStream_t st) {
  if (batch <= 0 || n <= 0) return cudaSuccess;
  const long long rows = (long long)batch * n;
  const long long g = (rows + 7) / 8;
  ProfScope ps(KC_MOVE, st, 2.0 * (double)rows * n * sizeof(T));
  note_launch();
  row_equilibrate_kernel<T><<<(unsigned)g, 256, 0, st>>>(rows, n, A, lda, sA, s);
  return cudaGetLastError();
}

template <class T>
cudaError_t col_scale(int batch, int n, T* X, long long ldx, long long sX, const double* s, cudaStream_t st) {
  if (batch <= 0 || n <= 0) return cudaSuccess;
  long long g = ((long long)batch * n * n + 255) / 256;
  if (g > 16384) g = 16384;
  ProfScope ps(KC_MOVE, st, 2.0 * (double)batch * n * n * sizeof(T));
  note_launch();
  col_scale_kernel<T><<<(int)g, 256, 0, st>>>(batch, n, X, ldx, sX, s);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Permuted block copies for the two-colour inverse of the ItI merge matrix:
//   gather:  out[b][i][j] = M[b][perm[r0+i]][perm[c0+j]]
//   scatter: M[b][perm[r0+i]][perm[c0+j]] = in[b][i][j] (+1 on i == j)
//   add_identity: X[b][i][i] += 1
// ---------------------------------------------------------------------------
template <class T>
__global__ void perm_gather_kernel(int n, int nr, int nc, const T* __restrict__ M, long long sM,
                                   const int* __restrict__ perm, int r0, int c0, T* out, long long sO) {
  const long long b = blockIdx.y;
  const long long tot = (long long)nr * nc;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e / nc), j = (int)(e % nc);
    out[b * sO + e] = M[b * sM + (long long)perm[r0 + i] * n + perm[c0 + j]];
  }
}

template <class T>
__global__ void perm_scatter_kernel(int n, int nr, int nc, T* M, long long sM, const int* __restrict__ perm, int r0,
                                    int c0, const T* __restrict__ in, long long sI, int add_identity) {
  const long long b = blockIdx.y;
  const long long tot = (long long)nr * nc;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e / nc), j = (int)(e % nc);
    T v = in[b * sI + e];
    if (add_identity && i == j) v = add(v, one<T>());
    M[b * sM + (long long)perm[r0 + i] * n + perm[c0 + j]] = v;
  }
}

template <class T>
__global__ void add_identity_kernel(int n, T* X, long long sX) {
  const long long b = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    X[b * sX + (long long)i * n + i] = add(X[b * sX + (long long)i * n + i], one<T>());
}

static inline int blocks_for(long long work) {
  long long g = (work + 255) / 256;
  return (int)(g < 1 ? 1 : (g > 1024 ? 1024 : g));
}

template <class T>
cudaError_t perm_gather(int batch, int n, int nr, int nc, const T* M, long long sM, const int* perm, int r0, int c0,
                        T* out, long long sO, cudaStream_t st) {
  const int gx = blocks_for((long long)nr * nc);
  for (int b0 = 0; b0 < batch; b0 += 65535) {
    const int nb = batch - b0 < 65535 ? batch - b0 : 65535;
    ProfScope ps(KC_MOVE, st, 2.0 * sizeof(T) * (double)nr * nc * nb);
    note_launch();
    perm_gather_kernel<T><<<dim3(gx, nb), 256, 0, st>>>(n, nr, nc, M + b0 * sM, sM, perm, r0, c0, out + b0 * sO, sO);
  }
  return cudaGetLastError();
}

template <class T>
cudaError_t perm_scatter(int batch, int n, int nr, int nc, T* M, long long sM, const int* perm, int r0, int c0,
                         const T* in, long long sI, int add_identity, cudaStream_t st) {
  const int gx = blocks_for((long long)nr * nc);
  for (int b0 = 0; b0 < batch; b0 += 65535) {
    const int nb = batch - b0 < 65535 ? batch - b0 : 65535;
    ProfScope ps(KC_MOVE, st, 2.0 * sizeof(T) * (double)nr * nc * nb);
    note_launch();
    perm_scatter_kernel<T><<<dim3(gx, nb), 256, 0, st>>>(n, nr, nc, M + b0 * sM, sM, perm, r0, c0, in + b0 * sI, sI,
                                                         add_identity);
  }
  return cudaGetLastError();
}

template <class T>
cudaError_t add_identity(int batch, int n, T* X, long long sX, cudaStream_t st) {
  const int gx = blocks_for(n);
  for (int b0 = 0; b0 < batch; b0 += 65535) {
    const int nb = batch - b0 < 65535 ? batch - b0 : 65535;
    note_launch();
    add_identity_kernel<T><<<dim3(gx, nb), 256, 0, st>>>(n, X + b0 * sX, sX);
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Merge gather  (reference: merge/_uniform_2D_DtN.py:206-475,
// merge/_schur_complement.py:182-237, 3D: merge/_schur_complement.py:293-774)
//
// Children of merge m are nodes m*nch .. m*nch+nch-1, each with a boundary
// of nb points.  Index maps (shared by all merges of a level):
//   int_c/int_l [2*n_int] : the two (child, local) copies of interface i
//   ext_c/ext_l [n_ext]   : (child, local) of exterior point e (final order)
//   loc [nch*n_int]       : local index of interface i in child c, or -1
// Outputs per merge:
//   D[i][j]  = sum over the children holding both i and j of T_c[i][j]
//   C[i][e]  = T_c(e)[i][e]        B[e][j] = T_c(e)[e][j]
//   Tout[e][f] = T_c[e][f] if e, f on the same child else 0   (the A blocks)
//   dh[i]    = sum of the two children's h at i,   hext[e] = h_c(e)[e]
// ---------------------------------------------------------------------------
// Rows are handled by groups of gw lanes (gw = the column count rounded up to
// a power of two, at most 32; several short rows share a warp): each group
// looks up its row's child and local index once and strides over the
// columns, so no element pays a division for its (row, column) pair.
__device__ __forceinline__ int row_group_width(int cols) {
  int w = 1;
  while (w < cols && w < 32) w <<= 1;
  return w;
}

template <class T>
__global__ void merge_gather_kernel(int nch, int nb, int n_int, int n_ext, int ns, const T* __restrict__ Tc,
                                    const T* __restrict__ hc, const int* __restrict__ int_c,
                                    const int* __restrict__ int_l, const int* __restrict__ ext_c,
                                    const int* __restrict__ ext_l, const int* __restrict__ loc, T* D, T* C,
                                    T* B, T* Tout, T* dh, T* hext, int skip_zero, long long m_base, int seg0) {
  const long long m = blockIdx.y + m_base;
  const int seg = (int)blockIdx.z + seg0;
  const long long nbb = (long long)nb * nb;
  const T* Tm = Tc ? Tc + m * nch * nbb : nullptr;
  const T* hm = hc ? hc + m * nch * (long long)nb * ns : nullptr;
  int rows, cols;
  switch (seg) {
    case 0: rows = Tm ? n_int : 0; cols = n_int; break;
    case 1: rows = Tm ? n_int : 0; cols = n_ext; break;
    case 2: rows = Tm ? n_ext : 0; cols = n_int; break;
    case 3: rows = (Tm && Tout) ? n_ext : 0; cols = n_ext; break;
    case 4: rows = hm ? n_int : 0; cols = ns; break;
    default: rows = hm ? n_ext : 0; cols = ns; break;
  }
  const int gw = row_group_width(cols);
  const int lane = threadIdx.x & 31, gl = lane & (gw - 1);
  const int groups = (blockDim.x >> 5) * (32 / gw);
  const int g = (threadIdx.x >> 5) * (32 / gw) + lane / gw;
  for (int r = blockIdx.x * groups + g; r < rows; r += gridDim.x * groups) {
    const long long o = (long long)r * cols;
    if (seg == 0) {
      const int c0 = int_c[2 * r], c1 = int_c[2 * r + 1];
      const T* t0 = c0 >= 0 ? Tm + c0 * nbb + (long long)int_l[2 * r] * nb : nullptr;
      const T* t1 = c1 >= 0 ? Tm + c1 * nbb + (long long)int_l[2 * r + 1] * nb : nullptr;
      const int* loc0 = loc + (c0 >= 0 ? c0 : 0) * n_int;
      const int* loc1 = loc + (c1 >= 0 ? c1 : 0) * n_int;
      T* out = D + m * n_int * (long long)n_int + o;
      for (int j = gl; j < cols; j += gw) {
        T v = zero<T>();
        if (t0) { const int lj = loc0[j]; if (lj >= 0) v = add(v, t0[lj]); }
        if (t1) { const int lj = loc1[j]; if (lj >= 0) v = add(v, t1[lj]); }
        out[j] = v;
      }
    } else if (seg == 1) {
      T* out = C + m * n_int * (long long)n_ext + o;
      for (int x = gl; x < cols; x += gw) {
        const int c = ext_c[x];
        const int li = loc[c * n_int + r];
        const T v = li >= 0 ? Tm[c * nbb + (long long)li * nb + ext_l[x]] : zero<T>();
        if (li >= 0 || !(skip_zero & 1)) out[x] = v;
      }
    } else if (seg == 2) {
      const int c = ext_c[r];
      const T* t = Tm + c * nbb + (long long)ext_l[r] * nb;
      const int* lc = loc + c * n_int;
      T* out = B + m * n_ext * (long long)n_int + o;
      for (int j = gl; j < cols; j += gw) {
        const int lj = lc[j];
        if (lj >= 0) out[j] = t[lj];
        else if (!(skip_zero & 2)) out[j] = zero<T>();
      }
    } else if (seg == 3) {
      const int c = ext_c[r];
      const T* t = Tm + c * nbb + (long long)ext_l[r] * nb;
      T* out = Tout + m * n_ext * (long long)n_ext + o;
      for (int y = gl; y < cols; y += gw) out[y] = ext_c[y] == c ? t[ext_l[y]] : zero<T>();
    } else if (seg == 4) {
      const int c0 = int_c[2 * r], c1 = int_c[2 * r + 1];
      const T* h0 = c0 >= 0 ? hm + (c0 * (long long)nb + int_l[2 * r]) * ns : nullptr;
      const T* h1 = c1 >= 0 ? hm + (c1 * (long long)nb + int_l[2 * r + 1]) * ns : nullptr;
      T* out = dh + m * n_int * (long long)ns + o;
      for (int s = gl; s < cols; s += gw) {
        T v = zero<T>();
        if (h0) v = add(v, h0[s]);
        if (h1) v = add(v, h1[s]);
        out[s] = v;
      }
    } else {
      const T* h = hm + (ext_c[r] * (long long)nb + ext_l[r]) * ns;
      T* out = hext + m * n_ext * (long long)ns + o;
      for (int s = gl; s < cols; s += gw) out[s] = h[s];
    }
  }
}

// Launch geometry of the ItI merge gather: x blocks of 256 threads over the
// largest segment of one merge.  When the launch would
// hold far more CTAs than the GPU runs at once (152 SMs x 8 CTAs of 256
// threads), each thread takes about four elements (the kernels stride over
// their segment): these segments are short, and with one element per thread
// scheduling the CTAs cost more than moving the data.
static int gather_blocks(long long big, long long ctas_per_x) {
  long long gx = (big + 255) / 256;
  if (gx * ctas_per_x > 16LL * 152 * 8) gx = (big + 1023) / 1024;
  if (gx < 1) gx = 1;
  if (gx > 512) gx = 512;
  return (int)gx;
}

// Launch geometry of the row-wise gathers and the down-pass scatter: groups
// of lanes per row as in the kernels (256 threads), one row per group; when
// the launch would hold far more CTAs than the GPU runs at once each group
// takes about four rows.
static int row_blocks(long long rows, long long cols, long long ctas_per_x) {
  long long gw = 1;
  while (gw < cols && gw < 32) gw <<= 1;
  const long long groups = 8 * (32 / gw);
  long long gx = (rows + groups - 1) / groups;
  if (gx * ctas_per_x > 16LL * 152 * 8) gx = (rows + 4 * groups - 1) / (4 * groups);
  if (gx < 1) gx = 1;
  if (gx > 512) gx = 512;
  return (int)gx;
}

// Segments 0-3 gather operator blocks (present with the children's
// operators), 4-5 the children's h (present with hc): the first segment
// launched and the number of segments, and the largest segment's size.
static void gather_segments(bool ops, bool has_tout, bool has_h, long long n_int, long long n_ext, long long ns,
                            int* seg0, int* nseg, long long* big) {
  *seg0 = ops ? 0 : 4;
  *nseg = (ops ? 4 : 0) + (has_h ? 2 : 0);
  long long b = 0;
  if (ops) {
    b = n_int * n_int;
    if (n_int * n_ext > b) b = n_int * n_ext;
    if (has_tout && n_ext * n_ext > b) b = n_ext * n_ext;
  }
  if (has_h) {
    const long long bh = (n_int > n_ext ? n_int : n_ext) * ns;
    if (bh > b) b = bh;
  }
  *big = b;
}

template <class T>
cudaError_t merge_gather(int n_merges, int nch, int nb, int n_int, int n_ext, int ns, const T* Tc, const T* hc,
                         const int* int_c, const int* int_l, const int* ext_c, const int* ext_l,
                         const int* loc, T* D, T* C, T* B, T* Tout, T* dh, T* hext, int skip_zero,
                         cudaStream_t st) {
  int seg0, nseg;
  long long big;
  gather_segments(Tc != nullptr, Tout != nullptr, hc != nullptr, n_int, n_ext, ns, &seg0, &nseg, &big);
  if (nseg == 0 || big == 0) return cudaSuccess;
  // the row blocks of the widest segment launched (segments 0-3: the
  // operator blocks, 4-5: h; rows x columns as in the kernel)
  const long long seg_rows[6] = {n_int, n_int, n_ext, n_ext, n_int, n_ext};
  const long long seg_cols[6] = {n_int, n_ext, n_int, n_ext, ns, ns};
  for (int m0 = 0; m0 < n_merges; m0 += 65535) {
    const int nm = n_merges - m0 < 65535 ? n_merges - m0 : 65535;
    int gx = 1;
    for (int sg = seg0; sg < seg0 + nseg; ++sg) {
      if (sg == 3 && !Tout) continue;
      const int b = row_blocks(seg_rows[sg], seg_cols[sg], (long long)nm * nseg);
      if (b > gx) gx = b;
    }
    const double outs =
        Tc ? ((double)n_int * n_int + 2.0 * n_int * n_ext + (Tout ? (double)n_ext * n_ext : 0.0)) : 0.0;
    ProfScope ps(KC_MOVE, st, 2.0 * sizeof(T) * nm * (outs + (hc ? (double)(n_int + n_ext) * ns : 0.0)));
    note_launch();
    merge_gather_kernel<T><<<dim3(gx, nm, nseg), 256, 0, st>>>(nch, nb, n_int, n_ext, ns, Tc, hc, int_c, int_l,
                                                               ext_c, ext_l, loc, D, C, B, Tout, dh, hext, skip_zero,
                                                               m0, seg0);
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// ItI merge gather  (reference: merge/_uniform_2D_ItI.py:182-375 with
// merge/_schur_complement.py:6-41, 78-114)
//
// Interface unknown u is child own_c[u]'s incoming impedance at local point
// own_l[u]; its equation is  t_u + (R t + h)_{partner}[par_l[u]] = 0  with
// the partner child par_c[u] across the interface.  int_c/int_l hold
// (own, partner) pairs.  Outputs as for the DtN gather, with
//   D[u][v] = delta_uv + R_{par(u)}[par_l(u)][own_l(v)]  if own_c(v) == par_c(u)
//   C[u][e] = R_{par(u)}[par_l(u)][ext_l(e)]            if ext_c(e) == par_c(u)
//   B[e][v] = R_{c(e)}[ext_l(e)][own_l(v)]              if own_c(v) == ext_c(e)
//   dh[u]   = h_{par(u)}[par_l(u)]
// ---------------------------------------------------------------------------
template <class T>
__global__ void merge_gather_iti_kernel(int nch, int nb, int n_int, int n_ext, int ns, const T* __restrict__ Rc,
                                        const T* __restrict__ hc, const int* __restrict__ int_c,
                                        const int* __restrict__ int_l, const int* __restrict__ ext_c,
                                        const int* __restrict__ ext_l, T* D, T* C, T* B, T* Tout, T* dh, T* hext,
                                        int skip_zero, long long m_base, int seg0) {
  const long long m = blockIdx.y + m_base;
  const int seg = (int)blockIdx.z + seg0;
  const long long nbb = (long long)nb * nb;
  const T* Rm = Rc ? Rc + m * nch * nbb : nullptr;
  const T* hm = hc ? hc + m * nch * (long long)nb * ns : nullptr;
  long long cnt;
  switch (seg) {
    case 0: cnt = Rm ? (long long)n_int * n_int : 0; break;
    case 1: cnt = Rm ? (long long)n_int * n_ext : 0; break;
    case 2: cnt = Rm ? (long long)n_ext * n_int : 0; break;
    case 3: cnt = (Rm && Tout) ? (long long)n_ext * n_ext : 0; break;
    case 4: cnt = hm ? (long long)n_int * ns : 0; break;
    default: cnt = hm ? (long long)n_ext * ns : 0; break;
  }
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < cnt;
       e += (long long)gridDim.x * blockDim.x) {
    T v = zero<T>();
    if (seg == 0) {
      const int u = (int)(e / n_int), w = (int)(e % n_int);
      const int pc = int_c[2 * u + 1];
      if (int_c[2 * w] == pc) v = Rm[pc * nbb + (long long)int_l[2 * u + 1] * nb + int_l[2 * w]];
      if (u == w) v = add(v, one<T>());
      D[m * n_int * (long long)n_int + e] = v;
    } else if (seg == 1) {
      const int u = (int)(e / n_ext), x = (int)(e % n_ext);
      const int pc = int_c[2 * u + 1];
      const bool nz = ext_c[x] == pc;
      if (nz) v = Rm[pc * nbb + (long long)int_l[2 * u + 1] * nb + ext_l[x]];
      if (nz || !(skip_zero & 1)) C[m * n_int * (long long)n_ext + e] = v;
    } else if (seg == 2) {
      const int x = (int)(e / n_int), w = (int)(e % n_int);
      const int c = ext_c[x];
      const bool nz = int_c[2 * w] == c;
      if (nz) v = Rm[c * nbb + (long long)ext_l[x] * nb + int_l[2 * w]];
      if (nz || !(skip_zero & 2)) B[m * n_ext * (long long)n_int + e] = v;
    } else if (seg == 3) {
      const int x = (int)(e / n_ext), y = (int)(e % n_ext);
      const int c = ext_c[x];
      if (ext_c[y] == c) v = Rm[c * nbb + (long long)ext_l[x] * nb + ext_l[y]];
      Tout[m * n_ext * (long long)n_ext + e] = v;
    } else if (seg == 4) {
      const int u = (int)(e / ns), s = (int)(e % ns);
      v = hm[(int_c[2 * u + 1] * (long long)nb + int_l[2 * u + 1]) * ns + s];
      dh[m * n_int * (long long)ns + e] = v;
    } else {
      const int x = (int)(e / ns), s = (int)(e % ns);
      v = hm[(ext_c[x] * (long long)nb + ext_l[x]) * ns + s];
      hext[m * n_ext * (long long)ns + e] = v;
    }
  }
}

template <class T>
cudaError_t merge_gather_iti(int n_merges, int nch, int nb, int n_int, int n_ext, int ns, const T* Rc, const T* hc,
                             const int* int_c, const int* int_l, const int* ext_c, const int* ext_l, T* D, T* C, T* B,
                             T* Tout, T* dh, T* hext, int skip_zero, cudaStream_t st) {
  int seg0, nseg;
  long long big;
  gather_segments(Rc != nullptr, Tout != nullptr, hc != nullptr, n_int, n_ext, ns, &seg0, &nseg, &big);
  if (nseg == 0 || big == 0) return cudaSuccess;
  for (int m0 = 0; m0 < n_merges; m0 += 65535) {
    const int nm = n_merges - m0 < 65535 ? n_merges - m0 : 65535;
    const int gx = gather_blocks(big, (long long)nm * nseg);
    ProfScope ps(KC_MOVE, st, 2.0 * sizeof(T) * nm * ((Rc ? (double)n_int * n_int + 2.0 * n_int * n_ext : 0.0) +
                                                       ((Rc && Tout) ? (double)n_ext * n_ext : 0.0) +
                                                       (hc ? (double)(n_int + n_ext) * ns : 0.0)));
    note_launch();
    merge_gather_iti_kernel<T><<<dim3(gx, nm, nseg), 256, 0, st>>>(nch, nb, n_int, n_ext, ns, Rc, hc, int_c, int_l,
                                                                   ext_c, ext_l, D, C, B, Tout, dh, hext, skip_zero,
                                                                   m0, seg0);
  }
  return cudaGetLastError();
}
template cudaError_t merge_gather_iti<c64>(int, int, int, int, int, int, const c64*, const c64*, const int*,
                                           const int*, const int*, const int*, c64*, c64*, c64*, c64*, c64*, c64*,
                                           int, cudaStream_t);
template cudaError_t merge_gather_iti<c128>(int, int, int, int, int, int, const c128*, const c128*, const int*,
                                            const int*, const int*, const int*, c128*, c128*, c128*, c128*, c128*,
                                            c128*, int, cudaStream_t);
template cudaError_t merge_gather_iti<float>(int, int, int, int, int, int, const float*, const float*, const int*,
                                             const int*, const int*, const int*, float*, float*, float*, float*,
                                             float*, float*, int, cudaStream_t);
template cudaError_t merge_gather_iti<double>(int, int, int, int, int, int, const double*, const double*, const int*,
                                              const int*, const int*, const int*, double*, double*, double*, double*,
                                              double*, double*, int, cudaStream_t);

// ---------------------------------------------------------------------------
// Down-pass scatter  (reference: down_pass/_uniform_2D_DtN.py:125-189)
// child boundary point (c, k) takes parent exterior value code>=0 or
// interface value -(code+1).
// ---------------------------------------------------------------------------
template <class T>
__global__ void down_scatter_kernel(int nch, int nb, int n_ext, int n_int, int ns, const int* __restrict__ code,
                                    const T* __restrict__ gpar, const T* __restrict__ gint, T* gch,
                                    long long m_base) {
  const long long m = blockIdx.y + m_base;
  const int rows = nch * nb;   // child boundary points (c*nb + k)
  const int gw = row_group_width(ns);
  const int lane = threadIdx.x & 31, gl = lane & (gw - 1);
  const int groups = (blockDim.x >> 5) * (32 / gw);
  const int g = (threadIdx.x >> 5) * (32 / gw) + lane / gw;
  for (int r = blockIdx.x * groups + g; r < rows; r += gridDim.x * groups) {
    const int cd = code[r];
    // HPS_CODE_PAD marks padding slots of a child with fewer boundary points
    const T* src = (cd == HPS_CODE_PAD) ? nullptr
                   : (cd >= 0) ? gpar + (m * n_ext + cd) * ns : gint + (m * n_int + (-cd - 1)) * ns;
    T* out = gch + (m * rows + r) * (long long)ns;
    for (int s = gl; s < ns; s += gw) out[s] = src ? src[s] : zero<T>();
  }
}

template <class T>
cudaError_t down_scatter(int n_merges, int nch, int nb, int n_ext, int n_int, int ns, const int* code,
                         const T* gpar, const T* gint, T* gch, cudaStream_t st) {
  const long long cnt = (long long)nch * nb * ns;
  for (int m0 = 0; m0 < n_merges; m0 += 65535) {
    const int nm = n_merges - m0 < 65535 ? n_merges - m0 : 65535;
    const int gx = row_blocks((long long)nch * nb, ns, nm);
    ProfScope ps(KC_MOVE, st, 2.0 * sizeof(T) * nm * (double)cnt);
    note_launch();
    down_scatter_kernel<T><<<dim3(gx, nm), 256, 0, st>>>(nch, nb, n_ext, n_int, ns, code, gpar, gint, gch, m0);
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Element-type conversion (f64 <-> f32, c128 <-> c64)
// ---------------------------------------------------------------------------
template <class S, class D>
__global__ void convert_kernel(long long n, const S* __restrict__ src, D* __restrict__ dst) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    if constexpr (sizeof(S) == sizeof(D) * 2 && sizeof(D) == 4) dst[e] = (D)src[e];
    else if constexpr (sizeof(D) == sizeof(S) * 2 && sizeof(S) == 4) dst[e] = (D)src[e];
    else if constexpr (sizeof(S) == 16) dst[e] = D{(float)src[e].x, (float)src[e].y};
    else dst[e] = D{(double)src[e].x, (double)src[e].y};
  }
}

template <class S, class D>
cudaError_t convert(long long n, const S* src, D* dst, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  long long g = (n + 255) / 256;
  if (g > 4096) g = 4096;
  note_launch();
  convert_kernel<S, D><<<(int)g, 256, 0, st>>>(n, src, dst);
  return cudaGetLastError();
}

// explicit instantiations
#define HPS_INST_K(T)                                                                                          \
  template cudaError_t leaf_assemble<T, double>(int, int, int, int, int, int, const double*, const double*, T*, \
                                                long long, long long, T*, long long, long long, cudaStream_t);  \
  template cudaError_t leaf_assemble<T, c128>(int, int, int, int, int, int, const double*, const c128*, T*,     \
                                              long long, long long, T*, long long, long long, cudaStream_t);    \
  template cudaError_t set_rows<T>(int, int, int, const T*, long long, T*, long long, long long, cudaStream_t); \
  template cudaError_t row_equilibrate<T>(int, int, T*, long long, long long, double*, cudaStream_t);              \
  template cudaError_t col_scale<T>(int, int, T*, long long, long long, const double*, cudaStream_t);           \
  template cudaError_t perm_gather<T>(int, int, int, int, const T*, long long, const int*, int, int, T*,       \
                                      long long, cudaStream_t);                                                  \
  template cudaError_t perm_scatter<T>(int, int, int, int, T*, long long, const int*, int, int, const T*,       \
                                       long long, int, cudaStream_t);                                            \
  template cudaError_t add_identity<T>(int, int, T*, long long, cudaStream_t);                                 \
  template cudaError_t merge_gather<T>(int, int, int, int, int, int, const T*, const T*, const int*, const int*, \
                                       const int*, const int*, const int*, T*, T*, T*, T*, T*, T*, int,           \
                                       cudaStream_t);                                                           \
  template cudaError_t down_scatter<T>(int, int, int, int, int, int, const int*, const T*, const T*, T*,        \
                                       cudaStream_t);
HPS_INST_K(float)
HPS_INST_K(double)
HPS_INST_K(c64)
HPS_INST_K(c128)
template cudaError_t convert<double, float>(long long, const double*, float*, cudaStream_t);
template cudaError_t convert<float, double>(long long, const float*, double*, cudaStream_t);
template cudaError_t convert<c128, c64>(long long, const c128*, c64*, cudaStream_t);
template cudaError_t convert<c64, c128>(long long, const c64*, c128*, cudaStream_t);

}  // namespace hps
