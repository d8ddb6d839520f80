/*
 * jaxhps_gb300 — C ABI of the GB300-native HPS build/solve path.
 *
 * The reference (meliao/jaxhps) is pure JAX and binds no native code; its
 * hot path is three families of stage functions that this library replaces
 * one for one:
 *
 *   local_solve_stage_uniform_{2D,3D}_DtN  src/jaxhps/local_solve/_uniform_2D_DtN.py:9-102
 *                                          (get_DtN :228-273), _uniform_3D_DtN.py:13-106
 *   local_solve_stage_uniform_2D_ItI       src/jaxhps/local_solve/_uniform_2D_ItI.py:10-117
 *                                          (get_ItI :120-186)
 *   merge_stage_uniform_{2D,3D}_DtN        src/jaxhps/merge/_uniform_2D_DtN.py:13-203
 *                                          (one level = vmapped_uniform_quad_merge_DtN :358-381)
 *   merge_stage_uniform_2D_ItI             src/jaxhps/merge/_uniform_2D_ItI.py:19-179
 *   down_pass_uniform_{2D,3D}_DtN / _ItI   src/jaxhps/down_pass/_uniform_2D_DtN.py:7-122
 *                                          (one level = _propagate_down_2D_DtN :125-189)
 *
 * Python host code (jaxhps_gb300/_native.py) binds these symbols with ctypes.
 *
 * Conventions
 *  - Every pointer argument is a device pointer unless stated otherwise.
 *    Arrays are dense row-major; batch strides are in elements.
 *  - The library never allocates device memory: callers pass a workspace
 *    sized by the matching *_workspace_size() call.
 *  - `stream` is a cudaStream_t passed as void*; work is enqueued, the call
 *    returns without synchronising.
 *  - Return value: HPS_OK (0) or an error code; hps_last_error() gives the
 *    message of the most recent failure in the calling thread.
 */
#ifndef JAXHPS_GB300_H
#define JAXHPS_GB300_H

#include <stddef.h>

#if defined(__GNUC__)
#define HPS_API __attribute__((visibility("default")))
#else
#define HPS_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* element types */
enum { HPS_F64 = 0, HPS_F32 = 1, HPS_C128 = 2, HPS_C64 = 3 };

/* status codes */
enum {
  HPS_OK = 0,
  HPS_ERR_ARG = 1,        /* invalid argument (shape, null pointer, dtype) */
  HPS_ERR_SINGULAR = 2,   /* reserved: a zero pivot (reported through info arrays) */
  HPS_ERR_WORKSPACE = 4,  /* workspace too small */
  HPS_ERR_CUDA = 5        /* a CUDA launch or runtime call failed */
};

/* Library version string (static storage). */
HPS_API const char* hps_version(void);

/* Number of CUDA kernels this library has enqueued since it was loaded.
 * No counterpart in the reference (instrumentation). */
HPS_API long long hps_launch_count(void);

/* Non-zero if a tensor-core GEMM launch of this process ever hit its bounded
 * wait (its output is then invalid).  Synchronises with the device.  No
 * counterpart in the reference. */
HPS_API int hps_gemm_tc_status(void);

/* hps_gemm_tc_status, and the flag cleared: the Python build and solve call
 * it after their work so that a flag raised by one call is reported once.
 * Synchronises with the device.  No counterpart in the reference. */
HPS_API int hps_gemm_tc_status_reset(void);

/* Poll limits of the library's bounded device waits, on the current device:
 * the multi-CTA inverse panel's grid barrier (default 2^24 polls of >= 100 ns;
 * a barrier that runs out marks its matrix with info = -1 and the inverse's
 * remaining kernels run to completion on in-range indices) and the
 * tensor-core kernels' mbarrier waits (GEMM and tensor-memory inverse;
 * default 2^22 polls, never set below 2^20: a CTA that gives up waits once
 * more, with the same limit, for its MMAs in flight before freeing their
 * tensor memory).  A negative value keeps a limit; the previous values are
 * returned through the pointers that are not NULL.  Process-wide for the
 * device, not meant to change while work is in flight.  No counterpart in
 * the reference (it has no device waits). */
HPS_API int hps_set_spin_limits(long long panel_barrier_polls, long long tc_wait_polls, long long* prev_panel,
                                long long* prev_tc);

/* Which FP32 inversions of 64 < n <= 224 use the kernel that keeps the
 * Gauss-Jordan tableau in tensor memory and runs its rank-32 trailing updates
 * as tcgen05 MMAs on operands split into three TF32 parts (no workspace):
 * 0 none (SIMT kernels only), 1 (default) the leaf stage's inverses of
 * hps_local_solve_dtn, 2 every one, hps_inverse_batched and the merges
 * included (the tensor core accumulates the update in FP32 with its own
 * rounding, which on the merges' interface matrices costs the mixed-precision
 * solve refinement steps; 2 is for tests and measurements).  Returns the
 * previous policy, or -1 for an invalid one.  HPS_INVERSE_TC=0 in the
 * environment starts a process at 0.  Process-wide; not meant to change while
 * work is in flight.  No counterpart in the reference (which calls
 * jnp.linalg.inv). */
HPS_API int hps_inverse_policy(int policy);

/* Whether the FP32 interface-matrix inverses of the DtN merges
 * (hps_merge_level_dtn, n >= 224) use the recursive 2 x 2 block inversion:
 * two half-size inversions and six half-size batched products per level,
 * down to blocks of n < 224 inverted by pivoted Gauss-Jordan, with no
 * pivoting across blocks (the leading blocks of an interface matrix are
 * interface operators themselves).  1 on (default; HPS_INVERSE_RECURSIVE=0 in
 * the environment starts a process at 0), 0 off (pivoted Gauss-Jordan over the
 * whole matrix), -1 query.  Returns the previous policy.  hps_inverse_batched
 * itself always pivots over the whole matrix.  Process-wide; not meant to
 * change while work is in flight.  No counterpart in the reference (which
 * calls jnp.linalg.inv). */
HPS_API int hps_inverse_block_policy(int policy);

/* Which batched products run on the tcgen05 kernel: 0 none (SIMT kernels
 * only), 1 the shapes where it was measured faster (default; HPS_GEMM_TC=0 in
 * the environment starts a process at 0), 2 every FP32 and complex64 product
 * (for tests and measurements), 3 none and the FP32 8x8 SIMT tiles with 4-byte
 * shared-memory loads instead of the 16-byte-load tiles (for comparisons;
 * identical results).  Returns the previous policy, or -1 for an
 * invalid one.  Process-wide; not meant to change while work is in flight.
 * No counterpart in the reference. */
HPS_API int hps_gemm_policy(int policy);

/* Autotuning of the FP32 batched products (the leaf, merge, refinement and
 * down-pass products; not the N <= 8 ones).  Kernel variants: 0 tcgen05
 * 3xTF32, 1 / 2 / 3 SIMT 8x8 register tiles of 128x128 / 128x64 / 64x64,
 * 4 / 5 / 6 64x64 tiles with K split over a 2 / 4 / 8-CTA cluster, 7 SIMT 4x4
 * register tiles of 64x64, 8 the warp-specialised TMA + tcgen05 3xTF32 kernel
 * for N <= 64 (16-byte aligned operands; other shapes run variant 3; policy 1
 * also picks it for such products with at least 608 row tiles of 128).
 * hps_gemm_tune_set stores the variant for an
 * (M, N, K, batch) shape (-1 removes it); products of a stored shape run that
 * variant, the others the built-in rules.  hps_gemm_tune_clear empties the
 * table.  hps_gemm_force_variant(v) runs every FP32 product with variant v
 * (-1: off; for timing), returning the previous one.  hps_gemm_shapes(mode,
 * out, cap): mode 1 clears the record and starts recording the distinct
 * product shapes, 0 stops, -1 only reads; returns the number recorded and
 * writes up to cap of them to out, 13 values each (M, N, K, batch, lda,
 * strideA, ldb, strideB, ldc, strideC, ldd, strideD, has C).  The table and
 * switches are process-wide.  jaxhps_gb300/autotune.py drives them.  No
 * counterpart in the reference (XLA chooses its own kernels). */
HPS_API int hps_gemm_tune_set(int M, int N, int K, int batch, int variant);
HPS_API int hps_gemm_tune_clear(void);
HPS_API int hps_gemm_force_variant(int variant);
HPS_API long long hps_gemm_shapes(int mode, long long* out, long long cap);

/* Live profiler.  hps_profile_begin(mask) arms CUDA-event timing of every
 * later launch whose kernel class c has bit (1 << c) set in mask (classes:
 * 1 GEMM (SIMT and the 3xTF32 tcgen05 kernel), 2 inverse, 3
 * gather/scatter/assembly, 4 FP64 refinement residual, 5 the TMA GEMM of the
 * N <= 64 products, 6 the FP32-pair residual update, 7 the tensor-memory leaf
 * inverse), recorded on the launch's own stream.  A launch inside another
 * recorded one (an inversion's products) counts for the outer one only.
 * hps_profile_end() synchronises on those events and fills arrays of 8
 * entries indexed by class: summed kernel time (ms), number of launches and
 * summed algorithmic work (flops for 1, 2, 4, 7; bytes for 3, 5, 6), then
 * disarms.  No counterpart in the reference. */
HPS_API int hps_profile_begin(int class_mask);
HPS_API int hps_profile_end(double* total_ms, long long* launches, double* work);

/* Copies the last error message of this thread into buf (NUL-terminated).
 * Returns the full message length.  No counterpart in the reference (whose
 * stages raise Python exceptions; the Python layer raises NativeError). */
HPS_API int hps_last_error(char* buf, size_t len);

/* ---------------------------------------------------------------------------
 * Batched primitives
 * ------------------------------------------------------------------------- */

/* D[b] = alpha * A[b] @ B[b] + beta * C[b]  (row-major, m x k times k x n).
 * alpha/beta are host pointers to {re, im}.  C may be NULL (beta ignored)
 * and may alias D.  A batch stride of 0 broadcasts that operand.
 * Replaces the `@` / einsum products of get_DtN (_uniform_2D_DtN.py:264-271),
 * _assemble_merge_outputs (merge/_schur_complement.py:222-235) and the down
 * pass (down_pass/_uniform_2D_DtN.py:114-120, :149). */
HPS_API int hps_gemm_batched(int dtype, int m, int n, int k, const double* alpha, const void* A, long long lda,
                     long long strideA, const void* B, long long ldb, long long strideB, const double* beta,
                     const void* C, long long ldc, long long strideC, void* D, long long ldd, long long strideD,
                     int batch, void* stream);

/* Workspace bytes for hps_inverse_batched (0 for small n); sizing only, the
 * inverse replaces jnp.linalg.inv (local_solve/_uniform_2D_DtN.py:257). */
HPS_API size_t hps_inverse_workspace_size(int dtype, int n, int batch);

/* X[b] = inv(A[b]) by Gauss-Jordan elimination with partial pivoting.
 * X may alias A.  info[b] (device, may be NULL) = 0 or k+1 for a zero pivot
 * at step k, or -1 when the multi-CTA panel used for few large matrices hit
 * its barrier time limit (X[b] is then invalid).  Replaces jnp.linalg.inv at local_solve/_uniform_2D_DtN.py:257
 * and merge/_schur_complement.py:107,146. */
HPS_API int hps_inverse_batched(int dtype, int n, const void* A, long long lda, long long strideA, void* X,
                        long long ldx, long long strideX, int batch, int* info, void* workspace,
                        size_t workspace_bytes, void* stream);

/* The inverse hps_merge_level_dtn applies to its interface matrices: as
 * hps_inverse_batched, except that FP32 matrices of n >= 224 use the
 * recursive 2 x 2 block inversion while hps_inverse_block_policy is 1 (zero
 * pivots of its blocks reported in info with the block's column offset).
 * Same workspace size.  Replaces jnp.linalg.inv at
 * merge/_schur_complement.py:146. */
HPS_API int hps_inverse_interface(int dtype, int n, const void* A, long long lda, long long strideA, void* X,
                                  long long ldx, long long strideX, int batch, int* info, void* workspace,
                                  size_t workspace_bytes, void* stream);

/* Size of the fixed scratch behind hps_inverse_batched_static: 64 MiB. */
#define HPS_STATIC_SCRATCH_BYTES (64u << 20)

/* hps_inverse_batched without a workspace argument, for callers that cannot
 * allocate device memory (no cudaMalloc available to them, or all device
 * memory owned by a pool that only hands out their inputs and outputs).
 * No counterpart in the reference: it exists for such callers only.
 * Scratch is a static device array of HPS_STATIC_SCRATCH_BYTES that every
 * GPU loading the library holds until exit; the call allocates nothing.
 * Returns HPS_ERR_WORKSPACE when hps_inverse_workspace_size(dtype, n, batch)
 * exceeds that size; that size counts 256 bytes of alignment slack, which the
 * already aligned array does not need, so the usable limit is
 * HPS_STATIC_SCRATCH_BYTES - 256 bytes of scratch proper.  All calls share the
 * array: calls that overlap on the GPU (other streams or host threads, same
 * device) race.  The first call on a device looks up the array's address and
 * should come before any stream capture.  The address is kept per device
 * index for the life of the process, which assumes the runtime's primary
 * context throughout (no cudaDeviceReset between calls). */
HPS_API int hps_inverse_batched_static(int dtype, int n, const void* A, long long lda, long long strideA,
                                       void* X, long long ldx, long long strideX, int batch, int* info,
                                       void* stream);

/* Element-type conversion of n contiguous elements (f64<->f32, c128<->c64);
 * the mixed-precision builds' casts, no counterpart in the reference. */
HPS_API int hps_convert(int dtype_src, int dtype_dst, long long n, const void* src, void* dst, void* stream);

/* ---------------------------------------------------------------------------
 * Leaf stage (DtN).  Replaces local_solve_stage_uniform_2D_DtN /
 * local_solve_stage_uniform_3D_DtN (get_DtN, _uniform_2D_DtN.py:228-273):
 *   A   = sum_o diag(coeffs[o]) ops[o]            (assemble_diff_operator :182-218)
 *   Y   = [P ; -inv(A_ii) A_ie P],  T = Q Y,
 *   v   = [0 ; inv(A_ii) f_int],     h = Q v.
 * ------------------------------------------------------------------------- */
typedef struct {
  int dtype;          /* HPS_F64 or HPS_F32 (HPS_C128/HPS_C64 for complex coefficients) */
  int coef_complex;   /* 0: coeffs are float64, 1: complex128 */
  int n_leaves;
  int n_pts;          /* p^d Chebyshev points per leaf */
  int n_cb;           /* Chebyshev boundary points (exterior-first prefix) */
  int n_gauss;        /* Gauss boundary points (4q in 2D, 6q^2 in 3D) */
  int nsrc;           /* number of right-hand sides (0: no source) */
  int n_ops;          /* number of active coefficient/operator pairs */
  const double* ops;  /* (n_ops, n_pts, n_pts) float64 */
  const void* coeffs; /* (n_ops, n_leaves, n_pts) float64 or complex128 */
  const void* source; /* (n_leaves, n_pts, nsrc) in dtype, or NULL */
  const void* P;      /* (n_cb, n_gauss) in dtype */
  const void* Q;      /* (n_gauss, n_pts) in dtype */
  void* Y;            /* out (n_leaves, n_pts, n_gauss) */
  void* T;            /* out (n_leaves, n_gauss, n_gauss) */
  void* v;            /* out (n_leaves, n_pts, nsrc) or NULL */
  void* h;            /* out (n_leaves, n_gauss, nsrc) or NULL */
  void* Aii_inv;      /* out (n_leaves, n_i, n_i), n_i = n_pts - n_cb */
  int* info;          /* out (n_leaves) pivot status, or NULL */
  void* workspace;
  size_t workspace_bytes;
} hps_leaf_dtn_args;

HPS_API size_t hps_local_solve_dtn_workspace_size(const hps_leaf_dtn_args* a);
HPS_API int hps_local_solve_dtn(const hps_leaf_dtn_args* a, void* stream);

/* ---------------------------------------------------------------------------
 * Leaf stage (ItI, 2D).  Replaces get_ItI (local_solve/_uniform_2D_ItI.py:120-186):
 *   B = [G ; A[n_cb:, :]],  Binv = inv(B),
 *   Y = Binv[:, :n_cb] P,   v = Binv[:, n_cb:] f_int,   T = QH Y,  h = QH v.
 * ------------------------------------------------------------------------- */
typedef struct {
  int dtype;          /* HPS_C128 or HPS_C64 */
  int coef_complex;
  int n_leaves, n_pts, n_cb, n_gauss, nsrc, n_ops;
  const double* ops;  /* (n_ops, n_pts, n_pts) float64 */
  const void* coeffs; /* (n_ops, n_leaves, n_pts) float64 or complex128 */
  const void* source; /* (n_leaves, n_pts, nsrc) in dtype, or NULL */
  const void* G;      /* (n_cb, n_pts) in dtype */
  const void* P;      /* (n_cb, n_gauss) in dtype */
  const void* QH;     /* (n_gauss, n_pts) in dtype */
  void* Y;            /* out (n_leaves, n_pts, n_gauss) */
  void* T;            /* out (n_leaves, n_gauss, n_gauss) */
  void* v;            /* out (n_leaves, n_pts, nsrc) or NULL */
  void* h;            /* out (n_leaves, n_gauss, nsrc) or NULL */
  void* B_inv;        /* out (n_leaves, n_pts, n_pts) */
  int* info;
  void* workspace;
  size_t workspace_bytes;
} hps_leaf_iti_args;

HPS_API size_t hps_local_solve_iti_workspace_size(const hps_leaf_iti_args* a);
HPS_API int hps_local_solve_iti(const hps_leaf_iti_args* a, void* stream);

/* ---------------------------------------------------------------------------
 * One merge level (DtN, quad or oct).  Replaces vmapped_uniform_quad_merge_DtN
 * (merge/_uniform_2D_DtN.py:358-381) and _uniform_oct_merge_DtN
 * (merge/_uniform_3D_DtN.py:127-187):
 *   gather B, C, D, A-blocks from the children's T  (index maps),
 *   D_inv = inv(D),  S = -D_inv C,  g~ = -D_inv dh,
 *   T_out = A + B S,  h_out = h_ext + B g~.
 * The exterior ordering of T_out / h_out / S columns is the final one
 * (the reference's roll by -n_int, :343-346, is folded into ext_c/ext_l).
 * ------------------------------------------------------------------------- */
typedef struct {
  int dtype;
  int n_merges;
  int nch;            /* children per merge: 4 (2D) or 8 (3D) */
  int nb;             /* boundary points of one child */
  int n_int;          /* interface points of one merge */
  int n_ext;          /* exterior points of one merge */
  int nsrc;           /* 0 for no source */
  const void* T_children; /* (n_merges*nch, nb, nb) */
  const void* h_children; /* (n_merges*nch, nb, nsrc) or NULL */
  const int* int_c;   /* (2*n_int) child of each copy of interface point i */
  const int* int_l;   /* (2*n_int) local index in that child */
  const int* ext_c;   /* (n_ext) */
  const int* ext_l;   /* (n_ext) */
  const int* loc;     /* (nch*n_int) local index of interface i in child c, -1 if absent */
  void* S;            /* out (n_merges, n_int, n_ext) */
  void* g_tilde;      /* out (n_merges, n_int, nsrc) or NULL */
  void* T_out;        /* out (n_merges, n_ext, n_ext), or NULL: the merged map is not formed
                         (a top level whose map nobody reads) */
  void* h_out;        /* out (n_merges, n_ext, nsrc) or NULL */
  void* D_inv;        /* out (n_merges, n_int, n_int), or NULL to keep it in the workspace */
  void* BD_inv;       /* out (n_merges, n_ext, n_int) = B D_inv, or NULL (no-source up pass) */
  void* B_out;        /* out (n_merges, n_ext, n_int) = B, or NULL (kept for the refinement up pass) */
  int* info;          /* (n_merges) or NULL */
  void* workspace;
  size_t workspace_bytes;
  /* Optional block structure (host arrays; counts 0 = dense products).  C is
   * zero outside c_rects, rows (i0, n_i) x columns (e0, n_e); B is zero
   * outside b_rects, rows (e0, n_e) x columns (i0, n_i).  `first` marks the
   * first rectangle over its column range (C) or row range (B); together the
   * rectangles must cover every exterior index.  The products S = -D^-1 C,
   * T_out += B S, h_out += B g~ and B D^-1 then run on the rectangles only
   * (a row of C touches only the exterior of the children sharing that
   * interface point: 1/4 of it in the ItI and 3D merges, 1/2 in 2D DtN). */
  int n_c_rects;
  const int* c_rects; /* (n_c_rects, 5): i0, n_i, e0, n_e, first */
  int n_b_rects;
  const int* b_rects; /* (n_b_rects, 5): e0, n_e, i0, n_i, first */
  /* Optional two-colour structure of D (ItI merges; n_x = 0: none).  With
   * the unknowns permuted by colour_perm (device, n_int: original index of
   * each permuted position, the first n_x of colour X), D = [[I, D12],
   * [D21, I]]; D^-1 is then formed from the inverse of the n_x x n_x matrix
   * W = I - D12 D21 (the reference's _invert_D_ItI,
   * merge/_schur_complement.py:78-114) instead of inverting D itself.
   * Requires n_int - n_x == n_x. */
  int n_x;
  const int* colour_perm;
} hps_merge_args;

HPS_API size_t hps_merge_level_dtn_workspace_size(const hps_merge_args* a);
HPS_API int hps_merge_level_dtn(const hps_merge_args* a, void* stream);

/* One ItI merge level.  Replaces vmapped_uniform_quad_merge_ItI
 * (merge/_uniform_2D_ItI.py:182-405): the interface unknowns are the
 * children's incoming impedances on both sides of every interface, in the
 * reference's final order; int_c/int_l hold (own, partner) pairs per unknown
 * (loc is unused).  D = I + R-coupling is inverted directly; the rest is as
 * hps_merge_level_dtn.  Workspace: hps_merge_level_dtn_workspace_size(). */
HPS_API int hps_merge_level_iti(const hps_merge_args* a, void* stream);

/* ---------------------------------------------------------------------------
 * One down-pass level.  Replaces _propagate_down_2D_DtN
 * (down_pass/_uniform_2D_DtN.py:125-189), _propogate_down_2D_ItI
 * (down_pass/_uniform_2D_ItI.py:121-192), _propogate_down_oct_DtN
 * (down_pass/_uniform_3D_DtN.py:116-246):
 *   g_int = S g_parent + g~ ;  child boundary data gathered through `code`
 *   (code >= 0: parent exterior index, code < 0: interface -(code+1)).
 * ------------------------------------------------------------------------- */
typedef struct {
  int dtype;
  int n_merges, nch, nb, n_int, n_ext, nsrc;
  const void* S;        /* (n_merges, n_int, n_ext) */
  const void* g_tilde;  /* (n_merges, n_int, nsrc) or NULL */
  const void* g_parent; /* (n_merges, n_ext, nsrc) */
  const int* code;      /* (nch*nb) */
  void* g_int;          /* scratch/out (n_merges, n_int, nsrc) */
  void* g_children;     /* out (n_merges*nch, nb, nsrc) */
} hps_down_args;

HPS_API int hps_down_level(const hps_down_args* a, void* stream);

/* ---------------------------------------------------------------------------
 * One up-pass level for new leaf data without rebuilding (the reference's
 * up_pass_uniform_2D_DtN / _ItI, up_pass/_uniform_2D_DtN.py:8-173):
 *   dh = h_a + h_b on every interface (ItI: the partner side's h),
 *   g~ = -D_inv dh,
 *   h_out = h_ext + B g~            (B the merge's B), or
 *   h_out = h_ext - B dh            (flags & HPS_UP_B_IS_BD_INV: B holds B D_inv,
 *                                    as stored by the no-source build).
 * Uses the D_inv and B (or B D_inv) kept from the merge stage.
 * ------------------------------------------------------------------------- */
#define HPS_UP_B_IS_BD_INV 1
#define HPS_UP_ITI 2
typedef struct {
  int dtype;
  int n_merges, nch, nb, n_int, n_ext, nsrc;
  const void* h_children; /* (n_merges*nch, nb, nsrc) */
  const int *int_c, *int_l, *ext_c, *ext_l;
  const void* D_inv;      /* (n_merges, n_int, n_int) */
  const void* B;          /* (n_merges, n_ext, n_int) */
  void* dh;               /* scratch (n_merges, n_int, nsrc) */
  void* g_tilde;          /* out (n_merges, n_int, nsrc) */
  void* h_out;            /* out (n_merges, n_ext, nsrc) */
  int flags;              /* HPS_UP_B_IS_BD_INV | HPS_UP_ITI */
} hps_up_args;

HPS_API int hps_up_level(const hps_up_args* a, void* stream);

/* ---------------------------------------------------------------------------
 * Iterative refinement (mixed precision).  No reference counterpart: the
 * reference solves in FP64 only.  These compute, in FP64, the residual of
 * the discrete system that the HPS solver solves directly:
 *   leaf rows       r_int = f_int - A_ii u_int - A_ie P g   (get_DtN's system,
 *                   local_solve/_uniform_2D_DtN.py:228-273)
 *   interface rows  flux continuity of Q u across shared Gauss nodes
 *                   (the merge equations, merge/_schur_complement.py:182-237)
 *   boundary rows   g - g_given on the domain boundary.
 * ------------------------------------------------------------------------- */
typedef struct {
  int n_leaves, p, q, nsrc, n_ops;
  int op_kind[10];         /* host values: 0 D_xx, 1 D_xy, 2 D_yy, 3 D_x, 4 D_y, 5 I */
  const double* coeffs;    /* (n_ops, n_leaves, p*p) on the exterior-first leaf points */
  const double* inv_half;  /* (n_leaves) 2 / leaf side length */
  const double* D1;        /* (p, p) Chebyshev differentiation on [-1, 1] */
  const double* D2;        /* (p, p) D1 @ D1 */
  const double* Pside;     /* (p, q) Gauss -> Chebyshev interpolation on one side */
  const double* Qside;     /* (q, p) Chebyshev -> Gauss interpolation on one side */
  const int* perm;         /* (p*p) meshgrid index of every exterior-first point */
  const double* u_int;     /* (n_leaves, n_i, nsrc) interior values */
  const double* g;         /* (n_leaves, 4q, nsrc) leaf boundary Gauss values */
  const double* f;         /* (n_leaves, p*p, nsrc) source, or NULL for a zero source */
  float* r_int;            /* out (n_leaves, n_i, nsrc) leaf-row residual, rounded to FP32 */
  double* r_int64;         /* out, same in FP64, or NULL */
  double* flux;            /* out (n_leaves, 4q, nsrc) outward normal derivative at the Gauss nodes */
  double* u_full;          /* out (n_leaves, p*p, nsrc) full leaf solution, or NULL */
} hps_residual2d_args;

HPS_API int hps_residual_2d(const hps_residual2d_args* a, void* stream);

/* Incremental update of the residual for corrections du (n_leaves, n_i, nsrc)
 * and dg (n_leaves, 4q, nsrc), both FP32:
 *   a->r_int64 -= (A du_full)_int   (FP64, in/out; a->r_int gets its FP32 copy)
 *   a->flux    += Q du_full          (FP64, in/out)
 * with du_full = [P dg ; du], evaluated in double-float (FP32-pair)
 * arithmetic on the FP32 pipe.  Refinement only: no counterpart in the
 * reference, which solves in FP64 directly. */
HPS_API int hps_residual_update_2d(const hps_residual2d_args* a, const float* du, const float* dg, void* stream);

/* hps_residual_2d with the FP64 leaf-row residual r also stored as an FP32
 * pair: a->r_int = fl32(r) and r_lo = fl32(r - a->r_int) (a->r_int64 may be
 * NULL).  With u_int32 not NULL the interior values are read from it (FP32,
 * same layout) instead of a->u_int.  The starting point of
 * hps_residual_update_2d_df.  Refinement only: no counterpart in the
 * reference. */
HPS_API int hps_residual_2d_df(const hps_residual2d_args* a, const float* u_int32, float* r_lo, void* stream);

/* y += x with y held as an FP32 pair (y_hi, y_lo; TwoSum, no FP64
 * arithmetic) and out[0] = max |x|, out[1] = max |y_hi| (FP64, device); n a
 * multiple of 4, arrays 16-byte aligned.  The refined solution's interior
 * accumulator.  No counterpart in the reference. */
HPS_API int hps_accumulate_max_df(long long n, const float* x, float* y_hi, float* y_lo, double* out, void* stream);

/* hps_assemble_u_2d with the interior values given as an FP32 pair
 * (u_hi + u_lo, summed in FP64).  No counterpart in the reference. */
HPS_API int hps_assemble_u_2d_df(int n_leaves, int p, int q, int nsrc, const double* Pside, const float* u_hi,
                                 const float* u_lo, const double* g, double* u_full, void* stream);

/* The incremental update of hps_residual_update_2d with the leaf-row
 * residual held as an FP32 pair (a->r_int = hi, r_lo = lo, both in/out; no
 * FP64 arithmetic on it) and a->flux += Q du_full (FP64, in/out); a->r_int64,
 * a->coeffs and the FP64 operators are not read: `prep` holds them as FP32
 * pairs, written once per solve by hps_residual_df_prepare (its size in bytes
 * from hps_residual_df_prep_size).  Each thread keeps one grid line in
 * registers.  Supported for q = p - 2 with p in 8, 10, 12, 14, 16
 * (hps_residual_df_supported); HPS_ERR_ARG otherwise.  Refinement only: no
 * counterpart in the reference. */
HPS_API size_t hps_residual_df_prep_size(int n_leaves, int p, int q, int n_ops);
HPS_API int hps_residual_df_prepare(const hps_residual2d_args* a, float* prep, void* stream);
HPS_API int hps_residual_update_2d_df(const hps_residual2d_args* a, const float* prep, const float* du,
                                      const float* dg, float* r_lo, void* stream);
HPS_API int hps_residual_df_supported(int p, int q);

/* u_full = [P g ; u_int] per leaf (FP64), exterior-first leaf order: the
 * leaf solution u = Y g + v of the down pass (down_pass/_uniform_2D_DtN.py
 * :125-189) in the refinement's unknowns. */
HPS_API int hps_assemble_u_2d(int n_leaves, int p, int q, int nsrc, const double* Pside, const double* u_int,
                              const double* g, double* u_full, void* stream);

/* The device address of page-locked host memory (cudaHostAlloc'd or
 * registered; mapped for the device), or HPS_ERR_ARG when `host` is not such
 * memory.  A kernel may write its output there directly: hps_assemble_u_2d
 * with u_full in a caller's page-locked buffer forms the solution and moves it
 * to the host in one pass, without a device copy or a separate transfer
 * (synchronise the stream before reading it).  No counterpart in the
 * reference. */
HPS_API int hps_mapped_pointer(const void* host, void** device);

/* out[l][i][j] = sum_o coeffs[o][l][row0+i] * ops[o][row0+i][j] for rows
 * row0 .. row0+n_rows-1 of every leaf's operator A (FP64; row stride ld,
 * leaf stride `stride`).  The assembly of assemble_diff_operator
 * (local_solve/_uniform_2D_DtN.py:182-218), kept for FP64 residuals. */
HPS_API int hps_assemble_rows(int n_leaves, int n_pts, int row0, int n_rows, int n_ops, const double* ops,
                              const double* coeffs, double* out, long long ld, long long stride, void* stream);

/* ---------------------------------------------------------------------------
 * Adaptive merges (merge/_adaptive_3D_DtN.py:30-565,
 * merge/_utils_adaptive_3D_DtN.py:647-743, down_pass/_adaptive_3D_DtN.py).
 * ------------------------------------------------------------------------- */

/* Index-map code of a padding slot: a child with fewer boundary points than
 * the merge's common child size leaves its tail slots unused. */
#define HPS_CODE_PAD (-2147483647 - 1)

/* Panel map along one axis of a batch of matrices.  mode 0 (rows):
 * out[b][i][c] for i < n_out, c < n_other; mode 1 (columns): out[b][r][j] for
 * r < n_other, j < n_out.  table (n_out x 4 int, 16-byte aligned) gives per
 * output index {kind, in_start, local, n_k}: kind 0 copies input index
 * in_start + local; kind 1 combines input indices in_start .. in_start+n_k-1
 * with row `local` of M (mode 0: M is m_len x n_k) or column `local` of M
 * (mode 1: M is n_k x m_len).  Compresses four fine interface panels into
 * one (L_1f4 on rows, L_4f1 on columns) and expands them back (L_4f1). */
HPS_API int hps_panel_map(int dtype, int mode, int batch, int n_out, int n_other, int m_len, const int* table,
                          const void* M, const void* in, long long ld_in, long long stride_in, void* out,
                          long long ld_out, long long stride_out, void* stream);

/* x[b][:] *= scale[b] (scale FP64 on the device) for n_per elements per batch:
 * the per-leaf side-length scaling of the adaptive leaf operators
 * (local_solve/_adaptive_3D_DtN.py:130-168). */
HPS_API int hps_scale_batched(int dtype, int batch, long long n_per, const double* scale, void* x, void* stream);

/* ---------------------------------------------------------------------------
 * Adaptive octree refinement check.  Replaces the per-node check of
 * generate_adaptive_mesh_level_restriction (_adaptive_discretization_3D.py
 * :34-210, :424-503): evaluate f on a node's grid and its eight children's
 * grids, interpolate node -> children (L_8f1) and compare.
 * ------------------------------------------------------------------------- */

/* pts (n_nodes, 9, p^3, 3): for every node (bounds (n_nodes, 6) = xmin, xmax,
 * ymin, ymax, zmin, zmax) its own Chebyshev points then those of children
 * a..h, each grid in exterior-first order (perm[k] = raster index
 * ix p^2 + iy p + iz of position k; cheb = 1D points on [-1, 1]). */
HPS_API int hps_refine_points_3d(int n_nodes, int p, const double* bounds, const double* cheb, const int* perm,
                                 double* pts, void* stream);

/* From f at those points (f_values (n_nodes, 9, p^3)): diff_max[n] =
 * max |L_8f1 f_node - f_children|, ref_max[n] = max |f_children|, and
 * (l2_err may be NULL) the Clenshaw-Curtis weighted squared L2 norm of the
 * difference over the children.  interp_lo/hi (p x p): 1D interpolation
 * from the node's points to a child's lower/upper half points; iperm =
 * inverse of perm; cc_weights = Clenshaw-Curtis weights on [-1, 1]. */
HPS_API int hps_refine_check_3d(int n_nodes, int p, const double* f_values, const int* perm, const int* iperm,
                                const double* interp_lo, const double* interp_hi, const double* cc_weights,
                                const double* bounds, double* diff_max, double* ref_max, double* l2_err,
                                void* stream);

/* 2D analogues (reference _adaptive_discretization_2D.py:34-197): per node 5
 * blocks of p^2 points (the node, then children a..d = SW, SE, NE, NW), pts
 * (n_nodes, 5, p^2, 2); bounds (n_nodes, 4); the check compares the node's
 * values interpolated to the four children with f there. */
HPS_API int hps_refine_points_2d(int n_nodes, int p, const double* bounds, const double* cheb, const int* perm,
                                 double* pts, void* stream);
HPS_API int hps_refine_check_2d(int n_nodes, int p, const double* f_values, const int* perm, const int* iperm,
                                const double* I_lo, const double* I_hi, const double* w_ref, const double* bounds,
                                double* diff_max, double* ref_max, double* l2, void* stream);

/* ---------------------------------------------------------------------------
 * Learned refinement proposal: a 513 -> 64 -> 64 -> 1 MLP (ReLU) over 8^3
 * uniform samples of f per octree node plus its depth.  No counterpart in
 * the reference: it proposes refinements for the adaptive meshing above,
 * whose plain criterion still decides every accepted leaf.  Parameters are
 * one FP32 vector of hps_mlp_param_count() entries: W1 (64 x 513), b1, W2
 * (64 x 64), b2, w3 (64), b3.
 * ------------------------------------------------------------------------- */
HPS_API int hps_mlp_param_count(void);
/* pts (n, 512, 3): cell-centred 8x8x8 sample points of each node's bounds (n, 6). */
HPS_API int hps_mlp_sample_points(int n, const double* bounds, double* pts, void* stream);
/* X (n, 513) FP32 = [f_samples / scale, depth / 16]. */
HPS_API int hps_mlp_features(int n, const double* f_samples, const int* depth, double scale, float* X, void* stream);
/* logit (n); H1, H2 (n, 64) hidden activations (may be NULL for inference). */
HPS_API int hps_mlp_forward(int n, const float* X, const float* params, float* H1, float* H2, float* logit,
                            void* stream);
/* Binary cross-entropy with logits (weight pos_weight on label 1): dlogit =
 * d(mean loss)/dlogit; *loss_sum (may be NULL) += summed weighted loss. */
HPS_API int hps_mlp_bce(int n, const float* logit, const float* labels, float pos_weight, float* dlogit,
                        float* loss_sum, void* stream);
/* grad += d(loss)/d(params) for the rows given dlogit (grad zeroed by the caller). */
HPS_API int hps_mlp_backward(int n, const float* X, const float* params, const float* H1, const float* H2,
                             const float* dlogit, float* grad, void* stream);
/* One Adam step (step counts from 1). */
HPS_API int hps_mlp_adam(float* params, const float* grad, float* m, float* v, float lr, float beta1, float beta2,
                         float eps, int step, void* stream);

/* As hps_assemble_rows with complex128 coefficients and output
 * (assemble_diff_operator, local_solve/_uniform_2D_DtN.py:182-218). */
HPS_API int hps_assemble_rows_complex(int n_leaves, int n_pts, int row0, int n_rows, int n_ops, const double* ops,
                                      const void* coeffs, void* out, long long ld, long long stride, void* stream);

/* ItI refinement interface terms (complex128 in, complex64 out; node = leaf*4q + k):
 *   hcorr[node] = t_out[node] + t_in[nbr[node]]  (0 where nbr < 0),
 *   r_bdry[b]   = t_given[b] - t_in[bdry_node[b]]  (t_given NULL: zero data).
 * t_out = outgoing impedance QH u, t_in = incoming impedance state; hcorr is
 * minus the residual of the partner's interface equation t_in(a) + t_out(b) = 0
 * (the coupling of the ItI merges, merge/_uniform_2D_ItI.py:182-375). */
HPS_API int hps_iti_combine(long long n_nodes, int nsrc, const int* nbr, const void* t_out, const void* t_in,
                            void* hcorr, int n_bdry, const int* bdry_node, const void* t_given, void* r_bdry,
                            void* stream);

/* Residual of the ItI leaf and interface system (complex128; no counterpart
 * in the reference, which solves in complex128 directly).  Per leaf, with u
 * the values at all p^2 points (exterior-first) and t_in the incoming
 * impedance at the 4q Gauss nodes (get_ItI's system,
 * local_solve/_uniform_2D_ItI.py:120-186):
 *   r[:n_cb]  = P t_in - G u        (G = N~ + i eta I, the incoming impedance)
 *   r[n_cb:]  = f_int - A_int u     (tensor-product derivatives)
 *   t_out     = QH u                (outgoing impedance at the Gauss nodes)
 * r is written as complex64, t_out as complex128. */
typedef struct {
  int n_leaves, p, q, nsrc, n_ops;
  int op_kind[10];         /* as in hps_residual2d_args */
  int coef_complex;        /* 1: coeffs are complex128, 0: float64 */
  double eta;
  const void* coeffs;      /* (n_ops, n_leaves, p*p) */
  const double* inv_half;  /* (n_leaves) 2 / leaf side length */
  const double* D1;        /* (p, p) */
  const double* D2;        /* (p, p) */
  const double* Pside;     /* (p, q) */
  const double* Qside;     /* (q, p) */
  const int* perm;         /* (p*p) */
  const void* u;           /* (n_leaves, p*p, nsrc) complex128 */
  const void* t_in;        /* (n_leaves, 4q, nsrc) complex128 */
  const void* f;           /* (n_leaves, p*p, nsrc) complex128, or NULL for a zero source */
  void* r;                 /* out (n_leaves, p*p, nsrc) complex64 */
  void* t_out;             /* out (n_leaves, 4q, nsrc) complex128 */
} hps_residual_iti2d_args;

HPS_API int hps_residual_iti_2d(const hps_residual_iti2d_args* a, void* stream);

/* ------------------------------------------------------------------------
 * Interpolation between the HPS grid and rectangular grids (replaces the
 * reference's _interpolation_methods.py:23-340 behind Domain.interp_*).
 * Barycentric Lagrange interpolation with the reference's coincident-point
 * rule: a target equal to a source node is moved off it by DBL_EPSILON.
 * ------------------------------------------------------------------------ */

/* out[r][k] = 1 / (d_k w_k nf_r), d_k = to_pts[r] - src_pts[k], nf_r =
 * sum_k 1 / (w_k d_k): row r of the 1D interpolation matrix from src_pts
 * (weights src_weights) to to_pts[r].  transposed != 0 writes each group of
 * rows_per_group rows as columns: out[g][k][r % rows_per_group]. */
HPS_API int hps_interp_rows(long long n_rows, int n_src, const double* to_pts, const double* src_pts,
                            const double* src_weights, double* out, int rows_per_group, int transposed, void* stream);

/* out[g][c] = in[g][idx[c]] for c < n_out (in: n_groups x n_in): the
 * reordering step of interp_to_hps (_interpolation_methods.py:23-340). */
HPS_API int hps_gather_cols(long long n_groups, int n_in, int n_out, const int* idx, const double* in, double* out,
                            void* stream);

/* Values at n_targets points (targets: (n_targets, dim)) of the piecewise
 * polynomial given by f (n_leaves, p^dim, nsrc) on the leaves' Chebyshev
 * grids (exterior-first order, rearrange: meshgrid index of each point).
 * Each target takes the first leaf in leaf order whose closed box
 * (leaf_bounds (n_leaves, 2 dim): min, max per axis) contains it, or leaf 0;
 * cells (n_cells[0] x .. x n_cells[dim-1], device) maps the finest cells of
 * the box at cell_origin with sizes cell_size (host arrays) to a leaf.
 * leaf_nodes / leaf_weights (n_leaves, dim, p): each axis' interpolation
 * nodes and barycentric weights.  out (n_targets, nsrc).  p <= 32. */
HPS_API int hps_interp_from_leaves(int dim, long long n_targets, int nsrc, const double* targets, int p,
                                   const double* leaf_bounds, const double* leaf_nodes, const double* leaf_weights,
                                   const int* rearrange, const int* cells, const int* n_cells,
                                   const double* cell_origin, const double* cell_size, const double* f, double* out,
                                   void* stream);

/* r32 = f[:, n_cb:, :] rounded to FP32 (the residual at zero).  Refinement
 * only: no counterpart in the reference. */
HPS_API int hps_interior_f32(long long n_leaves, int n_pts, int n_cb, int nsrc, const double* f, float* r32,
                             void* stream);

/* hcorr[node] = (flux[node] + flux[nbr[node]]) / 2 (0 where nbr < 0);
 * r_bdry[b] = g_given[b] - g_state[bdry_node[b]] (g_given NULL: zero data).
 * Node = leaf*4q + k.  Refinement only (the DtN interface equations that the
 * reference's merges eliminate): no counterpart in the reference. */
HPS_API int hps_flux_combine(long long n_nodes, int nsrc, const int* nbr, const double* flux, float* hcorr,
                             int n_bdry, const int* bdry_node, const double* g_given, const double* g_state,
                             float* r_bdry, void* stream);

/* y += x elementwise (x FP32, y FP64).  Refinement only: no counterpart in
 * the reference. */
HPS_API int hps_accumulate(long long n, const float* x, double* y, void* stream);

/* y += x as hps_accumulate, and out[0] = max |x|, out[1] = max |y| after the
 * update (per element, or per complex (re, im) pair when pairs != 0; n counts
 * FP32 values): the refinement loop's convergence test in the same pass.
 * out (2 doubles, device) is overwritten.  No counterpart in the reference. */
HPS_API int hps_accumulate_max(long long n, int pairs, const float* x, double* y, double* out, void* stream);


#ifdef __cplusplus
}
#endif

#endif /* JAXHPS_GB300_H */
