// Incremental refinement residual with the leaf-row residual held as an FP32
// pair (uniform 2D DtN leaves, q = p - 2).
//
// After the first FP64 residual, refinement keeps the residual current by
//     r_int -= (A du_full)_int,   flux += Q du_full,   du_full = [P dg ; du]
// with du, dg the FP32 corrections.  This kernel does the same arithmetic as
// jx_update_2d_kernel (double-float TwoProd / TwoSum on the FP32 pipe) but
//   * keeps r_int as two FP32 planes (hi, lo): the update needs no FP64
//     operation, and hi is the FP32 residual the next correction reads;
//   * evaluates the interior rows line by line: a thread holds one grid line
//     (p values of one right-hand side) in registers and forms the 1D
//     derivative at every interior point of it, with the differentiation
//     matrices read as warp-uniform (broadcast) shared-memory operands.  The
//     x-derivatives go through shared memory to the thread that owns the
//     point's y-line, which adds the y-derivatives and the zeroth-order term
//     and updates r in place.
// Grid values live in shared memory in meshgrid order (ix, iy; iy = 0 the
// north row) with a 16-float pad per x-line, so that the two lines a warp
// reads in either pass sit in different banks.
#include "df32.cuh"
#include "hps_common.cuh"
#include "hps_internal.h"

namespace hps {

namespace {

constexpr int DF_SC = 16;   // right-hand sides per CTA
constexpr int DF_NT = 256;

enum : int { KD_XX = 0, KD_XY = 1, KD_YY = 2, KD_X = 3, KD_Y = 4, KD_I = 5 };

template <int P, int Q>
struct DfLayout {
  static constexpr int PP = P * P, NCB = 4 * (P - 1), NI = PP - NCB, NQ = 4 * Q, NL = P - 2, NL2 = NL * NL;
  static constexpr int ULINE = P * DF_SC + 16;   // padded x-line of grid values
  static constexpr int ALINE = NL * DF_SC + 16;  // padded x-line of interior partial sums
};

template <int P, int Q>
size_t jx_df_smem(int n_ops, int need_uy) {
  using Lt = DfLayout<P, Q>;
  const size_t f = (size_t)P * Lt::ULINE                               // uh
                   + 4 * (size_t)P * DF_SC                              // boundary lo parts
                   + (need_uy ? 2 * (size_t)P * Lt::ULINE : 0)          // uy pairs
                   + 4 * (size_t)Lt::PP + 4 * (size_t)P * Q             // D1, D2, Pside, Qside pairs
                   + 2 * (size_t)n_ops * Lt::NL2                        // coefficient pairs
                   + 2 * (size_t)Lt::NL * Lt::ALINE                     // x-derivative partial sums (pairs)
                   + (size_t)Lt::NQ * DF_SC                             // dg
                   + 8 * (size_t)P * DF_SC;                             // normal derivatives (pairs)
  return f * sizeof(float) + (size_t)Lt::PP * sizeof(int);
}

// Floats of the per-solve table: the FP32 pairs of D1, D2, Pside, Qside, then
// per leaf the pairs of every operator's coefficient times its 1/h scaling.
template <int P, int Q>
constexpr size_t df_table_floats() {
  return 4 * (size_t)P * P + 4 * (size_t)P * Q;
}
template <int P, int Q>
size_t df_prep_floats(int n_leaves, int n_ops) {
  return df_table_floats<P, Q>() + (size_t)n_leaves * 2 * n_ops * (size_t)(P - 2) * (P - 2);
}

// (hs, he) += sum_j (dh + dl)[j] * v_j over one grid line whose values are
// FP32 except at the two ends, which carry the lo parts c0, c1
template <int P>
__device__ __forceinline__ void line_dot(float& hs, float& he, const float* dh, const float* dl, const float (&v)[P],
                                         float c0, float c1) {
  df_mac2(hs, he, dh[0], dl[0], v[0], c0);
#pragma unroll
  for (int j = 1; j < P - 1; ++j) df_mac1(hs, he, dh[j], dl[j], v[j]);
  df_mac2(hs, he, dh[P - 1], dl[P - 1], v[P - 1], c1);
}

// One CTA per leaf: its coefficient pairs in the interior meshgrid layout
// ((ix-1)*(P-2) + iy-1); CTA n_leaves: the operator pairs.  The only FP64
// arithmetic of the pair residual, done once per solve.
template <int P, int Q>
__global__ void __launch_bounds__(DF_NT)
jx_df_prep_kernel(int n_leaves, int n_ops, unsigned long long kinds, const double* __restrict__ coeffs,
                  const double* __restrict__ inv_half, const double* __restrict__ D1g,
                  const double* __restrict__ D2g, const double* __restrict__ Pside_g,
                  const double* __restrict__ Qside_g, const int* __restrict__ perm_g, float* __restrict__ prep) {
  constexpr int PP = P * P, NCB = 4 * (P - 1), NI = PP - NCB, NL = P - 2, NL2 = NL * NL;
  const int l = blockIdx.x;
  if (l == n_leaves) {
    float* d1h = prep;
    float* d1l = d1h + PP;
    float* d2h = d1l + PP;
    float* d2l = d2h + PP;
    float* psh = d2l + PP;
    float* psl = psh + P * Q;
    float* qsh = psl + P * Q;
    float* qsl = qsh + Q * P;
    for (int e = threadIdx.x; e < PP; e += DF_NT) {
      const df32 a = df_split(D1g[e]), b = df_split(D2g[e]);
      d1h[e] = a.hi;
      d1l[e] = a.lo;
      d2h[e] = b.hi;
      d2l[e] = b.lo;
    }
    for (int e = threadIdx.x; e < P * Q; e += DF_NT) {
      const df32 a = df_split(Pside_g[e]), b = df_split(Qside_g[e]);
      psh[e] = a.hi;
      psl[e] = a.lo;
      qsh[e] = b.hi;
      qsl[e] = b.lo;
    }
    return;
  }
  const double ih = inv_half[l];
  float* cfh = prep + df_table_floats<P, Q>() + (size_t)l * 2 * n_ops * NL2;
  float* cfl = cfh + n_ops * NL2;
  for (int e = threadIdx.x; e < n_ops * NI; e += DF_NT) {
    const int o = e / NI, i = e % NI;
    double scl;
    switch ((int)((kinds >> (4 * o)) & 15ull)) {
      case KD_XX:
      case KD_YY: scl = ih * ih; break;
      case KD_X:
      case KD_XY: scl = ih; break;
      case KD_Y: scl = -ih; break;
      default: scl = 1.0;
    }
    const int idx = perm_g[NCB + i];
    const int m = (idx / P - 1) * NL + (idx % P - 1);
    const df32 c = df_split(scl * coeffs[(long long)o * n_leaves * PP + (long long)l * PP + NCB + i]);
    cfh[o * NL2 + m] = c.hi;
    cfl[o * NL2 + m] = c.lo;
  }
}

template <int P, int Q>
__global__ void __launch_bounds__(DF_NT, 3)
jx_df_kernel(int n_leaves, int nsrc, int n_ops, unsigned long long kinds, const float* __restrict__ prep,
             const double* __restrict__ inv_half, const int* __restrict__ perm_g, const float* __restrict__ du,
             const float* __restrict__ dg, float* __restrict__ r_hi, float* __restrict__ r_lo,
             double* __restrict__ flux, int need_uy) {
  using Lt = DfLayout<P, Q>;
  constexpr int PP = Lt::PP, NCB = Lt::NCB, NI = Lt::NI, NQ = Lt::NQ, NL = Lt::NL, NL2 = Lt::NL2;
  constexpr int SC = DF_SC, UL = Lt::ULINE, AL = Lt::ALINE;
  extern __shared__ float smf[];
  float* uh = smf;                       // grid values (hi), P x-lines of UL
  float* lx0 = uh + P * UL;              // lo parts on the boundary: x = 0 line (by iy)
  float* lx1 = lx0 + P * SC;             //                           x = P-1 line
  float* ly0 = lx1 + P * SC;             //                           y = 0 line (by ix)
  float* ly1 = ly0 + P * SC;             //                           y = P-1 line
  float* uyh = ly1 + P * SC;             // D_xy only: the scaled y-derivative, pairs
  float* uyl = uyh + (need_uy ? P * UL : 0);
  float* d1h = uyl + (need_uy ? P * UL : 0);
  float* d1l = d1h + PP;
  float* d2h = d1l + PP;
  float* d2l = d2h + PP;
  float* psh = d2l + PP;
  float* psl = psh + P * Q;
  float* qsh = psl + P * Q;
  float* qsl = qsh + Q * P;
  float* cfh = qsl + Q * P;              // (n_ops, NL2) coefficient x scale, pairs
  float* cfl = cfh + n_ops * NL2;
  float* ah = cfl + n_ops * NL2;         // x-derivative partial sums, NL x-lines of AL
  float* al = ah + NL * AL;
  float* gs = al + NL * AL;              // (NQ, SC) Gauss boundary corrections
  float* ndh = gs + NQ * SC;             // (4P, SC) outward normal derivatives, pairs
  float* ndl = ndh + 4 * P * SC;
  int* perm = reinterpret_cast<int*>(ndl + 4 * P * SC);

  // the right-hand-side chunks of a leaf are consecutive blocks, so that they
  // run together and share each 256-byte row segment in L2
  const int nch = (nsrc + SC - 1) / SC;
  const long long l = blockIdx.x / nch;
  const int s0 = (int)(blockIdx.x % nch) * SC;
  const int sc = min(SC, nsrc - s0);
  const int tid = threadIdx.x;
  const df32 ihd = df_split(inv_half[l]), mihd = df32{-ihd.hi, -ihd.lo};

  // operator slot of each kind (-1: absent)
  int sxx = -1, sx = -1, sxy = -1, syy = -1, sy = -1, si = -1;
  for (int o = 0; o < n_ops; ++o) {
    switch ((int)((kinds >> (4 * o)) & 15ull)) {
      case KD_XX: sxx = o; break;
      case KD_XY: sxy = o; break;
      case KD_YY: syy = o; break;
      case KD_X: sx = o; break;
      case KD_Y: sy = o; break;
      default: si = o;
    }
  }

  // operator pairs (contiguous d1h .. qsl) and this leaf's coefficient pairs (cfh, cfl)
  for (int e = tid; e < (int)df_table_floats<P, Q>(); e += DF_NT) d1h[e] = prep[e];
  {
    const float* src = prep + df_table_floats<P, Q>() + (size_t)l * 2 * n_ops * NL2;
    for (int e = tid; e < 2 * n_ops * NL2; e += DF_NT) cfh[e] = src[e];
  }
  for (int e = tid; e < PP; e += DF_NT) perm[e] = perm_g[e];
  for (int e = tid; e < NQ * SC; e += DF_NT) {
    const int k = e / SC, s = e % SC;
    gs[e] = (s < sc) ? dg[(l * NQ + k) * nsrc + s0 + s] : 0.f;
  }
  for (int e = tid; e < 4 * P * SC; e += DF_NT) lx0[e] = 0.f;   // lx0, lx1, ly0, ly1
  __syncthreads();
  for (int e = tid; e < NI * SC; e += DF_NT) {
    const int i = e / SC, s = e % SC;
    const int idx = perm[NCB + i];
    uh[(idx / P) * UL + (idx % P) * SC + s] = (s < sc) ? du[(l * NI + i) * nsrc + s0 + s] : 0.f;
  }
  // Chebyshev boundary values P dg (pairs); corners average their two sides
  for (int e = tid; e < NCB * SC; e += DF_NT) {
    const int k = e / SC, s = e % SC;
    float hs = 0.f, he = 0.f;
    int cnt = 0;
#pragma unroll
    for (int side = 0; side < 4; ++side) {
      int t = k - side * (P - 1);
      if (side == 3 && k == 0) t = P - 1;
      if (t < 0 || t > P - 1) continue;
      if (side == 3 && t == P - 1 && k != 0) continue;
#pragma unroll
      for (int j = 0; j < Q; ++j) df_mac1(hs, he, psh[t * Q + j], psl[t * Q + j], gs[(side * Q + j) * SC + s]);
      ++cnt;
    }
    if (cnt == 2) {
      hs *= 0.5f;
      he *= 0.5f;
    }
    const df32 v = df_norm(hs, he);
    const int idx = perm[k];
    const int ix = idx / P, iy = idx % P;
    uh[ix * UL + iy * SC + s] = v.hi;
    if (ix == 0) lx0[iy * SC + s] = v.lo;
    if (ix == P - 1) lx1[iy * SC + s] = v.lo;
    if (iy == 0) ly0[ix * SC + s] = v.lo;
    if (iy == P - 1) ly1[ix * SC + s] = v.lo;
  }
  __syncthreads();
  // lo part of a grid value (zero at interior points)
  auto ulo = [&](int ix, int iy, int s) -> float {
    if (ix == 0) return lx0[iy * SC + s];
    if (ix == P - 1) return lx1[iy * SC + s];
    if (iy == 0) return ly0[ix * SC + s];
    if (iy == P - 1) return ly1[ix * SC + s];
    return 0.f;
  };
  if (need_uy) {
    for (int e = tid; e < PP * SC; e += DF_NT) {
      const int idx = e / SC, s = e % SC;
      const int ix = idx / P, iy = idx % P;
      float hs = 0.f, he = 0.f;
      for (int k = 0; k < P; ++k) df_mac2(hs, he, d1h[iy * P + k], d1l[iy * P + k], uh[ix * UL + k * SC + s], ulo(ix, k, s));
      const df32 v = df_mul(mihd, df_norm(hs, he));
      uyh[ix * UL + iy * SC + s] = v.hi;
      uyl[ix * UL + iy * SC + s] = v.lo;
    }
    __syncthreads();
  }

  // x-derivatives: thread (s, iy) holds the x-line u(., iy) of right-hand side
  // s; it also forms the E and W normal derivatives of that line.  The
  // threads without a line form the normal derivatives of the four boundary
  // lines meanwhile.
  if (tid < NL * SC) {
    const int s = tid % SC, iy = 1 + tid / SC;
    float col[P];
#pragma unroll
    for (int j = 0; j < P; ++j) col[j] = uh[j * UL + iy * SC + s];
    const float c0 = lx0[iy * SC + s], c1 = lx1[iy * SC + s];
#pragma unroll 2
    for (int ix = 1; ix <= P - 2; ++ix) {
      const int m = (ix - 1) * NL + (iy - 1);
      float as = 0.f, ae = 0.f;
      if (sxx >= 0) {
        float hs = 0.f, he = 0.f;
        line_dot<P>(hs, he, d2h + ix * P, d2l + ix * P, col, c0, c1);
        df_mac(as, ae, df32{cfh[sxx * NL2 + m], cfl[sxx * NL2 + m]}, df32{hs, he});
      }
      if (sx >= 0) {
        float hs = 0.f, he = 0.f;
        line_dot<P>(hs, he, d1h + ix * P, d1l + ix * P, col, c0, c1);
        df_mac(as, ae, df32{cfh[sx * NL2 + m], cfl[sx * NL2 + m]}, df32{hs, he});
      }
      if (sxy >= 0) {
        float hs = 0.f, he = 0.f;
        for (int j = 0; j < P; ++j)
          df_mac2(hs, he, d1h[ix * P + j], d1l[ix * P + j], uyh[j * UL + iy * SC + s], uyl[j * UL + iy * SC + s]);
        df_mac(as, ae, df32{cfh[sxy * NL2 + m], cfl[sxy * NL2 + m]}, df32{hs, he});
      }
      ah[(ix - 1) * AL + (iy - 1) * SC + s] = as;
      al[(ix - 1) * AL + (iy - 1) * SC + s] = ae;
    }
    {  // E: u_x on ix = P-1 at t = P-1-iy;  W: -u_x on ix = 0 at t = iy
      float hs = 0.f, he = 0.f;
      line_dot<P>(hs, he, d1h + (P - 1) * P, d1l + (P - 1) * P, col, c0, c1);
      df32 v = df_mul(ihd, df_norm(hs, he));
      ndh[(P + P - 1 - iy) * SC + s] = v.hi;
      ndl[(P + P - 1 - iy) * SC + s] = v.lo;
      hs = he = 0.f;
      line_dot<P>(hs, he, d1h, d1l, col, c0, c1);
      v = df_mul(mihd, df_norm(hs, he));
      ndh[(3 * P + iy) * SC + s] = v.hi;
      ndl[(3 * P + iy) * SC + s] = v.lo;
    }
  } else {
    // normal derivatives along the boundary lines (every value has a lo part):
    // S and N at t = 0, P-1 (y-lines x = 0, P-1); E and W at t = 0, P-1 (x-lines y = 0, P-1)
    for (int e = tid - NL * SC; e < 8 * SC; e += DF_NT - NL * SC) {
      const int c = e / SC, s = e % SC;
      const int side = c >> 1, t = (c & 1) ? P - 1 : 0;
      float hs = 0.f, he = 0.f;
      if (side == 0 || side == 2) {   // y-line u(ix, .) with ix = t (S) or P-1-t (N)
        const int ix = (side == 0) ? t : P - 1 - t;
        const float* lo = (ix == 0) ? lx0 : lx1;
        const float* dh = (side == 0) ? d1h + (P - 1) * P : d1h;
        const float* dl = (side == 0) ? d1l + (P - 1) * P : d1l;
#pragma unroll
        for (int k = 0; k < P; ++k) df_mac2(hs, he, dh[k], dl[k], uh[ix * UL + k * SC + s], lo[k * SC + s]);
      } else {                        // x-line u(., iy) with iy = P-1-t (E) or t (W)
        const int iy = (side == 1) ? P - 1 - t : t;
        const float* lo = (iy == 0) ? ly0 : ly1;
        const float* dh = (side == 1) ? d1h + (P - 1) * P : d1h;
        const float* dl = (side == 1) ? d1l + (P - 1) * P : d1l;
#pragma unroll
        for (int j = 0; j < P; ++j) df_mac2(hs, he, dh[j], dl[j], uh[j * UL + iy * SC + s], lo[j * SC + s]);
      }
      const df32 v = df_mul(side < 2 ? ihd : mihd, df_norm(hs, he));
      ndh[(side * P + t) * SC + s] = v.hi;
      ndl[(side * P + t) * SC + s] = v.lo;
    }
  }
  __syncthreads();
  // y-derivatives and the zeroth-order term: thread (s, ix) holds the
  // y-line u(ix, .), completes every interior row of it and updates r; it
  // also forms the S and N normal derivatives of that line
  if (tid < NL * SC) {
    const int s = tid % SC, ix = 1 + tid / SC;
    float row[P];
#pragma unroll
    for (int j = 0; j < P; ++j) row[j] = uh[ix * UL + j * SC + s];
    const float c0 = ly0[ix * SC + s], c1 = ly1[ix * SC + s];
#pragma unroll 2
    for (int iy = 1; iy <= P - 2; ++iy) {
      const int m = (ix - 1) * NL + (iy - 1);
      float as = ah[(ix - 1) * AL + (iy - 1) * SC + s];
      float ae = al[(ix - 1) * AL + (iy - 1) * SC + s];
      if (syy >= 0) {
        float hs = 0.f, he = 0.f;
        line_dot<P>(hs, he, d2h + iy * P, d2l + iy * P, row, c0, c1);
        df_mac(as, ae, df32{cfh[syy * NL2 + m], cfl[syy * NL2 + m]}, df32{hs, he});
      }
      if (sy >= 0) {
        float hs = 0.f, he = 0.f;
        line_dot<P>(hs, he, d1h + iy * P, d1l + iy * P, row, c0, c1);
        df_mac(as, ae, df32{cfh[sy * NL2 + m], cfl[sy * NL2 + m]}, df32{hs, he});
      }
      if (si >= 0) df_mac1(as, ae, cfh[si * NL2 + m], cfl[si * NL2 + m], uh[ix * UL + iy * SC + s]);
      ah[(ix - 1) * AL + (iy - 1) * SC + s] = as;
      al[(ix - 1) * AL + (iy - 1) * SC + s] = ae;
    }
    {  // S: -u_y on iy = P-1 at t = ix;  N: u_y on iy = 0 at t = P-1-ix
      float hs = 0.f, he = 0.f;
      line_dot<P>(hs, he, d1h + (P - 1) * P, d1l + (P - 1) * P, row, c0, c1);
      df32 v = df_mul(ihd, df_norm(hs, he));
      ndh[ix * SC + s] = v.hi;
      ndl[ix * SC + s] = v.lo;
      hs = he = 0.f;
      line_dot<P>(hs, he, d1h, d1l, row, c0, c1);
      v = df_mul(mihd, df_norm(hs, he));
      ndh[(2 * P + P - 1 - ix) * SC + s] = v.hi;
      ndl[(2 * P + P - 1 - ix) * SC + s] = v.lo;
    }
  }
  __syncthreads();
  // r -= (A du)_int, coalesced over (interior point, right-hand side), with
  // many independent loads in flight per thread
  for (int e = tid; e < NI * SC; e += DF_NT) {
    const int i = e / SC, s = e % SC;
    if (s >= sc) continue;
    const int idx = perm[NCB + i];
    const int a = (idx / P - 1) * AL + (idx % P - 1) * SC + s;
    const long long o = ((long long)l * NI + i) * nsrc + s0 + s;
    const df32 r = df_sub(r_hi[o], r_lo[o], ah[a], al[a]);
    r_hi[o] = r.hi;
    r_lo[o] = r.lo;
  }
  // flux at the Gauss nodes: Q applied to each side's normal derivatives
  for (int e = tid; e < NQ * SC; e += DF_NT) {
    const int k = e / SC, s = e % SC;
    if (s >= sc) continue;
    const int side = k / Q, j = k % Q;
    float hs = 0.f, he = 0.f;
#pragma unroll
    for (int t = 0; t < P; ++t)
      df_mac2(hs, he, qsh[j * P + t], qsl[j * P + t], ndh[(side * P + t) * SC + s], ndl[(side * P + t) * SC + s]);
    flux[((long long)l * NQ + k) * nsrc + s0 + s] += df_join(hs, he);
  }
}

template <int P, int Q>
cudaError_t launch_jx_df_prep(int n_leaves, int n_ops, unsigned long long kinds, const double* coeffs,
                              const double* inv_half, const double* D1, const double* D2, const double* Pside,
                              const double* Qside, const int* perm, float* prep, cudaStream_t st) {
  note_launch();
  jx_df_prep_kernel<P, Q><<<n_leaves + 1, DF_NT, 0, st>>>(n_leaves, n_ops, kinds, coeffs, inv_half, D1, D2, Pside,
                                                          Qside, perm, prep);
  return cudaGetLastError();
}

template <int P, int Q>
cudaError_t launch_jx_df(int n_leaves, int nsrc, int n_ops, unsigned long long kinds, const float* prep,
                         const double* inv_half, const int* perm, const float* du, const float* dg, float* r_hi,
                         float* r_lo, double* flux, int need_uy, cudaStream_t st) {
  const size_t smem = jx_df_smem<P, Q>(n_ops, need_uy);
  cudaError_t e = cudaFuncSetAttribute(jx_df_kernel<P, Q>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const long long nblk = (long long)n_leaves * ((nsrc + DF_SC - 1) / DF_SC);
  if (nblk > 2147483647ll) return cudaErrorInvalidValue;
  const unsigned grid = (unsigned)nblk;
  // algorithmic bytes: du, dg, the residual pair read and written, the flux
  // (FP64) read and written, this leaf's coefficient pairs
  constexpr int NI = P * P - 4 * (P - 1), NQ = 4 * Q, NL2 = (P - 2) * (P - 2);
  const double bytes = (double)n_leaves * ((double)nsrc * (4.0 * NI + 4.0 * NQ + 16.0 * NI + 16.0 * NQ) +
                                           8.0 * n_ops * NL2);
  ProfScope ps(KC_RESIDUAL_DF, st, bytes);
  note_launch();
  jx_df_kernel<P, Q><<<grid, DF_NT, smem, st>>>(n_leaves, nsrc, n_ops, kinds, prep, inv_half, perm, du, dg, r_hi,
                                                r_lo, flux, need_uy);
  return cudaGetLastError();
}

}  // namespace

bool jx_df_supported(int p, int q) {
  return q == p - 2 && (p == 8 || p == 10 || p == 12 || p == 14 || p == 16);
}

size_t jx_df_prep_floats(int n_leaves, int p, int q, int n_ops) {
#define HPS_JX_DF(PV) \
  if (p == PV && q == PV - 2) return df_prep_floats<PV, PV - 2>(n_leaves, n_ops);
  HPS_JX_DF(8)
  HPS_JX_DF(10)
  HPS_JX_DF(12)
  HPS_JX_DF(14)
  HPS_JX_DF(16)
#undef HPS_JX_DF
  return 0;
}

cudaError_t jx_df_prepare(int n_leaves, int p, int q, int n_ops, unsigned long long kinds, const double* coeffs,
                          const double* inv_half, const double* D1, const double* D2, const double* Pside,
                          const double* Qside, const int* perm, float* prep, cudaStream_t st) {
#define HPS_JX_DF(PV)                                                                                         \
  if (p == PV && q == PV - 2)                                                                                 \
    return launch_jx_df_prep<PV, PV - 2>(n_leaves, n_ops, kinds, coeffs, inv_half, D1, D2, Pside, Qside, perm, \
                                         prep, st);
  HPS_JX_DF(8)
  HPS_JX_DF(10)
  HPS_JX_DF(12)
  HPS_JX_DF(14)
  HPS_JX_DF(16)
#undef HPS_JX_DF
  return cudaErrorInvalidValue;
}

cudaError_t jx_df_update_2d(int n_leaves, int p, int q, int nsrc, int n_ops, unsigned long long kinds,
                            const float* prep, const double* inv_half, const int* perm, const float* du,
                            const float* dg, float* r_hi, float* r_lo, double* flux, int need_uy, cudaStream_t st) {
#define HPS_JX_DF(PV)                                                                                             \
  if (p == PV && q == PV - 2)                                                                                     \
    return launch_jx_df<PV, PV - 2>(n_leaves, nsrc, n_ops, kinds, prep, inv_half, perm, du, dg, r_hi, r_lo, flux, \
                                    need_uy, st);
  HPS_JX_DF(8)
  HPS_JX_DF(10)
  HPS_JX_DF(12)
  HPS_JX_DF(14)
  HPS_JX_DF(16)
#undef HPS_JX_DF
  return cudaErrorInvalidValue;
}

// ---------------------------------------------------------------------------
// The refined solution's interior values as an FP32 pair (hi, lo): the
// corrections are accumulated by TwoSum on the FP32 pipe (the FP64 version
// spends its time on the 1/64-rate FP64 add and conversion), with the
// convergence maxima max |dx| and max |x| (of hi) as integer bit patterns.
// ---------------------------------------------------------------------------
__global__ void accumulate_pair_max_kernel(long long n, const float4* __restrict__ x, float4* hi, float4* lo,
                                           unsigned long long* out) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __shared__ unsigned int sx[32], sy[32];
  unsigned int bx = 0, by = 0;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += stride) {
    const float4 d = x[e];
    float4 h = hi[e], l = lo[e];
    const float dv[4] = {d.x, d.y, d.z, d.w};
    float hv[4] = {h.x, h.y, h.z, h.w}, lv[4] = {l.x, l.y, l.z, l.w};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const float t = hv[j] + dv[j];
      const float bb = t - hv[j];
      const float err = (hv[j] - (t - bb)) + (dv[j] - bb);
      const df32 r = df_norm(t, lv[j] + err);
      hv[j] = r.hi;
      lv[j] = r.lo;
      bx = max(bx, __float_as_uint(dv[j]) & 0x7fffffffu);
      by = max(by, __float_as_uint(r.hi) & 0x7fffffffu);
    }
    hi[e] = make_float4(hv[0], hv[1], hv[2], hv[3]);
    lo[e] = make_float4(lv[0], lv[1], lv[2], lv[3]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    bx = max(bx, __shfl_xor_sync(0xffffffffu, bx, o));
    by = max(by, __shfl_xor_sync(0xffffffffu, by, o));
  }
  if (lane == 0) {
    sx[warp] = bx;
    sy[warp] = by;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned int ax = sx[0], ay = sy[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
      ax = max(ax, sx[w]);
      ay = max(ay, sy[w]);
    }
    // as FP64 bit patterns, the layout the FP64 version reports
    atomicMax(out, (unsigned long long)__double_as_longlong((double)__uint_as_float(ax)));
    atomicMax(out + 1, (unsigned long long)__double_as_longlong((double)__uint_as_float(ay)));
  }
}

cudaError_t accumulate_pair_max(long long n, const float* x, float* hi, float* lo, double* out, cudaStream_t st) {
  if (n % 4 || (reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(hi) | reinterpret_cast<uintptr_t>(lo)) & 15)
    return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(out, 0, 2 * sizeof(double), st);
  if (e != cudaSuccess) return e;
  long long g = (n / 4 + 255) / 256;
  if (g > 8192) g = 8192;
  if (g < 1) g = 1;
  ProfScope ps(KC_MOVE, st, 20.0 * (double)n);
  note_launch();
  accumulate_pair_max_kernel<<<(int)g, 256, 0, st>>>(n / 4, reinterpret_cast<const float4*>(x),
                                                     reinterpret_cast<float4*>(hi), reinterpret_cast<float4*>(lo),
                                                     reinterpret_cast<unsigned long long*>(out));
  return cudaGetLastError();
}

// u_full[l][k] = (P g)[k] on the Chebyshev boundary and hi + lo on the
// interior (FP64), exterior-first leaf order.  One CTA per leaf.  The
// interior is the exact FP64 sum of the pair (contiguous, no index
// arithmetic).  The boundary interpolation (q terms per side and point, two
// sides at the corners) runs in double-float on the FP32 pipe: P's pairs are
// staged once per CTA and the leaf's boundary data once per chunk of sc
// right-hand sides, so each FP64 input is split once instead of once per
// product (relative error about 2^-46 of sum |P||g|, against the FP64 pipe's
// 1/64 rate for q multiply-adds per point).
__global__ void assemble_u_pair_2d_kernel(int n_leaves, int p, int q, int nsrc, int sc,
                                          const double* __restrict__ Pside, const float* __restrict__ u_hi,
                                          const float* __restrict__ u_lo, const double* __restrict__ g,
                                          double* u_full) {
  extern __shared__ df32 au_smem[];
  df32* Pp = au_smem;            // [p][q]
  df32* gp = au_smem + p * q;    // [4q][sc]
  const int pp = p * p, ncb = 4 * (p - 1), ni = pp - ncb, nq = 4 * q;
  const long long l = blockIdx.x;
  for (int e = threadIdx.x; e < p * q; e += blockDim.x) Pp[e] = df_split(Pside[e]);
  {
    const float* hl = u_hi + l * ni * (long long)nsrc;
    const float* ll = u_lo + l * ni * (long long)nsrc;
    double* out = u_full + (l * pp + ncb) * (long long)nsrc;
    for (int e = threadIdx.x; e < ni * nsrc; e += blockDim.x) out[e] = (double)hl[e] + (double)ll[e];
  }
  for (int s0 = 0; s0 < nsrc; s0 += sc) {
    const int ns = min(sc, nsrc - s0);
    __syncthreads();   // P staged; the previous chunk's readers are done with gp
    for (int e = threadIdx.x; e < nq * ns; e += blockDim.x) {
      const int b = e / ns, s = e - b * ns;
      gp[b * sc + s] = df_split(g[(l * nq + b) * nsrc + s0 + s]);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < ncb * ns; e += blockDim.x) {
      const int k = e / ns, s = e - k * ns;
      float sh = 0.f, se = 0.f;
      int cnt = 0;
      for (int side = 0; side < 4; ++side) {
        int t = k - side * (p - 1);
        if (side == 3 && k == 0) t = p - 1;
        if (t < 0 || t > p - 1) continue;
        if (side == 3 && t == p - 1 && k != 0) continue;
        const df32* pr = Pp + t * q;
        const df32* gc = gp + side * q * sc + s;
        for (int j = 0; j < q; ++j) df_mac(sh, se, pr[j], gc[j * sc]);
        ++cnt;
      }
      const double v = df_join(sh, se);
      u_full[(l * pp + k) * (long long)nsrc + s0 + s] = (cnt == 2) ? 0.5 * v : v;
    }
  }
}

cudaError_t assemble_u_pair_2d(int n_leaves, int p, int q, int nsrc, const double* Pside, const float* u_hi,
                               const float* u_lo, const double* g, double* u_full, cudaStream_t st) {
  // right-hand sides per chunk: up to 32, fewer when P and the chunk's
  // boundary data would not fit 160 KB of shared memory
  const size_t budget = 160 * 1024, pbytes = sizeof(df32) * (size_t)p * q;
  if (pbytes + sizeof(df32) * 4 * (size_t)q > budget) return cudaErrorNotSupported;
  int sc = nsrc < 32 ? nsrc : 32;
  while (sc > 1 && pbytes + sizeof(df32) * 4 * (size_t)q * sc > budget) sc >>= 1;
  const size_t smem = pbytes + sizeof(df32) * 4 * (size_t)q * sc;
  if (smem > 48 * 1024) {
    const cudaError_t e = cudaFuncSetAttribute(assemble_u_pair_2d_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)smem);
    if (e != cudaSuccess) return e;
  }
  ProfScope ps(KC_MOVE, st, 8.0 * n_leaves * (double)p * p * nsrc * 2.0);
  note_launch();
  assemble_u_pair_2d_kernel<<<n_leaves, 256, smem, st>>>(n_leaves, p, q, nsrc, sc, Pside, u_hi, u_lo, g, u_full);
  return cudaGetLastError();
}

}  // namespace hps
