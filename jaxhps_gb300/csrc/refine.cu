// FP64 residual of the discrete HPS system and the bookkeeping kernels of
// mixed-precision iterative refinement.
//
// The HPS direct solver (leaf solves, merges, down pass) solves, for every
// leaf, the collocation equations at the interior Chebyshev points
//     A_ii u_int + A_ie (P g) = f_int                       (leaf rows)
// together with continuity of the outward normal derivative (Q u) across
// every interior interface Gauss node and the Dirichlet data on the domain
// boundary.  With the solver operators built in FP32, refinement iterates
//     r = b - J x   (FP64, this file),   x += HPS_fp32(r)
// until x is the FP64 discrete solution.  The residual uses the tensor
// structure of the spectral operators: derivatives are 1D Chebyshev
// differentiation along one grid axis (p MACs per point and operator)
// instead of dense p^2 x p^2 products.
#include "df32.cuh"
#include "hps_common.cuh"
#include "hps_internal.h"

namespace hps {

// op kinds (2D), matching the reference's coefficient stacking order
// (local_solve/_uniform_2D_DtN.py:59-68)
enum OpKind2D : int { OP_XX = 0, OP_XY = 1, OP_YY = 2, OP_X = 3, OP_Y = 4, OP_I = 5 };

constexpr int RES_SC = 16;   // right-hand sides per CTA
constexpr int RES_NT = 256;

// One CTA per (leaf, chunk of RES_SC right-hand sides).
// Grid values are kept in shared memory in the natural meshgrid layout
// u[(ix*p + iy)*RES_SC + s]  (iy = 0 is the north row, y decreasing).
__global__ void __launch_bounds__(RES_NT)
residual_2d_kernel(int n_leaves, int p, int q, int nsrc, int n_ops, unsigned long long kinds,
                   const double* __restrict__ coeffs, const double* __restrict__ inv_half,
                   const double* __restrict__ D1g, const double* __restrict__ D2g,
                   const double* __restrict__ Pside_g, const double* __restrict__ Qside_g,
                   const int* __restrict__ perm_g, const double* __restrict__ u_int,
                   const double* __restrict__ g, const double* __restrict__ f, float* r_int, double* r_int64,
                   float* r_lo, double* flux, double* u_full, int need_uy, const float* __restrict__ u_int32) {
  extern __shared__ double sm[];
  const int pp = p * p;
  const int ncb = 4 * (p - 1);
  const int ni = pp - ncb;
  const int nq = 4 * q;
  double* u = sm;                         // pp * SC
  double* uy = u + pp * RES_SC;           // pp * SC (only when D_xy is active)
  double* gs = uy + (need_uy ? pp * RES_SC : 0);  // nq * SC
  double* nd = gs + nq * RES_SC;          // 4p * SC
  double* D1 = nd + 4 * p * RES_SC;       // p*p
  double* D2 = D1 + pp;                   // p*p
  double* Ps = D2 + pp;                   // p*q
  double* Qs = Ps + p * q;                // q*p
  int* perm = reinterpret_cast<int*>(Qs + q * p);  // pp

  // the right-hand-side chunks of a leaf are consecutive blocks (shared L2 rows)
  const int nch = (nsrc + RES_SC - 1) / RES_SC;
  const long long l = blockIdx.x / nch;
  const int s0 = (int)(blockIdx.x % nch) * RES_SC;
  const int sc = min(RES_SC, nsrc - s0);
  const int tid = threadIdx.x;
  const double ih = inv_half[l];
  const double ih2 = ih * ih;

  for (int e = tid; e < pp; e += RES_NT) {
    D1[e] = D1g[e];
    D2[e] = D2g[e];
    perm[e] = perm_g[e];
  }
  for (int e = tid; e < p * q; e += RES_NT) {
    Ps[e] = Pside_g[e];
    Qs[e] = Qside_g[e];
  }
  for (int e = tid; e < nq * RES_SC; e += RES_NT) {
    const int k = e / RES_SC, s = e % RES_SC;
    gs[e] = (s < sc) ? g[(l * nq + k) * nsrc + s0 + s] : 0.0;
  }
  __syncthreads();
  // interior values
  for (int e = tid; e < ni * RES_SC; e += RES_NT) {
    const int i = e / RES_SC, s = e % RES_SC;
    const long long o = (l * ni + i) * nsrc + s0 + s;
    u[perm[ncb + i] * RES_SC + s] = (s < sc) ? (u_int32 ? (double)u_int32[o] : u_int[o]) : 0.0;
  }
  // Chebyshev boundary values u_b = P g: side t-th point interpolated from
  // the side's q Gauss values; the four corners average their two sides
  // (_precompute_operators_2D.py:48-79).
  for (int e = tid; e < ncb * RES_SC; e += RES_NT) {
    const int k = e / RES_SC, s = e % RES_SC;
    double acc = 0.0;
    int cnt = 0;
#pragma unroll
    for (int side = 0; side < 4; ++side) {
      int t = k - side * (p - 1);
      if (side == 3 && k == 0) t = p - 1;
      if (t < 0 || t > p - 1) continue;
      if (side == 3 && t == p - 1 && k != 0) continue;
      double v = 0.0;
      for (int j = 0; j < q; ++j) v = fma(Ps[t * q + j], gs[(side * q + j) * RES_SC + s], v);
      acc += v;
      ++cnt;
    }
    u[perm[k] * RES_SC + s] = (cnt == 2) ? 0.5 * acc : acc;
  }
  __syncthreads();
  if (need_uy) {
    for (int e = tid; e < pp * RES_SC; e += RES_NT) {
      const int idx = e / RES_SC, s = e % RES_SC;
      const int ix = idx / p, iy = idx % p;
      double v = 0.0;
      for (int k = 0; k < p; ++k) v = fma(D1[iy * p + k], u[(ix * p + k) * RES_SC + s], v);
      uy[e] = -ih * v;
    }
    __syncthreads();
  }
  // leaf rows: r = f - sum_o c_o * (D_o u) at the interior points
  for (int e = tid; e < ni * RES_SC; e += RES_NT) {
    const int i = e / RES_SC, s = e % RES_SC;
    if (s >= sc) continue;
    const int idx = perm[ncb + i];
    const int ix = idx / p, iy = idx % p;
    const long long pt = (long long)l * pp + ncb + i;
    double acc = f ? f[pt * nsrc + s0 + s] : 0.0;
    for (int o = 0; o < n_ops; ++o) {
      const double c = coeffs[(long long)o * n_leaves * pp + pt];
      double fld = 0.0;
      switch ((int)((kinds >> (4 * o)) & 15ull)) {
        case OP_XX:
          for (int j = 0; j < p; ++j) fld = fma(D2[ix * p + j], u[(j * p + iy) * RES_SC + s], fld);
          fld *= ih2;
          break;
        case OP_YY:
          for (int j = 0; j < p; ++j) fld = fma(D2[iy * p + j], u[(ix * p + j) * RES_SC + s], fld);
          fld *= ih2;
          break;
        case OP_X:
          for (int j = 0; j < p; ++j) fld = fma(D1[ix * p + j], u[(j * p + iy) * RES_SC + s], fld);
          fld *= ih;
          break;
        case OP_Y:
          for (int j = 0; j < p; ++j) fld = fma(D1[iy * p + j], u[(ix * p + j) * RES_SC + s], fld);
          fld *= -ih;
          break;
        case OP_XY:
          for (int j = 0; j < p; ++j) fld = fma(D1[ix * p + j], uy[(j * p + iy) * RES_SC + s], fld);
          fld *= ih;
          break;
        default:
          fld = u[idx * RES_SC + s];
      }
      acc = fma(-c, fld, acc);
    }
    const long long o = ((long long)l * ni + i) * nsrc + s0 + s;
    const float rh = (float)acc;
    r_int[o] = rh;
    if (r_int64) r_int64[o] = acc;
    if (r_lo) r_lo[o] = (float)(acc - (double)rh);   // the residual as an FP32 pair
  }
  // outward normal derivatives at the Chebyshev points of each side
  // (rows of N, _precompute_operators_2D.py:132-163):
  //  S: -u_y on iy=p-1 (W->E)   E: u_x on ix=p-1 (S->N)
  //  N:  u_y on iy=0   (E->W)   W: -u_x on ix=0  (N->S)
  for (int e = tid; e < 4 * p * RES_SC; e += RES_NT) {
    const int st = e / RES_SC, s = e % RES_SC;
    const int side = st / p, t = st % p;
    double v = 0.0;
    if (side == 0) {
      for (int k = 0; k < p; ++k) v = fma(D1[(p - 1) * p + k], u[(t * p + k) * RES_SC + s], v);
      v *= ih;  // -u_y = +ih * sum D1[iy=p-1][k] u
    } else if (side == 1) {
      const int iy = p - 1 - t;
      for (int j = 0; j < p; ++j) v = fma(D1[(p - 1) * p + j], u[(j * p + iy) * RES_SC + s], v);
      v *= ih;
    } else if (side == 2) {
      const int ix = p - 1 - t;
      for (int k = 0; k < p; ++k) v = fma(D1[k], u[(ix * p + k) * RES_SC + s], v);
      v *= -ih;
    } else {
      const int iy = t;
      for (int j = 0; j < p; ++j) v = fma(D1[j], u[(j * p + iy) * RES_SC + s], v);
      v *= -ih;
    }
    nd[e] = v;
  }
  __syncthreads();
  for (int e = tid; e < nq * RES_SC; e += RES_NT) {
    const int k = e / RES_SC, s = e % RES_SC;
    if (s >= sc) continue;
    const int side = k / q, j = k % q;
    double v = 0.0;
    for (int t = 0; t < p; ++t) v = fma(Qs[j * p + t], nd[(side * p + t) * RES_SC + s], v);
    flux[((long long)l * nq + k) * nsrc + s0 + s] = v;
  }
  if (u_full) {
    for (int e = tid; e < pp * RES_SC; e += RES_NT) {
      const int k = e / RES_SC, s = e % RES_SC;
      if (s < sc) u_full[((long long)l * pp + k) * nsrc + s0 + s] = u[perm[k] * RES_SC + s];
    }
  }
}

size_t residual_2d_smem(int p, int q, int need_uy) {
  const int pp = p * p;
  size_t d = (size_t)pp * RES_SC * (need_uy ? 2 : 1) + (size_t)4 * q * RES_SC + (size_t)4 * p * RES_SC +
             2 * (size_t)pp + 2 * (size_t)p * q;
  return d * sizeof(double) + (size_t)pp * sizeof(int);
}

cudaError_t residual_2d(int n_leaves, int p, int q, int nsrc, int n_ops, unsigned long long kinds, const double* coeffs,
                        const double* inv_half, const double* D1, const double* D2, const double* Pside,
                        const double* Qside, const int* perm, const double* u_int, const double* g,
                        const double* f, float* r_int, double* r_int64, float* r_lo, double* flux, double* u_full,
                        int need_uy, cudaStream_t st, const float* u_int32) {
  const size_t smem = residual_2d_smem(p, q, need_uy);
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(residual_2d_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const long long nblk = (long long)n_leaves * ((nsrc + RES_SC - 1) / RES_SC);
  if (nblk > 2147483647ll) return cudaErrorInvalidValue;
  const unsigned grid = (unsigned)nblk;
  const double work = 2.0 * n_leaves * (double)nsrc * (p * p * (double)p * (n_ops + 2) + 8.0 * p * q);
  ProfScope ps(KC_RESIDUAL, st, work);
  note_launch();
  residual_2d_kernel<<<grid, RES_NT, smem, st>>>(n_leaves, p, q, nsrc, n_ops, kinds, coeffs, inv_half, D1, D2,
                                                 Pside, Qside, perm, u_int, g, f, r_int, r_int64, r_lo, flux,
                                                 u_full, need_uy, u_int32);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// ItI residual (complex128).  Unknowns per leaf: u at all p^2 points
// (exterior-first order) and the incoming impedance t_in at the 4q Gauss
// nodes.  The leaf system of get_ItI (local_solve/_uniform_2D_ItI.py:120-186)
// is B u = [P t_in ; f_int] with B = [G ; A_int], G = N~ + i eta I the
// incoming impedance at the Chebyshev boundary points
// (_precompute_operators_2D.py:243-265).  Written here:
//   r[k]      = (P t_in)[k] - (u_n + i eta u)(k)        k < 4(p-1)
//   r[ncb+i]  = f_int[i] - sum_o c_o (D_o u)(i)
//   t_out[j]  = Q (u_n - i eta u)   at the Gauss nodes (QH u,
//               _precompute_operators_2D.py:195-240)
// r is rounded to complex64 (the input of the complex64 correction); t_out
// stays complex128 for the interface equations.  Same tensor-product
// evaluation as residual_2d: derivatives act along one grid axis.
// ---------------------------------------------------------------------------
template <bool CPLX>
__global__ void __launch_bounds__(RES_NT)
residual_iti_2d_kernel(int n_leaves, int p, int q, int nsrc, int SC, int n_ops, unsigned long long kinds,
                       double eta, const void* __restrict__ coeffs_v, const double* __restrict__ inv_half,
                       const double* __restrict__ D1g, const double* __restrict__ D2g,
                       const double* __restrict__ Pside_g, const double* __restrict__ Qside_g,
                       const int* __restrict__ perm_g, const double2* __restrict__ u_g,
                       const double2* __restrict__ tin_g, const double2* __restrict__ f, float2* __restrict__ r,
                       double2* __restrict__ t_out, int need_uy) {
  extern __shared__ double sm[];
  const int pp = p * p;
  const int m = p - 1;
  const int ncb = 4 * m;
  const int ni = pp - ncb;
  const int nq = 4 * q;
  double2* u = reinterpret_cast<double2*>(sm);          // pp * SC (meshgrid layout)
  double2* uy = u + pp * SC;                            // pp * SC when D_xy is active
  double2* ts = uy + (need_uy ? pp * SC : 0);           // nq * SC
  double2* nd = ts + nq * SC;                           // 4p * SC
  double* D1 = reinterpret_cast<double*>(nd + 4 * p * SC);
  double* D2 = D1 + pp;
  double* Ps = D2 + pp;
  double* Qs = Ps + p * q;
  int* perm = reinterpret_cast<int*>(Qs + q * p);

  // the right-hand-side chunks of a leaf are consecutive blocks (shared L2 rows)
  const int nch = (nsrc + SC - 1) / SC;
  const long long l = blockIdx.x / nch;
  const int s0 = (int)(blockIdx.x % nch) * SC;
  const int sc = min(SC, nsrc - s0);
  const int tid = threadIdx.x;
  const double ih = inv_half[l];
  const double ih2 = ih * ih;
  for (int e = tid; e < pp; e += RES_NT) {
    D1[e] = D1g[e];
    D2[e] = D2g[e];
    perm[e] = perm_g[e];
  }
  for (int e = tid; e < p * q; e += RES_NT) {
    Ps[e] = Pside_g[e];
    Qs[e] = Qside_g[e];
  }
  for (int e = tid; e < nq * SC; e += RES_NT) {
    const int k = e / SC, s = e % SC;
    ts[e] = (s < sc) ? tin_g[(l * nq + k) * nsrc + s0 + s] : make_double2(0.0, 0.0);
  }
  __syncthreads();
  for (int e = tid; e < pp * SC; e += RES_NT) {
    const int k = e / SC, s = e % SC;
    u[perm[k] * SC + s] = (s < sc) ? u_g[(l * pp + k) * nsrc + s0 + s] : make_double2(0.0, 0.0);
  }
  __syncthreads();
  if (need_uy) {
    for (int e = tid; e < pp * SC; e += RES_NT) {
      const int idx = e / SC, s = e % SC;
      const int ix = idx / p, iy = idx % p;
      double2 v = make_double2(0.0, 0.0);
      for (int k = 0; k < p; ++k) {
        const double d = D1[iy * p + k];
        const double2 w = u[(ix * p + k) * SC + s];
        v.x = fma(d, w.x, v.x);
        v.y = fma(d, w.y, v.y);
      }
      uy[e] = make_double2(-ih * v.x, -ih * v.y);
    }
    __syncthreads();
  }
  // PDE rows
  for (int e = tid; e < ni * SC; e += RES_NT) {
    const int i = e / SC, s = e % SC;
    if (s >= sc) continue;
    const int idx = perm[ncb + i];
    const int ix = idx / p, iy = idx % p;
    const long long pt = (long long)l * pp + ncb + i;
    double2 acc = f ? f[pt * nsrc + s0 + s] : make_double2(0.0, 0.0);
    for (int o = 0; o < n_ops; ++o) {
      double2 fld = make_double2(0.0, 0.0);
      const double2* src = u;
      int base = 0, stride = 0;
      const double* Dm = D1;
      double fac = 1.0;
      bool ident = false;
      switch ((int)((kinds >> (4 * o)) & 15ull)) {
        case OP_XX: Dm = D2 + ix * p; base = iy; stride = p; fac = ih2; break;
        case OP_YY: Dm = D2 + iy * p; base = ix * p; stride = 1; fac = ih2; break;
        case OP_X:  Dm = D1 + ix * p; base = iy; stride = p; fac = ih; break;
        case OP_Y:  Dm = D1 + iy * p; base = ix * p; stride = 1; fac = -ih; break;
        case OP_XY: Dm = D1 + ix * p; base = iy; stride = p; fac = ih; src = uy; break;
        default: ident = true;
      }
      if (ident) {
        fld = u[idx * SC + s];
      } else {
        for (int j = 0; j < p; ++j) {
          const double2 w = src[(base + j * stride) * SC + s];
          fld.x = fma(Dm[j], w.x, fld.x);
          fld.y = fma(Dm[j], w.y, fld.y);
        }
        fld.x *= fac;
        fld.y *= fac;
      }
      double cr, ci = 0.0;
      if (CPLX) {
        const double2 c = reinterpret_cast<const double2*>(coeffs_v)[(long long)o * n_leaves * pp + pt];
        cr = c.x;
        ci = c.y;
      } else {
        cr = reinterpret_cast<const double*>(coeffs_v)[(long long)o * n_leaves * pp + pt];
      }
      acc.x -= cr * fld.x - ci * fld.y;
      acc.y -= cr * fld.y + ci * fld.x;
    }
    r[((long long)l * pp + ncb + i) * nsrc + s0 + s] = make_float2((float)acc.x, (float)acc.y);
  }
  // outward normal derivative at the p points of each side:
  //  S: -u_y on iy=p-1 (W->E)   E: u_x on ix=p-1 (S->N)
  //  N:  u_y on iy=0   (E->W)   W: -u_x on ix=0  (N->S)
  for (int e = tid; e < 4 * p * SC; e += RES_NT) {
    const int st = e / SC, s = e % SC;
    const int side = st / p, t = st % p;
    const double* Dm;
    int base, stride;
    double fac;
    if (side == 0) { Dm = D1 + (p - 1) * p; base = t * p; stride = 1; fac = ih; }
    else if (side == 1) { Dm = D1 + (p - 1) * p; base = p - 1 - t; stride = p; fac = ih; }
    else if (side == 2) { Dm = D1; base = (p - 1 - t) * p; stride = 1; fac = -ih; }
    else { Dm = D1; base = t; stride = p; fac = -ih; }
    double2 v = make_double2(0.0, 0.0);
    for (int j = 0; j < p; ++j) {
      const double2 w = u[(base + j * stride) * SC + s];
      v.x = fma(Dm[j], w.x, v.x);
      v.y = fma(Dm[j], w.y, v.y);
    }
    nd[e] = make_double2(fac * v.x, fac * v.y);
  }
  __syncthreads();
  // impedance rows at the Chebyshev boundary points (side's t-th point, t < p-1)
  for (int e = tid; e < ncb * SC; e += RES_NT) {
    const int k = e / SC, s = e % SC;
    if (s >= sc) continue;
    const int side = k / m, t = k % m;
    double2 pt = make_double2(0.0, 0.0);
    for (int j = 0; j < q; ++j) {
      const double w = Ps[t * q + j];
      const double2 g = ts[(side * q + j) * SC + s];
      pt.x = fma(w, g.x, pt.x);
      pt.y = fma(w, g.y, pt.y);
    }
    const double2 un = nd[(side * p + t) * SC + s];
    const double2 uv = u[perm[k] * SC + s];
    // (u_n + i eta u) = (un.x - eta uv.y) + i (un.y + eta uv.x)
    const double gx = un.x - eta * uv.y, gy = un.y + eta * uv.x;
    r[((long long)l * pp + k) * nsrc + s0 + s] = make_float2((float)(pt.x - gx), (float)(pt.y - gy));
  }
  // outgoing impedance at the Gauss nodes
  for (int e = tid; e < nq * SC; e += RES_NT) {
    const int k = e / SC, s = e % SC;
    if (s >= sc) continue;
    const int side = k / q, j = k % q;
    double2 v = make_double2(0.0, 0.0);
    for (int t = 0; t < p; ++t) {
      const double2 un = nd[(side * p + t) * SC + s];
      const double2 uv = u[perm[(side * m + t) % ncb] * SC + s];
      // (u_n - i eta u) = (un.x + eta uv.y) + i (un.y - eta uv.x)
      const double w = Qs[j * p + t];
      v.x = fma(w, un.x + eta * uv.y, v.x);
      v.y = fma(w, un.y - eta * uv.x, v.y);
    }
    t_out[((long long)l * nq + k) * nsrc + s0 + s] = v;
  }
}

size_t residual_iti_2d_smem(int p, int q, int SC, int need_uy) {
  const int pp = p * p;
  size_t z = (size_t)pp * SC * (need_uy ? 2 : 1) + (size_t)4 * q * SC + (size_t)4 * p * SC;
  size_t d = 2 * (size_t)pp + 2 * (size_t)p * q;
  return z * sizeof(double2) + d * sizeof(double) + (size_t)pp * sizeof(int);
}

cudaError_t residual_iti_2d(int n_leaves, int p, int q, int nsrc, int n_ops, unsigned long long kinds, int cplx,
                            double eta, const void* coeffs, const double* inv_half, const double* D1,
                            const double* D2, const double* Pside, const double* Qside, const int* perm,
                            const void* u, const void* t_in, const void* f, void* r, void* t_out, int need_uy,
                            cudaStream_t st) {
  const int SC = nsrc < RES_SC ? nsrc : RES_SC;
  const size_t smem = residual_iti_2d_smem(p, q, SC, need_uy);
  if (smem > 200 * 1024) return cudaErrorInvalidValue;
  if (smem > 48 * 1024) {
    cudaFuncSetAttribute(residual_iti_2d_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(residual_iti_2d_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  }
  const long long nblk = (long long)n_leaves * ((nsrc + SC - 1) / SC);
  if (nblk > 2147483647ll) return cudaErrorInvalidValue;
  const unsigned grid = (unsigned)nblk;
  const double work = 8.0 * n_leaves * (double)nsrc * (p * p * (double)p * (n_ops + 2) + 8.0 * p * q);
  ProfScope ps(KC_RESIDUAL, st, work);
  note_launch();
  if (cplx)
    residual_iti_2d_kernel<true><<<grid, RES_NT, smem, st>>>(
        n_leaves, p, q, nsrc, SC, n_ops, kinds, eta, coeffs, inv_half, D1, D2, Pside, Qside, perm,
        (const double2*)u, (const double2*)t_in, (const double2*)f, (float2*)r, (double2*)t_out, need_uy);
  else
    residual_iti_2d_kernel<false><<<grid, RES_NT, smem, st>>>(
        n_leaves, p, q, nsrc, SC, n_ops, kinds, eta, coeffs, inv_half, D1, D2, Pside, Qside, perm,
        (const double2*)u, (const double2*)t_in, (const double2*)f, (float2*)r, (double2*)t_out, need_uy);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Interface flux mismatch and boundary-data residual.
//   hcorr[l][k] = (F[l][k] + F[nbr(l,k)]) / 2   for interior interface nodes,
//               0                               on the domain boundary;
//   r_bdry[b]   = g_given[b] - g[bdry_node(b)].
// Adding -R/2 = hcorr to the h of both leaves at a node enforces the flux
// residual R = -(F_a + F_b) in the next merge up-pass.
// ---------------------------------------------------------------------------
__global__ void flux_combine_kernel(long long n_nodes, int nsrc, const int* __restrict__ nbr,
                                    const double* __restrict__ flux, float* hcorr, int n_bdry,
                                    const int* __restrict__ bdry_node, const double* __restrict__ g_given,
                                    const double* __restrict__ g_state, float* r_bdry) {
  const long long total = n_nodes * nsrc;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long node = e / nsrc;
    const int s = (int)(e % nsrc);
    const int nb = nbr[node];
    hcorr[e] = (nb >= 0) ? (float)(0.5 * (flux[e] + flux[(long long)nb * nsrc + s])) : 0.0f;
  }
  const long long tb = (long long)n_bdry * nsrc;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tb;
       e += (long long)gridDim.x * blockDim.x) {
    const long long b = e / nsrc;
    const int s = (int)(e % nsrc);
    r_bdry[e] = (float)((g_given ? g_given[e] : 0.0) - g_state[(long long)bdry_node[b] * nsrc + s]);
  }
}

cudaError_t flux_combine(long long n_nodes, int nsrc, const int* nbr, const double* flux, float* hcorr, int n_bdry,
                         const int* bdry_node, const double* g_given, const double* g_state, float* r_bdry,
                         cudaStream_t st) {
  long long g = (n_nodes * nsrc + 255) / 256;
  if (g > 8192) g = 8192;
  if (g < 1) g = 1;
  ProfScope ps(KC_MOVE, st, (double)n_nodes * nsrc * (8.0 + 8.0 + 4.0) + (double)n_bdry * nsrc * 20.0);
  note_launch();
  flux_combine_kernel<<<(int)g, 256, 0, st>>>(n_nodes, nsrc, nbr, flux, hcorr, n_bdry, bdry_node, g_given, g_state,
                                              r_bdry);
  return cudaGetLastError();
}

// ItI interface terms (complex, interleaved re/im):
//   hcorr[node] = t_out[node] + t_in[nbr[node]]   (0 where nbr < 0), complex64
//   r_bdry[b]   = t_given[b] - t_in[bdry_node[b]],                     complex64
// hcorr is minus the residual of the partner node's interface equation
// t_in(a) + t_out(b) = 0, folded into b's outgoing data for the up pass.
__global__ void iti_combine_kernel(long long n_nodes, int nsrc, const int* __restrict__ nbr,
                                   const double2* __restrict__ t_out, const double2* __restrict__ t_in,
                                   float2* __restrict__ hcorr, int n_bdry, const int* __restrict__ bdry_node,
                                   const double2* __restrict__ t_given, float2* __restrict__ r_bdry) {
  const long long total = n_nodes * nsrc;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long node = e / nsrc;
    const int s = (int)(e % nsrc);
    const int nb = nbr[node];
    float2 h = make_float2(0.f, 0.f);
    if (nb >= 0) {
      const double2 a = t_out[e], b = t_in[(long long)nb * nsrc + s];
      h = make_float2((float)(a.x + b.x), (float)(a.y + b.y));
    }
    hcorr[e] = h;
  }
  const long long tb = (long long)n_bdry * nsrc;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tb;
       e += (long long)gridDim.x * blockDim.x) {
    const long long b = e / nsrc;
    const int s = (int)(e % nsrc);
    const double2 g = t_given ? t_given[e] : make_double2(0.0, 0.0);
    const double2 t = t_in[(long long)bdry_node[b] * nsrc + s];
    r_bdry[e] = make_float2((float)(g.x - t.x), (float)(g.y - t.y));
  }
}

cudaError_t iti_combine(long long n_nodes, int nsrc, const int* nbr, const void* t_out, const void* t_in, void* hcorr,
                        int n_bdry, const int* bdry_node, const void* t_given, void* r_bdry, cudaStream_t st) {
  long long g = (n_nodes * nsrc + 255) / 256;
  if (g > 8192) g = 8192;
  if (g < 1) g = 1;
  ProfScope ps(KC_MOVE, st, (double)n_nodes * nsrc * 40.0 + (double)n_bdry * nsrc * 40.0);
  note_launch();
  iti_combine_kernel<<<(int)g, 256, 0, st>>>(n_nodes, nsrc, nbr, (const double2*)t_out, (const double2*)t_in,
                                             (float2*)hcorr, n_bdry, bdry_node, (const double2*)t_given,
                                             (float2*)r_bdry);
  return cudaGetLastError();
}

// y[i] += x[i] (x FP32, y FP64), for n elements; returns nothing.
__global__ void accumulate_kernel(long long n, const float* __restrict__ x, double* y) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
    y[e] += (double)x[e];
}

// y += x (n FP32 values into FP64), with the largest |x| and the largest
// updated |y| (per element, or per (re, im) pair when pairs != 0) written to
// out[0], out[1]: the refinement's convergence test in the same pass.
// Non-negative doubles compare like their bit patterns, so the block maxima
// combine through atomicMax on the 64-bit words.
// max that keeps a NaN once seen (fmax would drop it and a NaN correction
// could pass the convergence test)
__device__ __forceinline__ double nanmax(double a, double b) {
  return (a != a) ? a : ((b != b || b > a) ? b : a);
}

__global__ void accumulate_max_kernel(long long n, int pairs, const float* __restrict__ x, double* y,
                                      unsigned long long* out) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __shared__ unsigned long long sx[32], sy[32];
  if (pairs) {
    // complex magnitudes in FP64 (the complex refinement's vectors are short)
    double mx = 0.0, my = 0.0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n / 2; e += stride) {
      const float xr = x[2 * e], xi = x[2 * e + 1];
      const double yr = y[2 * e] + (double)xr, yi = y[2 * e + 1] + (double)xi;
      y[2 * e] = yr;
      y[2 * e + 1] = yi;
      mx = nanmax(mx, sqrt((double)xr * xr + (double)xi * xi));
      my = nanmax(my, sqrt(yr * yr + yi * yi));
    }
    for (int o = 16; o > 0; o >>= 1) {
      mx = nanmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
      my = nanmax(my, __shfl_xor_sync(0xffffffffu, my, o));
    }
    if (lane == 0) {
      sx[warp] = (unsigned long long)__double_as_longlong(mx);
      sy[warp] = (unsigned long long)__double_as_longlong(my);
    }
  } else {
    // magnitudes compared as integer bit patterns (sign cleared): no FP64
    // compares on the FP64 pipe; a NaN sorts above every number and stays
    unsigned int bx = 0;
    unsigned long long by = 0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += stride) {
      const float xv = x[e];
      const double v = y[e] + (double)xv;
      y[e] = v;
      bx = max(bx, __float_as_uint(xv) & 0x7fffffffu);
      by = max(by, (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull);
    }
    for (int o = 16; o > 0; o >>= 1) {
      bx = max(bx, __shfl_xor_sync(0xffffffffu, bx, o));
      by = max(by, (unsigned long long)__shfl_xor_sync(0xffffffffu, (long long)by, o));
    }
    if (lane == 0) {
      const float fx = __uint_as_float(bx);
      sx[warp] = (unsigned long long)__double_as_longlong((double)fx);
      sy[warp] = by;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long ax = sx[0], ay = sy[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
      ax = max(ax, sx[w]);
      ay = max(ay, sy[w]);
    }
    atomicMax(out, ax);
    atomicMax(out + 1, ay);
  }
}

cudaError_t accumulate_max(long long n, int pairs, const float* x, double* y, double* out, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(out, 0, 2 * sizeof(double), st);
  if (e != cudaSuccess) return e;
  long long g = (n + 255) / 256;
  if (g > 8192) g = 8192;
  if (g < 1) g = 1;
  ProfScope ps(KC_MOVE, st, 20.0 * (double)n);
  note_launch();
  accumulate_max_kernel<<<(int)g, 256, 0, st>>>(n, pairs, x, y, reinterpret_cast<unsigned long long*>(out));
  return cudaGetLastError();
}

cudaError_t accumulate(long long n, const float* x, double* y, cudaStream_t st) {
  long long g = (n + 255) / 256;
  if (g > 8192) g = 8192;
  if (g < 1) g = 1;
  ProfScope ps(KC_MOVE, st, 20.0 * (double)n);
  note_launch();
  accumulate_kernel<<<(int)g, 256, 0, st>>>(n, x, y);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Incremental residual update in double-float arithmetic.
//
// After the first FP64 residual, refinement keeps the residual current by
//     r_int -= (A du)_int,   flux += Q du_full,
// where du (FP32 interior values) and dg (FP32 Gauss boundary values) are the
// FP32 corrections.  Products and sums use unevaluated pairs of FP32 numbers
// (hi + lo, ~48-bit significands) with the error-free transformations
// TwoProd (by FMA) and TwoSum (Knuth), so the work runs on the FP32 pipe;
// every correction after the first is at most a few percent of the solution,
// so the pair arithmetic's rounding enters the residual far below FP64 level.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(RES_NT)
jx_update_2d_kernel(int n_leaves, int p, int q, int nsrc, int n_ops, unsigned long long kinds,
                    const double* __restrict__ coeffs, const double* __restrict__ inv_half,
                    const double* __restrict__ D1g, const double* __restrict__ D2g,
                    const double* __restrict__ Pside_g, const double* __restrict__ Qside_g,
                    const int* __restrict__ perm_g, const float* __restrict__ du, const float* __restrict__ dg,
                    double* r_int, float* r32, double* flux, int need_uy) {
  extern __shared__ float smf[];
  const int pp = p * p;
  const int ncb = 4 * (p - 1);
  const int ni = pp - ncb;
  const int nq = 4 * q;
  df32* u = reinterpret_cast<df32*>(smf);          // pp * SC
  df32* uy = u + pp * RES_SC;                       // pp * SC when D_xy is active
  df32* nd = uy + (need_uy ? pp * RES_SC : 0);      // 4p * SC; before that, the coefficient pairs
  df32* cf = nd;                                    // n_ops * ni: c * scale of every interior point
  const int ndr = max(4 * p * RES_SC, n_ops * ni);
  df32* D1 = nd + ndr;
  df32* D2 = D1 + pp;
  df32* Ps = D2 + pp;
  df32* Qs = Ps + p * q;
  float* gs = reinterpret_cast<float*>(Qs + q * p);  // nq * SC
  int* perm = reinterpret_cast<int*>(gs + nq * RES_SC);

  // the right-hand-side chunks of a leaf are consecutive blocks (shared L2 rows)
  const int nch = (nsrc + RES_SC - 1) / RES_SC;
  const long long l = blockIdx.x / nch;
  const int s0 = (int)(blockIdx.x % nch) * RES_SC;
  const int sc = min(RES_SC, nsrc - s0);
  const int tid = threadIdx.x;
  const double ih = inv_half[l];
  const double ih2 = ih * ih;
  const df32 ihd = df_split(ih), mihd = df32{-ihd.hi, -ihd.lo};

  for (int e = tid; e < pp; e += RES_NT) {
    D1[e] = df_split(D1g[e]);
    D2[e] = df_split(D2g[e]);
    perm[e] = perm_g[e];
  }
  // the FP64 coefficient times the operator's 1/h scaling, split once per
  // point (not per right-hand side): the only FP64 arithmetic of the PDE rows
  for (int e = tid; e < n_ops * ni; e += RES_NT) {
    const int o = e / ni, i = e % ni;
    double sc;
    switch ((int)((kinds >> (4 * o)) & 15ull)) {
      case OP_XX:
      case OP_YY: sc = ih2; break;
      case OP_X:
      case OP_XY: sc = ih; break;
      case OP_Y: sc = -ih; break;
      default: sc = 1.0;
    }
    cf[e] = df_split(sc * coeffs[(long long)o * n_leaves * pp + (long long)l * pp + ncb + i]);
  }
  for (int e = tid; e < p * q; e += RES_NT) {
    Ps[e] = df_split(Pside_g[e]);
    Qs[e] = df_split(Qside_g[e]);
  }
  for (int e = tid; e < nq * RES_SC; e += RES_NT) {
    const int k = e / RES_SC, s = e % RES_SC;
    gs[e] = (s < sc) ? dg[(l * nq + k) * nsrc + s0 + s] : 0.f;
  }
  __syncthreads();
  for (int e = tid; e < ni * RES_SC; e += RES_NT) {
    const int i = e / RES_SC, s = e % RES_SC;
    u[perm[ncb + i] * RES_SC + s] = df32{(s < sc) ? du[(l * ni + i) * nsrc + s0 + s] : 0.f, 0.f};
  }
  for (int e = tid; e < ncb * RES_SC; e += RES_NT) {
    const int k = e / RES_SC, s = e % RES_SC;
    float hs = 0.f, he = 0.f;
    int cnt = 0;
#pragma unroll
    for (int side = 0; side < 4; ++side) {
      int t = k - side * (p - 1);
      if (side == 3 && k == 0) t = p - 1;
      if (t < 0 || t > p - 1) continue;
      if (side == 3 && t == p - 1 && k != 0) continue;
      for (int j = 0; j < q; ++j) df_mac(hs, he, Ps[t * q + j], df32{gs[(side * q + j) * RES_SC + s], 0.f});
      ++cnt;
    }
    if (cnt == 2) {
      hs *= 0.5f;
      he *= 0.5f;
    }
    u[perm[k] * RES_SC + s] = df_norm(hs, he);
  }
  __syncthreads();
  if (need_uy) {
    for (int e = tid; e < pp * RES_SC; e += RES_NT) {
      const int idx = e / RES_SC, s = e % RES_SC;
      const int ix = idx / p, iy = idx % p;
      float hs = 0.f, he = 0.f;
      for (int k = 0; k < p; ++k) df_mac(hs, he, D1[iy * p + k], u[(ix * p + k) * RES_SC + s]);
      uy[e] = df_mul(mihd, df_norm(hs, he));
    }
    __syncthreads();
  }
  for (int e = tid; e < ni * RES_SC; e += RES_NT) {
    const int i = e / RES_SC, s = e % RES_SC;
    if (s >= sc) continue;
    const int idx = perm[ncb + i];
    const int ix = idx / p, iy = idx % p;
    float as = 0.f, ae = 0.f;   // sum over the operators, as a pair
    for (int o = 0; o < n_ops; ++o) {
      float hs = 0.f, he = 0.f;
      switch ((int)((kinds >> (4 * o)) & 15ull)) {
        case OP_XX:
          for (int j = 0; j < p; ++j) df_mac(hs, he, D2[ix * p + j], u[(j * p + iy) * RES_SC + s]);
          break;
        case OP_YY:
          for (int j = 0; j < p; ++j) df_mac(hs, he, D2[iy * p + j], u[(ix * p + j) * RES_SC + s]);
          break;
        case OP_X:
          for (int j = 0; j < p; ++j) df_mac(hs, he, D1[ix * p + j], u[(j * p + iy) * RES_SC + s]);
          break;
        case OP_Y:
          for (int j = 0; j < p; ++j) df_mac(hs, he, D1[iy * p + j], u[(ix * p + j) * RES_SC + s]);
          break;
        case OP_XY:
          for (int j = 0; j < p; ++j) df_mac(hs, he, D1[ix * p + j], uy[(j * p + iy) * RES_SC + s]);
          break;
        default:
          hs = u[idx * RES_SC + s].hi;
          he = u[idx * RES_SC + s].lo;
      }
      df_mac(as, ae, cf[o * ni + i], df32{hs, he});
    }
    const long long o = ((long long)l * ni + i) * nsrc + s0 + s;
    const double r = r_int[o] - df_join(as, ae);
    r_int[o] = r;
    r32[o] = (float)r;
  }
  __syncthreads();   // nd below reuses the coefficient pairs' storage
  for (int e = tid; e < 4 * p * RES_SC; e += RES_NT) {
    const int st = e / RES_SC, s = e % RES_SC;
    const int side = st / p, t = st % p;
    float hs = 0.f, he = 0.f;
    df32 sg;
    if (side == 0) {
      for (int k = 0; k < p; ++k) df_mac(hs, he, D1[(p - 1) * p + k], u[(t * p + k) * RES_SC + s]);
      sg = ihd;
    } else if (side == 1) {
      const int iy = p - 1 - t;
      for (int j = 0; j < p; ++j) df_mac(hs, he, D1[(p - 1) * p + j], u[(j * p + iy) * RES_SC + s]);
      sg = ihd;
    } else if (side == 2) {
      const int ix = p - 1 - t;
      for (int k = 0; k < p; ++k) df_mac(hs, he, D1[k], u[(ix * p + k) * RES_SC + s]);
      sg = mihd;
    } else {
      for (int j = 0; j < p; ++j) df_mac(hs, he, D1[j], u[(j * p + t) * RES_SC + s]);
      sg = mihd;
    }
    nd[e] = df_mul(sg, df_norm(hs, he));
  }
  __syncthreads();
  for (int e = tid; e < nq * RES_SC; e += RES_NT) {
    const int k = e / RES_SC, s = e % RES_SC;
    if (s >= sc) continue;
    const int side = k / q, j = k % q;
    float hs = 0.f, he = 0.f;
    for (int t = 0; t < p; ++t) df_mac(hs, he, Qs[j * p + t], nd[(side * p + t) * RES_SC + s]);
    flux[((long long)l * nq + k) * nsrc + s0 + s] += df_join(hs, he);
  }
}

size_t jx_update_2d_smem(int p, int q, int need_uy, int n_ops) {
  const int pp = p * p;
  const size_t ni = (size_t)pp - 4 * (size_t)(p - 1);
  const size_t ndr = (size_t)4 * p * RES_SC > n_ops * ni ? (size_t)4 * p * RES_SC : n_ops * ni;
  size_t pairs = (size_t)pp * RES_SC * (need_uy ? 2 : 1) + ndr + 2 * (size_t)pp + 2 * (size_t)p * q;
  return pairs * sizeof(df32) + (size_t)4 * q * RES_SC * sizeof(float) + (size_t)pp * sizeof(int);
}

cudaError_t jx_update_2d(int n_leaves, int p, int q, int nsrc, int n_ops, unsigned long long kinds,
                         const double* coeffs, const double* inv_half, const double* D1, const double* D2,
                         const double* Pside, const double* Qside, const int* perm, const float* du, const float* dg,
                         double* r_int, float* r32, double* flux, int need_uy, cudaStream_t st) {
  const size_t smem = jx_update_2d_smem(p, q, need_uy, n_ops);
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(jx_update_2d_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const long long nblk = (long long)n_leaves * ((nsrc + RES_SC - 1) / RES_SC);
  if (nblk > 2147483647ll) return cudaErrorInvalidValue;
  const unsigned grid = (unsigned)nblk;
  const int ni = p * p - 4 * (p - 1);
  const double work = 2.0 * n_leaves * (double)nsrc * ((double)ni * p * n_ops + 8.0 * p * q);
  ProfScope ps(KC_RESIDUAL, st, work);
  note_launch();
  jx_update_2d_kernel<<<grid, RES_NT, smem, st>>>(n_leaves, p, q, nsrc, n_ops, kinds, coeffs, inv_half, D1, D2, Pside,
                                                  Qside, perm, du, dg, r_int, r32, flux, need_uy);
  return cudaGetLastError();
}

// u_full[l][k] = (P g)[k] on the Chebyshev boundary and u_int on the interior
// (FP64), written in the exterior-first leaf order.
__global__ void assemble_u_2d_kernel(int n_leaves, int p, int q, int nsrc, const double* __restrict__ Pside,
                                     const double* __restrict__ u_int, const double* __restrict__ g, double* u_full) {
  const int pp = p * p, ncb = 4 * (p - 1), ni = pp - ncb, nq = 4 * q;
  const long long l = blockIdx.x;
  for (int e = threadIdx.x; e < pp * nsrc; e += blockDim.x) {
    const int k = e / nsrc, s = e % nsrc;
    double v;
    if (k >= ncb) {
      v = u_int[(l * ni + (k - ncb)) * nsrc + s];
    } else {
      double acc = 0.0;
      int cnt = 0;
      for (int side = 0; side < 4; ++side) {
        int t = k - side * (p - 1);
        if (side == 3 && k == 0) t = p - 1;
        if (t < 0 || t > p - 1) continue;
        if (side == 3 && t == p - 1 && k != 0) continue;
        for (int j = 0; j < q; ++j) acc = fma(Pside[t * q + j], g[(l * nq + side * q + j) * nsrc + s], acc);
        ++cnt;
      }
      v = (cnt == 2) ? 0.5 * acc : acc;
    }
    u_full[(l * pp + k) * nsrc + s] = v;
  }
}

cudaError_t assemble_u_2d(int n_leaves, int p, int q, int nsrc, const double* Pside, const double* u_int,
                          const double* g, double* u_full, cudaStream_t st) {
  ProfScope ps(KC_MOVE, st, 8.0 * n_leaves * (double)p * p * nsrc * 2.0);
  note_launch();
  assemble_u_2d_kernel<<<n_leaves, 256, 0, st>>>(n_leaves, p, q, nsrc, Pside, u_int, g, u_full);
  return cudaGetLastError();
}

// r32[l][i][s] = f[l][n_cb + i][s]  (the residual at x = 0, rounded to FP32)
__global__ void interior_f32_kernel(long long n_leaves, int pp, int ncb, int nsrc, const double* __restrict__ f,
                                    float* r32) {
  const int ni = pp - ncb;
  const long long n = n_leaves * ni * nsrc;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const long long l = e / ((long long)ni * nsrc);
    const long long rem = e % ((long long)ni * nsrc);
    r32[e] = (float)f[l * pp * nsrc + (long long)ncb * nsrc + rem];
  }
}

cudaError_t interior_f32(long long n_leaves, int pp, int ncb, int nsrc, const double* f, float* r32, cudaStream_t st) {
  long long n = n_leaves * (pp - ncb) * nsrc;
  long long g = (n + 255) / 256;
  if (g > 8192) g = 8192;
  if (g < 1) g = 1;
  note_launch();
  interior_f32_kernel<<<(int)g, 256, 0, st>>>(n_leaves, pp, ncb, nsrc, f, r32);
  return cudaGetLastError();
}

}  // namespace hps
