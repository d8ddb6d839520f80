// Interpolation between the HPS grid and rectangular grids
// (reference: _interpolation_methods.py:23-340, Domain.interp_* in
// _domain.py:99-294).
//
// Both directions use barycentric Lagrange interpolation in tensor-product
// form, with the reference's handling of coincident points (a target equal
// to a source node is moved off it by EPS, quadrature/_interpolation.py
// :117-213).
//
//  * from the HPS grid (interp_from_leaves_kernel): every target point is
//    located in the first leaf, in leaf order, whose closed box contains it
//    (the reference's argmax over containment tests; outside every leaf it
//    falls back to leaf 0), through a table of the finest-level cells; its
//    value is sum_c ax[i(c)] ay[j(c)] (az[k(c)]) f_leaf[c] over the leaf's
//    points c in exterior-first order.
//  * to the HPS grid: the per-leaf 1D interpolation rows are formed here
//    (interp_rows_kernel) and contracted with the samples by GEMMs, then
//    the leaf values are put in exterior-first order (gather_cols_kernel).
#include "hps_common.cuh"
#include "hps_internal.h"

namespace hps {

__device__ __forceinline__ double nudge(double d) { return d == 0.0 ? 2.220446049250313e-16 : d; }

// out[r][k] = 1 / (d_k w_k nf_r), d_k = to[r] - src[k] (nudged), nf_r = sum_k 1 / (w_k d_k);
// transposed: out[(r / rpg) * n_src * rpg + k * rpg + r % rpg] (rows of a group as columns)
__global__ void interp_rows_kernel(long long n_rows, int n_src, const double* __restrict__ to,
                                   const double* __restrict__ src, const double* __restrict__ w, double* out,
                                   int rpg, int transposed) {
  const long long row = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= n_rows) return;
  const double t = to[row];
  double nf = 0.0;
  for (int k = lane; k < n_src; k += 32) nf += 1.0 / (w[k] * nudge(t - src[k]));
  for (int o = 16; o > 0; o >>= 1) nf += __shfl_xor_sync(0xffffffffu, nf, o);
  const long long g = row / rpg;
  const int rr = (int)(row % rpg);
  for (int k = lane; k < n_src; k += 32) {
    const double v = 1.0 / (nudge(t - src[k]) * w[k] * nf);
    if (transposed)
      out[(g * n_src + k) * rpg + rr] = v;
    else
      out[row * n_src + k] = v;
  }
}

// out[g][c] = in[g][idx[c]]
__global__ void gather_cols_kernel(long long n_groups, int n_in, int n_out, const int* __restrict__ idx,
                                   const double* __restrict__ in, double* out) {
  const long long tot = n_groups * n_out;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
    const long long g = e / n_out;
    out[e] = in[g * n_in + idx[e % n_out]];
  }
}

constexpr int IP_MAXP = 32;

// DIM = 2 or 3.  bounds (n_leaves, 2*DIM) as (min, max) per axis; nodes
// (n_leaves, DIM, p) the leaf's interpolation nodes per axis (2D: y
// descending, as the leaf grid) and wts the matching barycentric weights;
// cell table (nc[0] x nc[1] (x nc[2])) of leaf indices on the finest cells of
// the root box [lo, lo + nc h].
template <int DIM>
__global__ void interp_from_leaves_kernel(long long n_t, int nsrc, const double* __restrict__ tpts, int p, int ppd,
                                          const double* __restrict__ bounds, const double* __restrict__ nodes,
                                          const double* __restrict__ wts, const int* __restrict__ rearr,
                                          const int* __restrict__ cells, int nc0, int nc1, int nc2, double lo0,
                                          double lo1, double lo2, double h0, double h1, double h2,
                                          const double* __restrict__ f, double* out) {
  const long long tot = n_t * nsrc;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
    const long long t = e / nsrc;
    const int s = (int)(e % nsrc);
    double x[3];
    x[0] = tpts[t * DIM + 0];
    x[1] = tpts[t * DIM + 1];
    x[2] = DIM == 3 ? tpts[t * DIM + 2] : 0.0;
    const int nc[3] = {nc0, nc1, nc2};
    const double lo[3] = {lo0, lo1, lo2}, hh[3] = {h0, h1, h2};
    int base[3];
    for (int a = 0; a < DIM; ++a) {
      double c = floor((x[a] - lo[a]) / hh[a]);
      c = c < 0.0 ? 0.0 : (c > nc[a] - 1 ? (double)(nc[a] - 1) : c);
      base[a] = (int)c;
    }
    long long leaf = -1;
    const int span2 = DIM == 3 ? 1 : 0;
    for (int dx = -1; dx <= 1; ++dx)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dz = -span2; dz <= span2; ++dz) {
          const int i0 = base[0] + dx, i1 = base[1] + dy, i2 = base[2] + dz;
          if (i0 < 0 || i0 >= nc0 || i1 < 0 || i1 >= nc1) continue;
          if (DIM == 3 && (i2 < 0 || i2 >= nc2)) continue;
          const long long cidx = DIM == 3 ? ((long long)i0 * nc1 + i1) * nc2 + i2 : (long long)i0 * nc1 + i1;
          const int l = cells[cidx];
          const double* b = bounds + (long long)l * 2 * DIM;
          bool in = true;
          for (int a = 0; a < DIM; ++a) in = in && x[a] >= b[2 * a] && x[a] <= b[2 * a + 1];
          if (in && (leaf < 0 || l < leaf)) leaf = l;
        }
    if (leaf < 0) leaf = 0;
    // 1D barycentric factors on the leaf's nodes
    double fac[3][IP_MAXP];
    for (int a = 0; a < DIM; ++a) {
      const double* nd = nodes + (leaf * DIM + a) * p;
      const double* wt = wts + (leaf * DIM + a) * p;
      double nf = 0.0;
      for (int i = 0; i < p; ++i) nf += 1.0 / (wt[i] * nudge(x[a] - nd[i]));
      for (int i = 0; i < p; ++i) fac[a][i] = 1.0 / (nudge(x[a] - nd[i]) * wt[i] * nf);
    }
    const double* fl = f + leaf * (long long)ppd * nsrc + s;
    double acc = 0.0;
    for (int c = 0; c < ppd; ++c) {
      const int m = rearr[c];
      double wgt;
      if (DIM == 2)
        wgt = fac[0][m / p] * fac[1][m % p];
      else
        wgt = fac[0][m / (p * p)] * fac[1][(m / p) % p] * fac[2][m % p];
      acc = fma(wgt, fl[(long long)c * nsrc], acc);
    }
    out[e] = acc;
  }
}

cudaError_t interp_rows(long long n_rows, int n_src, const double* to, const double* src, const double* w,
                        double* out, int rpg, int transposed, cudaStream_t st) {
  if (n_rows <= 0 || n_src <= 0) return cudaSuccess;
  const long long g = (n_rows + 7) / 8;
  ProfScope ps(KC_MOVE, st, 8.0 * (double)n_rows * n_src);
  note_launch();
  interp_rows_kernel<<<(unsigned)g, 256, 0, st>>>(n_rows, n_src, to, src, w, out, rpg, transposed);
  return cudaGetLastError();
}

cudaError_t gather_cols(long long n_groups, int n_in, int n_out, const int* idx, const double* in, double* out,
                        cudaStream_t st) {
  if (n_groups <= 0 || n_out <= 0) return cudaSuccess;
  long long g = (n_groups * n_out + 255) / 256;
  if (g > 16384) g = 16384;
  ProfScope ps(KC_MOVE, st, 16.0 * (double)n_groups * n_out);
  note_launch();
  gather_cols_kernel<<<(int)g, 256, 0, st>>>(n_groups, n_in, n_out, idx, in, out);
  return cudaGetLastError();
}

cudaError_t interp_from_leaves(int dim, long long n_t, int nsrc, const double* tpts, int p, const double* bounds,
                               const double* nodes, const double* wts, const int* rearr, const int* cells,
                               const int* nc, const double* lo, const double* h, const double* f, double* out,
                               cudaStream_t st) {
  if (n_t <= 0 || nsrc <= 0) return cudaSuccess;
  if (p < 2 || p > IP_MAXP || (dim != 2 && dim != 3)) return cudaErrorInvalidValue;
  const int ppd = dim == 2 ? p * p : p * p * p;
  long long g = (n_t * nsrc + 127) / 128;
  if (g > 65535) g = 65535;
  ProfScope ps(KC_MOVE, st, (double)n_t * nsrc * (2.0 * ppd + 8.0 * dim * p));
  note_launch();
  if (dim == 2)
    interp_from_leaves_kernel<2><<<(int)g, 128, 0, st>>>(n_t, nsrc, tpts, p, ppd, bounds, nodes, wts, rearr, cells,
                                                        nc[0], nc[1], 1, lo[0], lo[1], 0.0, h[0], h[1], 1.0, f, out);
  else
    interp_from_leaves_kernel<3><<<(int)g, 128, 0, st>>>(n_t, nsrc, tpts, p, ppd, bounds, nodes, wts, rearr, cells,
                                                        nc[0], nc[1], nc[2], lo[0], lo[1], lo[2], h[0], h[1], h[2],
                                                        f, out);
  return cudaGetLastError();
}

}  // namespace hps
