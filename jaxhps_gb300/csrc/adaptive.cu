// Adaptive octree refinement check (reference: _adaptive_discretization_3D.py
// generate_adaptive_mesh_level_restriction :34-210, the L-infinity check
// check_current_discretization_global_linf_norm :475-503 and the L2 check
// get_squared_l2_norm_eight_voxels :424-472).
//
// For every queued node the reference evaluates f on the node's p^3
// Chebyshev grid and on its eight children's grids, interpolates the node
// values to the children with the dense (8p^3 x p^3) operator L_8f1 and
// compares.  Here the interpolation is applied as three 1D passes
// (x, y, z: the operator is a Kronecker product per child), ~28 p^4 flops
// per node instead of 16 p^6, in FP64.
//
// Point layout (both kernels): per node 9 blocks of p^3 points, block 0 the
// node itself and blocks 1..8 the children a..h, each in the exterior-first
// order of the leaf grids (perm[k] = raster index ix*p^2 + iy*p + iz of
// position k).
#include "hps_common.cuh"
#include "hps_internal.h"

namespace hps {

// (x, y, z) half of children a..h: a-d upper z, each half (lo,lo) (hi,lo) (hi,hi) (lo,hi).
__constant__ int c_child_bits[8][3] = {{0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1},
                                      {0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}};

__global__ void refine_points_3d_kernel(int n_nodes, int p, const double* __restrict__ bounds,
                                        const double* __restrict__ cheb, const int* __restrict__ perm,
                                        double* __restrict__ pts) {
  const long long node = blockIdx.y;
  const int np3 = p * p * p;
  const double* b = bounds + node * 6;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < 9 * np3; e += gridDim.x * blockDim.x) {
    const int blk = e / np3, k = e % np3;
    const int r = perm[k];
    const int ix = r / (p * p), iy = (r / p) % p, iz = r % p;
    const int idx[3] = {ix, iy, iz};
    double* out = pts + ((node * 9 + blk) * np3 + k) * 3;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      double lo = b[2 * d], hi = b[2 * d + 1];
      if (blk > 0) {
        const double mid = (lo + hi) / 2;
        if (c_child_bits[blk - 1][d]) lo = mid;
        else hi = mid;
      }
      out[d] = 0.5 * (hi - lo) * cheb[idx[d]] + 0.5 * (lo + hi);
    }
  }
}

// One CTA per node.  Outputs: diff[node] = max |interp - f_child| over the
// eight children, ref[node] = max |f_child|, l2[node] = sum over the
// children of the Clenshaw-Curtis weighted squared difference.
constexpr int RC_NT = 256;

__global__ void __launch_bounds__(RC_NT)
refine_check_3d_kernel(int n_nodes, int p, const double* __restrict__ fv, const int* __restrict__ perm,
                       const int* __restrict__ iperm, const double* __restrict__ Ilo,
                       const double* __restrict__ Ihi, const double* __restrict__ wref,
                       const double* __restrict__ bounds, double* __restrict__ diff_out,
                       double* __restrict__ ref_out, double* __restrict__ l2_out) {
  extern __shared__ double rc_sm[];
  const int np3 = p * p * p, pp = p * p;
  double* F = rc_sm;          // node values, raster order
  double* T1 = F + np3;
  double* T2 = T1 + np3;
  const long long node = blockIdx.x;
  const double* fnode = fv + node * 9 * (long long)np3;
  const double* b = bounds + node * 6;
  const int tid = threadIdx.x;
  for (int k = tid; k < np3; k += RC_NT) F[perm[k]] = fnode[k];
  double dmax = 0.0, rmax = 0.0, l2 = 0.0;
  for (int c = 0; c < 8; ++c) {
    const double* Ix = c_child_bits[c][0] ? Ihi : Ilo;
    const double* Iy = c_child_bits[c][1] ? Ihi : Ilo;
    const double* Iz = c_child_bits[c][2] ? Ihi : Ilo;
    __syncthreads();
    for (int e = tid; e < np3; e += RC_NT) {   // along z
      const int a = e / pp, bb = (e / p) % p, kz = e % p;
      double s = 0.0;
      for (int j = 0; j < p; ++j) s = fma(Iz[kz * p + j], F[a * pp + bb * p + j], s);
      T1[e] = s;
    }
    __syncthreads();
    for (int e = tid; e < np3; e += RC_NT) {   // along y
      const int a = e / pp, ky = (e / p) % p, kz = e % p;
      double s = 0.0;
      for (int j = 0; j < p; ++j) s = fma(Iy[ky * p + j], T1[a * pp + j * p + kz], s);
      T2[e] = s;
    }
    __syncthreads();
    const double hx = 0.25 * (b[1] - b[0]), hy = 0.25 * (b[3] - b[2]), hz = 0.25 * (b[5] - b[4]);
    const double* fc = fnode + (long long)(c + 1) * np3;
    for (int e = tid; e < np3; e += RC_NT) {   // along x, compare
      const int kx = e / pp, ky = (e / p) % p, kz = e % p;
      double s = 0.0;
      for (int j = 0; j < p; ++j) s = fma(Ix[kx * p + j], T2[j * pp + ky * p + kz], s);
      const double fvv = fc[iperm[e]];
      const double d = fabs(s - fvv);
      dmax = fmax(dmax, d);
      rmax = fmax(rmax, fabs(fvv));
      l2 += (hx * wref[kx]) * (hy * wref[ky]) * (hz * wref[kz]) * d * d;
    }
  }
  // block reductions
  __shared__ double red[3][RC_NT / 32];
#pragma unroll
  for (int off = 16; off; off >>= 1) {
    dmax = fmax(dmax, __shfl_xor_sync(0xffffffffu, dmax, off));
    rmax = fmax(rmax, __shfl_xor_sync(0xffffffffu, rmax, off));
    l2 += __shfl_xor_sync(0xffffffffu, l2, off);
  }
  const int lane = tid & 31, warp = tid >> 5;
  if (lane == 0) {
    red[0][warp] = dmax;
    red[1][warp] = rmax;
    red[2][warp] = l2;
  }
  __syncthreads();
  if (tid == 0) {
    double a = 0.0, r = 0.0, s = 0.0;
    for (int w = 0; w < RC_NT / 32; ++w) {
      a = fmax(a, red[0][w]);
      r = fmax(r, red[1][w]);
      s += red[2][w];
    }
    diff_out[node] = a;
    ref_out[node] = r;
    if (l2_out) l2_out[node] = s;
  }
}

// ---------------------------------------------------------------------------
// 2D (reference _adaptive_discretization_2D.py:34-197): per node 5 blocks of
// p^2 points, block 0 the node and blocks 1..4 the children a..d (SW, SE, NE,
// NW), each in the leaf grids' exterior-first order; raster index
// perm[k] = ix*p + iy with y descending (meshgrid(x, flipud(y), 'ij')).
// ---------------------------------------------------------------------------
__constant__ int c_quad_bits[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};

__global__ void refine_points_2d_kernel(int n_nodes, int p, const double* __restrict__ bounds,
                                        const double* __restrict__ cheb, const int* __restrict__ perm,
                                        double* __restrict__ pts) {
  const long long node = blockIdx.y;
  const int np2 = p * p;
  const double* b = bounds + node * 4;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < 5 * np2; e += gridDim.x * blockDim.x) {
    const int blk = e / np2, k = e % np2;
    const int r = perm[k];
    const int idx[2] = {r / p, p - 1 - (r % p)};
    double* out = pts + ((node * 5 + blk) * np2 + k) * 2;
#pragma unroll
    for (int d = 0; d < 2; ++d) {
      double lo = b[2 * d], hi = b[2 * d + 1];
      if (blk > 0) {
        const double mid = (lo + hi) / 2;
        if (c_quad_bits[blk - 1][d]) lo = mid;
        else hi = mid;
      }
      out[d] = 0.5 * (hi - lo) * cheb[idx[d]] + 0.5 * (lo + hi);
    }
  }
}

// One CTA per node: as refine_check_3d_kernel with two 1D passes (y, then x).
__global__ void __launch_bounds__(RC_NT)
refine_check_2d_kernel(int n_nodes, int p, const double* __restrict__ fv, const int* __restrict__ perm,
                       const int* __restrict__ iperm, const double* __restrict__ Ilo,
                       const double* __restrict__ Ihi, const double* __restrict__ wref,
                       const double* __restrict__ bounds, double* __restrict__ diff_out,
                       double* __restrict__ ref_out, double* __restrict__ l2_out) {
  extern __shared__ double rc2_sm[];
  const int np2 = p * p;
  double* F = rc2_sm;          // node values, raster order (y descending)
  double* T1 = F + np2;
  const long long node = blockIdx.x;
  const double* fnode = fv + node * 5 * (long long)np2;
  const double* b = bounds + node * 4;
  const int tid = threadIdx.x;
  for (int k = tid; k < np2; k += RC_NT) F[perm[k]] = fnode[k];
  double dmax = 0.0, rmax = 0.0, l2 = 0.0;
  const double hx = 0.25 * (b[1] - b[0]), hy = 0.25 * (b[3] - b[2]);
  for (int c = 0; c < 4; ++c) {
    const double* Ix = c_quad_bits[c][0] ? Ihi : Ilo;
    const double* Iy = c_quad_bits[c][1] ? Ihi : Ilo;
    __syncthreads();
    for (int e = tid; e < np2; e += RC_NT) {   // along y, both grids descending
      const int a = e / p, ky = e % p;
      double s = 0.0;
      for (int j = 0; j < p; ++j) s = fma(Iy[(p - 1 - ky) * p + (p - 1 - j)], F[a * p + j], s);
      T1[e] = s;
    }
    __syncthreads();
    const double* fc = fnode + (long long)(c + 1) * np2;
    for (int e = tid; e < np2; e += RC_NT) {   // along x, compare
      const int kx = e / p, ky = e % p;
      double s = 0.0;
      for (int j = 0; j < p; ++j) s = fma(Ix[kx * p + j], T1[j * p + ky], s);
      const double fvv = fc[iperm[e]];
      const double d = fabs(s - fvv);
      dmax = fmax(dmax, d);
      rmax = fmax(rmax, fabs(fvv));
      l2 += (hx * wref[kx]) * (hy * wref[ky]) * d * d;
    }
  }
  __shared__ double red2[3][RC_NT / 32];
#pragma unroll
  for (int off = 16; off; off >>= 1) {
    dmax = fmax(dmax, __shfl_xor_sync(0xffffffffu, dmax, off));
    rmax = fmax(rmax, __shfl_xor_sync(0xffffffffu, rmax, off));
    l2 += __shfl_xor_sync(0xffffffffu, l2, off);
  }
  const int lane = tid & 31, warp = tid >> 5;
  if (lane == 0) {
    red2[0][warp] = dmax;
    red2[1][warp] = rmax;
    red2[2][warp] = l2;
  }
  __syncthreads();
  if (tid == 0) {
    double a = 0.0, r = 0.0, s = 0.0;
    for (int w = 0; w < RC_NT / 32; ++w) {
      a = fmax(a, red2[0][w]);
      r = fmax(r, red2[1][w]);
      s += red2[2][w];
    }
    diff_out[node] = a;
    ref_out[node] = r;
    if (l2_out) l2_out[node] = s;
  }
}

cudaError_t refine_points_2d(int n_nodes, int p, const double* bounds, const double* cheb, const int* perm,
                             double* pts, cudaStream_t st) {
  const int np2 = p * p;
  int gx = (5 * np2 + 255) / 256;
  if (gx > 64) gx = 64;
  for (int n0 = 0; n0 < n_nodes; n0 += 65535) {
    const int nn = n_nodes - n0 < 65535 ? n_nodes - n0 : 65535;
    ProfScope ps(KC_MOVE, st, 8.0 * 4 * nn + 8.0 * 2 * 5 * np2 * nn);
    note_launch();
    refine_points_2d_kernel<<<dim3(gx, nn), 256, 0, st>>>(nn, p, bounds + (long long)n0 * 4, cheb, perm,
                                                          pts + (long long)n0 * 10 * np2);
  }
  return cudaGetLastError();
}

cudaError_t refine_check_2d(int n_nodes, int p, const double* fv, const int* perm, const int* iperm,
                            const double* Ilo, const double* Ihi, const double* wref, const double* bounds,
                            double* diff, double* ref, double* l2, cudaStream_t st) {
  const int np2 = p * p;
  const size_t smem = 2 * sizeof(double) * (size_t)np2;
  if (smem > 200 * 1024) return cudaErrorInvalidValue;
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(refine_check_2d_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  ProfScope ps(KC_RESIDUAL, st, 2.0 * 4 * 2 * (double)np2 * p * n_nodes);
  note_launch();
  refine_check_2d_kernel<<<n_nodes, RC_NT, smem, st>>>(n_nodes, p, fv, perm, iperm, Ilo, Ihi, wref, bounds, diff,
                                                        ref, l2);
  return cudaGetLastError();
}

cudaError_t refine_points_3d(int n_nodes, int p, const double* bounds, const double* cheb, const int* perm,
                             double* pts, cudaStream_t st) {
  const int np3 = p * p * p;
  int gx = (9 * np3 + 255) / 256;
  if (gx > 64) gx = 64;
  for (int n0 = 0; n0 < n_nodes; n0 += 65535) {
    const int nn = n_nodes - n0 < 65535 ? n_nodes - n0 : 65535;
    ProfScope ps(KC_MOVE, st, 8.0 * 6 * nn + 8.0 * 3 * 9 * np3 * nn);
    note_launch();
    refine_points_3d_kernel<<<dim3(gx, nn), 256, 0, st>>>(nn, p, bounds + (long long)n0 * 6, cheb, perm,
                                                          pts + (long long)n0 * 27 * np3);
  }
  return cudaGetLastError();
}

cudaError_t refine_check_3d(int n_nodes, int p, const double* fv, const int* perm, const int* iperm,
                            const double* Ilo, const double* Ihi, const double* wref, const double* bounds,
                            double* diff, double* ref, double* l2, cudaStream_t st) {
  const int np3 = p * p * p;
  const size_t smem = 3 * sizeof(double) * (size_t)np3;
  if (smem > 200 * 1024) return cudaErrorInvalidValue;
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(refine_check_3d_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  // flops: 8 children x 3 passes x p^4 FMAs
  ProfScope ps(KC_RESIDUAL, st, 2.0 * 8 * 3 * (double)np3 * p * n_nodes);
  note_launch();
  refine_check_3d_kernel<<<n_nodes, RC_NT, smem, st>>>(n_nodes, p, fv, perm, iperm, Ilo, Ihi, wref, bounds, diff,
                                                        ref, l2);
  return cudaGetLastError();
}

}  // namespace hps
