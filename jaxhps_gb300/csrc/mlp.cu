// Refinement-proposal network: a 513 -> 64 -> 64 -> 1 multilayer perceptron
// (ReLU hidden layers, one logit out) that predicts, from 8^3 uniform
// samples of f over an octree node plus the node's depth, whether the
// adaptive meshing criterion will refine the node.  This component has no
// counterpart in the reference; it proposes refinements, and the plain
// interpolation criterion (_adaptive_discretization_3D.py:475-503) still
// decides every accepted leaf.
//
// Parameters are one FP32 vector: W1 (64 x 513, row = hidden unit), b1 (64),
// W2 (64 x 64, row = output unit), b2 (64), w3 (64), b3 (1).
// Forward and backward work on tiles of MLP_R rows per CTA; gradients are
// summed with atomics into a zeroed gradient vector; Adam updates in place.
#include "hps_common.cuh"
#include "hps_internal.h"

namespace hps {

constexpr int MLP_IN = 513;
constexpr int MLP_H = 64;
constexpr int MLP_R = 32;
constexpr int MLP_NT = 256;
constexpr int OFF_W1 = 0;
constexpr int OFF_B1 = OFF_W1 + MLP_H * MLP_IN;
constexpr int OFF_W2 = OFF_B1 + MLP_H;
constexpr int OFF_B2 = OFF_W2 + MLP_H * MLP_H;
constexpr int OFF_W3 = OFF_B2 + MLP_H;
constexpr int OFF_B3 = OFF_W3 + MLP_H;
constexpr int MLP_NPARAM = OFF_B3 + 1;

int mlp_param_count() { return MLP_NPARAM; }

// Uniform cell-centred 8x8x8 sample points of every node: pts (n, 512, 3),
// sample s = (i*8 + j)*8 + k at x = xmin + (i + 1/2) (xmax - xmin) / 8, ...
__global__ void mlp_sample_points_kernel(int n, const double* __restrict__ bounds, double* __restrict__ pts) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)n * 512) return;
  const long long node = e / 512;
  const int s = (int)(e % 512);
  const int ijk[3] = {s / 64, (s / 8) % 8, s % 8};
  const double* b = bounds + node * 6;
#pragma unroll
  for (int d = 0; d < 3; ++d) pts[e * 3 + d] = b[2 * d] + (ijk[d] + 0.5) * (b[2 * d + 1] - b[2 * d]) / 8.0;
}

// X (n, 513): samples / scale, then depth / 16.
__global__ void mlp_features_kernel(int n, const double* __restrict__ fvals, const int* __restrict__ depth,
                                    double inv_scale, float* __restrict__ X) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)n * MLP_IN) return;
  const long long r = e / MLP_IN;
  const int k = (int)(e % MLP_IN);
  X[e] = (k < 512) ? (float)(fvals[r * 512 + k] * inv_scale) : (float)depth[r] * (1.0f / 16.0f);
}

__global__ void __launch_bounds__(MLP_NT)
mlp_forward_kernel(int n, const float* __restrict__ X, const float* __restrict__ P, float* __restrict__ H1,
                   float* __restrict__ H2, float* __restrict__ logit) {
  extern __shared__ float mlp_sm[];
  float* xs = mlp_sm;                                  // [MLP_R][513]: odd stride, conflict-free column reads
  float(*h1s)[MLP_H + 1] = reinterpret_cast<float(*)[MLP_H + 1]>(xs + MLP_R * MLP_IN);
  float(*h2s)[MLP_H + 1] = h1s + MLP_R;
  float(*w2s)[MLP_H + 1] = h2s + MLP_R;
  const int tid = threadIdx.x;
  const long long r0 = (long long)blockIdx.x * MLP_R;
  const int nr = (int)min((long long)MLP_R, (long long)n - r0);
  for (int e = tid; e < MLP_R * MLP_IN; e += MLP_NT) {
    const int r = e / MLP_IN;
    xs[e] = (r < nr) ? X[(r0 + r) * MLP_IN + (e % MLP_IN)] : 0.f;
  }
  for (int e = tid; e < MLP_H * MLP_H; e += MLP_NT) w2s[e / MLP_H][e % MLP_H] = P[OFF_W2 + e];
  __syncthreads();
  // layer 1: lanes of a warp take 32 rows of the same unit (W1 reads broadcast)
  for (int o = tid; o < MLP_R * MLP_H; o += MLP_NT) {
    const int j = o / MLP_R, r = o % MLP_R;
    const float* w = P + OFF_W1 + j * MLP_IN;
    float s = P[OFF_B1 + j];
    for (int k = 0; k < MLP_IN; ++k) s = fmaf(__ldg(w + k), xs[r * MLP_IN + k], s);
    h1s[r][j] = fmaxf(s, 0.f);
  }
  __syncthreads();
  for (int o = tid; o < MLP_R * MLP_H; o += MLP_NT) {
    const int j = o / MLP_R, r = o % MLP_R;
    float s = P[OFF_B2 + j];
    for (int k = 0; k < MLP_H; ++k) s = fmaf(w2s[j][k], h1s[r][k], s);
    h2s[r][j] = fmaxf(s, 0.f);
  }
  __syncthreads();
  if (tid < MLP_R && tid < nr) {
    float s = P[OFF_B3];
    for (int k = 0; k < MLP_H; ++k) s = fmaf(P[OFF_W3 + k], h2s[tid][k], s);
    logit[r0 + tid] = s;
  }
  for (int e = tid; e < nr * MLP_H; e += MLP_NT) {
    const int r = e / MLP_H, j = e % MLP_H;
    if (H1) H1[(r0 + r) * MLP_H + j] = h1s[r][j];
    if (H2) H2[(r0 + r) * MLP_H + j] = h2s[r][j];
  }
}

// Binary cross-entropy with logits, weight wpos on positive labels; writes
// dlogit = d(mean loss)/dlogit and adds the summed loss to *loss.
__global__ void mlp_bce_kernel(int n, const float* __restrict__ logit, const float* __restrict__ y, float wpos,
                               float* __restrict__ dlogit, float* __restrict__ loss) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.f;
  if (i < n) {
    const float z = logit[i], t = y[i];
    const float w = t > 0.5f ? wpos : 1.f;
    const float pz = 1.f / (1.f + expf(-z));
    l = w * (fmaxf(z, 0.f) - z * t + log1pf(expf(-fabsf(z))));
    dlogit[i] = w * (pz - t) / (float)n;
  }
#pragma unroll
  for (int off = 16; off; off >>= 1) l += __shfl_xor_sync(0xffffffffu, l, off);
  if ((threadIdx.x & 31) == 0 && loss) atomicAdd(loss, l);
}

__global__ void __launch_bounds__(MLP_NT)
mlp_backward_kernel(int n, const float* __restrict__ X, const float* __restrict__ P, const float* __restrict__ H1,
                    const float* __restrict__ H2, const float* __restrict__ dlogit, float* __restrict__ G) {
  extern __shared__ float mlp_sm[];
  float* xs = mlp_sm;
  float(*h1s)[MLP_H + 1] = reinterpret_cast<float(*)[MLP_H + 1]>(xs + MLP_R * MLP_IN);
  float(*h2s)[MLP_H + 1] = h1s + MLP_R;
  float(*d2)[MLP_H + 1] = h2s + MLP_R;
  float(*d1)[MLP_H + 1] = d2 + MLP_R;
  __shared__ float dl[MLP_R];
  const int tid = threadIdx.x;
  const long long r0 = (long long)blockIdx.x * MLP_R;
  const int nr = (int)min((long long)MLP_R, (long long)n - r0);
  for (int e = tid; e < MLP_R * MLP_IN; e += MLP_NT) {
    const int r = e / MLP_IN;
    xs[e] = (r < nr) ? X[(r0 + r) * MLP_IN + (e % MLP_IN)] : 0.f;
  }
  for (int e = tid; e < MLP_R * MLP_H; e += MLP_NT) {
    const int r = e / MLP_H, j = e % MLP_H;
    h1s[r][j] = (r < nr) ? H1[(r0 + r) * MLP_H + j] : 0.f;
    h2s[r][j] = (r < nr) ? H2[(r0 + r) * MLP_H + j] : 0.f;
  }
  if (tid < MLP_R) dl[tid] = (tid < nr) ? dlogit[r0 + tid] : 0.f;
  __syncthreads();
  for (int e = tid; e < MLP_R * MLP_H; e += MLP_NT) {
    const int r = e / MLP_H, j = e % MLP_H;
    d2[r][j] = (h2s[r][j] > 0.f) ? dl[r] * P[OFF_W3 + j] : 0.f;
  }
  __syncthreads();
  for (int e = tid; e < MLP_R * MLP_H; e += MLP_NT) {
    const int r = e / MLP_H, i = e % MLP_H;
    float s = 0.f;
    for (int j = 0; j < MLP_H; ++j) s = fmaf(P[OFF_W2 + j * MLP_H + i], d2[r][j], s);
    d1[r][i] = (h1s[r][i] > 0.f) ? s : 0.f;
  }
  __syncthreads();
  // parameter gradients summed over this CTA's rows
  for (int e = tid; e < MLP_H * MLP_IN; e += MLP_NT) {
    const int i = e / MLP_IN, k = e % MLP_IN;
    float s = 0.f;
    for (int r = 0; r < nr; ++r) s = fmaf(d1[r][i], xs[r * MLP_IN + k], s);
    atomicAdd(G + OFF_W1 + e, s);
  }
  for (int e = tid; e < MLP_H * MLP_H; e += MLP_NT) {
    const int j = e / MLP_H, i = e % MLP_H;
    float s = 0.f;
    for (int r = 0; r < nr; ++r) s = fmaf(d2[r][j], h1s[r][i], s);
    atomicAdd(G + OFF_W2 + e, s);
  }
  if (tid < MLP_H) {
    float sb1 = 0.f, sb2 = 0.f, sw3 = 0.f;
    for (int r = 0; r < nr; ++r) {
      sb1 += d1[r][tid];
      sb2 += d2[r][tid];
      sw3 = fmaf(dl[r], h2s[r][tid], sw3);
    }
    atomicAdd(G + OFF_B1 + tid, sb1);
    atomicAdd(G + OFF_B2 + tid, sb2);
    atomicAdd(G + OFF_W3 + tid, sw3);
  }
  if (tid == 0) {
    float s = 0.f;
    for (int r = 0; r < nr; ++r) s += dl[r];
    atomicAdd(G + OFF_B3, s);
  }
}

__global__ void mlp_adam_kernel(int n, float* __restrict__ P, const float* __restrict__ G, float* __restrict__ M,
                                float* __restrict__ V, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float g = G[i];
  const float m = b1 * M[i] + (1.f - b1) * g;
  const float v = b2 * V[i] + (1.f - b2) * g * g;
  M[i] = m;
  V[i] = v;
  P[i] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
}

cudaError_t mlp_sample_points(int n, const double* bounds, double* pts, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const long long tot = (long long)n * 512;
  note_launch();
  mlp_sample_points_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(n, bounds, pts);
  return cudaGetLastError();
}

cudaError_t mlp_features(int n, const double* fvals, const int* depth, double inv_scale, float* X, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const long long tot = (long long)n * MLP_IN;
  note_launch();
  mlp_features_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(n, fvals, depth, inv_scale, X);
  return cudaGetLastError();
}

cudaError_t mlp_forward(int n, const float* X, const float* P, float* H1, float* H2, float* logit, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const size_t smem = sizeof(float) * ((size_t)MLP_R * MLP_IN + 2 * MLP_R * (MLP_H + 1) + MLP_H * (MLP_H + 1));
  cudaFuncSetAttribute(mlp_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  ProfScope ps(KC_GEMM, st, 2.0 * n * (MLP_IN * MLP_H + MLP_H * MLP_H + MLP_H));
  note_launch();
  mlp_forward_kernel<<<(n + MLP_R - 1) / MLP_R, MLP_NT, smem, st>>>(n, X, P, H1, H2, logit);
  return cudaGetLastError();
}

cudaError_t mlp_bce(int n, const float* logit, const float* y, float wpos, float* dlogit, float* loss,
                    cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  note_launch();
  mlp_bce_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, logit, y, wpos, dlogit, loss);
  return cudaGetLastError();
}

cudaError_t mlp_backward(int n, const float* X, const float* P, const float* H1, const float* H2,
                         const float* dlogit, float* G, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const size_t smem = sizeof(float) * ((size_t)MLP_R * MLP_IN + 4 * MLP_R * (MLP_H + 1));
  cudaFuncSetAttribute(mlp_backward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  ProfScope ps(KC_GEMM, st, 4.0 * n * (MLP_IN * MLP_H + MLP_H * MLP_H + MLP_H));
  note_launch();
  mlp_backward_kernel<<<(n + MLP_R - 1) / MLP_R, MLP_NT, smem, st>>>(n, X, P, H1, H2, dlogit, G);
  return cudaGetLastError();
}

cudaError_t mlp_adam(float* P, const float* G, float* M, float* V, float lr, float b1, float b2, float eps, int step,
                     cudaStream_t st) {
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  note_launch();
  mlp_adam_kernel<<<(MLP_NPARAM + 255) / 256, 256, 0, st>>>(MLP_NPARAM, P, G, M, V, lr, b1, b2, eps, c1, c2);
  return cudaGetLastError();
}

}  // namespace hps
