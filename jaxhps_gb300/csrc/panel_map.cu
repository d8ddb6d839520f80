// Panel maps for adaptive merges (reference: merge/_utils_adaptive_3D_DtN.py
// _compress_rows_from_lst / _compress_cols_from_lst :647-743 and the
// de-projection of down_pass/_adaptive_3D_DtN.py _deproject_merge_interface_3D).
//
// Where an interface has four fine panels on one side and one coarse panel
// on the other, the fine side's rows are compressed with L_1f4 (q^2 x 4q^2),
// its columns with L_4f1 (4q^2 x q^2), and in the down pass its data is
// expanded back with L_4f1.  Every output index i along the mapped axis has
// a table entry {kind, in_start, local, n_k}:
//   kind 0: out[i] = in[in_start + local]
//   kind 1: rows mode   out[i] = sum_k M[local][k] in[in_start + k]   (k < n_k)
//           cols mode   out[i] = sum_k in[in_start + k] M[k][local]
// (M row-major with n_k columns in rows mode, n_k rows in cols mode; its
// other dimension is the segment's output length m_len).
#include "hps_common.cuh"
#include "hps_internal.h"

namespace hps {

template <class T>
__global__ void panel_map_rows_kernel(int n_out, int n_other, const int4* __restrict__ tab, const T* __restrict__ M,
                                      const T* __restrict__ in, long long ld_in, long long s_in, T* __restrict__ out,
                                      long long ld_out, long long s_out) {
  const long long b = blockIdx.y;
  const T* ib = in + b * s_in;
  T* ob = out + b * s_out;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)n_out * n_other;
       e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e / n_other), col = (int)(e % n_other);
    const int4 t = tab[i];
    T v;
    if (t.x == 0) {
      v = ib[(long long)(t.y + t.z) * ld_in + col];
    } else {
      v = zero<T>();
      const T* mrow = M + (long long)t.z * t.w;
      for (int k = 0; k < t.w; ++k) v = fma_(mrow[k], ib[(long long)(t.y + k) * ld_in + col], v);
    }
    ob[(long long)i * ld_out + col] = v;
  }
}

template <class T>
__global__ void panel_map_cols_kernel(int n_out, int n_other, int m_len, const int4* __restrict__ tab,
                                      const T* __restrict__ M, const T* __restrict__ in, long long ld_in,
                                      long long s_in, T* __restrict__ out, long long ld_out, long long s_out) {
  const long long b = blockIdx.y;
  const T* ib = in + b * s_in;
  T* ob = out + b * s_out;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)n_out * n_other;
       e += (long long)gridDim.x * blockDim.x) {
    const int row = (int)(e / n_out), j = (int)(e % n_out);
    const int4 t = tab[j];
    const T* irow = ib + (long long)row * ld_in;
    T v;
    if (t.x == 0) {
      v = irow[t.y + t.z];
    } else {
      v = zero<T>();
      for (int k = 0; k < t.w; ++k) v = fma_(irow[t.y + k], M[(long long)k * m_len + t.z], v);
    }
    ob[(long long)row * ld_out + j] = v;
  }
}

template <class T>
cudaError_t panel_map(int mode, int batch, int n_out, int n_other, int m_len, const int* tab, const T* M, const T* in,
                      long long ld_in, long long s_in, T* out, long long ld_out, long long s_out, cudaStream_t st) {
  if (batch <= 0 || n_out <= 0 || n_other <= 0) return cudaSuccess;
  const long long tot = (long long)n_out * n_other;
  int gx = (int)((tot + 255) / 256);
  if (gx > 1024) gx = 1024;
  for (int b0 = 0; b0 < batch; b0 += 65535) {
    const int nb = batch - b0 < 65535 ? batch - b0 : 65535;
    ProfScope ps(KC_MOVE, st, 2.0 * sizeof(T) * (double)tot * nb);
    note_launch();
    if (mode == 0)
      panel_map_rows_kernel<T><<<dim3(gx, nb), 256, 0, st>>>(n_out, n_other, reinterpret_cast<const int4*>(tab), M,
                                                             in + (long long)b0 * s_in, ld_in, s_in,
                                                             out + (long long)b0 * s_out, ld_out, s_out);
    else
      panel_map_cols_kernel<T><<<dim3(gx, nb), 256, 0, st>>>(n_out, n_other, m_len,
                                                             reinterpret_cast<const int4*>(tab), M,
                                                             in + (long long)b0 * s_in, ld_in, s_in,
                                                             out + (long long)b0 * s_out, ld_out, s_out);
  }
  return cudaGetLastError();
}

template <class T>
__global__ void scale_batched_kernel(long long n_per, const double* __restrict__ scale, T* __restrict__ x) {
  const long long b = blockIdx.y;
  const double s = scale[b];
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n_per; e += (long long)gridDim.x * blockDim.x)
    x[b * n_per + e] = mul(x[b * n_per + e], from_real<T>(s));
}

template <class T>
cudaError_t scale_batched(int batch, long long n_per, const double* scale, T* x, cudaStream_t st) {
  if (batch <= 0 || n_per <= 0) return cudaSuccess;
  int gx = (int)((n_per + 255) / 256);
  if (gx > 256) gx = 256;
  for (int b0 = 0; b0 < batch; b0 += 65535) {
    const int nb = batch - b0 < 65535 ? batch - b0 : 65535;
    note_launch();
    scale_batched_kernel<T><<<dim3(gx, nb), 256, 0, st>>>(n_per, scale + b0, x + (long long)b0 * n_per);
  }
  return cudaGetLastError();
}

#define HPS_INST_PM(T)                                                                                         \
  template cudaError_t panel_map<T>(int, int, int, int, int, const int*, const T*, const T*, long long, long long, \
                                    T*, long long, long long, cudaStream_t);                                   \
  template cudaError_t scale_batched<T>(int, long long, const double*, T*, cudaStream_t);
HPS_INST_PM(float)
HPS_INST_PM(double)
HPS_INST_PM(c64)
HPS_INST_PM(c128)

}  // namespace hps
