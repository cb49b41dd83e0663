// Launch layer shared by the dispatch unit and the per-size kernel units: block-shape rules
// and the declarations of the per-size launchers (defined in gf_inst_n.cuh, instantiated one
// FFT length and precision per translation unit so that the build parallelises).
#pragma once
#include "gf_fft.cuh"
#include "gf_internal.h"

namespace gf {

constexpr int SMEM_CAP = 200 * 1024;

inline int num_sms() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 152;
  }
  return n;
}

// Columns per column-kernel block: aim at ~512 threads, but shrink until the grid has at
// least two blocks per SM; keep shared memory under SMEM_CAP.  smem(C) gives the block's
// dynamic shared-memory bytes for C columns.
template <class F>
inline int pick_C(int NY, int R, int nkr, F smem, int nb = 1) {
  const int TPF = NY / R;
  int C = 512 / TPF;
  if (C < 1) C = 1;
  if (C > 16) C = 16;
  while (C > 1 && (C * TPF > 512 || smem(C) > (size_t)SMEM_CAP)) C /= 2;
  while (C > 1 && (size_t)nb * ((nkr + C - 1) / C) < (size_t)2 * num_sms()) C /= 2;
  return C;
}
// Row pairs per row-kernel block (same rule: >= 2 blocks per SM when possible).
inline int pick_B(int NX, int R, size_t elem, int nbufs, int npairs, int nb = 1) {
  const int TPF = NX / R;
  int B = 256 / TPF;
  if (B < 1) B = 1;
  while (B > 1 && ((size_t)B * (NX + NX / R) * elem * nbufs > SMEM_CAP || B * TPF > 256 || npairs % B != 0)) B /= 2;
  while (B > 1 && (size_t)nb * (npairs / B) < (size_t)2 * num_sms()) B /= 2;
  return B;
}

// Largest column-kernel block: the one-layer path without bottom drag on FP32 columns of
// >= 1024 points allows 640 threads (e.g. five radix-16 columns of 2048, one block per SM at
// 96 registers a thread: the wide instantiation), everything else 512.
inline int col_max_threads(size_t real_bytes, int NY, const ModArgs& m, int nl) {
  return (real_bytes == 4 && NY >= 1024 && nl == 1 && !m.drag) ? 640 : 512;
}

// The column-kernel instantiation (its MAXT) a launch of `threads` threads runs: 640, the
// wide FP32 one-layer instantiation above 512 threads; 256, the narrow df64 one (one layer,
// no bottom drag, two product fields, columns >= 1024, at most 256 threads: three blocks per
// SM at 80 registers in two shared-memory buffers; IEEE FP64 is ALU-bound and measured slower
// there); 512 otherwise.
inline int col_variant(bool df64, int NY, const ModArgs& m, int nl, int threads) {
  if (threads > 512) return 640;
  if (df64 && NY >= 1024 && threads <= 256 && nl == 1 && !m.drag && 1 + m.hasB + m.hasC <= 2) return 256;
  return 512;
}

// The wide and narrow instantiations run the one-layer path without bottom drag and with at
// most two product fields in two shared-memory buffers (three otherwise, and in the
// 512-thread instantiation).
inline bool col_two_buffers(const ModArgs& m, int nl, int threads, bool df64, int NY) {
  return col_variant(df64, NY, m, nl, threads) != 512 && nl == 1 && !m.drag && 1 + m.hasB + m.hasC <= 2;
}

// shared-memory bytes of col_stage_kernel for C columns with column stride cs and `threads`
// threads (elem: complex element bytes): one layer without bottom drag F0, F1 (, F2);
// otherwise F0, F1, F2 and the X of every layer
__host__ __forceinline__ size_t col_stage_smem(int NY, int C, int cs, const ModArgs& m, int nl, size_t elem,
                                               int threads, bool df64) {
  if (nl == 1 && !m.drag) return (size_t)(col_two_buffers(m, nl, threads, df64, NY) ? 2 : 3) * C * cs * elem;
  if (nl > 1) return (size_t)3 * C * cs * elem;  // layer split: X of every layer in global memory
  return ((size_t)3 * C * cs + (size_t)nl * NY * C) * elem;
}

// Whether B row pairs per block fit the row kernel (threads, shared memory, pair count).
inline bool row_shape_ok(int NX, int R, size_t elem, int nbufs, int npairs, int B) {
  const int TPF = NX / R;
  return B >= 1 && B * TPF <= 256 && (size_t)B * (NX + NX / R) * elem * nbufs <= SMEM_CAP && npairs % B == 0;
}

// Column stride of the column kernels' work buffers: NY slots, staggered so that the C
// columns a wavefront touches in the element mapping fall into disjoint banks.
template <class T>
inline int col_stride(int NY, int C) {
  const int unit = wave_threads<T>();
  return C > 1 ? NY + (unit / C > 1 ? unit / C : 1) : NY;
}

// Opt in to large dynamic shared memory and ask for the maximum shared-memory carveout
// (the FFT kernels are shared-memory bound; L1 is not used for reuse here).
template <class K>
inline cudaError_t set_smem(K kernel, size_t bytes) {
  static_assert(sizeof(K) > 0, "");
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  if (e != cudaSuccess) return e;
  // the 48 KB default limit covers static + dynamic shared memory: opt in well below it
  if (bytes > 32 * 1024) return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  return cudaSuccess;
}

// Radix of the Stockham passes (FP32 tunable at build time; FP64 uses 8).
#ifndef GF_RADIX_F32
#define GF_RADIX_F32 8
#endif
template <class T>
constexpr int RADIX = sizeof(T) == 4 ? GF_RADIX_F32 : 8;

// per-size launchers (NN = FFT length along the transformed direction)
template <class T, int NN> cudaError_t launch_row_n(const Geom&, const ModArgs&, const Bufs&, cudaStream_t);
template <class T, int NN, int R> cudaError_t launch_row_nr(const Geom&, const ModArgs&, const Bufs&, cudaStream_t);
template <class T, int NN, int R>
cudaError_t launch_col_nr(const Geom&, const ModArgs&, const StepArgs&, const Bufs&, cudaStream_t);
template <class T, int NN, int R> cudaError_t launch_adj_row_nr(const Geom&, const AdjArgs&, const Bufs&, cudaStream_t);
template <class T, int NN, int R>
cudaError_t launch_adj_col_nr(const Geom&, const ModArgs&, const AdjArgs&, const Bufs&, cudaStream_t);
// FFT radices of the FP32 step kernels that the autotuner may pick, per length
constexpr bool f32_radix_built(int N, int R) { return R == 8 || (R == 16) || (R == 4 && N <= 1024); }
template <class T, int NN> cudaError_t launch_col_n(const Geom&, const ModArgs&, const StepArgs&, const Bufs&, cudaStream_t);
template <class T, int NN> cudaError_t launch_col_inv_n(const Geom&, const ModArgs&, const void*, int, int, const Bufs&,
                                                        cudaStream_t);
template <class T, int NN> cudaError_t launch_row_c2r_n(const Geom&, const Bufs&, int, void*, cudaStream_t);
template <class T, int NN> cudaError_t launch_row_r2c_n(const Geom&, const Bufs&, int, const void*, cudaStream_t);
template <class T, int NN> cudaError_t launch_col_fwd_n(const Geom&, const Bufs&, int, void*, int, cudaStream_t);
template <class T, int NN> cudaError_t launch_adj_row_n(const Geom&, const AdjArgs&, const Bufs&, cudaStream_t);
template <class T, int NN> cudaError_t launch_adj_col_n(const Geom&, const ModArgs&, const AdjArgs&, const Bufs&,
                                                        cudaStream_t);
template <class T, int NN>
cudaError_t launch_adj_col_ml_n(const Geom&, const ModArgs&, const AdjArgs&, const Bufs&, cudaStream_t);

}  // namespace gf
