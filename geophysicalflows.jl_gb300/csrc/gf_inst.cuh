// Launch wrappers: pick the compile-time FFT lengths and the block shapes for one
// precision T.  Included once per precision by gf_f32.cu / gf_f64.cu.
#pragma once
#include "gf_kernels.cuh"

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
inline int pick_C(int NY, int R, int nkr, F smem) {
  const int TPF = NY / R;
  int C = 512 / TPF;
  if (C < 1) C = 1;
  if (C > 16) C = 16;
  while (C > 1 && (C * TPF > 512 || smem(C) > (size_t)SMEM_CAP)) C /= 2;
  while (C > 1 && (nkr + C - 1) / C < 2 * num_sms()) C /= 2;
  return C;
}
// Row pairs per row-kernel block (same rule: >= 2 blocks per SM when possible).
inline int pick_B(int NX, int R, size_t elem, int nbufs, int npairs) {
  const int TPF = NX / R;
  int B = 256 / TPF;
  if (B < 1) B = 1;
  while (B > 1 && ((size_t)B * (NX + NX / R) * elem * nbufs > SMEM_CAP || B * TPF > 256 || npairs % B != 0)) B /= 2;
  while (B > 1 && npairs / B < 2 * num_sms()) B /= 2;
  return B;
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
  if (bytes > 48 * 1024) return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  return cudaSuccess;
}

#define GF_SWITCH_N(n, ...)                                     \
  switch (n) {                                                   \
    case 32: { constexpr int NN = 32; __VA_ARGS__; } break;             \
    case 64: { constexpr int NN = 64; __VA_ARGS__; } break;             \
    case 128: { constexpr int NN = 128; __VA_ARGS__; } break;           \
    case 256: { constexpr int NN = 256; __VA_ARGS__; } break;           \
    case 512: { constexpr int NN = 512; __VA_ARGS__; } break;           \
    case 1024: { constexpr int NN = 1024; __VA_ARGS__; } break;         \
    case 2048: { constexpr int NN = 2048; __VA_ARGS__; } break;         \
    default: return cudaErrorInvalidValue;                       \
  }

// Radix of the Stockham passes (FP32 tunable at build time; FP64 uses 8).
#ifndef GF_RADIX_F32
#define GF_RADIX_F32 8
#endif
template <class T>
constexpr int RADIX = sizeof(T) == 4 ? GF_RADIX_F32 : 8;

template <class T>
cudaError_t launch_row(const Geom& g, const ModArgs& m, const Bufs& b, cudaStream_t st) {
  cudaError_t err = cudaSuccess;
  const size_t e = sizeof(cplx<T>);
  GF_SWITCH_N(g.nx, {
    const int B = pick_B(NN, RADIX<T>, e, 3, g.ny / 2);
    const size_t sm = (size_t)B * 3 * row_stride<T>(NN, NN / RADIX<T>) * e;
    auto k = row_nl_kernel<T, NN, RADIX<T>>;
    if ((err = set_smem(k, sm)) != cudaSuccess) return err;
    k<<<g.ny / 2 / B, B * (NN / RADIX<T>), sm, st>>>(g, m, b, B);
  });
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_col(const Geom& g, const ModArgs& m, const StepArgs& s, const Bufs& b, cudaStream_t st) {
  cudaError_t err = cudaSuccess;
  const size_t e = sizeof(cplx<T>);
  GF_SWITCH_N(g.ny, {
    const int C = pick_C(NN, RADIX<T>, g.nkr, [&](int c) { return col_stage_smem(NN, c, col_stride<T>(NN, c), g.nl, e); });
    Geom g2 = g;
    g2.cs = col_stride<T>(NN, C);
    const size_t sm = col_stage_smem(NN, C, g2.cs, g.nl, e);
    auto k = col_stage_kernel<T, NN, RADIX<T>>;
    if ((err = set_smem(k, sm)) != cudaSuccess) return err;
    k<<<(g.nkr + C - 1) / C, C * (NN / RADIX<T>), sm, st>>>(g2, m, s, b, C);
  });
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_col_inv(const Geom& g, const ModArgs& m, const void* src, int kind, int mask, const Bufs& b,
                           cudaStream_t st) {
  cudaError_t err;
  const size_t e = sizeof(cplx<T>);
  GF_SWITCH_N(g.ny, {
    const int C = pick_C(NN, RADIX<T>, g.nkr, [&](int c) { return (size_t)c * col_stride<T>(NN, c) * e; });
    Geom g2 = g;
    g2.cs = col_stride<T>(NN, C);
    const size_t sm = (size_t)C * g2.cs * e;
    auto k = col_inv_generic<T, NN, RADIX<T>>;
    if ((err = set_smem(k, sm)) != cudaSuccess) return err;
    k<<<(g.nkr + C - 1) / C, C * (NN / RADIX<T>), sm, st>>>(g2, m, src, kind, mask, b, C);
  });
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_row_c2r(const Geom& g, const Bufs& b, int nf, void* out, cudaStream_t st) {
  cudaError_t err;
  const size_t e = sizeof(cplx<T>);
  GF_SWITCH_N(g.nx, {
    const int B = pick_B(NN, RADIX<T>, e, 1, g.ny / 2);
    const size_t sm = (size_t)B * row_stride<T>(NN, NN / RADIX<T>) * e;
    auto k = row_c2r_generic<T, NN, RADIX<T>>;
    if ((err = set_smem(k, sm)) != cudaSuccess) return err;
    k<<<g.ny / 2 / B, B * (NN / RADIX<T>), sm, st>>>(g, b, nf, static_cast<T*>(out), B);
  });
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_row_r2c(const Geom& g, const Bufs& b, int nf, const void* in, cudaStream_t st) {
  cudaError_t err;
  const size_t e = sizeof(cplx<T>);
  GF_SWITCH_N(g.nx, {
    const int B = pick_B(NN, RADIX<T>, e, 1, g.ny / 2);
    const size_t sm = (size_t)B * row_stride<T>(NN, NN / RADIX<T>) * e;
    auto k = row_r2c_generic<T, NN, RADIX<T>>;
    if ((err = set_smem(k, sm)) != cudaSuccess) return err;
    k<<<g.ny / 2 / B, B * (NN / RADIX<T>), sm, st>>>(g, b, nf, static_cast<const T*>(in), B);
  });
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_col_fwd(const Geom& g, const Bufs& b, int nf, void* out, int zero_mean, cudaStream_t st) {
  cudaError_t err;
  const size_t e = sizeof(cplx<T>);
  GF_SWITCH_N(g.ny, {
    const int C = pick_C(NN, RADIX<T>, g.nkr, [&](int c) { return (size_t)c * col_stride<T>(NN, c) * e; });
    Geom g2 = g;
    g2.cs = col_stride<T>(NN, C);
    const size_t sm = (size_t)C * g2.cs * e;
    auto k = col_fwd_generic<T, NN, RADIX<T>>;
    if ((err = set_smem(k, sm)) != cudaSuccess) return err;
    k<<<(g.nkr + C - 1) / C, C * (NN / RADIX<T>), sm, st>>>(g2, b, nf, static_cast<cplx<T>*>(out), zero_mean, C);
  });
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_diag(const Geom& g, const ModArgs& m, const void* sol, const void* prevsol, const void* Fh,
                        uint32_t mask, double* partial, int nblocks, cudaStream_t st) {
  diag_kernel<T><<<nblocks, DIAG_BLOCK, 0, st>>>(g, m, static_cast<const cplx<T>*>(sol),
                                                 static_cast<const cplx<T>*>(prevsol),
                                                 static_cast<const cplx<T>*>(Fh), mask, partial);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_mask_inplace(const Geom& g, void* sol, cudaStream_t st) {
  mask_inplace_kernel<T><<<256, 256, 0, st>>>(g, static_cast<cplx<T>*>(sol));
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_spec_apply(const Geom& g, const ModArgs& m, const void* in, void* out, int op, cudaStream_t st) {
  spec_apply_kernel<T><<<256, 256, 0, st>>>(g, m, static_cast<const cplx<T>*>(in), static_cast<cplx<T>*>(out), op);
  return cudaGetLastError();
}

#define GF_INSTANTIATE_COL(T)                                                                                  \
  template cudaError_t launch_col<T>(const Geom&, const ModArgs&, const StepArgs&, const Bufs&, cudaStream_t); \
  template cudaError_t launch_col_inv<T>(const Geom&, const ModArgs&, const void*, int, int, const Bufs&,      \
                                         cudaStream_t);                                                        \
  template cudaError_t launch_col_fwd<T>(const Geom&, const Bufs&, int, void*, int, cudaStream_t);            \
  template cudaError_t launch_diag<T>(const Geom&, const ModArgs&, const void*, const void*, const void*,     \
                                      uint32_t, double*, int, cudaStream_t);                                   \
  template cudaError_t launch_mask_inplace<T>(const Geom&, void*, cudaStream_t);                              \
  template cudaError_t launch_spec_apply<T>(const Geom&, const ModArgs&, const void*, void*, int, cudaStream_t);

#define GF_INSTANTIATE_ROW(T)                                                                                  \
  template cudaError_t launch_row<T>(const Geom&, const ModArgs&, const Bufs&, cudaStream_t);                 \
  template cudaError_t launch_row_c2r<T>(const Geom&, const Bufs&, int, void*, cudaStream_t);                 \
  template cudaError_t launch_row_r2c<T>(const Geom&, const Bufs&, int, const void*, cudaStream_t);

}  // namespace gf
