// Per-size launchers: block shapes for one FFT length NN and precision T, and the launch.
#pragma once
#include <type_traits>
#include "gf_adjoint.cuh"
#include "gf_launch.cuh"
#include "gf_tma.cuh"

namespace gf {

// TMA column stage with C columns per block (tensor-map pair ci of the context).
template <class T, int NN, int R, int C>
cudaError_t launch_col_tma_c(const Geom& g, const ModArgs& m, const StepArgs& s, const Bufs& b, cudaStream_t st,
                             int ci) {
  cudaError_t err;
  Geom g2 = g;
  g2.cs = col_stride<T>(NN, C);
  const size_t sm = col_tma_smem(C, g2.cs, sizeof(cplx<T>));
  auto k = col_tma_kernel<T, NN, R, C>;
  if ((err = set_smem(k, sm)) != cudaSuccess) return err;
  const int ncols = g.kout > 0 ? g.kout : g.nkr;
  const CUtensorMap* mp = reinterpret_cast<const CUtensorMap*>(b.tma->p[ci]);
  const CUtensorMap* mw = reinterpret_cast<const CUtensorMap*>(b.tma->w[ci]);
  k<<<dim3((ncols + C - 1) / C, g.nb), C * (NN / R), sm, st>>>(g2, m, s, b, *mp, *mw, b.derr);
  return cudaGetLastError();
}

// Whether the TMA column stage runs this launch: one layer, no bottom drag, at most two
// product fields, tensor maps built, and a column count chosen (Geom::tmaC) that has maps.
// Returns the tensor-map pair index, or -1.
inline int col_tma_pair(const Geom& g, const ModArgs& m, const Bufs& b) {
  if (!b.tma || !b.tma->ok || g.tmaC <= 0 || g.nl != 1 || m.drag || 1 + m.hasB + m.hasC > 2) return -1;
  return g.tmaC == b.tma->Cs[0] ? 0 : g.tmaC == b.tma->Cs[1] ? 1 : -1;
}

template <class T, int NN, int R>
cudaError_t launch_col_tma(const Geom& g, const ModArgs& m, const StepArgs& s, const Bufs& b, cudaStream_t st,
                           int ci) {
  // the candidate column counts: 2 and 4 columns of 8-byte elements (16- and 32-byte box
  // rows), 1 and 2 columns of 16-byte elements
  constexpr int C0 = sizeof(cplx<T>) == 8 ? 2 : 1;
  if (ci == 0) return launch_col_tma_c<T, NN, R, C0>(g, m, s, b, st, ci);
  return launch_col_tma_c<T, NN, R, 2 * C0>(g, m, s, b, st, ci);
}

// Row kernel with FFT radix R; B row pairs per block from the autotuner when it fits.
template <class T, int NN, int R>
cudaError_t launch_row_nr(const Geom& g, const ModArgs& m, const Bufs& b, cudaStream_t st) {
  cudaError_t err = cudaSuccess;
  const size_t e = sizeof(cplx<T>);
  int B = pick_B(NN, R, e, 3, g.ny / 2, g.nb);
  if (g.tuneB > 0 && row_shape_ok(NN, R, e, 3, g.ny / 2, g.tuneB)) B = g.tuneB;
  // df64 rows of >= 1024 with the two products (u q', v q') only: the two-buffer
  // instantiation, three blocks per SM
  const bool two = std::is_same<T, df64>::value && NN >= 1024 && m.hasB && !m.hasC && !m.ql && B * (NN / R) <= 256;
  const size_t sm = (size_t)B * (two ? 2 : 3) * row_stride<T>(NN, NN / R) * e;
  auto k = row_nl_kernel<T, NN, R>;
  if constexpr (std::is_same<T, df64>::value && NN >= 1024)
    if (two) k = row_nl_kernel<T, NN, R, true>;
  if ((err = set_smem(k, sm)) != cudaSuccess) return err;
  k<<<dim3(g.ny / 2 / B, g.nb), B * (NN / R), sm, st>>>(g, m, b, B);
  return cudaGetLastError();
}

// Column kernel with FFT radix R; C columns per block from the autotuner when it fits.
template <class T, int NN, int R>
cudaError_t launch_col_nr(const Geom& g, const ModArgs& m, const StepArgs& s, const Bufs& b, cudaStream_t st) {
  cudaError_t err = cudaSuccess;
  if (const int ci = col_tma_pair(g, m, b); ci >= 0) return launch_col_tma<T, NN, R>(g, m, s, b, st, ci);
  const size_t e = sizeof(cplx<T>);
  constexpr bool is_df64 = std::is_same<T, df64>::value;
  auto smem = [&](int c) { return col_stage_smem(NN, c, col_stride<T>(NN, c), m, g.nl, e, c * (NN / R), is_df64); };
  int C = pick_C(NN, R, g.nkr, smem, g.nb);
  if (g.tuneC > 0) {
    // the tuned columns per block; launches of observed steps (every column, every mode: a
    // grid of nkr columns) stay within 512-thread blocks
    const int maxT = g.kout > 0 ? col_max_threads(sizeof(T), NN, m, g.nl) : 512;
    const int tc = std::min(g.tuneC, maxT / (NN / R));
    if (tc >= 1 && smem(tc) <= (size_t)SMEM_CAP) C = tc;
  }
  Geom g2 = g;
  g2.cs = col_stride<T>(NN, C);
  const size_t sm = smem(C);
  auto k = col_stage_kernel<T, NN, R>;
  const int variant = col_variant(is_df64, NN, m, g.nl, C * (NN / R));
  if constexpr (sizeof(T) == 4 && NN >= 1024)
    if (variant == 640) k = col_stage_kernel<T, NN, R, 640>;
  if constexpr (is_df64 && NN >= 1024)
    if (variant == 256) k = col_stage_kernel<T, NN, R, 256>;
  if ((err = set_smem(k, sm)) != cudaSuccess) return err;
  const int ncols = g.kout > 0 ? g.kout : g.nkr;
  if (g.nl == 1) {
    k<<<dim3((ncols + C - 1) / C, g.nb), C * (NN / R), sm, st>>>(g2, m, s, b, C);
    return cudaGetLastError();
  }
  // several layers: one launch for the forward half (every (column block, layer)), one for
  // the inverse half (column blocks below kcut, every layer)
  StepArgs sf = s;
  sf.layer_split = 1;
  if (s.do_fwd) {
    sf.do_inv = 0;
    k<<<dim3((ncols + C - 1) / C, g.nb, g.nl), C * (NN / R), sm, st>>>(g2, m, sf, b, C);
    if ((err = cudaGetLastError()) != cudaSuccess) return err;
  }
  if (s.do_inv) {
    StepArgs si = sf;
    si.do_fwd = 0;
    si.do_inv = 1;
    if (s.do_fwd) si.sol = s.Xg;
    k<<<dim3((std::min(ncols, g.kcut) + C - 1) / C, g.nb, g.nl), C * (NN / R), sm, st>>>(g2, m, si, b, C);
  }
  return cudaGetLastError();
}

template <class T, int NN>
cudaError_t launch_row_n(const Geom& g, const ModArgs& m, const Bufs& b, cudaStream_t st) {
  return launch_row_nr<T, NN, RADIX<T>>(g, m, b, st);
}

template <class T, int NN>
cudaError_t launch_col_n(const Geom& g, const ModArgs& m, const StepArgs& s, const Bufs& b, cudaStream_t st) {
  return launch_col_nr<T, NN, RADIX<T>>(g, m, s, b, st);
}

template <class T, int NN>
cudaError_t launch_col_inv_n(const Geom& g, const ModArgs& m, const void* src, int kind, int mask, const Bufs& b,
                           cudaStream_t st) {

  cudaError_t err;
  const size_t e = sizeof(cplx<T>);
  const int C = pick_C(NN, RADIX<T>, g.nkr, [&](int c) { return (size_t)c * col_stride<T>(NN, c) * e; }, g.nb);
  Geom g2 = g;
  g2.cs = col_stride<T>(NN, C);
  const size_t sm = (size_t)C * g2.cs * e;
  auto k = col_inv_generic<T, NN, RADIX<T>>;
  if ((err = set_smem(k, sm)) != cudaSuccess) return err;
  k<<<dim3((g.nkr + C - 1) / C, g.nb), C * (NN / RADIX<T>), sm, st>>>(g2, m, src, kind, mask, b, C);
  return cudaGetLastError();
}

template <class T, int NN>
cudaError_t launch_row_c2r_n(const Geom& g, const Bufs& b, int nf, void* out, cudaStream_t st) {

  cudaError_t err;
  const size_t e = sizeof(cplx<T>);
  const int B = pick_B(NN, RADIX<T>, e, 1, g.ny / 2, g.nb);
  const size_t sm = (size_t)B * row_stride<T>(NN, NN / RADIX<T>) * e;
  auto k = row_c2r_generic<T, NN, RADIX<T>>;
  if ((err = set_smem(k, sm)) != cudaSuccess) return err;
  k<<<dim3(g.ny / 2 / B, g.nb), B * (NN / RADIX<T>), sm, st>>>(g, b, nf, static_cast<T*>(out), B);
  return cudaGetLastError();
}

template <class T, int NN>
cudaError_t launch_row_r2c_n(const Geom& g, const Bufs& b, int nf, const void* in, cudaStream_t st) {

  cudaError_t err;
  const size_t e = sizeof(cplx<T>);
  const int B = pick_B(NN, RADIX<T>, e, 1, g.ny / 2, g.nb);
  const size_t sm = (size_t)B * row_stride<T>(NN, NN / RADIX<T>) * e;
  auto k = row_r2c_generic<T, NN, RADIX<T>>;
  if ((err = set_smem(k, sm)) != cudaSuccess) return err;
  k<<<dim3(g.ny / 2 / B, g.nb), B * (NN / RADIX<T>), sm, st>>>(g, b, nf, static_cast<const T*>(in), B);
  return cudaGetLastError();
}

template <class T, int NN>
cudaError_t launch_col_fwd_n(const Geom& g, const Bufs& b, int nf, void* out, int zero_mean, cudaStream_t st) {

  cudaError_t err;
  const size_t e = sizeof(cplx<T>);
  const int C = pick_C(NN, RADIX<T>, g.nkr, [&](int c) { return (size_t)c * col_stride<T>(NN, c) * e; }, g.nb);
  Geom g2 = g;
  g2.cs = col_stride<T>(NN, C);
  const size_t sm = (size_t)C * g2.cs * e;
  auto k = col_fwd_generic<T, NN, RADIX<T>>;
  if ((err = set_smem(k, sm)) != cudaSuccess) return err;
  k<<<dim3((g.nkr + C - 1) / C, g.nb), C * (NN / RADIX<T>), sm, st>>>(g2, b, nf, static_cast<cplx<T>*>(out), zero_mean, C);
  return cudaGetLastError();
}

// Adjoint kernels with FFT radix R; the context's tuned tiles when they fit.
template <class T, int NN, int R>
cudaError_t launch_adj_row_nr(const Geom& g, const AdjArgs& a, const Bufs& b, cudaStream_t st) {
  cudaError_t err;
  const size_t e = sizeof(cplx<T>);
  int B = pick_B(NN, R, e, 3, g.ny / 2, 1);
  if (g.tuneB > 0 && row_shape_ok(NN, R, e, 3, g.ny / 2, g.tuneB)) B = g.tuneB;
  const size_t sm = (size_t)B * 3 * row_stride<T>(NN, NN / R) * e;
  auto k = adj_row_kernel<T, NN, R>;
  if ((err = set_smem(k, sm)) != cudaSuccess) return err;
  k<<<g.ny / 2 / B, B * (NN / R), sm, st>>>(g, a, b, B);
  return cudaGetLastError();
}

template <class T, int NN, int R>
cudaError_t launch_adj_col_nr(const Geom& g, const ModArgs& m, const AdjArgs& a, const Bufs& b, cudaStream_t st) {
  cudaError_t err;
  const size_t e = sizeof(cplx<T>);
  auto smem = [&](int c) { return adj_col_smem(c, col_stride<T>(NN, c), e); };
  int C = pick_C(NN, R, g.nkr, smem, 1);
  if (g.tuneC > 0 && g.tuneC * (NN / R) <= 512 && smem(g.tuneC) <= (size_t)SMEM_CAP) C = g.tuneC;
  Geom g2 = g;
  g2.cs = col_stride<T>(NN, C);
  const size_t sm = smem(C);
  auto k = adj_col_kernel<T, NN, R>;
  if ((err = set_smem(k, sm)) != cudaSuccess) return err;
  k<<<(g.nkr + C - 1) / C, C * (NN / R), sm, st>>>(g2, m, a, b, C);
  return cudaGetLastError();
}

// the several-layer adjoint column kernel: every layer of C columns per block (C from the
// shared-memory budget: 3 x nl x C columns)
template <class T, int NN>
cudaError_t launch_adj_col_ml_n(const Geom& g, const ModArgs& m, const AdjArgs& a, const Bufs& b, cudaStream_t st) {
  cudaError_t err;
  const size_t e = sizeof(cplx<T>);
  constexpr int R = RADIX<T>;
  auto smem = [&](int c) { return (size_t)3 * g.nl * c * col_stride<T>(NN, c) * e; };
  const int C = pick_C(NN, R, g.nkr, smem, 1);
  if (smem(C) > (size_t)SMEM_CAP) return cudaErrorInvalidConfiguration;
  Geom g2 = g;
  g2.cs = col_stride<T>(NN, C);
  auto k = adj_col_ml_kernel<T, NN, R>;
  if ((err = set_smem(k, smem(C))) != cudaSuccess) return err;
  k<<<(g.nkr + C - 1) / C, C * (NN / R), smem(C), st>>>(g2, m, a, b, C);
  return cudaGetLastError();
}

template <class T, int NN>
cudaError_t launch_adj_row_n(const Geom& g, const AdjArgs& a, const Bufs& b, cudaStream_t st) {
  return launch_adj_row_nr<T, NN, RADIX<T>>(g, a, b, st);
}

template <class T, int NN>
cudaError_t launch_adj_col_n(const Geom& g, const ModArgs& m, const AdjArgs& a, const Bufs& b, cudaStream_t st) {
  return launch_adj_col_nr<T, NN, RADIX<T>>(g, m, a, b, st);
}

// the step kernels at another FFT radix (autotuner candidates)
#define GF_INST_NR(T, NN, R)                                                                                   \
  template cudaError_t launch_row_nr<T, NN, R>(const Geom&, const ModArgs&, const Bufs&, cudaStream_t);         \
  template cudaError_t launch_col_nr<T, NN, R>(const Geom&, const ModArgs&, const StepArgs&, const Bufs&,       \
                                               cudaStream_t);                                                  \
  template cudaError_t launch_adj_row_nr<T, NN, R>(const Geom&, const AdjArgs&, const Bufs&, cudaStream_t);     \
  template cudaError_t launch_adj_col_nr<T, NN, R>(const Geom&, const ModArgs&, const AdjArgs&, const Bufs&,    \
                                                   cudaStream_t);

#define GF_INST_N(T, NN)                                                                                       \
  template cudaError_t launch_row_n<T, NN>(const Geom&, const ModArgs&, const Bufs&, cudaStream_t);             \
  template cudaError_t launch_col_n<T, NN>(const Geom&, const ModArgs&, const StepArgs&, const Bufs&,           \
                                           cudaStream_t);                                                      \
  template cudaError_t launch_col_inv_n<T, NN>(const Geom&, const ModArgs&, const void*, int, int, const Bufs&, \
                                               cudaStream_t);                                                  \
  template cudaError_t launch_row_c2r_n<T, NN>(const Geom&, const Bufs&, int, void*, cudaStream_t);             \
  template cudaError_t launch_row_r2c_n<T, NN>(const Geom&, const Bufs&, int, const void*, cudaStream_t);       \
  template cudaError_t launch_col_fwd_n<T, NN>(const Geom&, const Bufs&, int, void*, int, cudaStream_t);        \
  template cudaError_t launch_adj_row_n<T, NN>(const Geom&, const AdjArgs&, const Bufs&, cudaStream_t);         \
  template cudaError_t launch_adj_col_n<T, NN>(const Geom&, const ModArgs&, const AdjArgs&, const Bufs&,        \
                                               cudaStream_t);                                                  \
  template cudaError_t launch_adj_col_ml_n<T, NN>(const Geom&, const ModArgs&, const AdjArgs&, const Bufs&,     \
                                                  cudaStream_t);

}  // namespace gf
