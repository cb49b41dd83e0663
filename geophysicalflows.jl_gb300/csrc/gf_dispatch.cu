// Dispatch from runtime sizes to the per-size launchers, and the element-wise / reduction
// launchers (the FFT kernels themselves are instantiated in the gf_k_<type>_<n>.cu units).
#include "gf_kernels.cuh"
#include "gf_launch.cuh"

#include <type_traits>

namespace gf {

// FP32: the autotuner's radix (4, 8 or 16) when one was chosen; otherwise RADIX<T>
#define GF_ROW_CASE(N)                                                                      \
  case N:                                                                                   \
    if constexpr (std::is_same<T, float>::value) {                                          \
      if (g.tuneRr == 16) return launch_row_nr<float, N, 16>(g, m, b, st);                  \
      if constexpr (N <= 1024)                                                              \
        if (g.tuneRr == 4) return launch_row_nr<float, N, 4>(g, m, b, st);                  \
    }                                                                                       \
    return launch_row_n<T, N>(g, m, b, st);
#define GF_COL_CASE(N)                                                                      \
  case N:                                                                                   \
    if constexpr (std::is_same<T, float>::value) {                                          \
      if (g.tuneRc == 16) return launch_col_nr<float, N, 16>(g, m, s, b, st);               \
      if constexpr (N <= 1024)                                                              \
        if (g.tuneRc == 4) return launch_col_nr<float, N, 4>(g, m, s, b, st);               \
    }                                                                                       \
    return launch_col_n<T, N>(g, m, s, b, st);

template <class T>
cudaError_t launch_row(const Geom& g, const ModArgs& m, const Bufs& b, cudaStream_t st) {
  if (g.rtx) return launch_row_rt<T>(g, m, b, st);
  if (g.fpR) return launch_row_fp<T>(g, m, b, st);
  switch (g.nx) {
    GF_ROW_CASE(32) GF_ROW_CASE(64) GF_ROW_CASE(128) GF_ROW_CASE(256) GF_ROW_CASE(512) GF_ROW_CASE(1024)
    GF_ROW_CASE(2048)
    default: return cudaErrorInvalidValue;
  }
}

template <class T>
cudaError_t launch_col(const Geom& g, const ModArgs& m, const StepArgs& s, const Bufs& b, cudaStream_t st) {
  if (g.rty) return launch_col_rt<T>(g, m, s, b, st);
  if (g.fpRc) return launch_col_fp<T>(g, m, s, b, st);
  switch (g.ny) {
    GF_COL_CASE(32) GF_COL_CASE(64) GF_COL_CASE(128) GF_COL_CASE(256) GF_COL_CASE(512) GF_COL_CASE(1024)
    GF_COL_CASE(2048)
    default: return cudaErrorInvalidValue;
  }
}

template <class T>
cudaError_t launch_col_inv(const Geom& g, const ModArgs& m, const void* src, int kind, int mask, const Bufs& b,
                           cudaStream_t st) {
  if (g.rty) return launch_col_inv_rt<T>(g, m, src, kind, mask, b, st);
  switch (g.ny) {
    case 32: return launch_col_inv_n<T, 32>(g, m, src, kind, mask, b, st);
    case 64: return launch_col_inv_n<T, 64>(g, m, src, kind, mask, b, st);
    case 128: return launch_col_inv_n<T, 128>(g, m, src, kind, mask, b, st);
    case 256: return launch_col_inv_n<T, 256>(g, m, src, kind, mask, b, st);
    case 512: return launch_col_inv_n<T, 512>(g, m, src, kind, mask, b, st);
    case 1024: return launch_col_inv_n<T, 1024>(g, m, src, kind, mask, b, st);
    case 2048: return launch_col_inv_n<T, 2048>(g, m, src, kind, mask, b, st);
    default: return cudaErrorInvalidValue;
  }
}

template <class T>
cudaError_t launch_row_c2r(const Geom& g, const Bufs& b, int nf, void* out, cudaStream_t st) {
  if (g.rtx) return launch_row_c2r_rt<T>(g, b, nf, out, st);
  switch (g.nx) {
    case 32: return launch_row_c2r_n<T, 32>(g, b, nf, out, st);
    case 64: return launch_row_c2r_n<T, 64>(g, b, nf, out, st);
    case 128: return launch_row_c2r_n<T, 128>(g, b, nf, out, st);
    case 256: return launch_row_c2r_n<T, 256>(g, b, nf, out, st);
    case 512: return launch_row_c2r_n<T, 512>(g, b, nf, out, st);
    case 1024: return launch_row_c2r_n<T, 1024>(g, b, nf, out, st);
    case 2048: return launch_row_c2r_n<T, 2048>(g, b, nf, out, st);
    default: return cudaErrorInvalidValue;
  }
}

template <class T>
cudaError_t launch_row_r2c(const Geom& g, const Bufs& b, int nf, const void* in, cudaStream_t st) {
  if (g.rtx) return launch_row_r2c_rt<T>(g, b, nf, in, st);
  switch (g.nx) {
    case 32: return launch_row_r2c_n<T, 32>(g, b, nf, in, st);
    case 64: return launch_row_r2c_n<T, 64>(g, b, nf, in, st);
    case 128: return launch_row_r2c_n<T, 128>(g, b, nf, in, st);
    case 256: return launch_row_r2c_n<T, 256>(g, b, nf, in, st);
    case 512: return launch_row_r2c_n<T, 512>(g, b, nf, in, st);
    case 1024: return launch_row_r2c_n<T, 1024>(g, b, nf, in, st);
    case 2048: return launch_row_r2c_n<T, 2048>(g, b, nf, in, st);
    default: return cudaErrorInvalidValue;
  }
}

template <class T>
cudaError_t launch_col_fwd(const Geom& g, const Bufs& b, int nf, void* out, int zero_mean, cudaStream_t st) {
  if (g.rty) return launch_col_fwd_rt<T>(g, b, nf, out, zero_mean, st);
  switch (g.ny) {
    case 32: return launch_col_fwd_n<T, 32>(g, b, nf, out, zero_mean, st);
    case 64: return launch_col_fwd_n<T, 64>(g, b, nf, out, zero_mean, st);
    case 128: return launch_col_fwd_n<T, 128>(g, b, nf, out, zero_mean, st);
    case 256: return launch_col_fwd_n<T, 256>(g, b, nf, out, zero_mean, st);
    case 512: return launch_col_fwd_n<T, 512>(g, b, nf, out, zero_mean, st);
    case 1024: return launch_col_fwd_n<T, 1024>(g, b, nf, out, zero_mean, st);
    case 2048: return launch_col_fwd_n<T, 2048>(g, b, nf, out, zero_mean, st);
    default: return cudaErrorInvalidValue;
  }
}

template <class T>
cudaError_t launch_diag(const Geom& g, const ModArgs& m, const void* sol, const void* prevsol, const void* Fh,
                        uint32_t mask, double* partial, int nblocks, cudaStream_t st) {
  diag_kernel<T><<<dim3(nblocks, g.nb), DIAG_BLOCK, 0, st>>>(g, m, static_cast<const cplx<T>*>(sol),
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
  spec_apply_kernel<T><<<dim3(256, g.nb), 256, 0, st>>>(g, m, static_cast<const cplx<T>*>(in), static_cast<cplx<T>*>(out), op);
  return cudaGetLastError();
}

#define GF_ADJ_ROW_CASE(N)                                                                  \
  case N:                                                                                   \
    if constexpr (std::is_same<T, float>::value) {                                          \
      if (g.tuneRr == 16) return launch_adj_row_nr<float, N, 16>(g, a, b, st);              \
      if constexpr (N <= 1024)                                                              \
        if (g.tuneRr == 4) return launch_adj_row_nr<float, N, 4>(g, a, b, st);              \
    }                                                                                       \
    return launch_adj_row_n<T, N>(g, a, b, st);
#define GF_ADJ_COL_CASE(N)                                                                  \
  case N:                                                                                   \
    if constexpr (std::is_same<T, float>::value) {                                          \
      if (g.tuneRc == 16) return launch_adj_col_nr<float, N, 16>(g, m, a, b, st);           \
      if constexpr (N <= 1024)                                                              \
        if (g.tuneRc == 4) return launch_adj_col_nr<float, N, 4>(g, m, a, b, st);           \
    }                                                                                       \
    return launch_adj_col_n<T, N>(g, m, a, b, st);

// the adjoint kernels follow the context's tuned radix and tiles (FP32), and its
// field-parallel setting
template <class T>
cudaError_t launch_adj_row(const Geom& g, const AdjArgs& a, const Bufs& b, cudaStream_t st) {
  if (g.fpR) return launch_adj_row_fp<T>(g, a, b, st);
  switch (g.nx) {
    GF_ADJ_ROW_CASE(32) GF_ADJ_ROW_CASE(64) GF_ADJ_ROW_CASE(128) GF_ADJ_ROW_CASE(256) GF_ADJ_ROW_CASE(512)
    GF_ADJ_ROW_CASE(1024) GF_ADJ_ROW_CASE(2048)
    default: return cudaErrorInvalidValue;
  }
}

template <class T>
cudaError_t launch_adj_col(const Geom& g, const ModArgs& m, const AdjArgs& a, const Bufs& b, cudaStream_t st) {
  if (g.nl > 1 || m.drag) {  // MultiLayerQG: every layer of a column in one block
    switch (g.ny) {
      case 32: return launch_adj_col_ml_n<T, 32>(g, m, a, b, st);
      case 64: return launch_adj_col_ml_n<T, 64>(g, m, a, b, st);
      case 128: return launch_adj_col_ml_n<T, 128>(g, m, a, b, st);
      case 256: return launch_adj_col_ml_n<T, 256>(g, m, a, b, st);
      case 512: return launch_adj_col_ml_n<T, 512>(g, m, a, b, st);
      case 1024: return launch_adj_col_ml_n<T, 1024>(g, m, a, b, st);
      case 2048: return launch_adj_col_ml_n<T, 2048>(g, m, a, b, st);
      default: return cudaErrorInvalidValue;
    }
  }
  if (g.fpRc) return launch_adj_col_fp<T>(g, m, a, b, st);
  switch (g.ny) {
    GF_ADJ_COL_CASE(32) GF_ADJ_COL_CASE(64) GF_ADJ_COL_CASE(128) GF_ADJ_COL_CASE(256) GF_ADJ_COL_CASE(512)
    GF_ADJ_COL_CASE(1024) GF_ADJ_COL_CASE(2048)
    default: return cudaErrorInvalidValue;
  }
}

// op 0: out = w K^2 f^2 in / (nx ny)^2, the gradient of the kinetic energy
//       sum_full K^2 |f in|^2 / (2 (nx ny)^2) with respect to in (real (Re, Im) pairs);
// op 1: out = M in nx ny / w, so that the normalised c2r of out is rfft^T(M in), the
//       gradient with respect to the physical field whose rfft (dealiased) is the state.
// w = 2 on interior kr columns, 1 on kr = 0 and Nyquist; f the PV-inversion factor.
template <class T>
__global__ void adj_spec_kernel(Geom g, ModArgs m, const cplx<T>* in, cplx<T>* out, int op) {
  const size_t n = (size_t)g.ny * g.nkr;
  const T dky = sel<T>(g.dky, g.dky_f, g.dky_l), dkx = sel<T>(g.dkx, g.dkx_f, g.dkx_l);
  const T ell2 = sel<T>(m.ell_inv2, m.ell_inv2_f, m.ell_inv2_l), inv_n = sel<T>(g.inv_nxny, g.inv_nxny_f, g.inv_nxny_l);
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int kr = (int)(e % g.nkr), j = (int)(e / g.nkr);
    const size_t ti = (size_t)j * g.ldk + kr;
    const bool edge = (kr == 0) || (2 * kr == g.nx);
    const cplx<T> x = in[ti];
    if (op == 0) {
      const T krT = T(kr) * dkx, lv = T(lidx(g, j)) * dky;
      const T K2 = krT * krT + lv * lv;
      const T f = psi_factor<T>(m.psi_kind, K2, ell2, m.mult, ti);
      const T w = edge ? T(1) : T(2);
      out[ti] = ((w * K2 * f * f) * inv_n * inv_n) * x;
    } else {
      const T nn = T((double)g.nx * (double)g.ny);
      out[ti] = kept(g, kr, j) ? ((edge ? T(1) : T(0.5)) * nn) * x : czero<T>();
    }
  }
}

template <class T>
cudaError_t launch_adj_spec(const Geom& g, const ModArgs& m, const void* in, void* out, int op, cudaStream_t st) {
  adj_spec_kernel<T><<<256, 256, 0, st>>>(g, m, static_cast<const cplx<T>*>(in), static_cast<cplx<T>*>(out), op);
  return cudaGetLastError();
}

// MultiLayerQG (every layer at an element): op 0, the gradient of the total kinetic energy
// sum_j H_j / sum(H) sum_full K^2 |psi_j|^2 / (2 (nx ny)^2), psi = S^-1 X:
//   out = S^-T (H_j / sum(H) w K^2 psi_j / (nx ny)^2);
// op 1: out = M in nx ny / w with the k = 0 mode zeroed (set_q! zeroes it), every layer.
template <class T>
__global__ void adj_spec_ml_kernel(Geom g, ModArgs m, LayerWeights hw, const cplx<T>* in, cplx<T>* out, int op) {
  const size_t n = (size_t)g.ny * g.nkr, lstride = (size_t)g.ny * g.ldk;
  const int nl = g.nl;
  const T dky = sel<T>(g.dky, g.dky_f, g.dky_l), dkx = sel<T>(g.dkx, g.dkx_f, g.dkx_l);
  const T ell2 = sel<T>(m.ell_inv2, m.ell_inv2_f, m.ell_inv2_l), inv_n = sel<T>(g.inv_nxny, g.inv_nxny_f, g.inv_nxny_l);
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int kr = (int)(e % g.nkr), j = (int)(e / g.nkr);
    const size_t ti = (size_t)j * g.ldk + kr;
    const bool edge = (kr == 0) || (2 * kr == g.nx);
    if (op == 1) {
      const T nn = T((double)g.nx * (double)g.ny);
      const bool z = !kept(g, kr, j) || (kr == 0 && j == 0);
      for (int L = 0; L < nl; ++L)
        out[L * lstride + ti] = z ? czero<T>() : ((edge ? T(1) : T(0.5)) * nn) * in[L * lstride + ti];
      continue;
    }
    const T krT = T(kr) * dkx, lv = T(lidx(g, j)) * dky;
    const T K2 = krT * krT + lv * lv;
    cplx<T> X[MAXL], P[MAXL];
    for (int L = 0; L < nl; ++L) X[L] = in[L * lstride + ti];
    psi_all<T>(m, nl, K2, X, P, ti);
    const T w = edge ? T(1) : T(2);
    for (int L = 0; L < nl; ++L) P[L] = ((T(hw.w[L]) * w * K2) * inv_n * inv_n) * P[L];
    if (m.psi_kind == PSI_EIGEN) {  // S^-T = Vinv^T diag(1/(lam - K^2)) V^T
      for (int r = 0; r < nl; ++r) {
        cplx<T> x = czero<T>();
        if (K2 != T(0))
          for (int q = 0; q < nl; ++q) {
            cplx<T> sq = czero<T>();
            for (int L = 0; L < nl; ++L) sq = sq + T(m.V[L * MAXL + q]) * P[L];
            x = x + (T(m.Vinv[q * MAXL + r]) * (T(1) / (T(m.lam[q]) - K2))) * sq;
          }
        out[r * lstride + ti] = x;
      }
    } else {
      const T f = psi_factor<T>(m.psi_kind, K2, ell2, m.mult, ti);
      for (int L = 0; L < nl; ++L) out[L * lstride + ti] = f * P[L];
    }
  }
}

template <class T>
cudaError_t launch_adj_spec_ml(const Geom& g, const ModArgs& m, const LayerWeights& hw, const void* in, void* out,
                               int op, cudaStream_t st) {
  adj_spec_ml_kernel<T><<<256, 256, 0, st>>>(g, m, hw, static_cast<const cplx<T>*>(in), static_cast<cplx<T>*>(out), op);
  return cudaGetLastError();
}

// out -= a + b (physical arrays of n elements)
template <class T>
__global__ void sub2_kernel(size_t n, T* out, const T* a, const T* b) {
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
    out[e] = out[e] - (a[e] + b[e]);
}

template <class T>
cudaError_t launch_sub2(size_t n, void* out, const void* a, const void* b, cudaStream_t st) {
  sub2_kernel<T><<<256, 256, 0, st>>>(n, static_cast<T*>(out), static_cast<const T*>(a), static_cast<const T*>(b));
  return cudaGetLastError();
}

template <class T> __device__ __forceinline__ double to_double(T x) { return (double)x; }
template <> __device__ __forceinline__ double to_double<df64>(df64 x) { return (double)x.hi + (double)x.lo; }

// Partial sums of the MultiLayerQG fluxes per block and instance (blockIdx.y): slot L < nl
// sum U_L v_L uy_L, slot nl + L sum (U_L - U_{L+1}) v_{L+1} psi_L; physical fields
// [instance][layer][j][i], U [layer][j] in FP64.
template <class T>
__global__ void __launch_bounds__(256) flux_kernel(Geom g, const T* __restrict__ v, const T* __restrict__ uy,
                                                   const T* __restrict__ psi, const double* __restrict__ U,
                                                   double* partial) {
  __shared__ double red[256];
  const int ib = blockIdx.y, nl = g.nl, nq = 2 * nl - 1;
  const size_t np = (size_t)g.ny * g.nx, off = (size_t)ib * nl * np;
  for (int q = 0; q < nq; ++q) {
    const bool lat = q < nl;
    const int L = lat ? q : q - nl;
    double s = 0, comp = 0;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < np; e += (size_t)gridDim.x * blockDim.x) {
      const int j = (int)(e / g.nx);
      const double x = lat ? U[(size_t)L * g.ny + j] * to_double(v[off + L * np + e]) * to_double(uy[off + L * np + e])
                           : (U[(size_t)L * g.ny + j] - U[(size_t)(L + 1) * g.ny + j]) *
                                 to_double(v[off + (L + 1) * np + e]) * to_double(psi[off + L * np + e]);
      const double t = s + x;
      comp += (fabs(s) >= fabs(x)) ? (s - t) + x : (x - t) + s;
      s = t;
    }
    red[threadIdx.x] = s + comp;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
      if ((int)threadIdx.x < st) red[threadIdx.x] += red[threadIdx.x + st];
      __syncthreads();
    }
    if (threadIdx.x == 0) partial[((size_t)q * gridDim.y + ib) * gridDim.x + blockIdx.x] = red[0];
    __syncthreads();
  }
}

template <class T>
cudaError_t launch_flux(const Geom& g, const void* v, const void* uy, const void* psi, const double* U, double* partial,
                        int nblocks, cudaStream_t st) {
  flux_kernel<T><<<dim3(nblocks, g.nb), 256, 0, st>>>(g, static_cast<const T*>(v), static_cast<const T*>(uy),
                                                      static_cast<const T*>(psi), U, partial);
  return cudaGetLastError();
}

#define GF_INST_DISPATCH(T)                                                                                    \
  template cudaError_t launch_row<T>(const Geom&, const ModArgs&, const Bufs&, cudaStream_t);                   \
  template cudaError_t launch_col<T>(const Geom&, const ModArgs&, const StepArgs&, const Bufs&, cudaStream_t);  \
  template cudaError_t launch_col_inv<T>(const Geom&, const ModArgs&, const void*, int, int, const Bufs&,       \
                                         cudaStream_t);                                                        \
  template cudaError_t launch_row_c2r<T>(const Geom&, const Bufs&, int, void*, cudaStream_t);                   \
  template cudaError_t launch_row_r2c<T>(const Geom&, const Bufs&, int, const void*, cudaStream_t);             \
  template cudaError_t launch_col_fwd<T>(const Geom&, const Bufs&, int, void*, int, cudaStream_t);              \
  template cudaError_t launch_diag<T>(const Geom&, const ModArgs&, const void*, const void*, const void*,       \
                                      uint32_t, double*, int, cudaStream_t);                                   \
  template cudaError_t launch_mask_inplace<T>(const Geom&, void*, cudaStream_t);                                \
  template cudaError_t launch_spec_apply<T>(const Geom&, const ModArgs&, const void*, void*, int, cudaStream_t); \
  template cudaError_t launch_adj_row<T>(const Geom&, const AdjArgs&, const Bufs&, cudaStream_t);               \
  template cudaError_t launch_adj_col<T>(const Geom&, const ModArgs&, const AdjArgs&, const Bufs&, cudaStream_t); \
  template cudaError_t launch_adj_spec<T>(const Geom&, const ModArgs&, const void*, void*, int, cudaStream_t);      \
  template cudaError_t launch_sub2<T>(size_t, void*, const void*, const void*, cudaStream_t);                     \
  template cudaError_t launch_adj_spec_ml<T>(const Geom&, const ModArgs&, const LayerWeights&, const void*, void*, \
                                             int, cudaStream_t);                                               \
  template cudaError_t launch_flux<T>(const Geom&, const void*, const void*, const void*, const double*, double*,   \
                                      int, cudaStream_t);

GF_INST_DISPATCH(float)
GF_INST_DISPATCH(double)
GF_INST_DISPATCH(df64)

}  // namespace gf
