// Launchers of the generic-length kernels (gf_rt.cuh) for FP32, FP64 and df64.
#include <algorithm>

#include "gf_launch.cuh"
#include "gf_rt.cuh"

namespace gf {

// threads per block: a quarter of the length (at least 64, at most 256)
inline int rt_threads(int n) { return std::min(256, std::max(64, (n / 4 + 31) / 32 * 32)); }

template <class T>
cudaError_t launch_row_rt(const Geom& g, const ModArgs& m, const Bufs& b, cudaStream_t st) {
  const size_t sm = (size_t)4 * g.nx * sizeof(cplx<T>);
  cudaError_t err = set_smem(row_nl_rt<T>, sm);
  if (err != cudaSuccess) return err;
  row_nl_rt<T><<<dim3(g.ny / 2, g.nb), rt_threads(g.nx), sm, st>>>(g, m, b);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_col_rt(const Geom& g, const ModArgs& m, const StepArgs& s, const Bufs& b, cudaStream_t st) {
  const size_t sm = (size_t)5 * g.ny * sizeof(cplx<T>);
  cudaError_t err = set_smem(col_stage_rt<T>, sm);
  if (err != cudaSuccess) return err;
  const int ncols = g.kout > 0 ? g.kout : g.nkr;
  const int nt = rt_threads(g.ny);
  if (g.nl == 1) {
    col_stage_rt<T><<<dim3(ncols, g.nb), nt, sm, st>>>(g, m, s, b);
    return cudaGetLastError();
  }
  // several layers: forward launch over (column, instance, layer) writing X to s.Xg, then the
  // inverse launch over the columns below kcut reading the X of every layer from there
  if (s.do_fwd) {
    StepArgs sf = s;
    sf.do_inv = 0;
    col_stage_rt<T><<<dim3(ncols, g.nb, g.nl), nt, sm, st>>>(g, m, sf, b);
    if ((err = cudaGetLastError()) != cudaSuccess) return err;
  }
  if (s.do_inv) {
    StepArgs si = s;
    si.do_fwd = 0;
    si.do_inv = 1;
    if (s.do_fwd) si.sol = s.Xg;
    col_stage_rt<T><<<dim3(std::min(ncols, g.kcut), g.nb, g.nl), nt, sm, st>>>(g, m, si, b);
  }
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_col_inv_rt(const Geom& g, const ModArgs& m, const void* src, int kind, int mask, const Bufs& b,
                              cudaStream_t st) {
  const size_t sm = (size_t)2 * g.ny * sizeof(cplx<T>);
  cudaError_t err = set_smem(col_inv_rt<T>, sm);
  if (err != cudaSuccess) return err;
  col_inv_rt<T><<<dim3(g.nkr, g.nb), rt_threads(g.ny), sm, st>>>(g, m, src, kind, mask, b);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_row_c2r_rt(const Geom& g, const Bufs& b, int nf, void* out, cudaStream_t st) {
  const size_t sm = (size_t)2 * g.nx * sizeof(cplx<T>);
  cudaError_t err = set_smem(row_c2r_rt<T>, sm);
  if (err != cudaSuccess) return err;
  row_c2r_rt<T><<<dim3(g.ny / 2, g.nb), rt_threads(g.nx), sm, st>>>(g, b, nf, static_cast<T*>(out));
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_row_r2c_rt(const Geom& g, const Bufs& b, int nf, const void* in, cudaStream_t st) {
  const size_t sm = (size_t)2 * g.nx * sizeof(cplx<T>);
  cudaError_t err = set_smem(row_r2c_rt<T>, sm);
  if (err != cudaSuccess) return err;
  row_r2c_rt<T><<<dim3(g.ny / 2, g.nb), rt_threads(g.nx), sm, st>>>(g, b, nf, static_cast<const T*>(in));
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_col_fwd_rt(const Geom& g, const Bufs& b, int nf, void* out, int zero_mean, cudaStream_t st) {
  const size_t sm = (size_t)2 * g.ny * sizeof(cplx<T>);
  cudaError_t err = set_smem(col_fwd_rt<T>, sm);
  if (err != cudaSuccess) return err;
  col_fwd_rt<T><<<dim3(g.nkr, g.nb), rt_threads(g.ny), sm, st>>>(g, b, nf, static_cast<cplx<T>*>(out), zero_mean);
  return cudaGetLastError();
}

#define GF_INST_RT(T)                                                                                           \
  template cudaError_t launch_row_rt<T>(const Geom&, const ModArgs&, const Bufs&, cudaStream_t);                \
  template cudaError_t launch_col_rt<T>(const Geom&, const ModArgs&, const StepArgs&, const Bufs&, cudaStream_t); \
  template cudaError_t launch_col_inv_rt<T>(const Geom&, const ModArgs&, const void*, int, int, const Bufs&,    \
                                            cudaStream_t);                                                     \
  template cudaError_t launch_row_c2r_rt<T>(const Geom&, const Bufs&, int, void*, cudaStream_t);                \
  template cudaError_t launch_row_r2c_rt<T>(const Geom&, const Bufs&, int, const void*, cudaStream_t);          \
  template cudaError_t launch_col_fwd_rt<T>(const Geom&, const Bufs&, int, void*, int, cudaStream_t);

GF_INST_RT(float)
GF_INST_RT(double)
GF_INST_RT(df64)

}  // namespace gf
