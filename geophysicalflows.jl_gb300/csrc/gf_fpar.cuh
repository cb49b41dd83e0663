// Field-parallel step kernels for grids too small to fill the GPU with the row-pair and column
// blocks of the classic kernels (row_nl_kernel / col_stage_kernel).
//
// A single 128^2 run has 64 row pairs and 65 columns.  In the classic kernels one group of N/R
// threads transforms all fields of its row pair or column -- one field after the other in
// FP64/df64, in lockstep in FP32 -- so at 128 points and radix 8 a block is one half-warp whose
// dependent instruction chain is the whole work of the block, and a stage costs 30-50 us on a
// GPU that is almost idle.  Here a block has three groups of N/R threads, one per field:
//   row:    the three inverse x-transforms (q, u, v) of the row pair run concurrently, the
//           physical-space products are spread over all threads, and the two or three product
//           transforms run concurrently (a group without a product transforms a buffer that
//           is not stored, so that every thread passes the same barriers);
//   column: the product y-transforms run concurrently, N, the stage epilogue and the next
//           stage's (q, u, v) are spread over all threads, and the three inverse y-transforms
//           run concurrently.
// Radix 2 or 4 puts more threads on each transform (shorter dependent chains, more passes).
// The arithmetic per element is that of the classic kernels (the same epilogue, products and
// PV inversion functions); the transforms differ in their radix, so results agree to
// rounding.  One layer without bottom drag (the column kernel holds the three fields of one
// layer); lengths 32 ... 512.
#pragma once
#include "gf_adjoint.cuh"
#include "gf_kernels.cuh"
#include "gf_launch.cuh"

namespace gf {

template <class T, int NX, int R>
__global__ void __launch_bounds__(FP_MAXT)
    row_fp_kernel(const __grid_constant__ Geom g, const __grid_constant__ ModArgs m, const __grid_constant__ Bufs b) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int TPF = NX / R, NT = 3 * TPF, M = NX / 2;
  constexpr int PS = row_stride<T>(NX, TPF);
  const int tid = threadIdx.x, f = tid / TPF, t = tid % TPF;
  const int j0 = 2 * blockIdx.x;
  cplx<T>* buf = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* mine = buf + f * PS;  // the group's field
  const cplx<T>* tw = static_cast<const cplx<T>*>(b.twid);
  const cplx<T>* W = static_cast<const cplx<T>*>(b.W) + blockIdx.y * g.bs_w;
  cplx<T>* P = static_cast<cplx<T>*>(b.P) + blockIdx.y * g.bs_p;
  const T* U1D = static_cast<const T*>(m.U1D);
  const T* Qy1D = static_cast<const T*>(m.Qy1D);
  const int nslot = 1 + m.hasB + m.hasC;
  const int kout = g.kout > 0 ? g.kout : g.nkr;
  // x-inverse transform of field f (q, u, v) of the packed row pair
  const cplx<T>* Wa = W + (size_t)f * g.ny * g.ldw + (size_t)j0 * g.ldw;
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const int k = t + i * TPF;
    mine[swz<T>(k)] = packed_spec<T>(Wa, Wa + g.ldw, k, NX, g.kcut);
  }
  __syncthreads();
  fft_smem<T, NX, R, +1>(mine, t, tw);
  // physical-space products, every thread on its own columns x
  const cplx<T> Up = mk<T>(U1D ? U1D[j0] : T(0), U1D ? U1D[j0 + 1] : T(0));
  const cplx<T> Qp = mk<T>(Qy1D ? Qy1D[j0] : T(0), Qy1D ? Qy1D[j0 + 1] : T(0));
  for (int x = tid; x < NX; x += NT) {
    const int px = swz<T>(x);
    cplx<T> A, Bv, Cv;
    pair_products<T>(g, m, b, W, 0, j0, x, NX, Up, Qp, true, buf[px], buf[PS + px], buf[2 * PS + px], A, Bv, Cv);
    buf[px] = A;
    if (m.hasB) {
      buf[PS + px] = Bv;
      if (m.hasC) buf[2 * PS + px] = Cv;
    } else {
      buf[PS + px] = Cv;
    }
  }
  __syncthreads();
  // x-forward transforms of the products; groups f >= nslot transform a buffer not stored
  fft_smem<T, NX, R, -1>(mine, t, tw);
  if (f < nslot) {
    cplx<T>* Pa = P + (size_t)f * g.ny * g.ldk + (size_t)j0 * g.ldk;
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int k = t + i * TPF;
      if (k <= M && k < kout) unpack_store<T>(mine, k, NX, Pa, Pa + g.ldk);
    }
  }
}

// C columns per block (3 x C x NY/R threads); buffers: field f of column c at F0 + (f C + c) cs.
template <class T, int NY, int R>
__global__ void __launch_bounds__(FP_MAXT)
    col_fp_kernel(const __grid_constant__ Geom g, const __grid_constant__ ModArgs m, const __grid_constant__ StepArgs s,
                  const __grid_constant__ Bufs b, int C) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int TPF = NY / R;
  const int NT = blockDim.x, CN = C * NY;
  const int cs = g.cs;
  cplx<T>* F0 = reinterpret_cast<cplx<T>*>(smem_raw);
  const int tid = threadIdx.x, cf = tid / TPF, tf = tid % TPF;
  const int bx = blockIdx.x;
  const size_t ib = blockIdx.y;
  const bool prune = g.kout > 0;  // unobserved step: products for kr < kout, state at kept modes
  const int kend = prune ? g.kout : g.nkr;
  const cplx<T>* tw = static_cast<const cplx<T>*>(b.twid);
  const size_t lstride = (size_t)g.ny * g.ldk;
  const size_t ioff = ib * g.bs_spec;
  cplx<T>* Dp = m.D ? static_cast<cplx<T>*>(m.D) + ib * g.bs_d : nullptr;
  const T dky = sel<T>(g.dky, g.dky_f, g.dky_l), dkx = sel<T>(g.dkx, g.dkx_f, g.dkx_l);
  const T dt = sel<T>(s.dt, s.dt_f, s.dt_l), ell2 = sel<T>(m.ell_inv2, m.ell_inv2_f, m.ell_inv2_l);
  uint64_t step = s.step;
  T fscale = sel<T>(s.fscale, s.fscale_f, s.fscale_l);
  int ab3_euler = s.ab3_euler;
  if (s.clk) {
    step = (uint64_t)s.clk->step;
    const int k = s.stage >= 1 ? s.stage - 1 : 0;
    fscale = sel<T>(s.clk->fs[k], s.clk->fs_f[k], s.clk->fs_l[k]);
    ab3_euler = s.clk->step < 3;
  }
  const T U0 = sel<T>(m.U0, m.U0_f, m.U0_l);
  const T sc = sel<T>(g.inv_nxny, g.inv_nxny_f, g.inv_nxny_l);
  cplx<T>* W = static_cast<cplx<T>*>(b.W) + ib * g.bs_w;
  const int nslot = 1 + m.hasB + m.hasC;
  if (s.do_fwd) {
    const cplx<T>* P = static_cast<const cplx<T>*>(b.P) + ib * g.bs_p;
    for (int e = tid; e < nslot * CN; e += NT) {
      const int f = e / CN, r = e - f * CN, c = r % C, j = r / C, kr = bx * C + c;
      cplx<T>* dst = F0 + (size_t)(f * C + c) * cs + swz<T>(j);
      if (kr < kend) cp_async_elem<T>(dst, P + (size_t)f * lstride + (size_t)j * g.ldk + kr);
      else *dst = czero<T>();
    }
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();
    fft_smem<T, NY, R, -1>(F0 + (size_t)cf * cs, tf, tw);  // groups beyond nslot x C: not read
  }
  // N, the stage epilogue and the next stage's (q, u, v), each element by one thread, in place
  for (int e = tid; e < CN; e += NT) {
    const int c = e % C, j = e / C, kr = bx * C + c;
    const bool kin = kr < kend;
    const T krT = T(kr) * dkx;
    cplx<T> x = czero<T>();
    if (s.do_fwd) {
      if (kin && (!prune || kept(g, kr, j))) {
        const EpiCtx<T> ec{kr, krT, dky, dt, U0, fscale, step, ab3_euler, ioff, ib, lstride, 1, Dp};
        cplx<T> N = czero<T>();
        for (int f = 0; f < nslot; ++f) {
          const int slot = (f == 0) ? 0 : (f == 1 && m.hasB) ? 1 : 2;
          N = N + product_term<T>(ec, g, m, slot, j, F0[(size_t)(f * C + c) * cs + swz<T>(j)]);
        }
        x = stage_epilogue<T>(ec, g, m, s, 0, j, N);
      }
    } else if (kin && kept(g, kr, j)) {
      x = static_cast<const cplx<T>*>(s.sol)[ioff + (size_t)j * g.ldk + kr];
    }
    if (s.do_inv) {
      const T lv = T(lidx(g, j)) * dky;
      const T K2 = krT * krT + lv * lv;
      const cplx<T> p = psi_factor<T>(m.psi_kind, K2, ell2, m.mult, (size_t)j * g.ldk + (kin ? kr : 0)) * x;
      F0[(size_t)c * cs + swz<T>(j)] = sc * x;
      F0[(size_t)(C + c) * cs + swz<T>(j)] = sc * (lv * mul_mi(p));     // u = -i l psi
      F0[(size_t)(2 * C + c) * cs + swz<T>(j)] = sc * (krT * mul_i(p));  // v =  i kr psi
    }
  }
  if (!s.do_inv || bx * C >= g.kcut) return;  // whole block aliased: W is never read there
  __syncthreads();
  fft_smem<T, NY, R, +1>(F0 + (size_t)cf * cs, tf, tw);
  for (int e = tid; e < 3 * CN; e += NT) {
    const int f = e / CN, r = e - f * CN, c = r % C, j = r / C, kr = bx * C + c;
    if (kr < g.kcut) W[(size_t)f * g.ny * g.ldw + (size_t)j * g.ldw + kr] = F0[(size_t)(f * C + c) * cs + swz<T>(j)];
  }
}

// ---- adjoint (the transposed stage of gf_adjoint.cuh), same block structure
// Row: the x-c2r of (abar, bbar) by groups 0 and 1, the transposed products over all threads,
// the x-r2c of (qbar, ubar, vbar) by groups 0, 1, 2.
template <class T, int NX, int R>
__global__ void __launch_bounds__(FP_MAXT)
    adj_row_fp_kernel(const __grid_constant__ Geom g, const __grid_constant__ AdjArgs a, const __grid_constant__ Bufs b) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int TPF = NX / R, NT = 3 * TPF;
  constexpr int PS = row_stride<T>(NX, TPF);
  const int tid = threadIdx.x, f = tid / TPF, t = tid % TPF;
  const int j0 = 2 * blockIdx.x;
  cplx<T>* buf = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* mine = buf + f * PS;
  const cplx<T>* tw = static_cast<const cplx<T>*>(b.twid);
  const cplx<T>* Wb = static_cast<const cplx<T>*>(a.Wb);
  cplx<T>* Pb = static_cast<cplx<T>*>(a.Pb);
  if (f < (a.hasC ? 3 : 2)) {
    const cplx<T>* Wa = Wb + (size_t)f * g.ny * g.ldk + (size_t)j0 * g.ldk;
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int k = t + i * TPF;
      mine[swz<T>(k)] = packed_spec<T>(Wa, Wa + g.ldk, k, NX, g.nkr);
    }
  }
  __syncthreads();
  fft_smem<T, NX, R, +1>(mine, t, tw);  // group 2 without the U(y) product: a buffer overwritten below
  for (int x = tid; x < NX; x += NT) {
    const int px = swz<T>(x);
    adj_pair_products<T>(g, a, j0, x, NX, buf[px], buf[PS + px], a.hasC ? buf[2 * PS + px] : czero<T>(), buf[px],
                         buf[PS + px], buf[2 * PS + px]);
  }
  __syncthreads();
  fft_smem<T, NX, R, -1>(mine, t, tw);
  cplx<T>* Pa = Pb + (size_t)f * g.ny * g.ldk + (size_t)j0 * g.ldk;
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const int k = t + i * TPF;
    if (k < g.kcut) unpack_store<T>(mine, k, NX, Pa, Pa + g.ldk);
  }
}

// Column: the y-FFTs of the three adjoint products by groups, Xbar and the transposed stage
// combination element by element over all threads, the y-inverse FFTs of
// (i kr Nbar / w, i l Nbar / w) by groups 0 and 1 (C columns per block).
template <class T, int NY, int R>
__global__ void __launch_bounds__(FP_MAXT)
    adj_col_fp_kernel(const __grid_constant__ Geom g, const __grid_constant__ ModArgs m,
                      const __grid_constant__ AdjArgs a, const __grid_constant__ Bufs b, int C) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int TPF = NY / R;
  const int NT = blockDim.x, CN = C * NY;
  const int cs = g.cs;
  cplx<T>* F0 = reinterpret_cast<cplx<T>*>(smem_raw);
  const int tid = threadIdx.x, cf = tid / TPF, tf = tid % TPF;
  const int bx = blockIdx.x;
  const cplx<T>* tw = static_cast<const cplx<T>*>(b.twid);
  const T dky = sel<T>(g.dky, g.dky_f, g.dky_l), dkx = sel<T>(g.dkx, g.dkx_f, g.dkx_l);
  const T ell2 = sel<T>(m.ell_inv2, m.ell_inv2_f, m.ell_inv2_l);
  const T inv_n = sel<T>(g.inv_nxny, g.inv_nxny_f, g.inv_nxny_l);
  const bool fwd = a.stage <= 4 && bx * C < g.kcut;
  if (fwd) {
    const cplx<T>* P = static_cast<const cplx<T>*>(a.Pb);
    const size_t fs = (size_t)g.ny * g.ldk;
    for (int e = tid; e < 3 * CN; e += NT) {
      const int f = e / CN, r = e - f * CN, c = r % C, j = r / C, kr = bx * C + c;
      F0[(size_t)(f * C + c) * cs + swz<T>(j)] = (kr < g.kcut) ? P[f * fs + (size_t)j * g.ldk + kr] : czero<T>();
    }
    __syncthreads();
    fft_smem<T, NY, R, -1>(F0 + (size_t)cf * cs, tf, tw);
  }
  const bool out_w = !(a.stage == 1 && !a.head);
  for (int e = tid; e < CN; e += NT) {
    const int c = e % C, j = e / C, kr = bx * C + c;
    const bool kin = kr < g.nkr;
    const T krT = T(kr) * dkx;
    const bool edge = (kr == 0) || (2 * kr == g.nx);
    const T scale_in = edge ? inv_n : T(2) * inv_n;  // irfft^T: w / (nx ny)
    const T scale_out = edge ? T(1) : T(0.5);       // rfft^T via the c2r path: 1 / w
    const size_t ti = (size_t)j * g.ldk + kr;
    const bool keep = kin && kept(g, kr, j);
    cplx<T> xj = czero<T>();
    if (fwd && keep) {  // Xbar of this stage
      const T lv = T(lidx(g, j)) * dky;
      const T K2 = krT * krT + lv * lv;
      const T f = psi_factor<T>(m.psi_kind, K2, ell2, m.mult, ti);
      const cplx<T> Q = F0[(size_t)c * cs + swz<T>(j)], Ub = F0[(size_t)(C + c) * cs + swz<T>(j)],
                    Vb = F0[(size_t)(2 * C + c) * cs + swz<T>(j)];
      xj = scale_in * (Q + f * (lv * mul_i(Ub) - krT * mul_i(Vb)));
    }
    // transposed stage combination -> the next cotangent
    const cplx<T> nb = kin ? adj_stage_combine<T>(a, ti, keep, xj) : czero<T>();
    if (out_w) {
      F0[(size_t)c * cs + swz<T>(j)] = (scale_out * krT) * mul_i(nb);
      F0[(size_t)(C + c) * cs + swz<T>(j)] = (scale_out * (T(lidx(g, j)) * dky)) * mul_i(nb);
      if (a.hasC) F0[(size_t)(2 * C + c) * cs + swz<T>(j)] = (-scale_out) * nb;  // the U(y) product
    }
  }
  if (!out_w) return;
  __syncthreads();
  fft_smem<T, NY, R, +1>(F0 + (size_t)cf * cs, tf, tw);  // the third field: stored with the U(y) product
  cplx<T>* Wb = static_cast<cplx<T>*>(a.Wb);
  for (int e = tid; e < (a.hasC ? 3 : 2) * CN; e += NT) {
    const int f = e / CN, r = e - f * CN, c = r % C, j = r / C, kr = bx * C + c;
    if (kr < g.nkr) Wb[(size_t)f * g.ny * g.ldk + (size_t)j * g.ldk + kr] = F0[(size_t)(f * C + c) * cs + swz<T>(j)];
  }
}

template <class T, int NN, int R>
cudaError_t launch_row_fp_nr(const Geom& g, const ModArgs& m, const Bufs& b, cudaStream_t st) {
  const size_t sm = (size_t)3 * row_stride<T>(NN, NN / R) * sizeof(cplx<T>);
  auto k = row_fp_kernel<T, NN, R>;
  cudaError_t err = set_smem(k, sm);
  if (err != cudaSuccess) return err;
  k<<<dim3(g.ny / 2, g.nb), 3 * (NN / R), sm, st>>>(g, m, b);
  return cudaGetLastError();
}

template <class T, int NN, int R>
cudaError_t launch_col_fp_nr(const Geom& g, const ModArgs& m, const StepArgs& s, const Bufs& b, cudaStream_t st) {
  const int C = g.fpC > 0 ? g.fpC : 1;
  Geom g2 = g;
  g2.cs = col_stride<T>(NN, C);
  const size_t sm = (size_t)3 * C * g2.cs * sizeof(cplx<T>);
  auto k = col_fp_kernel<T, NN, R>;
  cudaError_t err = set_smem(k, sm);
  if (err != cudaSuccess) return err;
  const int ncols = g.kout > 0 ? g.kout : g.nkr;
  k<<<dim3((ncols + C - 1) / C, g.nb), 3 * C * (NN / R), sm, st>>>(g2, m, s, b, C);
  return cudaGetLastError();
}

template <class T, int NN, int R>
cudaError_t launch_adj_row_fp_nr(const Geom& g, const AdjArgs& a, const Bufs& b, cudaStream_t st) {
  const size_t sm = (size_t)3 * row_stride<T>(NN, NN / R) * sizeof(cplx<T>);
  auto k = adj_row_fp_kernel<T, NN, R>;
  cudaError_t err = set_smem(k, sm);
  if (err != cudaSuccess) return err;
  k<<<g.ny / 2, 3 * (NN / R), sm, st>>>(g, a, b);
  return cudaGetLastError();
}

template <class T, int NN, int R>
cudaError_t launch_adj_col_fp_nr(const Geom& g, const ModArgs& m, const AdjArgs& a, const Bufs& b, cudaStream_t st) {
  const int C = g.fpC > 0 ? g.fpC : 1;
  Geom g2 = g;
  g2.cs = col_stride<T>(NN, C);
  const size_t sm = (size_t)3 * C * g2.cs * sizeof(cplx<T>);
  auto k = adj_col_fp_kernel<T, NN, R>;
  cudaError_t err = set_smem(k, sm);
  if (err != cudaSuccess) return err;
  k<<<(g.nkr + C - 1) / C, 3 * C * (NN / R), sm, st>>>(g2, m, a, b, C);
  return cudaGetLastError();
}

// run-time length and radix -> instantiation (lengths 32 ... 256 at radix 2, 4, 8; 512 at 4, 8)
#define GF_FP_SWITCH(FN, N, R, ...)                                                     \
  switch (N * 16 + R) {                                                                 \
    case 32 * 16 + 2: return FN<T, 32, 2>(__VA_ARGS__);                                 \
    case 32 * 16 + 4: return FN<T, 32, 4>(__VA_ARGS__);                                 \
    case 32 * 16 + 8: return FN<T, 32, 8>(__VA_ARGS__);                                 \
    case 64 * 16 + 2: return FN<T, 64, 2>(__VA_ARGS__);                                 \
    case 64 * 16 + 4: return FN<T, 64, 4>(__VA_ARGS__);                                 \
    case 64 * 16 + 8: return FN<T, 64, 8>(__VA_ARGS__);                                 \
    case 128 * 16 + 2: return FN<T, 128, 2>(__VA_ARGS__);                               \
    case 128 * 16 + 4: return FN<T, 128, 4>(__VA_ARGS__);                               \
    case 128 * 16 + 8: return FN<T, 128, 8>(__VA_ARGS__);                               \
    case 256 * 16 + 2: return FN<T, 256, 2>(__VA_ARGS__);                               \
    case 256 * 16 + 4: return FN<T, 256, 4>(__VA_ARGS__);                               \
    case 256 * 16 + 8: return FN<T, 256, 8>(__VA_ARGS__);                               \
    case 512 * 16 + 4: return FN<T, 512, 4>(__VA_ARGS__);                               \
    case 512 * 16 + 8: return FN<T, 512, 8>(__VA_ARGS__);                               \
    default: return cudaErrorInvalidValue;                                              \
  }

template <class T>
cudaError_t launch_row_fp(const Geom& g, const ModArgs& m, const Bufs& b, cudaStream_t st) {
  GF_FP_SWITCH(launch_row_fp_nr, g.nx, g.fpR, g, m, b, st)
}

template <class T>
cudaError_t launch_col_fp(const Geom& g, const ModArgs& m, const StepArgs& s, const Bufs& b, cudaStream_t st) {
  GF_FP_SWITCH(launch_col_fp_nr, g.ny, g.fpRc, g, m, s, b, st)
}

template <class T>
cudaError_t launch_adj_row_fp(const Geom& g, const AdjArgs& a, const Bufs& b, cudaStream_t st) {
  GF_FP_SWITCH(launch_adj_row_fp_nr, g.nx, g.fpR, g, a, b, st)
}

template <class T>
cudaError_t launch_adj_col_fp(const Geom& g, const ModArgs& m, const AdjArgs& a, const Bufs& b, cudaStream_t st) {
  GF_FP_SWITCH(launch_adj_col_fp_nr, g.ny, g.fpRc, g, m, a, b, st)
}

}  // namespace gf
