// Fused kernels of the pseudospectral step.  One time-stepper stage of the reference
// (FourierFlows stepforward! -> calcN! -> stage combination) is two kernels here:
//
//   row kernel  : for a pair of rows j, j+1 and every layer: the x-direction c2r of the
//                 three inverse fields (q, u, v) packed two rows per complex FFT, the
//                 physical-space products (u q, v q, u Qx + v Qy, ...), and the x-direction
//                 r2c of the products.
//   column kernel: for a block of C adjacent kr columns: the y-direction forward FFT of
//                 the products, N = -i kr A - i l B - C (+ forcing, drag), the stepper's
//                 stage combination (RK4 / ETDRK4 / AB3 / ForwardEuler, filtered or not),
//                 the dealias mask, the PV inversion psi(X) and the y-direction inverse FFT
//                 of the next stage's (q, u, v) -- i.e. the first half of the next calcN!.
//
// So every stage costs one HBM sweep of the products and one of the pruned inverse fields,
// instead of the reference's 5-7 FFT library calls plus ~8 broadcast sweeps per calcN!.
// Per-element wavenumber arithmetic runs in the storage type T (FP64 only in the FP64 path).
#pragma once
#include <utility>

#include "gf_fft.cuh"
#include "gf_philox.cuh"
#include "gf_internal.h"

// Minimum resident blocks per SM requested for the FP32 step kernels (register budget):
// column kernel (512 threads) and row kernel (256 threads).
#ifndef GF_MINBLOCKS_F32
#define GF_MINBLOCKS_F32 1        // column lengths >= 1024
#endif
#ifndef GF_MINBLOCKS_SMALL_F32
#define GF_MINBLOCKS_SMALL_F32 2  // shorter columns (small grids, ensembles: many small blocks)
#endif
#ifndef GF_ROW_MINBLOCKS_F32
#define GF_ROW_MINBLOCKS_F32 3
#endif
#ifndef GF_ROW_MINBLOCKS_WIDE
#define GF_ROW_MINBLOCKS_WIDE 2   // FP64 and df64 row kernels (128 registers, no spills)
#endif
#ifndef GF_MINBLOCKS_WIDE_COL
#define GF_MINBLOCKS_WIDE_COL 1   // FP64 and df64 column kernels
#endif
// Elements per iteration of the column kernel's stage-epilogue loops (code size: the
// epilogue covers every stepper and forcing kind)
#ifndef GF_EPI_UNROLL
#define GF_EPI_UNROLL 1
#endif
// Column kernel, one layer: prefetch the stage input and accumulator of the element this many
// iterations ahead in the epilogue loop (0: off)
#ifndef GF_EPI_PREFETCH
#define GF_EPI_PREFETCH 1
#endif
// Elements per iteration of the wide column path's (q, u, v) fill loop
#ifndef GF_FILL_UNROLL
#define GF_FILL_UNROLL 16
#endif

namespace gf {

constexpr int EPI_UNROLL = GF_EPI_UNROLL;
constexpr int FILL_UNROLL = GF_FILL_UNROLL;

// ------------------------------------------------------------------------------ helpers
__device__ __forceinline__ bool kept(const Geom& g, int kr, int j) { return kr < g.kcut && (j < g.lA || j > g.lB); }
// signed wavenumber index of row j (fftfreq order)
__device__ __forceinline__ int lidx(const Geom& g, int j) { return j < g.ny / 2 ? j : j - g.ny; }

template <class T>
__device__ __forceinline__ cplx<T> ldc(const void* p, size_t i, int is_cplx) {
  if (is_cplx) return static_cast<const cplx<T>*>(p)[i];
  return mk<T>(static_cast<const T*>(p)[i], T(0));
}
template <class T>
__device__ __forceinline__ cplx<T> mulc(cplx<T> c, cplx<T> x, int is_cplx) {
  return is_cplx ? c * x : c.x * x;
}

// The per-layer psi factor f of single-layer modules (psi = f X) at |k|^2 = K2.
template <class T>
__device__ __forceinline__ T psi_factor(int kind, T K2, T ell2, const void* mult, size_t ti) {
  if (kind == PSI_INVK2) return K2 == T(0) ? T(0) : T(-1) / K2;
  if (kind == PSI_HELMHOLTZ) return T(-1) / (K2 + ell2);
  return -static_cast<const T*>(mult)[ti];
}

// MultiLayerQG: psi = V diag(1/(lam - K^2)) Vinv X (zero at K = 0); e = [lam | V | Vinv].
template <class T>
__device__ __forceinline__ void psi_eigen(int nl, const T* e, T K2, const cplx<T>* X, cplx<T>* psi) {
  if (K2 == T(0)) {
    for (int a = 0; a < nl; ++a) psi[a] = czero<T>();
    return;
  }
  const T* V = e + MAXL;
  const T* Vi = e + MAXL + MAXL * MAXL;
  cplx<T> y[MAXL];
  for (int a = 0; a < nl; ++a) {
    cplx<T> s = czero<T>();
    for (int q = 0; q < nl; ++q) s = s + Vi[a * MAXL + q] * X[q];
    y[a] = (T(1) / (e[a] - K2)) * s;
  }
  for (int a = 0; a < nl; ++a) {
    cplx<T> s = czero<T>();
    for (int q = 0; q < nl; ++q) s = s + V[a * MAXL + q] * y[q];
    psi[a] = s;
  }
}

// Row L of the same inversion: psi_L = sum_q V[L][q] / (lam_q - K^2) sum_r Vinv[q][r] X_r, with
// the layer values from Xat(r) (zero at K = 0); the same operations in the same order as
// psi_eigen, without per-layer arrays.
template <class T, class F>
__device__ __forceinline__ cplx<T> psi_eigen_row(int nl, const T* e, T K2, int L, F&& Xat) {
  cplx<T> p = czero<T>();
  if (K2 == T(0)) return p;
  const T* V = e + MAXL;
  const T* Vi = e + MAXL + MAXL * MAXL;
  for (int q = 0; q < nl; ++q) {
    cplx<T> s = czero<T>();
    for (int r = 0; r < nl; ++r) s = s + Vi[q * MAXL + r] * Xat(r);
    p = p + V[L * MAXL + q] * ((T(1) / (e[q] - K2)) * s);
  }
  return p;
}

// psi for all layers (any module) -- used outside the hot kernels, constants read from m
template <class T>
__device__ __forceinline__ void psi_all(const ModArgs& m, int nl, T K2, const cplx<T>* X, cplx<T>* psi, size_t ti) {
  if (m.psi_kind == PSI_EIGEN) {
    T e[MAXL + 2 * MAXL * MAXL];
    for (int a = 0; a < MAXL; ++a) e[a] = T(m.lam[a]);
    for (int a = 0; a < MAXL * MAXL; ++a) { e[MAXL + a] = T(m.V[a]); e[MAXL + MAXL * MAXL + a] = T(m.Vinv[a]); }
    psi_eigen<T>(nl, e, K2, X, psi);
    return;
  }
  const T f = psi_factor<T>(m.psi_kind, K2, T(m.ell_inv2), m.mult, ti);
  for (int a = 0; a < nl; ++a) psi[a] = f * X[a];
}

// ------------------------------------------------------------------- stage epilogue
// Per-thread constants of a column-kernel thread at column kr (shared by the column kernels).
template <class T>
struct EpiCtx {
  int kr;
  T krT, dky, dt, U0, fscale;
  uint64_t step;
  int ab3_euler;
  size_t ioff, ib, lstride;
  int nl;
  cplx<T>* Dp;
};

// Per-element stage epilogue at (layer L, row j) of column x.kr: forcing, U eta term, bottom
// drag, the stepper's stage combination; returns the next stage's X (zero where dealiased).
// Columns kr < kout only.
template <class T>
__device__ __forceinline__ cplx<T> stage_epilogue(const EpiCtx<T>& x, const Geom& g, const ModArgs& m,
                                                  const StepArgs& s, int L, int j, cplx<T> N) {
  const int kr = x.kr, nl = x.nl, ab3_euler = x.ab3_euler;
  const T krT = x.krT, dt = x.dt, U0 = x.U0, fscale = x.fscale;
  const uint64_t step = x.step;
  const size_t ioff = x.ioff, ib = x.ib, lstride = x.lstride;
  cplx<T>* Dp = x.Dp;
  cplx<T> xn = czero<T>();
  const size_t ti = (size_t)j * g.ldk + kr;       // table index
  const size_t si = ioff + (size_t)L * lstride + ti;  // state index
  const bool keep = kept(g, kr, j);
  if (m.Ueta) N = N - (U0 * krT) * mul_i(static_cast<const cplx<T>*>(m.etah)[ti]);
  if (m.drag && L == nl - 1) N = N + Dp[ti];
  cplx<T>* sol = static_cast<cplx<T>*>(s.sol);
  const cplx<T> solm = keep ? sol[si] : czero<T>();
  // forcing
  if (s.fkind == FK_STATIC) {
    N = N + static_cast<const cplx<T>*>(s.Fh)[si];
  } else if (s.fkind == FK_HARMONIC) {
    N = N + fscale * static_cast<const cplx<T>*>(s.Fh)[si];
  } else if (s.fkind == FK_STOCH || s.fkind == FK_STOCH_PHASE) {
    cplx<T> Fv;
    if (s.draw) {
      const T sp = static_cast<const T*>(s.fspec)[ti];
      const uint64_t e = (uint64_t)kr + (uint64_t)g.nkr * ((uint64_t)j + (uint64_t)g.ny * L);
      Fv = czero<T>();
      const bool zero_mean = (s.fkind == FK_STOCH_PHASE) && kr == 0 && j == 0;
      if (sp != T(0) && !zero_mean) Fv = sp * draw<T>(e, step, s.seed + ib, s.fkind == FK_STOCH_PHASE);
      static_cast<cplx<T>*>(s.Fstore)[si] = Fv;
      static_cast<cplx<T>*>(s.prevsol)[si] = solm;
    } else {
      Fv = static_cast<const cplx<T>*>(s.Fh)[si];
    }
    N = N + Fv;
  }
  auto Lmul = [&](cplx<T> v) { return mulc(ldc<T>(s.Ltab, ti, s.cplxL), v, s.cplxL); };
  auto finish = [&](cplx<T> v) {
    if (s.filtered) v = static_cast<const T*>(s.filt)[ti] * v;
    sol[si] = v;
    return v;
  };
  if (s.kind == SK_NOUT) {
    static_cast<cplx<T>*>(s.acc)[si] = N;
  } else if (s.kind == SK_FE) {
    cplx<T> Rv = N;
    if (s.hasL) Rv = Rv + Lmul(solm);
    xn = finish(solm + dt * Rv);
  } else if (s.kind == SK_RK4) {
    cplx<T>* X = static_cast<cplx<T>*>(s.X);
    cplx<T>* acc = static_cast<cplx<T>*>(s.acc);
    cplx<T> Rv = N;
    if (s.hasL) Rv = Rv + Lmul(s.stage == 1 ? solm : (keep ? X[si] : czero<T>()));
    if (s.stage == 1) {
      acc[si] = T(1.0 / 6.0) * Rv;
      xn = solm + T(0.5) * dt * Rv;
    } else if (s.stage < 4) {
      acc[si] = acc[si] + T(1.0 / 3.0) * Rv;
      xn = solm + (s.stage == 2 ? T(0.5) * dt : dt) * Rv;
    } else {
      xn = finish(solm + dt * (acc[si] + T(1.0 / 6.0) * Rv));
    }
    if (s.hasL && s.stage < 4) X[si] = keep ? xn : czero<T>();
  } else if (s.kind == SK_ETDRK4) {
    const int cx = s.cplxL;
    cplx<T>* acc = static_cast<cplx<T>*>(s.acc);
    if (s.stage == 1) {
      xn = mulc(ldc<T>(s.e2, ti, cx), solm, cx) + mulc(ldc<T>(s.zeta, ti, cx), N, cx);
      static_cast<cplx<T>*>(s.s1)[si] = keep ? xn : czero<T>();
      static_cast<cplx<T>*>(s.N1)[si] = N;
      acc[si] = mulc(ldc<T>(s.alpha, ti, cx), N, cx);
    } else if (s.stage == 2) {
      xn = mulc(ldc<T>(s.e2, ti, cx), solm, cx) + mulc(ldc<T>(s.zeta, ti, cx), N, cx);
      acc[si] = acc[si] + T(2) * mulc(ldc<T>(s.beta, ti, cx), N, cx);
    } else if (s.stage == 3) {
      const cplx<T> s1 = static_cast<const cplx<T>*>(s.s1)[si];
      const cplx<T> n1 = static_cast<const cplx<T>*>(s.N1)[si];
      xn = mulc(ldc<T>(s.e2, ti, cx), s1, cx) + mulc(ldc<T>(s.zeta, ti, cx), T(2) * N - n1, cx);
      acc[si] = acc[si] + T(2) * mulc(ldc<T>(s.beta, ti, cx), N, cx);
    } else {
      xn = finish(mulc(ldc<T>(s.e, ti, cx), solm, cx) + acc[si] + mulc(ldc<T>(s.gamma, ti, cx), N, cx));
    }
  } else {  // AB3
    cplx<T> Rv = N;
    if (s.hasL) Rv = Rv + Lmul(solm);
    cplx<T> upd;
    if (ab3_euler) {
      upd = Rv;
    } else {
      const cplx<T> r1 = static_cast<const cplx<T>*>(s.Rm1)[si];
      const cplx<T> r2 = static_cast<const cplx<T>*>(s.Rm2)[si];
      upd = T(23.0 / 12.0) * Rv - T(16.0 / 12.0) * r1 + T(5.0 / 12.0) * r2;
    }
    static_cast<cplx<T>*>(s.Rout)[si] = Rv;
    xn = finish(solm + dt * upd);
  }
  if (!keep) xn = czero<T>();
  return xn;
}

// One product slot's term of N at row j of column x.kr: -i kr A, -i l B, -C (or -i l C of
// the zonal mean).
template <class T>
__device__ __forceinline__ cplx<T> product_term(const EpiCtx<T>& x, const Geom& g, const ModArgs& m, int slot, int j,
                                                cplx<T> v) {
  cplx<T> d;
  if (slot == 0) d = x.krT * mul_mi(v);
  else if (slot == 1) d = (T(lidx(g, j)) * x.dky) * mul_mi(v);
  else if (m.ql) d = (T(lidx(g, j)) * x.dky) * mul_mi(v);
  else d = czero<T>() - v;
  if (m.ql && ((x.kr == 0) != (slot == 2))) d = czero<T>();  // mean: C only; eddies: A, B
  return d;
}

// The epilogue constants of the column-kernel thread at column kr of instance ib.
template <class T>
__device__ __forceinline__ EpiCtx<T> epi_ctx(const Geom& g, const ModArgs& m, const StepArgs& s, int kr, size_t ib) {
  EpiCtx<T> x;
  x.kr = kr;
  x.krT = T(kr) * sel<T>(g.dkx, g.dkx_f, g.dkx_l);
  x.dky = sel<T>(g.dky, g.dky_f, g.dky_l);
  x.dt = sel<T>(s.dt, s.dt_f, s.dt_l);
  x.U0 = sel<T>(m.U0, m.U0_f, m.U0_l);
  // clock-dependent values: from the device clock when the launch is part of a graph
  x.step = s.step;
  x.fscale = sel<T>(s.fscale, s.fscale_f, s.fscale_l);
  x.ab3_euler = s.ab3_euler;
  if (s.clk) {
    x.step = (uint64_t)s.clk->step;
    const int k = s.stage >= 1 ? s.stage - 1 : 0;
    x.fscale = sel<T>(s.clk->fs[k], s.clk->fs_f[k], s.clk->fs_l[k]);
    x.ab3_euler = s.clk->step < 3;
  }
  x.ib = ib;
  x.ioff = ib * g.bs_spec;
  x.lstride = (size_t)g.ny * g.ldk;
  x.nl = g.nl;
  x.Dp = m.D ? static_cast<cplx<T>*>(m.D) + ib * g.bs_d : nullptr;
  return x;
}

// ------------------------------------------------------------------------ column kernel
// Block: C adjacent kr columns x (NY/R) threads per column.  Two thread mappings:
//   element mapping (global loads/stores, epilogue): c = tid % C, t = tid / C, so a warp's
//     global accesses are C-wide contiguous; thread (c, t) owns rows j = t + i (NY/R);
//   FFT mapping: column cf = tid / TPF, butterfly index tf = tid % TPF, so a warp works on
//     one column and the swizzled Stockham accesses are conflict-free.
// Shared memory, one layer without bottom drag: work buffers F0/F1 (C columns of g.cs slots
// each; F2 too with three product fields) for the product and inverse FFTs, N and the next X
// in registers.  Otherwise: F0/F1/F2 (a layer's product fields, then its (q, u, v), each
// set transformed in lockstep) and Xs (N, then the next stage X; nl x NY x C interleaved,
// thread-owned); the PV inversion of every element is recomputed from Xs where u and v of a
// layer are formed.
// MAXT: largest block the instantiation is compiled for (register budget); 640 is the wide
// FP32 variant for five radix-16 columns of 2048 (or radix-8 columns of 1024) per block, 256
// the narrow FP64 / df64 variant (one radix-8 column of 2048, three blocks per SM); both run
// the one-layer path only, with the two-buffer inverse pass.
// The column kernel's work for block (bx, by, bz) -- column block, instance, layer -- with
// its shared memory; shared by col_stage_kernel and the persistent ensemble kernel.
template <class T, int NY, int R, int MAXT = 512, bool ENS = false>
__device__ __forceinline__ void col_stage_body(const Geom& g, const ModArgs& m, const StepArgs& s, const Bufs& b, int C,
                                               int ens_bx, int ens_by, unsigned char* smem_raw, T* eig) {
  // ENS: the block index comes from (ens_bx, ens_by) (persistent ensemble launch, one layer)
  const int bx = ENS ? ens_bx : (int)blockIdx.x, by = ENS ? ens_by : (int)blockIdx.y;
  const int bz = ENS ? 0 : (int)blockIdx.z;
  constexpr int TPF = NY / R;
  const int cs = g.cs;
  const int nl = g.nl;
  cplx<T>* F0 = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* F1 = F0 + C * cs;
  cplx<T>* F2 = F1 + C * cs;  // third work buffer (not in the wide instantiation)
  cplx<T>* Xs = F2 + C * cs;  // the general path's N / next-X of every layer
  const int tid = threadIdx.x, c = tid % C, t = tid / C;
  const int cf = tid / TPF, tf = tid % TPF;
  const int kr = bx * C + c;
  // unobserved step (kout set): the products exist only for kr < kout = kcut, and the state is
  // updated only at kept modes -- the aliased modes of the state are zeroed by the next
  // stage's dealias before anything reads them, so the step's kept modes (and every later
  // state) are the same as when every mode is computed
  const bool prune = g.kout > 0;
  const bool kin = kr < (prune ? g.kout : g.nkr);
  const cplx<T>* tw = static_cast<const cplx<T>*>(b.twid);
  const size_t lstride = (size_t)g.ny * g.ldk;
  const size_t ib = by;                          // ensemble instance
  const size_t ioff = ib * g.bs_spec;                    // its state arrays
  cplx<T>* Dp = m.D ? static_cast<cplx<T>*>(m.D) + ib * g.bs_d : nullptr;
  const T dky = sel<T>(g.dky, g.dky_f, g.dky_l), krT = T(kr) * sel<T>(g.dkx, g.dkx_f, g.dkx_l);
  const T dt = sel<T>(s.dt, s.dt_f, s.dt_l), ell2 = sel<T>(m.ell_inv2, m.ell_inv2_f, m.ell_inv2_l), muT = sel<T>(m.mu, m.mu_f, m.mu_l);
  // clock-dependent values: from the device clock when the launch is part of a graph
  uint64_t step = s.step;
  T fscale = sel<T>(s.fscale, s.fscale_f, s.fscale_l);
  int ab3_euler = s.ab3_euler;
  if (s.clk) {
    step = (uint64_t)s.clk->step;
    const int k = s.stage >= 1 ? s.stage - 1 : 0;
    fscale = sel<T>(s.clk->fs[k], s.clk->fs_f[k], s.clk->fs_l[k]);
    ab3_euler = s.clk->step < 3;
  }
  if (m.psi_kind == PSI_EIGEN) {
    for (int a = tid; a < MAXL + 2 * MAXL * MAXL; a += blockDim.x)
      eig[a] = a < MAXL ? sel<T>(m.lam[a], m.lam_f[a], m.lam_l[a])
             : a < MAXL + MAXL * MAXL ? sel<T>(m.V[a - MAXL], m.V_f[a - MAXL], m.V_l[a - MAXL])
                                      : sel<T>(m.Vinv[a - MAXL - MAXL * MAXL], m.Vinv_f[a - MAXL - MAXL * MAXL],
                                               m.Vinv_l[a - MAXL - MAXL * MAXL]);
  }

  const T U0 = sel<T>(m.U0, m.U0_f, m.U0_l);
  const EpiCtx<T> ec{kr, krT, dky, dt, U0, fscale, step, ab3_euler, ioff, ib, lstride, nl, Dp};
  auto epilogue = [&](int L, int j, cplx<T> N) -> cplx<T> { return stage_epilogue<T>(ec, g, m, s, L, j, N); };
  auto slot_term = [&](int slot, int j, cplx<T> v) -> cplx<T> { return product_term<T>(ec, g, m, slot, j, v); };
  cplx<T>* W = static_cast<cplx<T>*>(b.W) + ib * g.bs_w;
  const T sc = sel<T>(g.inv_nxny, g.inv_nxny_f, g.inv_nxny_l);

  if (nl == 1 && !m.drag) {
    // ---- one layer: the product FFTs (in lockstep where the registers allow), N and the
    // next X in registers, then the three inverse FFTs of (q, u, v) -- in lockstep from three
    // buffers, or from two in the wide and narrow instantiations (which the host launches
    // for one layer without bottom drag only)
    cplx<T> xr[R];
    if (s.do_fwd) {
      const cplx<T>* P = static_cast<const cplx<T>*>(b.P) + ib * g.bs_p;
      const int nslot = 1 + m.hasB + m.hasC;
      for (int f = 0; f < nslot; ++f) {  // one cp.async group per product field
        const cplx<T>* Pf = P + (size_t)f * lstride + kr;
        cplx<T>* Fc = F0 + (size_t)f * C * cs + c * cs;
#pragma unroll
        for (int i = 0; i < R; ++i) {
          const int j = t + i * TPF;
          if (kin) cp_async_elem<T>(Fc + swz<T>(j), Pf + (size_t)j * g.ldk);
          else Fc[swz<T>(j)] = czero<T>();
        }
        cp_async_commit();
      }
      if constexpr (GF_FFT_MULTI && sizeof(T) == 4 && 3 * R <= 24) {
        // lockstep FFTs of all fields once every load has landed
        cp_async_wait<0>();
        __syncthreads();
        if (nslot == 3) fft_smem_group<T, NY, R, -1, 3>(F0 + cf * cs, C * cs, tf, tw);
        else if (nslot == 2) fft_smem_group<T, NY, R, -1, 2>(F0 + cf * cs, C * cs, tf, tw);
        else fft_smem<T, NY, R, -1>(F0 + cf * cs, tf, tw);
      } else {
        // field f's FFT while the later fields' loads are still in flight
        for (int f = 0; f < nslot; ++f) {
          const int pending = nslot - 1 - f;
          if (pending >= 2) cp_async_wait<2>();
          else if (pending == 1) cp_async_wait<1>();
          else cp_async_wait<0>();
          __syncthreads();
          fft_smem<T, NY, R, -1>(F0 + (size_t)f * C * cs + cf * cs, tf, tw);
        }
      }
#pragma unroll (EPI_UNROLL)
      for (int i = 0; i < R; ++i) {
        const int j = t + i * TPF;
        constexpr int PF = MAXT > 512 ? 0 : GF_EPI_PREFETCH;  // measured: slower in the wide blocks
        if constexpr (PF > 0) {
          if (kin && i + PF < R) {  // the state of a later element towards L1
            const size_t sn = ioff + (size_t)(j + PF * TPF) * g.ldk + kr;
            asm volatile("prefetch.global.L1 [%0];" ::"l"(static_cast<const cplx<T>*>(s.sol) + sn));
            if (s.acc) asm volatile("prefetch.global.L1 [%0];" ::"l"(static_cast<const cplx<T>*>(s.acc) + sn));
          }
        }
        xr[i] = czero<T>();
        if (!kin || (prune && !kept(g, kr, j))) continue;
        cplx<T> N = czero<T>();
        for (int f = 0; f < nslot; ++f) {
          const int slot = (f == 0) ? 0 : (f == 1 && m.hasB) ? 1 : 2;
          N = N + slot_term(slot, j, F0[(size_t)f * C * cs + c * cs + swz<T>(j)]);
        }
        xr[i] = epilogue(0, j, N);
      }
    } else {
      const cplx<T>* sol = static_cast<const cplx<T>*>(s.sol);
#pragma unroll
      for (int i = 0; i < R; ++i) {
        const int j = t + i * TPF;
        xr[i] = (kin && kept(g, kr, j)) ? sol[ioff + (size_t)j * g.ldk + kr] : czero<T>();
      }
    }
    if (!s.do_inv) return;
    if ((int)bx * C >= g.kcut) return;  // whole block aliased: W is never read there
    if constexpr (MAXT != 512) {
      // the wide and narrow instantiations, two buffers: q (F0) and u (F1) filled, then the
      // inverse FFTs of q, u and -- filled into F0 once q is stored, psi formed again from
      // the registers -- v, one after the other from a single call site (instruction cache)
#pragma unroll 1
      for (int k = 0; k < 3; ++k) {
        if (k != 1) {
#pragma unroll (FILL_UNROLL)
          for (int i = 0; i < R; ++i) {
            const int j = t + i * TPF;
            const T lv = T(lidx(g, j)) * dky;
            const T K2 = krT * krT + lv * lv;
            const cplx<T> x = xr[i];
            const cplx<T> p = psi_factor<T>(m.psi_kind, K2, ell2, m.mult, (size_t)j * g.ldk + (kin ? kr : 0)) * x;
            if (k == 0) {
              F0[c * cs + swz<T>(j)] = sc * x;
              F1[c * cs + swz<T>(j)] = sc * (lv * mul_mi(p));   // u = -i l psi
            } else {
              F0[c * cs + swz<T>(j)] = sc * (krT * mul_i(p));   // v =  i kr psi
            }
          }
        }
        __syncthreads();  // (k = 2: every thread's reads of q in F0 were before the k = 1 barrier)
        cplx<T>* Fb = (k == 1) ? F1 : F0;
        fft_smem<T, NY, R, +1>(Fb + cf * cs, tf, tw);
        if (kr < g.kcut) {
          cplx<T>* Wf = W + (size_t)k * g.ny * g.ldw + kr;
#pragma unroll
          for (int i = 0; i < R; ++i) {
            const int j = t + i * TPF;
            Wf[(size_t)j * g.ldw] = Fb[c * cs + swz<T>(j)];
          }
        }
      }
    } else {
      // (q, u, v) of the next stage; each thread rewrites only the slots it read above
#pragma unroll
      for (int i = 0; i < R; ++i) {
        const int j = t + i * TPF;
        const T lv = T(lidx(g, j)) * dky;
        const T K2 = krT * krT + lv * lv;
        const cplx<T> x = xr[i];
        const cplx<T> p = psi_factor<T>(m.psi_kind, K2, ell2, m.mult, (size_t)j * g.ldk + (kin ? kr : 0)) * x;
        F0[c * cs + swz<T>(j)] = sc * x;
        F1[c * cs + swz<T>(j)] = sc * (lv * mul_mi(p));   // u = -i l psi
        F2[c * cs + swz<T>(j)] = sc * (krT * mul_i(p));   // v =  i kr psi
      }
      __syncthreads();
      fft_smem_group<T, NY, R, +1, 3>(F0 + cf * cs, C * cs, tf, tw);
      if (kr < g.kcut) {
#pragma unroll
        for (int f = 0; f < 3; ++f) {
          cplx<T>* Wf = W + (size_t)f * g.ny * g.ldw + kr;
          const cplx<T>* Fe = F0 + (size_t)f * C * cs + c * cs;
#pragma unroll
          for (int i = 0; i < R; ++i) {
            const int j = t + i * TPF;
            Wf[(size_t)j * g.ldw] = Fe[swz<T>(j)];
          }
        }
      }
    }
    return;
  }

  if constexpr (MAXT == 512) {  // several layers or bottom drag (the wide and narrow instantiations are one-layer only)
    // Work buffers F0, F1, F2 and Xs (N, then the next stage's X of every layer: nl x NY x C,
    // thread-owned).  Per layer: the product fields of the layer in one cp.async group, their
    // FFTs in lockstep, N and the stage epilogue; then per layer the inverse FFTs of (q, u, v)
    // in lockstep.
    // Layer split (several layers, s.layer_split): one block per (column block, layer L =
    // bz) and two launches per stage -- the forward launch writes the next stage's X
    // of its layer to s.Xg; the inverse launch (do_fwd = 0, s.sol = s.Xg) reads the X of
    // every layer at each element from there for the PV inversion of its layer.  Three times
    // the blocks, and no Xs in shared memory.
    const bool split = s.layer_split;
    const int L0 = split ? bz : 0, L1 = split ? L0 + 1 : nl;
    if (s.do_fwd) {
      const cplx<T>* P = static_cast<const cplx<T>*>(b.P) + ib * g.bs_p;
      const int nslot = 1 + m.hasB + m.hasC;
      for (int L = L0; L < L1; ++L) {
        for (int f = 0; f < nslot; ++f) {  // one cp.async group per field
          const cplx<T>* Pf = P + ((size_t)f * nl + L) * lstride + kr;
          cplx<T>* Fc = F0 + (size_t)f * C * cs + c * cs;
  #pragma unroll
          for (int i = 0; i < R; ++i) {
            const int j = t + i * TPF;
            if (kin) cp_async_elem<T>(Fc + swz<T>(j), Pf + (size_t)j * g.ldk);
            else Fc[swz<T>(j)] = czero<T>();
          }
          cp_async_commit();
        }
        if constexpr (GF_FFT_MULTI && sizeof(T) == 4 && 3 * R <= 24) {
          cp_async_wait<0>();
          __syncthreads();
          if (nslot == 3) fft_smem_group<T, NY, R, -1, 3>(F0 + cf * cs, C * cs, tf, tw);
          else if (nslot == 2) fft_smem_group<T, NY, R, -1, 2>(F0 + cf * cs, C * cs, tf, tw);
          else fft_smem<T, NY, R, -1>(F0 + cf * cs, tf, tw);
        } else {
          // field f's FFT while the later fields' loads are still in flight
          for (int f = 0; f < nslot; ++f) {
            const int pending = nslot - 1 - f;
            if (pending >= 2) cp_async_wait<2>();
            else if (pending == 1) cp_async_wait<1>();
            else cp_async_wait<0>();
            __syncthreads();
            fft_smem<T, NY, R, -1>(F0 + (size_t)f * C * cs + cf * cs, tf, tw);
          }
        }
        // N of layer L and the stage epilogue (rolled: GF_EPI_UNROLL elements per iteration;
        // each thread writes only its own Xs slots)
        cplx<T>* XL = Xs + L * NY * C + c;
  #pragma unroll (EPI_UNROLL)
        for (int i = 0; i < R; ++i) {
          const int j = t + i * TPF;
          if constexpr (GF_EPI_PREFETCH > 0 && sizeof(T) == 8) {  // measured: FP32 is better without
            if (kin && i + GF_EPI_PREFETCH < R) {  // the state of a later element towards L1
              const size_t sn = ioff + (size_t)L * lstride + (size_t)(j + GF_EPI_PREFETCH * TPF) * g.ldk + kr;
              asm volatile("prefetch.global.L1 [%0];" ::"l"(static_cast<const cplx<T>*>(s.sol) + sn));
              if (s.acc) asm volatile("prefetch.global.L1 [%0];" ::"l"(static_cast<const cplx<T>*>(s.acc) + sn));
            }
          }
          cplx<T> xn = czero<T>();
          if (kin && (!prune || kept(g, kr, j))) {
            cplx<T> N = czero<T>();
            for (int f = 0; f < nslot; ++f) {
              const int slot = (f == 0) ? 0 : (f == 1 && m.hasB) ? 1 : 2;
              N = N + slot_term(slot, j, F0[(size_t)f * C * cs + c * cs + swz<T>(j)]);
            }
            xn = epilogue(L, j, N);
          }
          if (!split) XL[j * C] = xn;
          else if (kin) static_cast<cplx<T>*>(s.Xg)[ioff + (size_t)L * lstride + (size_t)j * g.ldk + kr] = xn;
        }
        __syncthreads();  // the work buffers are the next layer's load targets
      }
    } else if (!split) {
      const cplx<T>* sol = static_cast<const cplx<T>*>(s.sol);
      for (int L = 0; L < nl; ++L) {
  #pragma unroll
        for (int i = 0; i < R; ++i) {
          const int j = t + i * TPF;
          cplx<T> xn = czero<T>();
          if (kin && kept(g, kr, j)) xn = sol[ioff + (size_t)L * lstride + (size_t)j * g.ldk + kr];
          Xs[(L * NY + j) * C + c] = xn;
        }
      }
    }
    if (!s.do_inv) return;
    if ((int)bx * C >= g.kcut) return;  // whole block aliased: W is never read there
    __syncthreads();  // eig[] filled

    // y-direction inverse FFTs of (q, u, v) of every layer, in lockstep; psi of layer L from
    // the X of all layers at the element (several layers: PV inversion); the bottom-drag term
    // of the next stage from the last layer's psi
    const cplx<T>* Xsrc = static_cast<const cplx<T>*>(s.sol) + ioff;  // layer split: X of every layer
    // layer split with up to three layers: the X of every layer staged into F0..F2 with
    // cp.async (all loads in flight); each thread later reads and overwrites only its own
    // elements there, so no barrier is needed before the fill
    const bool staged = split && nl <= 3;
    if (staged) {
      for (int a = 0; a < nl; ++a) {
        cplx<T>* Fa = F0 + (size_t)a * C * cs + c * cs;
  #pragma unroll
        for (int i = 0; i < R; ++i) {
          const int j = t + i * TPF;
          if (kin && kept(g, kr, j)) cp_async_elem<T>(Fa + swz<T>(j), Xsrc + (size_t)a * lstride + (size_t)j * g.ldk + kr);
          else Fa[swz<T>(j)] = czero<T>();
        }
      }
      cp_async_commit();
      cp_async_wait<0>();
    }
    for (int L = L0; L < L1; ++L) {
  #pragma unroll 2  // rolled: the PV inversion per element is long code (instruction cache)
      for (int i = 0; i < R; ++i) {
        const int j = t + i * TPF;
        const bool xin = kin && kept(g, kr, j);
        // X of layer a at this element
        auto Xat = [&](int a) -> cplx<T> {
          if (!split) return Xs[(a * NY + j) * C + c];
          if (staged) return F0[(size_t)a * C * cs + c * cs + swz<T>(j)];
          return xin ? Xsrc[(size_t)a * lstride + (size_t)j * g.ldk + kr] : czero<T>();
        };
        const cplx<T> x = Xat(L);
        const T lv = T(lidx(g, j)) * dky;
        const T K2 = krT * krT + lv * lv;
        const size_t ti = (size_t)j * g.ldk + (kin ? kr : 0);
        // psi of layer L only (one row of the inversion, no per-layer arrays: arrays indexed
        // by the run-time layer count would live in local memory)
        const cplx<T> p = (nl > 1 && m.psi_kind == PSI_EIGEN)
                              ? psi_eigen_row<T>(nl, eig, K2, L, Xat)
                              : psi_factor<T>(m.psi_kind, K2, ell2, m.mult, ti) * x;
        if (m.drag && kin && L == nl - 1) Dp[ti] = (muT * K2) * p;
        F0[c * cs + swz<T>(j)] = sc * x;
        F1[c * cs + swz<T>(j)] = sc * (lv * mul_mi(p));   // u = -i l psi
        F2[c * cs + swz<T>(j)] = sc * (krT * mul_i(p));   // v =  i kr psi
      }
      __syncthreads();
      fft_smem_group<T, NY, R, +1, 3>(F0 + cf * cs, C * cs, tf, tw);
      if (kr < g.kcut) {
  #pragma unroll
        for (int f = 0; f < 3; ++f) {
          cplx<T>* Wf = W + ((size_t)f * nl + L) * g.ny * g.ldw + kr;
          const cplx<T>* Fe = F0 + (size_t)f * C * cs + c * cs;
  #pragma unroll
          for (int i = 0; i < R; ++i) {
            const int j = t + i * TPF;
            Wf[(size_t)j * g.ldw] = Fe[swz<T>(j)];
          }
        }
      }
      __syncthreads();  // the next layer's fill overwrites the buffers
    }
  }
}


template <class T, int NY, int R, int MAXT = 512>
__global__ void __launch_bounds__(MAXT, MAXT > 512 ? 1 : MAXT < 512 ? 3 : sizeof(T) == 4 ? (NY >= 1024 ? GF_MINBLOCKS_F32 : GF_MINBLOCKS_SMALL_F32) : GF_MINBLOCKS_WIDE_COL)
    col_stage_kernel(const __grid_constant__ Geom g, const __grid_constant__ ModArgs m,
                     const __grid_constant__ StepArgs s, const __grid_constant__ Bufs b, int C) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ T eig[MAXL + 2 * MAXL * MAXL];
  col_stage_body<T, NY, R, MAXT>(g, m, s, b, C, 0, 0, smem_raw, eig);
}

// --------------------------------------------------------------------------- row kernel
// Slots per row-pair buffer: NX, staggered by TPF when several pairs share a wavefront.
template <class T>
__host__ __device__ constexpr int row_stride(int NX, int TPF) {
  return NX + (TPF < wave_threads<T>() ? TPF : 0);
}

// Block: B row pairs x (NX/R) threads; the pair (j0, j0+1) is packed as one complex
// length-NX FFT (row j0 in the real part, j0+1 in the imaginary part).
template <class T>
__device__ __forceinline__ cplx<T> packed_spec(const cplx<T>* Wa, const cplx<T>* Wb, int k, int NX, int kcut) {
  const int M = NX / 2;
  if (k <= M) {
    if (k >= kcut) return czero<T>();
    cplx<T> A = Wa[k], B = Wb[k];
    if (k == 0 || k == M) { A.y = T(0); B.y = T(0); }   // c2r uses the real part there
    return mk<T>(A.x - B.y, A.y + B.x);                  // A + i B
  }
  const int q = NX - k;
  if (q >= kcut) return czero<T>();
  const cplx<T> A = Wa[q], B = Wb[q];
  return mk<T>(A.x + B.y, B.x - A.y);                    // conj(A) + i conj(B)
}

// unpack the spectra of the two packed rows from the swizzled buf at kr index k
template <class T>
__device__ __forceinline__ void unpack_store(const cplx<T>* buf, int k, int NX, cplx<T>* Pa, cplx<T>* Pb) {
  const cplx<T> z = buf[swz<T>(k)], w = buf[swz<T>((NX - k) & (NX - 1))];
  Pa[k] = mk<T>(T(0.5) * (z.x + w.x), T(0.5) * (z.y - w.y));
  Pb[k] = mk<T>(T(0.5) * (z.y + w.y), T(0.5) * (w.x - z.x));
}

// Physical-space products at column x of the packed row pair (j0, j0 + 1) of layer L (row
// j0 in the real parts, j0 + 1 in the imaginary parts), from the inverse fields (q, u, v):
// A = (U + u) q' (U q' when linear), B = v q', C = (U + u) Qx + v Qy (when m.hasC), with
// q' = q + eta; BarotropicQGQL: (U z' + u' Z, v' Z, v' z') from the zonal means of W.
// Up / Qyp: the pair's U(y) and Qy(y) values.  Row length NX; also stores (q', U + u, v) for
// the adjoint when b.phys is set.
template <class T>
__device__ __forceinline__ void pair_products(const Geom& g, const ModArgs& m, const Bufs& b, const cplx<T>* W, int L,
                                              int j0, int x, int NX, cplx<T> Up, cplx<T> Qyp, bool last, cplx<T> q,
                                              cplx<T> u, cplx<T> v, cplx<T>& A, cplx<T>& Bv, cplx<T>& Cv) {
  const int nl = g.nl;
  const T* eta = static_cast<const T*>(m.eta);
  const T* Qx2D = static_cast<const T*>(m.Qx2D);
  const T* Qy2D = static_cast<const T*>(m.Qy2D);
  u = u + Up;
  if (eta) q = q + mk<T>(eta[(size_t)j0 * NX + x], eta[(size_t)(j0 + 1) * NX + x]);
  if (b.phys) {  // forward fields (q + eta, u, v) of this stage, kept for the adjoint
    T* ph = static_cast<T*>(b.phys) + (size_t)L * g.ny * NX;
    const size_t ia = (size_t)j0 * NX + x, fs = (size_t)nl * g.ny * NX;
    ph[ia] = q.x; ph[ia + NX] = q.y;
    ph[fs + ia] = u.x; ph[fs + ia + NX] = u.y;
    ph[2 * fs + ia] = v.x; ph[2 * fs + ia + NX] = v.y;
  }
  const cplx<T> au = m.linear ? Up : u;
  A = mk<T>(au.x * q.x, au.y * q.y);
  Bv = mk<T>(v.x * q.x, v.y * q.y);
  Cv = czero<T>();
  if (m.ql) {
    // zonal means Z, U of the two rows (x-constant: the kr = 0 inverse values) and eddies
    const cplx<T> Z = mk<T>(W[(size_t)j0 * g.ldw].x, W[(size_t)(j0 + 1) * g.ldw].x);
    const cplx<T>* Wu = W + (size_t)nl * g.ny * g.ldw;
    const cplx<T> Um = mk<T>(Wu[(size_t)j0 * g.ldw].x, Wu[(size_t)(j0 + 1) * g.ldw].x);
    const cplx<T> ze = q - Z, ue = u - Um;
    A = mk<T>(Um.x * ze.x + ue.x * Z.x, Um.y * ze.y + ue.y * Z.y);   // U z' + u' Z
    Bv = mk<T>(v.x * Z.x, v.y * Z.y);                                 // v' Z
    Cv = mk<T>(v.x * ze.x, v.y * ze.y);                               // v' z'
  } else if (m.hasC) {
    cplx<T> Qy = Qyp, Qx = czero<T>();
    if (last && Qy2D) Qy = Qy + mk<T>(Qy2D[(size_t)j0 * NX + x], Qy2D[(size_t)(j0 + 1) * NX + x]);
    if (last && Qx2D) Qx = mk<T>(Qx2D[(size_t)j0 * NX + x], Qx2D[(size_t)(j0 + 1) * NX + x]);
    Cv = mk<T>(u.x * Qx.x + v.x * Qy.x, u.y * Qx.y + v.y * Qy.y);
  }
}

// TWO: products (u q', v q') only, in two buffers per row pair -- q, then u with the first
// product, then v with the second, one c2r and one r2c call site -- so that three df64 blocks
// (80 registers, 64 KB at 2048) fit on an SM instead of two.
// The row kernel's work for block (ens_bx, ens_by) -- row-pair block, instance -- of the
// persistent ensemble launch (its arguments through references); row_nl_kernel below runs the
// same source (gf_row_body.inc) with its own arguments and blockIdx.
template <class T, int NX, int R, bool TWO = false>
__device__ __forceinline__ void row_nl_body(const Geom& g, const ModArgs& m, const Bufs& b, int B, unsigned ens_bx,
                                            unsigned ens_by, unsigned char* smem_raw) {
#define GF_ROW_BX ens_bx
#define GF_ROW_BY ens_by
#include "gf_row_body.inc"
#undef GF_ROW_BX
#undef GF_ROW_BY
}

template <class T, int NX, int R, bool TWO = false>
__global__ void __launch_bounds__(256, TWO ? 3 : sizeof(T) == 4 ? GF_ROW_MINBLOCKS_F32 : GF_ROW_MINBLOCKS_WIDE)
    row_nl_kernel(Geom g, ModArgs m, Bufs b, int B) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
#define GF_ROW_BX blockIdx.x
#define GF_ROW_BY blockIdx.y
#include "gf_row_body.inc"
#undef GF_ROW_BX
#undef GF_ROW_BY
}

// ------------------------------------------------------------------ generic transforms
// Spectral field `kind` of layer L at (kr, j) from the layer values S (instance base, [layer]
// [j][ldk]): X, psi, u, v, du/dy, d/dx, d/dy or the raw array; `mask`: dealias X first.
template <class T>
__device__ __forceinline__ cplx<T> spec_field_value(const Geom& g, const ModArgs& m, const cplx<T>* S, int kind,
                                                    int mask, int kr, int j, int L, T krT, T dky) {
  const int nl = g.nl;
  const size_t lstride = (size_t)g.ny * g.ldk;
  const size_t ti = (size_t)j * g.ldk + kr;
  cplx<T> X[MAXL], ps[MAXL];
  for (int a = 0; a < nl; ++a) X[a] = S[a * lstride + ti];
  if (mask && !kept(g, kr, j)) for (int a = 0; a < nl; ++a) X[a] = czero<T>();
  const T lv = T(lidx(g, j)) * dky;
  if (kind == SF_X || kind == SF_RAW) return X[L];
  if (kind == SF_DX) return krT * mul_i(X[L]);
  if (kind == SF_DY) return lv * mul_i(X[L]);
  psi_all<T>(m, nl, krT * krT + lv * lv, X, ps, ti);
  const cplx<T> p = ps[L];
  if (kind == SF_PSI) return p;
  if (kind == SF_U) return lv * mul_mi(p);   // u = -i l psi
  if (kind == SF_V) return krT * mul_i(p);   // v =  i kr psi
  return (lv * lv) * p;                      // du/dy = i l u = l^2 psi
}

// y-direction inverse FFT of a derived spectral field of every layer into W (full kr
// range, row stride ldk): kind selects X, psi, u, v, du/dy, d/dx, d/dy or the raw array.
template <class T, int NY, int R>
__global__ void __launch_bounds__(512) col_inv_generic(Geom g, ModArgs m, const void* src, int kind, int mask,
                                                        Bufs b, int C) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int TPF = NY / R;
  const int cs = g.cs;
  const int tid = threadIdx.x, c = tid % C, t = tid / C;
  const int cf = tid / TPF, tf = tid % TPF;
  const int kr = blockIdx.x * C + c;
  const bool kin = kr < g.nkr;
  cplx<T>* F = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* Fc = F + c * cs;
  const T krT = T(kr) * sel<T>(g.dkx, g.dkx_f, g.dkx_l), dky = sel<T>(g.dky, g.dky_f, g.dky_l);
  const cplx<T>* S = static_cast<const cplx<T>*>(src) + blockIdx.y * g.bs_spec;
  const cplx<T>* tw = static_cast<const cplx<T>*>(b.twid);
  cplx<T>* W = static_cast<cplx<T>*>(b.W) + blockIdx.y * g.bs_w;
  const size_t lstride = (size_t)g.ny * g.ldk;
  const int nl = g.nl;
  const T sc = sel<T>(g.inv_nxny, g.inv_nxny_f, g.inv_nxny_l);
  for (int L = 0; L < nl; ++L) {
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int j = t + i * TPF;
      Fc[swz<T>(j)] = sc * (kin ? spec_field_value<T>(g, m, S, kind, mask, kr, j, L, krT, dky) : czero<T>());
    }
    __syncthreads();
    fft_smem<T, NY, R, +1>(F + cf * cs, tf, tw);
    if (kin) {
#pragma unroll
      for (int i = 0; i < R; ++i) {
        const int j = t + i * TPF;
        W[(size_t)L * lstride + (size_t)j * g.ldk + kr] = Fc[swz<T>(j)];
      }
    }
    __syncthreads();
  }
}

// x-direction c2r of nf fields W (full spectrum, row stride ldk) into physical out[f][j][i]
template <class T, int NX, int R>
__global__ void __launch_bounds__(512) row_c2r_generic(Geom g, Bufs b, int nf, T* out, int B) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int TPF = NX / R;
  const int tid = threadIdx.x, bp = tid / TPF, t = tid % TPF;
  const int j0 = 2 * (blockIdx.x * B + bp);
  cplx<T>* buf = reinterpret_cast<cplx<T>*>(smem_raw) + (size_t)bp * row_stride<T>(NX, TPF);
  const cplx<T>* tw = static_cast<const cplx<T>*>(b.twid);
  const cplx<T>* W = static_cast<const cplx<T>*>(b.W) + blockIdx.y * g.bs_w;
  out += blockIdx.y * g.bs_phys;
  for (int f = 0; f < nf; ++f) {
    const cplx<T>* Wa = W + (size_t)f * g.ny * g.ldk + (size_t)j0 * g.ldk;
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int k = t + i * TPF;
      buf[swz<T>(k)] = packed_spec<T>(Wa, Wa + g.ldk, k, NX, g.nkr);
    }
    __syncthreads();
    fft_smem<T, NX, R, +1>(buf, t, tw);
    T* o = out + (size_t)f * g.ny * NX + (size_t)j0 * NX;
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int x = t + i * TPF;
      const cplx<T> z = buf[swz<T>(x)];
      o[x] = z.x;
      o[NX + x] = z.y;
    }
    __syncthreads();
  }
}

// x-direction r2c of nf physical fields in[f][j][i] into P (row stride ldk)
template <class T, int NX, int R>
__global__ void __launch_bounds__(512) row_r2c_generic(Geom g, Bufs b, int nf, const T* in, int B) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int TPF = NX / R;
  constexpr int M = NX / 2;
  const int tid = threadIdx.x, bp = tid / TPF, t = tid % TPF;
  const int j0 = 2 * (blockIdx.x * B + bp);
  cplx<T>* buf = reinterpret_cast<cplx<T>*>(smem_raw) + (size_t)bp * row_stride<T>(NX, TPF);
  const cplx<T>* tw = static_cast<const cplx<T>*>(b.twid);
  cplx<T>* P = static_cast<cplx<T>*>(b.P) + blockIdx.y * g.bs_p;
  in += blockIdx.y * g.bs_phys;
  for (int f = 0; f < nf; ++f) {
    const T* src = in + (size_t)f * g.ny * NX + (size_t)j0 * NX;
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int x = t + i * TPF;
      buf[swz<T>(x)] = mk<T>(src[x], src[NX + x]);
    }
    __syncthreads();
    fft_smem<T, NX, R, -1>(buf, t, tw);
    cplx<T>* Pa = P + (size_t)f * g.ny * g.ldk + (size_t)j0 * g.ldk;
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int k = t + i * TPF;
      if (k <= M) unpack_store<T>(buf, k, NX, Pa, Pa + g.ldk);
    }
    __syncthreads();
  }
}

// y-direction forward FFT of nf fields P into out[f][j][kr] (row stride ldk)
template <class T, int NY, int R>
__global__ void __launch_bounds__(512) col_fwd_generic(Geom g, Bufs b, int nf, cplx<T>* out, int zero_mean, int C) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int TPF = NY / R;
  const int cs = g.cs;
  const int tid = threadIdx.x, c = tid % C, t = tid / C;
  const int cf = tid / TPF, tf = tid % TPF;
  const int kr = blockIdx.x * C + c;
  const bool kin = kr < g.nkr;
  cplx<T>* F = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* Fc = F + c * cs;
  const cplx<T>* tw = static_cast<const cplx<T>*>(b.twid);
  const cplx<T>* P = static_cast<const cplx<T>*>(b.P) + blockIdx.y * g.bs_p;
  out += blockIdx.y * g.bs_spec;
  const size_t lstride = (size_t)g.ny * g.ldk;
  for (int f = 0; f < nf; ++f) {
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int j = t + i * TPF;
      Fc[swz<T>(j)] = kin ? P[(size_t)f * lstride + (size_t)j * g.ldk + kr] : czero<T>();
    }
    __syncthreads();
    fft_smem<T, NY, R, -1>(F + cf * cs, tf, tw);
    if (kin) {
#pragma unroll
      for (int i = 0; i < R; ++i) {
        const int j = t + i * TPF;
        cplx<T> v = Fc[swz<T>(j)];
        if (zero_mean && kr == 0 && j == 0) v = czero<T>();
        out[(size_t)f * lstride + (size_t)j * g.ldk + kr] = v;
      }
    }
    __syncthreads();
  }
}

// ----------------------------------------------------------------- elementwise helpers
template <class T>
__global__ void mask_inplace_kernel(Geom g, cplx<T>* sol) {
  const size_t n = (size_t)g.nl * g.nb * g.ny * g.nkr;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int kr = e % g.nkr;
    const size_t r = e / g.nkr;
    const int j = r % g.ny;
    const int L = r / g.ny;
    if (!kept(g, kr, j)) sol[((size_t)L * g.ny + j) * g.ldk + kr] = czero<T>();
  }
}

// op 0: out = S psi (MultiLayerQG pvfromstreamfunction!); op 1: out = psi(in)
template <class T>
__global__ void spec_apply_kernel(Geom g, ModArgs m, const cplx<T>* in, cplx<T>* out, int op) {
  in += blockIdx.y * g.bs_spec;
  out += blockIdx.y * g.bs_spec;
  const size_t n = (size_t)g.ny * g.nkr;
  const int nl = g.nl;
  const size_t lstride = (size_t)g.ny * g.ldk;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int kr = e % g.nkr, j = e / g.nkr;
    const size_t ti = (size_t)j * g.ldk + kr;
    const double krv = kr * g.dkx, lv = lidx(g, j) * g.dky, K2 = krv * krv + lv * lv;
    cplx<T> X[MAXL], Y[MAXL];
    for (int a = 0; a < nl; ++a) X[a] = in[a * lstride + ti];
    if (op == 1) {
      psi_all<T>(m, nl, T(K2), X, Y, ti);
    } else if (m.psi_kind == PSI_EIGEN) {
      // S = -K^2 I + F with F = V diag(lam) Vinv
      for (int a = 0; a < nl; ++a) {
        cplx<T> s = T(-K2) * X[a];
        for (int q = 0; q < nl; ++q) {
          double fa = 0;
          for (int r = 0; r < nl; ++r) fa += m.V[a * MAXL + r] * m.lam[r] * m.Vinv[r * MAXL + q];
          s = s + T(fa) * X[q];
        }
        Y[a] = s;
      }
    } else {
      for (int a = 0; a < nl; ++a) Y[a] = T(-K2) * X[a];
    }
    for (int a = 0; a < nl; ++a) out[a * lstride + ti] = Y[a];
  }
}

// ------------------------------------------------------------------------- diagnostics
// Per-element terms of the reference's Parseval-sum diagnostics, accumulated in FP64 with
// Neumaier compensation, one block partial per slot.  w = parsevalsum weight (1 for the
// kr = 0 and Nyquist columns, 2 otherwise).
struct NeumaierAcc {
  double s = 0, c = 0;
  __device__ __forceinline__ void add(double x) {
    const double t = s + x;
    c += (fabs(s) >= fabs(x)) ? (s - t) + x : (x - t) + s;
    s = t;
  }
};

__device__ __forceinline__ double powi(double x, int n) {
  if (n == 0) return 1.0;
  double r = 1.0, b = n > 0 ? x : 1.0 / x;
  int e = n > 0 ? n : -n;
  while (e) { if (e & 1) r *= b; b *= b; e >>= 1; }
  return r;
}

template <class T>
__global__ void __launch_bounds__(DIAG_BLOCK) diag_kernel(Geom g, ModArgs m, const cplx<T>* sol, const cplx<T>* prevsol,
                                                          const cplx<T>* Fh, uint32_t mask, double* partial) {
  NeumaierAcc acc[NDIAG];
  const size_t n = (size_t)g.ny * g.nkr;
  const int nl = g.nl;
  const size_t lstride = (size_t)g.ny * g.ldk;
  sol += blockIdx.y * g.bs_spec;
  if (prevsol) prevsol += blockIdx.y * g.bs_spec;
  if (Fh) Fh += blockIdx.y * g.bs_spec;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int kr = e % g.nkr, j = e / g.nkr;
    const size_t ti = (size_t)j * g.ldk + kr;
    const double w = (kr == 0 || (g.nx % 2 == 0 && kr == g.nkr - 1)) ? 1.0 : 2.0;
    const double krv = kr * g.dkx, lv = lidx(g, j) * g.dky, K2 = krv * krv + lv * lv;
    const double iK2 = K2 == 0.0 ? 0.0 : 1.0 / K2;
    const bool k0 = (kr == 0 && j == 0);
    if (m.module == MOD_MLQG) {
      // psi in double from the stored layer values
      cplx<double> Xd[MAXL], Pd[MAXL];
      for (int a = 0; a < nl; ++a) { const cplx<T> x = sol[a * lstride + ti]; Xd[a] = mk<double>(to_double(x.x), to_double(x.y)); }
      psi_all<double>(m, nl, K2, Xd, Pd, ti);
      for (int a = 0; a < nl; ++a) {
        const double pr = Pd[a].x, pi = Pd[a].y;
        if (mask & (1u << a)) acc[a].add(w * K2 * (pr * pr + pi * pi));
        if (a + 1 < nl && (mask & (1u << (nl + a)))) {
          const double dr = pr - Pd[a + 1].x, di = pi - Pd[a + 1].y;
          acc[nl + a].add(w * (dr * dr + di * di));
        }
      }
      continue;
    }
    const cplx<T> x0 = sol[ti];
    const double sr = to_double(x0.x), si = to_double(x0.y), s2 = sr * sr + si * si;
    // forcing work term Re(S conj(F)), S = sol or (prevsol + sol)/2
    double wr = 0;
    if (Fh) {
      double ar = sr, ai = si;
      if (prevsol) { ar = 0.5 * (sr + to_double(prevsol[ti].x)); ai = 0.5 * (si + to_double(prevsol[ti].y)); }
      const double fr = to_double(Fh[ti].x), fi = to_double(Fh[ti].y);
      wr = ar * fr + ai * fi;
    }
    const double nu = m.nu, mu = m.mu_visc;
    const int nnu = m.nnu, nmu = m.nmu;
    double v[NDIAG];
    for (int q = 0; q < NDIAG; ++q) v[q] = 0;
    if (m.module == MOD_TWODNS) {
      v[0] = 0.5 * iK2 * s2;
      v[1] = 0.5 * s2;
      v[2] = 0.5 * K2 * s2;
      v[3] = k0 ? 0.0 : -nu * powi(K2, nnu - 1) * s2;
      v[4] = k0 ? 0.0 : -mu * powi(K2, nmu - 1) * s2;
      v[5] = k0 ? 0.0 : -nu * powi(K2, nnu) * s2;
      v[6] = k0 ? 0.0 : -mu * powi(K2, nmu) * s2;
      v[7] = iK2 * wr;
      v[8] = wr;
    } else if (m.module == MOD_SLQG) {
      const double f = m.psi_kind == PSI_INVK2 ? -iK2 : -1.0 / (K2 + m.ell_inv2);
      const double p2 = f * f * s2;
      v[0] = 0.5 * K2 * p2;
      v[1] = 0.5 * m.ell_inv2 * p2;
      double er = sr, ei = si;
      if (m.etah) { er += to_double(static_cast<const cplx<T>*>(m.etah)[ti].x); ei += to_double(static_cast<const cplx<T>*>(m.etah)[ti].y); }
      v[2] = 0.5 * (er * er + ei * ei);
      v[3] = k0 ? 0.0 : nu * powi(K2, nnu - 1) * s2;
      v[4] = k0 ? 0.0 : nu * powi(K2, nnu) * s2;
      v[5] = iK2 * wr;
      v[6] = wr;
      v[7] = k0 ? 0.0 : mu * iK2 * s2;
      v[8] = k0 ? 0.0 : mu * s2;
    } else if (m.module == MOD_QGQL) {
      v[0] = 0.5 * iK2 * s2;
      v[1] = k0 ? 0.0 : 0.5 * s2;
      v[2] = k0 ? 0.0 : nu * powi(K2, nnu - 1) * s2;
      v[3] = iK2 * wr;
      v[4] = k0 ? 0.0 : mu * iK2 * s2;
    } else {  // SQG
      const double M = to_double(static_cast<const T*>(m.mult)[ti]);
      v[0] = 0.5 * K2 * M * M * s2;
      v[1] = s2;
      v[2] = 0.5 * M * s2;
      v[3] = k0 ? 0.0 : 2 * nu * powi(K2, nnu) * s2;
      v[4] = 2.0 * wr;  // forced: 2 sol conj(F); stochastic: (prevsol + sol) conj(F)
    }
#pragma unroll
    for (int q = 0; q < NDIAG; ++q)
      if (mask & (1u << q)) acc[q].add(w * v[q]);
  }
  // block reduction
  __shared__ double red[DIAG_BLOCK];
  for (int q = 0; q < NDIAG; ++q) {
    if (!(mask & (1u << q))) continue;
    red[threadIdx.x] = acc[q].s + acc[q].c;
    __syncthreads();
    for (int st = DIAG_BLOCK / 2; st > 0; st >>= 1) {
      if ((int)threadIdx.x < st) red[threadIdx.x] += red[threadIdx.x + st];
      __syncthreads();
    }
    if (threadIdx.x == 0) partial[((size_t)q * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] = red[0];
    __syncthreads();
  }
}

}  // namespace gf
