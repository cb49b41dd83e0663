// Generic-length transforms: the step and the field transforms for grid sizes that have no
// compiled-in FFT length (anything but the powers of two 32 ... 2048), e.g. the reference's
// own test grids 128 x 126, 64 x 66, 32 x 34 and 16 x 16.  FourierFlows' TwoDGrid takes any
// nx, ny (FFTW plans any length); this path accepts even lengths whose prime factors are at
// most MAXPRIME.
//
// FFT: Stockham passes over a run-time radix plan (Geom::plx / ply, product = the length):
// radices 2, 4, 8, 16 through the same exact in-register butterflies as the fixed-length
// kernels (dft in gf_fft.cuh), 3, 5, 7, 11, 13 as direct in-register DFTs with the length-n
// twiddle table, other primes up to MAXPRIME as a run-time direct DFT.  Each pass reads one
// shared buffer and writes the other (no in-register staging of a whole pass), so any
// length fits and a thread runs as many butterflies as the length needs.
//
// Kernels: one row pair (x direction) or one kr column (y direction) per block, with the
// physics shared with the fixed-length kernels (pair_products, product_term,
// stage_epilogue, spec_field_value), so both paths step the same equations.
#pragma once
#include "gf_kernels.cuh"

namespace gf {

// Direct DFT of compile-time length P: out[s] = sum_r v[r] w^(DIR rs), w = exp(-2 pi i / P),
// the powers read from the length-n table (n divisible by P).
template <class T, int P, int DIR>
__device__ __forceinline__ void dft_direct(cplx<T>* v, const cplx<T>* __restrict__ tw, int n) {
  const int st = n / P;
  cplx<T> out[P];
#pragma unroll
  for (int s = 0; s < P; ++s) {
    cplx<T> acc = v[0];
#pragma unroll
    for (int r = 1; r < P; ++r) acc = acc + v[r] * twiddle<DIR>(tw, st * ((r * s) % P));
    out[s] = acc;
  }
#pragma unroll
  for (int s = 0; s < P; ++s) v[s] = out[s];
}

// One radix-P butterfly j of a Stockham pass at stride Ns (m = n / P butterflies): reads
// src[j + r m], twiddles, DFT, writes dst[(j / Ns) Ns P + j % Ns + r Ns].
template <class T, int P, int DIR>
__device__ __forceinline__ void rt_bfly(const cplx<T>* src, cplx<T>* dst, int j, int m, int Ns, int n,
                                        const cplx<T>* __restrict__ tw) {
  const int k = j % Ns;
  cplx<T> v[P];
#pragma unroll
  for (int r = 0; r < P; ++r) v[r] = src[j + r * m];
  if (Ns > 1) {
    const int ts = n / (Ns * P);
#pragma unroll
    for (int r = 1; r < P; ++r) v[r] = tw_mul<false>(v[r], twiddle<DIR>(tw, r * k * ts));
  }
  if constexpr ((P & (P - 1)) == 0) dft<P, DIR>(v);
  else dft_direct<T, P, DIR>(v, tw, n);
  const int o = (j / Ns) * Ns * P + k;
#pragma unroll
  for (int r = 0; r < P; ++r) dst[o + r * Ns] = v[r];
}

// The same for a run-time prime P <= MAXPRIME (values in a local array).
template <class T, int DIR>
__device__ __noinline__ void rt_bfly_any(const cplx<T>* src, cplx<T>* dst, int j, int m, int Ns, int n, int P,
                                         const cplx<T>* __restrict__ tw) {
  const int k = j % Ns;
  cplx<T> v[MAXPRIME];
  for (int r = 0; r < P; ++r) {
    v[r] = src[j + r * m];
    if (Ns > 1 && r > 0) v[r] = v[r] * twiddle<DIR>(tw, r * k * (n / (Ns * P)));
  }
  const int st = n / P, o = (j / Ns) * Ns * P + k;
  for (int s = 0; s < P; ++s) {
    cplx<T> acc = v[0];
    for (int r = 1; r < P; ++r) acc = acc + v[r] * twiddle<DIR>(tw, st * ((r * s) % P));
    dst[o + s * Ns] = acc;
  }
}

// Length-n FFT over the radix plan by threads t in [0, nthr): passes alternate between a
// and b; returns the buffer that holds the result.  The caller synchronises the block before;
// every pass ends with a block barrier.
template <class T, int DIR>
__device__ cplx<T>* fft_rt(cplx<T>* a, cplx<T>* b, int n, const int* plan, int np, int t, int nthr,
                           const cplx<T>* __restrict__ tw) {
  int Ns = 1;
  for (int p = 0; p < np; ++p) {
    const int P = plan[p], m = n / P;
    for (int j = t; j < m; j += nthr) {
      switch (P) {
        case 2: rt_bfly<T, 2, DIR>(a, b, j, m, Ns, n, tw); break;
        case 3: rt_bfly<T, 3, DIR>(a, b, j, m, Ns, n, tw); break;
        case 4: rt_bfly<T, 4, DIR>(a, b, j, m, Ns, n, tw); break;
        case 5: rt_bfly<T, 5, DIR>(a, b, j, m, Ns, n, tw); break;
        case 7: rt_bfly<T, 7, DIR>(a, b, j, m, Ns, n, tw); break;
        case 8: rt_bfly<T, 8, DIR>(a, b, j, m, Ns, n, tw); break;
        case 11: rt_bfly<T, 11, DIR>(a, b, j, m, Ns, n, tw); break;
        case 13: rt_bfly<T, 13, DIR>(a, b, j, m, Ns, n, tw); break;
        case 16: rt_bfly<T, 16, DIR>(a, b, j, m, Ns, n, tw); break;
        default: rt_bfly_any<T, DIR>(a, b, j, m, Ns, n, P, tw);
      }
    }
    __syncthreads();
    cplx<T>* c = a;
    a = b;
    b = c;
    Ns *= P;
  }
  return a;
}

// FFT of buffer f in place (scratch s): copies the result back when it ends in s.
template <class T, int DIR>
__device__ __forceinline__ void fft_rt_inplace(cplx<T>* f, cplx<T>* s, int n, const int* plan, int np, int t,
                                               int nthr, const cplx<T>* __restrict__ tw) {
  const cplx<T>* r = fft_rt<T, DIR>(f, s, n, plan, np, t, nthr, tw);
  if (r != f) {
    for (int i = t; i < n; i += nthr) f[i] = r[i];
    __syncthreads();
  }
}

// --------------------------------------------------------------------------- row kernel
// One row pair (j0, j0 + 1) per block, packed as one complex length-nx FFT: the c2r of the
// three inverse fields of every layer from W (pruned, kr < kcut), the products
// (pair_products), the r2c of the products into P (kr < kout).  Shared: 4 x nx (three
// fields and the scratch).
template <class T>
__global__ void __launch_bounds__(256) row_nl_rt(Geom g, ModArgs m, Bufs b) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int NX = g.nx, M = NX / 2, t = threadIdx.x, nthr = blockDim.x;
  const int j0 = 2 * blockIdx.x;
  cplx<T>* F = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* S = F + 3 * NX;
  const cplx<T>* tw = static_cast<const cplx<T>*>(b.twx);
  const cplx<T>* W = static_cast<const cplx<T>*>(b.W) + blockIdx.y * g.bs_w;
  cplx<T>* P = static_cast<cplx<T>*>(b.P) + blockIdx.y * g.bs_p;
  const int nl = g.nl, nslot = 1 + m.hasB + m.hasC;
  const int kout = g.kout > 0 ? g.kout : g.nkr;
  const T* U1D = static_cast<const T*>(m.U1D);
  const T* Qy1D = static_cast<const T*>(m.Qy1D);
  for (int L = 0; L < nl; ++L) {
    for (int f = 0; f < 3; ++f) {
      const cplx<T>* Wa = W + ((size_t)f * nl + L) * g.ny * g.ldw + (size_t)j0 * g.ldw;
      for (int k = t; k < NX; k += nthr) F[f * NX + k] = packed_spec<T>(Wa, Wa + g.ldw, k, NX, g.kcut);
    }
    __syncthreads();
    for (int f = 0; f < 3; ++f) fft_rt_inplace<T, +1>(F + f * NX, S, NX, g.plx, g.npx, t, nthr, tw);
    const cplx<T> Up = mk<T>(U1D ? U1D[L * g.ny + j0] : T(0), U1D ? U1D[L * g.ny + j0 + 1] : T(0));
    const cplx<T> Qyp = mk<T>(Qy1D ? Qy1D[L * g.ny + j0] : T(0), Qy1D ? Qy1D[L * g.ny + j0 + 1] : T(0));
    for (int x = t; x < NX; x += nthr) {
      cplx<T> A, Bv, Cv;
      pair_products<T>(g, m, b, W, L, j0, x, NX, Up, Qyp, L == nl - 1, F[x], F[NX + x], F[2 * NX + x], A, Bv, Cv);
      F[x] = A;
      if (m.hasB) { F[NX + x] = Bv; if (m.hasC) F[2 * NX + x] = Cv; }
      else F[NX + x] = Cv;
    }
    __syncthreads();
    for (int f = 0; f < nslot; ++f) fft_rt_inplace<T, -1>(F + f * NX, S, NX, g.plx, g.npx, t, nthr, tw);
    for (int f = 0; f < nslot; ++f) {
      cplx<T>* Pa = P + ((size_t)f * nl + L) * g.ny * g.ldk + (size_t)j0 * g.ldk;
      const cplx<T>* Fb = F + f * NX;
      for (int k = t; k <= M && k < kout; k += nthr) {
        const cplx<T> z = Fb[k], w = Fb[k == 0 ? 0 : NX - k];
        Pa[k] = mk<T>(T(0.5) * (z.x + w.x), T(0.5) * (z.y - w.y));
        Pa[g.ldk + k] = mk<T>(T(0.5) * (z.y + w.y), T(0.5) * (w.x - z.x));
      }
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------------ column kernel
// One kr column per block (grid: columns x instances, x layers when several): the y-FFT of
// the products, N and the stage epilogue, then the PV inversion and the y-inverse FFTs of
// (q, u, v) into W.  One layer: both halves in one launch, X kept in shared memory.  Several
// layers: as the fixed-length kernels, a forward launch per (column, layer) writing X to
// s.Xg and an inverse launch (do_fwd = 0, s.sol = X of every layer) per (column, layer).
// Shared: 5 x ny (three fields, the scratch and X).
template <class T>
__global__ void __launch_bounds__(256) col_stage_rt(Geom g, ModArgs m, StepArgs s, Bufs b) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ T eig[MAXL + 2 * MAXL * MAXL];
  const int NY = g.ny, t = threadIdx.x, nthr = blockDim.x;
  cplx<T>* F = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* S = F + 3 * NY;
  cplx<T>* Xs = F + 4 * NY;
  const int kr = blockIdx.x;
  const size_t ib = blockIdx.y;
  const int nl = g.nl;
  const bool split = nl > 1;
  const int L = split ? (int)blockIdx.z : 0;
  const bool prune = g.kout > 0;
  const bool kin = kr < (prune ? g.kout : g.nkr);
  const cplx<T>* tw = static_cast<const cplx<T>*>(b.twy);
  const EpiCtx<T> ec = epi_ctx<T>(g, m, s, kr, ib);
  const size_t lstride = ec.lstride, ioff = ec.ioff;
  const T ell2 = sel<T>(m.ell_inv2, m.ell_inv2_f, m.ell_inv2_l), muT = sel<T>(m.mu, m.mu_f, m.mu_l);
  const T sc = sel<T>(g.inv_nxny, g.inv_nxny_f, g.inv_nxny_l);
  if (m.psi_kind == PSI_EIGEN) {
    for (int a = t; a < MAXL + 2 * MAXL * MAXL; a += nthr)
      eig[a] = a < MAXL ? sel<T>(m.lam[a], m.lam_f[a], m.lam_l[a])
             : a < MAXL + MAXL * MAXL ? sel<T>(m.V[a - MAXL], m.V_f[a - MAXL], m.V_l[a - MAXL])
                                      : sel<T>(m.Vinv[a - MAXL - MAXL * MAXL], m.Vinv_f[a - MAXL - MAXL * MAXL],
                                               m.Vinv_l[a - MAXL - MAXL * MAXL]);
  }
  if (s.do_fwd) {
    const cplx<T>* P = static_cast<const cplx<T>*>(b.P) + ib * g.bs_p;
    const int nslot = 1 + m.hasB + m.hasC;
    for (int f = 0; f < nslot; ++f)
      for (int j = t; j < NY; j += nthr)
        F[f * NY + j] = kin ? P[((size_t)f * nl + L) * lstride + (size_t)j * g.ldk + kr] : czero<T>();
    __syncthreads();
    for (int f = 0; f < nslot; ++f) fft_rt_inplace<T, -1>(F + f * NY, S, NY, g.ply, g.npy, t, nthr, tw);
    for (int j = t; j < NY; j += nthr) {
      cplx<T> xn = czero<T>();
      if (kin && (!prune || kept(g, kr, j))) {
        cplx<T> N = czero<T>();
        for (int f = 0; f < nslot; ++f) {
          const int slot = (f == 0) ? 0 : (f == 1 && m.hasB) ? 1 : 2;
          N = N + product_term<T>(ec, g, m, slot, j, F[f * NY + j]);
        }
        xn = stage_epilogue<T>(ec, g, m, s, L, j, N);
      }
      if (!split) Xs[j] = xn;
      else if (kin) static_cast<cplx<T>*>(s.Xg)[ioff + (size_t)L * lstride + (size_t)j * g.ldk + kr] = xn;
    }
  } else if (!split) {
    const cplx<T>* sol = static_cast<const cplx<T>*>(s.sol);
    for (int j = t; j < NY; j += nthr) Xs[j] = (kin && kept(g, kr, j)) ? sol[ioff + (size_t)j * g.ldk + kr] : czero<T>();
  }
  if (!s.do_inv) return;
  if (kr >= g.kcut) return;  // aliased column: W is never read there
  __syncthreads();
  const cplx<T>* Xsrc = static_cast<const cplx<T>*>(s.sol) + ioff;  // several layers: X of every layer
  const T krT = ec.krT, dky = ec.dky;
  cplx<T>* Dp = ec.Dp;
  for (int j = t; j < NY; j += nthr) {
    const bool xin = kin && kept(g, kr, j);
    const T lv = T(lidx(g, j)) * dky;
    const T K2 = krT * krT + lv * lv;
    const size_t ti = (size_t)j * g.ldk + (kin ? kr : 0);
    cplx<T> x, p;
    if (split) {
      cplx<T> X[MAXL], ps[MAXL];
      for (int a = 0; a < nl; ++a) X[a] = xin ? Xsrc[(size_t)a * lstride + (size_t)j * g.ldk + kr] : czero<T>();
      if (m.psi_kind == PSI_EIGEN) {
        psi_eigen<T>(nl, eig, K2, X, ps);
      } else {
        const T fk = psi_factor<T>(m.psi_kind, K2, ell2, m.mult, ti);
        for (int a = 0; a < nl; ++a) ps[a] = fk * X[a];
      }
      x = X[L];
      p = ps[L];
    } else {
      x = Xs[j];
      if (m.psi_kind == PSI_EIGEN) {
        cplx<T> ps[1];
        psi_eigen<T>(1, eig, K2, &x, ps);
        p = ps[0];
      } else {
        p = psi_factor<T>(m.psi_kind, K2, ell2, m.mult, ti) * x;
      }
    }
    if (m.drag && kin && L == nl - 1) Dp[ti] = (muT * K2) * p;
    F[j] = sc * x;
    F[NY + j] = sc * (lv * mul_mi(p));      // u = -i l psi
    F[2 * NY + j] = sc * (krT * mul_i(p));  // v =  i kr psi
  }
  __syncthreads();
  for (int f = 0; f < 3; ++f) fft_rt_inplace<T, +1>(F + f * NY, S, NY, g.ply, g.npy, t, nthr, tw);
  cplx<T>* W = static_cast<cplx<T>*>(b.W) + ib * g.bs_w;
  for (int f = 0; f < 3; ++f) {
    cplx<T>* Wf = W + ((size_t)f * nl + L) * g.ny * g.ldw + kr;
    for (int j = t; j < NY; j += nthr) Wf[(size_t)j * g.ldw] = F[f * NY + j];
  }
}

// ------------------------------------------------------------------ field transforms
// y-inverse FFT of a derived spectral field of every layer into W (full kr range, row stride
// ldk): one column per block (spec_field_value).
template <class T>
__global__ void __launch_bounds__(256) col_inv_rt(Geom g, ModArgs m, const void* src, int kind, int mask, Bufs b) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int NY = g.ny, t = threadIdx.x, nthr = blockDim.x, kr = blockIdx.x;
  cplx<T>* F = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* S = F + NY;
  const T krT = T(kr) * sel<T>(g.dkx, g.dkx_f, g.dkx_l), dky = sel<T>(g.dky, g.dky_f, g.dky_l);
  const T sc = sel<T>(g.inv_nxny, g.inv_nxny_f, g.inv_nxny_l);
  const cplx<T>* Sp = static_cast<const cplx<T>*>(src) + blockIdx.y * g.bs_spec;
  const cplx<T>* tw = static_cast<const cplx<T>*>(b.twy);
  cplx<T>* W = static_cast<cplx<T>*>(b.W) + blockIdx.y * g.bs_w;
  const size_t lstride = (size_t)g.ny * g.ldk;
  for (int L = 0; L < g.nl; ++L) {
    for (int j = t; j < NY; j += nthr) F[j] = sc * spec_field_value<T>(g, m, Sp, kind, mask, kr, j, L, krT, dky);
    __syncthreads();
    fft_rt_inplace<T, +1>(F, S, NY, g.ply, g.npy, t, nthr, tw);
    for (int j = t; j < NY; j += nthr) W[(size_t)L * lstride + (size_t)j * g.ldk + kr] = F[j];
    __syncthreads();
  }
}

// x-direction c2r of nf fields W (full spectrum, row stride ldk) into physical out[f][j][i]
template <class T>
__global__ void __launch_bounds__(256) row_c2r_rt(Geom g, Bufs b, int nf, T* out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int NX = g.nx, t = threadIdx.x, nthr = blockDim.x, j0 = 2 * blockIdx.x;
  cplx<T>* F = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* S = F + NX;
  const cplx<T>* tw = static_cast<const cplx<T>*>(b.twx);
  const cplx<T>* W = static_cast<const cplx<T>*>(b.W) + blockIdx.y * g.bs_w;
  out += blockIdx.y * g.bs_phys;
  for (int f = 0; f < nf; ++f) {
    const cplx<T>* Wa = W + (size_t)f * g.ny * g.ldk + (size_t)j0 * g.ldk;
    for (int k = t; k < NX; k += nthr) F[k] = packed_spec<T>(Wa, Wa + g.ldk, k, NX, g.nkr);
    __syncthreads();
    fft_rt_inplace<T, +1>(F, S, NX, g.plx, g.npx, t, nthr, tw);
    T* o = out + (size_t)f * g.ny * NX + (size_t)j0 * NX;
    for (int x = t; x < NX; x += nthr) {
      o[x] = F[x].x;
      o[NX + x] = F[x].y;
    }
    __syncthreads();
  }
}

// x-direction r2c of nf physical fields in[f][j][i] into P (row stride ldk)
template <class T>
__global__ void __launch_bounds__(256) row_r2c_rt(Geom g, Bufs b, int nf, const T* in) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int NX = g.nx, M = NX / 2, t = threadIdx.x, nthr = blockDim.x, j0 = 2 * blockIdx.x;
  cplx<T>* F = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* S = F + NX;
  const cplx<T>* tw = static_cast<const cplx<T>*>(b.twx);
  cplx<T>* P = static_cast<cplx<T>*>(b.P) + blockIdx.y * g.bs_p;
  in += blockIdx.y * g.bs_phys;
  for (int f = 0; f < nf; ++f) {
    const T* src = in + (size_t)f * g.ny * NX + (size_t)j0 * NX;
    for (int x = t; x < NX; x += nthr) F[x] = mk<T>(src[x], src[NX + x]);
    __syncthreads();
    fft_rt_inplace<T, -1>(F, S, NX, g.plx, g.npx, t, nthr, tw);
    cplx<T>* Pa = P + (size_t)f * g.ny * g.ldk + (size_t)j0 * g.ldk;
    for (int k = t; k <= M; k += nthr) {
      const cplx<T> z = F[k], w = F[k == 0 ? 0 : NX - k];
      Pa[k] = mk<T>(T(0.5) * (z.x + w.x), T(0.5) * (z.y - w.y));
      Pa[g.ldk + k] = mk<T>(T(0.5) * (z.y + w.y), T(0.5) * (w.x - z.x));
    }
    __syncthreads();
  }
}

// y-direction forward FFT of nf fields P into out[f][j][kr] (row stride ldk)
template <class T>
__global__ void __launch_bounds__(256) col_fwd_rt(Geom g, Bufs b, int nf, cplx<T>* out, int zero_mean) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int NY = g.ny, t = threadIdx.x, nthr = blockDim.x, kr = blockIdx.x;
  cplx<T>* F = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* S = F + NY;
  const cplx<T>* tw = static_cast<const cplx<T>*>(b.twy);
  const cplx<T>* P = static_cast<const cplx<T>*>(b.P) + blockIdx.y * g.bs_p;
  out += blockIdx.y * g.bs_spec;
  const size_t lstride = (size_t)g.ny * g.ldk;
  for (int f = 0; f < nf; ++f) {
    for (int j = t; j < NY; j += nthr) F[j] = P[(size_t)f * lstride + (size_t)j * g.ldk + kr];
    __syncthreads();
    fft_rt_inplace<T, -1>(F, S, NY, g.ply, g.npy, t, nthr, tw);
    for (int j = t; j < NY; j += nthr) {
      cplx<T> v = F[j];
      if (zero_mean && kr == 0 && j == 0) v = czero<T>();
      out[(size_t)f * lstride + (size_t)j * g.ldk + kr] = v;
    }
    __syncthreads();
  }
}

}  // namespace gf
