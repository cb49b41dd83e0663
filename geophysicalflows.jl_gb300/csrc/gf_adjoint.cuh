// Adjoint (reverse mode) of the fused ETDRK4 / FilteredETDRK4 and RK4 / FilteredRK4 steps of
// SingleLayerQG and TwoDNavierStokes (one layer, constant U or U(y)): the transpose of the discrete
// step that gf_kernels.cuh computes, stage by stage in reverse, with the same two-kernel
// structure (the stage combinations in adj_stage_combine).
//
// Forward calcN! at a dealiased stage input X (src/singlelayerqg.jl:356-382, 443-451):
//   psi = f X, u = irfft(-i l psi), v = irfft(i kr psi), q = irfft(X), qe = q + eta,
//   N = -i kr rfft(u qe) - i l rfft(v qe) - i kr U eta_hat.
// Its transpose for a cotangent Nbar (spectral arrays as real (Re, Im) vectors over the
// stored half spectrum, physical arrays plain):
//   abar = rfft^T(i kr Nbar), bbar = rfft^T(i l Nbar)                        [adj row kernel]
//   ubar = abar qe, vbar = bbar qe, qbar = abar u + bbar v, etabar += qbar + U abar
//   Xbar = irfft^T(qbar) + f (i l irfft^T(ubar) - i kr irfft^T(vbar))          [adj col kernel]
// With U(y) (src/singlelayerqg.jl:395-432) the products are u' q, v q and C = u' Qx + v Qy
// (u' = U + u, Qx = d(eta)/dx, Qy = d(eta)/dy - U_yy, no q + eta): cbar = rfft^T(-Nbar),
// ubar += cbar Qx, vbar += cbar Qy, and the cotangents of Qx, Qy (cbar u', cbar v), summed over
// every stage, give etabar = -d/dx(sum cbar u') - d/dy(sum cbar v) at the end of the sweep.
// with rfft^T(Y) = sum over the half spectrum of Re(Y e^{i k x}) (the c2r path applied to
// Y / w) and irfft^T(x) = w rfft(x) / (nx ny), w = 2 on interior kr columns, 1 on kr = 0 and
// the Nyquist column.  The column kernel also runs the transposed stage combination:
//   stage 4: Cbar = Xbar;  N3bar = 2 conj(b) ub + 2 conj(z) Cbar;  n1acc = conj(a) ub - conj(z) Cbar;
//            xaacc = conj(e2) Cbar
//   stage 3: Bbar = Xbar;  x1acc = conj(e) ub + conj(e2) Bbar;  N2bar = 2 conj(b) ub + conj(z) Bbar
//   stage 2: Abar = M (xaacc + Xbar);  x1acc += conj(e2) Abar;  N1bar = n1acc + conj(z) Abar
//   stage 1: ubar_n = M (x1acc + Xbar)
// where ub = filter * (cotangent of the step's result) and M the dealias mask, and writes the
// y-inverse transforms of (i kr Nbar / w, i l Nbar / w) of the next (earlier) stage.
#pragma once
#include "gf_kernels.cuh"

namespace gf {

// conj(c) x for a real (is_cplx = 0) or complex coefficient table
template <class T>
__device__ __forceinline__ cplx<T> mulcj(const void* p, size_t i, cplx<T> x, int is_cplx) {
  if (!is_cplx) return static_cast<const T*>(p)[i] * x;
  const cplx<T> c = static_cast<const cplx<T>*>(p)[i];
  return mk<T>(c.x * x.x + c.y * x.y, c.x * x.y - c.y * x.x);
}

// The transposed stage combination at element ti (kr < nkr; keep: a kept mode) given
// xj = J^T Nbar of this stage's calcN! (zero where not kept): updates the accumulators and
// returns the Nbar of the next (earlier) stage -- or, at stage 5, of stage 4 from ubar_in.
// RK4 (a.rk4): RHS_s = N(X_s) + L X_s, so Xbar_s = xj + conj(L) Rbar_s; with ub the filtered
// cotangent of the step's result and Y_s = M Xbar_s:
//   stage 5: Rbar4 = dt/6 ub
//   stage 4: x1acc = ub + Y4;  Rbar3 = dt/3 ub + dt Y4
//   stage 3: x1acc += Y3;      Rbar2 = dt/3 ub + dt/2 Y3
//   stage 2: x1acc += Y2;      Rbar1 = dt/6 ub + dt/2 Y2
//   stage 1: ubar_n = M (x1acc + xj + conj(L) Rbar1)
// (n1acc holds the current Rbar).  ETDRK4: the combination in the header comment.
template <class T>
__device__ __forceinline__ cplx<T> adj_stage_combine(const AdjArgs& a, size_t ti, bool keep, cplx<T> xj,
                                                     size_t si = ~size_t(0)) {
  if (si == ~size_t(0)) si = ti;  // one layer: the state index is the table index
  const int cx = a.cplx;
  cplx<T>* ub = static_cast<cplx<T>*>(a.ub);
  cplx<T>* n1 = static_cast<cplx<T>*>(a.n1acc);
  cplx<T>* x1 = static_cast<cplx<T>*>(a.x1acc);
  if (a.rk4) {
    const T dt = sel<T>(a.dt, a.dt_f, a.dt_l);
    auto start = [&](cplx<T> u) {  // cotangent of a step's result -> stage-4 Rbar
      const cplx<T> v = a.filtered ? static_cast<const T*>(a.filt)[ti] * u : u;
      ub[si] = v;
      const cplx<T> r = (dt / T(6)) * v;
      n1[si] = r;
      return r;
    };
    auto lt = [&](cplx<T> r) { return a.L ? mulcj<T>(a.L, ti, r, cx) : czero<T>(); };
    if (a.stage == 5) return start(static_cast<const cplx<T>*>(a.ubar_in)[si]);
    if (a.stage == 1) {
      const cplx<T> un = keep ? x1[si] + xj + lt(n1[si]) : czero<T>();
      static_cast<cplx<T>*>(a.ubar_out)[si] = un;
      return a.head ? start(un) : czero<T>();
    }
    const cplx<T> u = ub[si];
    const cplx<T> y = keep ? xj + lt(n1[si]) : czero<T>();
    cplx<T> r;
    if (a.stage == 4) {
      x1[si] = u + y;
      r = (dt / T(3)) * u + dt * y;
    } else if (a.stage == 3) {
      x1[si] = x1[si] + y;
      r = (dt / T(3)) * u + (dt / T(2)) * y;
    } else {
      x1[si] = x1[si] + y;
      r = (dt / T(6)) * u + (dt / T(2)) * y;
    }
    n1[si] = r;
    return r;
  }
  auto start = [&](cplx<T> u) {  // cotangent of a step's result -> stage-4 Nbar
    const cplx<T> v = a.filtered ? static_cast<const T*>(a.filt)[ti] * u : u;
    ub[si] = v;
    return mulcj<T>(a.gamma, ti, v, cx);
  };
  if (a.stage == 5) return start(static_cast<const cplx<T>*>(a.ubar_in)[si]);
  if (a.stage == 4) {
    const cplx<T> u = ub[si];
    n1[si] = mulcj<T>(a.alpha, ti, u, cx) - mulcj<T>(a.zeta, ti, xj, cx);
    static_cast<cplx<T>*>(a.xaacc)[si] = mulcj<T>(a.e2, ti, xj, cx);
    return T(2) * mulcj<T>(a.beta, ti, u, cx) + T(2) * mulcj<T>(a.zeta, ti, xj, cx);
  }
  if (a.stage == 3) {
    const cplx<T> u = ub[si];
    x1[si] = mulcj<T>(a.e, ti, u, cx) + mulcj<T>(a.e2, ti, xj, cx);
    return T(2) * mulcj<T>(a.beta, ti, u, cx) + mulcj<T>(a.zeta, ti, xj, cx);
  }
  if (a.stage == 2) {
    const cplx<T> Ab = keep ? static_cast<const cplx<T>*>(a.xaacc)[si] + xj : czero<T>();
    x1[si] = x1[si] + mulcj<T>(a.e2, ti, Ab, cx);
    return n1[si] + mulcj<T>(a.zeta, ti, Ab, cx);
  }
  const cplx<T> un = keep ? x1[si] + xj : czero<T>();  // stage 1
  static_cast<cplx<T>*>(a.ubar_out)[si] = un;
  return a.head ? start(un) : czero<T>();
}

// The transposed products at column x of the packed row pair (j0, j0 + 1) from the cotangents
// ab, bb (and cb) of the products A = u' qe, B = v qe (and C = u' Qx + v Qy) and the stored
// forward fields (qe, u' = U + u, v): qbar = ab u' + bb v, ubar = ab qe (+ cb Qx),
// vbar = bb qe (+ cb Qy); constant U: etabar += qbar + U ab (qe = q + eta and the -i kr U
// eta_hat term); U(y): the cotangents of Qx and Qy (cb u', cb v) accumulated for the
// topography gradient.  Each element is read and written by one thread.
template <class T>
__device__ __forceinline__ void adj_pair_products(const Geom& g, const AdjArgs& a, int j0, int x, int NX, cplx<T> ab,
                                                  cplx<T> bb, cplx<T> cb, cplx<T>& qb_out, cplx<T>& ub_out,
                                                  cplx<T>& vb_out, int L = 0) {
  const int nl = g.nl;
  const size_t np = (size_t)nl * g.ny * NX;  // field stride of the stored forward fields [3][layer][j][i]
  const T* ph = static_cast<const T*>(a.phys) + (size_t)L * g.ny * NX;
  const size_t ia = (size_t)j0 * NX + x, ibb = ia + NX;
  const cplx<T> qe = mk<T>(ph[ia], ph[ibb]);
  const cplx<T> u = mk<T>(ph[np + ia], ph[np + ibb]);
  const cplx<T> v = mk<T>(ph[2 * np + ia], ph[2 * np + ibb]);
  const cplx<T> qb = mk<T>(ab.x * u.x + bb.x * v.x, ab.y * u.y + bb.y * v.y);
  cplx<T> ub = mk<T>(ab.x * qe.x, ab.y * qe.y), vb = mk<T>(bb.x * qe.x, bb.y * qe.y);
  if (a.hasC) {
    const T* Qy1 = static_cast<const T*>(a.Qy1D);
    const T* Qx2 = static_cast<const T*>(a.Qx2D);
    const T* Qy2 = static_cast<const T*>(a.Qy2D);
    const bool last = L == nl - 1;  // the 2-D gradients act on the bottom layer
    cplx<T> Qx = czero<T>(), Qy = Qy1 ? mk<T>(Qy1[L * g.ny + j0], Qy1[L * g.ny + j0 + 1]) : czero<T>();
    if (last && Qx2) Qx = mk<T>(Qx2[ia], Qx2[ibb]);
    if (last && Qy2) Qy = Qy + mk<T>(Qy2[ia], Qy2[ibb]);
    ub = ub + mk<T>(cb.x * Qx.x, cb.y * Qx.y);
    vb = vb + mk<T>(cb.x * Qy.x, cb.y * Qy.y);
    if (a.qxb && last) {  // the topography gradient (it enters the bottom layer's Qx, Qy)
      T* qxb = static_cast<T*>(a.qxb);
      T* qyb = static_cast<T*>(a.qyb);
      qxb[ia] = qxb[ia] + cb.x * u.x;
      qxb[ibb] = qxb[ibb] + cb.y * u.y;
      qyb[ia] = qyb[ia] + cb.x * v.x;
      qyb[ibb] = qyb[ibb] + cb.y * v.y;
    }
  } else {
    const T U = sel<T>(a.U, a.U_f, a.U_l);
    T* etab = static_cast<T*>(a.etab);
    etab[ia] = etab[ia] + (qb.x + U * ab.x);
    etab[ibb] = etab[ibb] + (qb.y + U * ab.y);
  }
  qb_out = qb;
  ub_out = ub;
  vb_out = vb;
}

// Column kernel: y-direction FFT of the three adjoint products of stage a.stage (kr < kcut),
// the transposed stage combination, and the y-direction inverse FFT of the next cotangent's
// (i kr Nbar / w, i l Nbar / w) into Wb (all kr).  a.stage = 5: head only (start of a step
// from a.ubar_in).  Block: C adjacent kr columns x NY / R threads per column.
template <class T, int NY, int R>
__global__ void __launch_bounds__(512, 1) adj_col_kernel(Geom g, ModArgs m, AdjArgs a, Bufs b, int C) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int TPF = NY / R;
  const int cs = g.cs;
  cplx<T>* F0 = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* F1 = F0 + C * cs;
  cplx<T>* F2 = F1 + C * cs;
  const int tid = threadIdx.x, c = tid % C, t = tid / C;
  const int cf = tid / TPF, tf = tid % TPF;
  const int kr = blockIdx.x * C + c;
  const bool kin = kr < g.nkr;
  const cplx<T>* tw = static_cast<const cplx<T>*>(b.twid);
  const T dky = sel<T>(g.dky, g.dky_f, g.dky_l), krT = T(kr) * sel<T>(g.dkx, g.dkx_f, g.dkx_l);
  const T ell2 = sel<T>(m.ell_inv2, m.ell_inv2_f, m.ell_inv2_l);
  const T inv_n = sel<T>(g.inv_nxny, g.inv_nxny_f, g.inv_nxny_l);
  const bool edge = (kr == 0) || (2 * kr == g.nx);
  const T scale_in = edge ? inv_n : T(2) * inv_n;  // irfft^T: w / (nx ny)
  const T scale_out = edge ? T(1) : T(0.5);       // rfft^T via the c2r path: 1 / w

  // 1) Xbar of this stage: y-FFT of (qbar, ubar, vbar), combined and masked
  cplx<T> xj[R];
#pragma unroll
  for (int i = 0; i < R; ++i) xj[i] = czero<T>();
  if (a.stage <= 4 && (int)blockIdx.x * C < g.kcut) {
    const cplx<T>* P = static_cast<const cplx<T>*>(a.Pb);
    const size_t fs = (size_t)g.ny * g.ldk;
    cplx<T>* Fs[3] = {F0, F1, F2};
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      cplx<T>* Fc = Fs[f] + c * cs;
#pragma unroll
      for (int i = 0; i < R; ++i) {
        const int j = t + i * TPF;
        Fc[swz<T>(j)] = (kr < g.kcut) ? P[f * fs + (size_t)j * g.ldk + kr] : czero<T>();
      }
    }
    __syncthreads();
    fft_smem_group<T, NY, R, -1, 3>(F0 + cf * cs, C * cs, tf, tw);  // F0, F1, F2 are C * cs apart
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int j = t + i * TPF;
      if (kin && kept(g, kr, j)) {
        const T lv = T(lidx(g, j)) * dky;
        const T K2 = krT * krT + lv * lv;
        const T f = psi_factor<T>(m.psi_kind, K2, ell2, m.mult, (size_t)j * g.ldk + kr);
        const cplx<T> Q = F0[c * cs + swz<T>(j)], Ub = F1[c * cs + swz<T>(j)], Vb = F2[c * cs + swz<T>(j)];
        xj[i] = scale_in * (Q + f * (lv * mul_i(Ub) - krT * mul_i(Vb)));
      }
    }
    __syncthreads();  // F0..F2 are reused below
  }

  // 2) transposed stage combination -> the next cotangent Nbar
  cplx<T> nb[R];
  bool out_w = true;
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const int j = t + i * TPF;
    nb[i] = kin ? adj_stage_combine<T>(a, (size_t)j * g.ldk + kr, kept(g, kr, j), xj[i]) : czero<T>();
  }
  if (a.stage == 1 && !a.head) out_w = false;
  if (!out_w) return;

  // 3) y-inverse FFT of (i kr Nbar / w, i l Nbar / w) -- and of -Nbar / w for the U(y)
  // product -- into Wb (every kr column), in lockstep
  cplx<T>* Wb = static_cast<cplx<T>*>(a.Wb);
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const int j = t + i * TPF;
    F0[c * cs + swz<T>(j)] = (scale_out * krT) * mul_i(nb[i]);
    F1[c * cs + swz<T>(j)] = (scale_out * (T(lidx(g, j)) * dky)) * mul_i(nb[i]);
    if (a.hasC) F2[c * cs + swz<T>(j)] = (-scale_out) * nb[i];
  }
  __syncthreads();
  if (a.hasC) fft_smem_group<T, NY, R, +1, 3>(F0 + cf * cs, C * cs, tf, tw);
  else fft_smem_group<T, NY, R, +1, 2>(F0 + cf * cs, C * cs, tf, tw);
  if (kin) {
    const int nw = a.hasC ? 3 : 2;
    for (int f = 0; f < nw; ++f) {
      cplx<T>* Wf = Wb + (size_t)f * g.ny * g.ldk + kr;
      const cplx<T>* Fe = F0 + (size_t)f * C * cs + c * cs;
#pragma unroll
      for (int i = 0; i < R; ++i) {
        const int j = t + i * TPF;
        Wf[(size_t)j * g.ldk] = Fe[swz<T>(j)];
      }
    }
  }
}

// Several layers or bottom drag (MultiLayerQG): every layer of C columns in one block --
// buffers F(f, L, c) = F0 + ((f nl + L) C + c) cs for f = qbar, ubar, vbar.  The y-FFTs of the
// three cotangent products of every layer; then per element, with psibar_L = w/N (i l Ubar_L -
// i kr Vbar_L) (+ mu K^2 Nbar_n in the bottom layer, Nbar of this stage from a.nbar),
// Xbar_L = w/N Qbar_L + [S^-T psibar]_L at kept modes (S^-1 = V diag(1/(lam - K^2)) Vinv);
// the transposed stage combination of every layer (its Nbar also kept in a.nbar); the
// y-inverse FFTs of (i kr Nbar / w, i l Nbar / w, -Nbar / w) of every layer into Wb.
template <class T, int NY, int R>
__global__ void __launch_bounds__(512, 1) adj_col_ml_kernel(Geom g, ModArgs m, AdjArgs a, Bufs b, int C) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ T eig[MAXL + 2 * MAXL * MAXL];
  constexpr int TPF = NY / R;
  const int cs = g.cs, nl = g.nl;
  cplx<T>* F0 = reinterpret_cast<cplx<T>*>(smem_raw);
  auto Fb = [&](int f, int L, int c) { return F0 + ((size_t)(f * nl + L) * C + c) * cs; };
  const int tid = threadIdx.x, c = tid % C, t = tid / C;
  const int cf = tid / TPF, tf = tid % TPF;
  const int kr = blockIdx.x * C + c;
  const bool kin = kr < g.nkr;
  const cplx<T>* tw = static_cast<const cplx<T>*>(b.twid);
  const T dky = sel<T>(g.dky, g.dky_f, g.dky_l), krT = T(kr) * sel<T>(g.dkx, g.dkx_f, g.dkx_l);
  const T ell2 = sel<T>(m.ell_inv2, m.ell_inv2_f, m.ell_inv2_l), muT = sel<T>(m.mu, m.mu_f, m.mu_l);
  const T inv_n = sel<T>(g.inv_nxny, g.inv_nxny_f, g.inv_nxny_l);
  const bool edge = (kr == 0) || (2 * kr == g.nx);
  const T scale_in = edge ? inv_n : T(2) * inv_n;  // irfft^T: w / (nx ny)
  const T scale_out = edge ? T(1) : T(0.5);       // rfft^T via the c2r path: 1 / w
  const size_t lstride = (size_t)g.ny * g.ldk;
  if (m.psi_kind == PSI_EIGEN)
    for (int q = tid; q < MAXL + 2 * MAXL * MAXL; q += blockDim.x)
      eig[q] = q < MAXL ? sel<T>(m.lam[q], m.lam_f[q], m.lam_l[q])
             : q < MAXL + MAXL * MAXL ? sel<T>(m.V[q - MAXL], m.V_f[q - MAXL], m.V_l[q - MAXL])
                                      : sel<T>(m.Vinv[q - MAXL - MAXL * MAXL], m.Vinv_f[q - MAXL - MAXL * MAXL],
                                               m.Vinv_l[q - MAXL - MAXL * MAXL]);
  __syncthreads();
  const bool fwd = a.stage <= 4 && (int)blockIdx.x * C < g.kcut;
  if (fwd) {
    const cplx<T>* P = static_cast<const cplx<T>*>(a.Pb);
    for (int f = 0; f < 3; ++f)
      for (int L = 0; L < nl; ++L) {
        cplx<T>* Fc = Fb(f, L, c);
        for (int i = 0; i < R; ++i) {
          const int j = t + i * TPF;
          Fc[swz<T>(j)] = (kr < g.kcut) ? P[((size_t)f * nl + L) * lstride + (size_t)j * g.ldk + kr] : czero<T>();
        }
      }
    __syncthreads();
#pragma unroll 1
    for (int fl = 0; fl < 3 * nl; ++fl) fft_smem<T, NY, R, -1>(F0 + ((size_t)fl * C + cf) * cs, tf, tw);
  }
  const bool out_w = !(a.stage == 1 && !a.head);
  cplx<T>* nbar = static_cast<cplx<T>*>(a.nbar);
#pragma unroll 1
  for (int i = 0; i < R; ++i) {
    const int j = t + i * TPF;
    const size_t ti = (size_t)j * g.ldk + kr;
    const bool keep = kin && kept(g, kr, j);
    const T lv = T(lidx(g, j)) * dky;
    const T K2 = krT * krT + lv * lv;
    cplx<T> xj[MAXL];
    for (int L = 0; L < nl; ++L) xj[L] = czero<T>();
    if (fwd && keep) {
      cplx<T> pb[MAXL];
      for (int L = 0; L < nl; ++L)
        pb[L] = scale_in * (lv * mul_i(Fb(1, L, c)[swz<T>(j)]) - krT * mul_i(Fb(2, L, c)[swz<T>(j)]));
      if (m.drag) pb[nl - 1] = pb[nl - 1] + (muT * K2) * nbar[(size_t)(nl - 1) * lstride + ti];
      for (int r = 0; r < nl; ++r) {
        cplx<T> x = scale_in * Fb(0, r, c)[swz<T>(j)];
        if (m.psi_kind == PSI_EIGEN) {  // [S^-T pb]_r = sum_q Vinv[q][r] / (lam_q - K^2) sum_L V[L][q] pb_L
          if (K2 != T(0)) {
            const T* V = eig + MAXL;
            const T* Vi = eig + MAXL + MAXL * MAXL;
            for (int q = 0; q < nl; ++q) {
              cplx<T> sq = czero<T>();
              for (int L = 0; L < nl; ++L) sq = sq + V[L * MAXL + q] * pb[L];
              x = x + (Vi[q * MAXL + r] * (T(1) / (eig[q] - K2))) * sq;
            }
          }
        } else {
          x = x + psi_factor<T>(m.psi_kind, K2, ell2, m.mult, ti) * pb[r];
        }
        xj[r] = x;
      }
    }
    for (int L = 0; L < nl; ++L) {
      const size_t si = (size_t)L * lstride + ti;
      const cplx<T> nb = kin ? adj_stage_combine<T>(a, ti, keep, xj[L], si) : czero<T>();
      if (kin) nbar[si] = nb;
      if (out_w) {
        Fb(0, L, c)[swz<T>(j)] = (scale_out * krT) * mul_i(nb);
        Fb(1, L, c)[swz<T>(j)] = (scale_out * lv) * mul_i(nb);
        Fb(2, L, c)[swz<T>(j)] = (-scale_out) * nb;
      }
    }
  }
  if (!out_w) return;
  __syncthreads();
#pragma unroll 1
  for (int fl = 0; fl < 3 * nl; ++fl) fft_smem<T, NY, R, +1>(F0 + ((size_t)fl * C + cf) * cs, tf, tw);
  if (kin) {
    cplx<T>* Wb = static_cast<cplx<T>*>(a.Wb);
    for (int f = 0; f < 3; ++f)
      for (int L = 0; L < nl; ++L)
        for (int i = 0; i < R; ++i) {
          const int j = t + i * TPF;
          Wb[((size_t)f * nl + L) * lstride + (size_t)j * g.ldk + kr] = Fb(f, L, c)[swz<T>(j)];
        }
  }
}

// shared-memory bytes of adj_col_kernel for C columns with column stride cs
__host__ __forceinline__ size_t adj_col_smem(int C, int cs, size_t elem) { return (size_t)3 * C * cs * elem; }

// Row kernel: for the row pair (j0, j0+1) packed as one complex FFT, the x-direction c2r of
// (abar, bbar) from Wb, the transposed products against the stored forward fields
// (qe, u, v) of the stage, the etabar accumulation, and the x-direction r2c of
// (qbar, ubar, vbar) into Pb (kr < kcut).
template <class T, int NX, int R>
__global__ void __launch_bounds__(256, 1) adj_row_kernel(Geom g, AdjArgs a, Bufs b, int B) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int TPF = NX / R;
  constexpr int PS = row_stride<T>(NX, NX / R);
  const int tid = threadIdx.x, bp = tid / TPF, t = tid % TPF;
  const int j0 = 2 * (blockIdx.x * B + bp);
  cplx<T>* buf = reinterpret_cast<cplx<T>*>(smem_raw) + (size_t)bp * 3 * PS;
  const cplx<T>* tw = static_cast<const cplx<T>*>(b.twid);
  const cplx<T>* Wb = static_cast<const cplx<T>*>(a.Wb);
  cplx<T>* Pb = static_cast<cplx<T>*>(a.Pb);
  const int nin = a.hasC ? 3 : 2, nl = g.nl;
  for (int L = 0; L < nl; ++L) {  // Wb and Pb: [field][layer][j][ldk]
    for (int f = 0; f < nin; ++f) {
      const cplx<T>* Wa = Wb + ((size_t)f * nl + L) * g.ny * g.ldk + (size_t)j0 * g.ldk;
#pragma unroll
      for (int i = 0; i < R; ++i) {
        const int k = t + i * TPF;
        buf[f * PS + swz<T>(k)] = packed_spec<T>(Wa, Wa + g.ldk, k, NX, g.nkr);
      }
    }
    __syncthreads();
    if (a.hasC) fft_smem_group<T, NX, R, +1, 3>(buf, PS, t, tw);
    else fft_smem_group<T, NX, R, +1, 2>(buf, PS, t, tw);
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int x = t + i * TPF;
      const int px = swz<T>(x);
      adj_pair_products<T>(g, a, j0, x, NX, buf[px], buf[PS + px], a.hasC ? buf[2 * PS + px] : czero<T>(),
                           buf[px], buf[PS + px], buf[2 * PS + px], L);
    }
    __syncthreads();
    fft_smem_group<T, NX, R, -1, 3>(buf, PS, t, tw);
    for (int f = 0; f < 3; ++f) {
      cplx<T>* Pa = Pb + ((size_t)f * nl + L) * g.ny * g.ldk + (size_t)j0 * g.ldk;
#pragma unroll
      for (int i = 0; i < R; ++i) {
        const int k = t + i * TPF;
        if (k < g.kcut) unpack_store<T>(buf + f * PS, k, NX, Pa, Pa + g.ldk);
      }
    }
    __syncthreads();  // the next layer refills the buffers
  }
}

}  // namespace gf
