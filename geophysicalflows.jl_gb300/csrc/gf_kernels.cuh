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
#pragma once
#include <utility>

#include "gf_fft.cuh"
#include "gf_internal.h"

namespace gf {

// ------------------------------------------------------------------------------ helpers
__device__ __forceinline__ bool kept(const Geom& g, int kr, int j) { return kr < g.kcut && (j < g.lA || j > g.lB); }
__device__ __forceinline__ double lval(const Geom& g, int j) { return (j < g.ny / 2 ? j : j - g.ny) * g.dky; }

template <class T>
__device__ __forceinline__ cplx<T> ldc(const void* p, size_t i, int is_cplx) {
  if (is_cplx) return static_cast<const cplx<T>*>(p)[i];
  return mk<T>(static_cast<const T*>(p)[i], T(0));
}
template <class T>
__device__ __forceinline__ cplx<T> mulc(cplx<T> c, cplx<T> x, int is_cplx) {
  return is_cplx ? c * x : c.x * x;
}

// Philox4x32-10 (Salmon et al., SC'11): counter (e, step_lo, step_hi, tag), key = seed.
__device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r > 0) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    const uint32_t hi0 = __umulhi(0xD2511F53u, c[0]), lo0 = 0xD2511F53u * c[0];
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]), lo1 = 0xCD9E8D57u * c[2];
    const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
  }
}
constexpr uint32_t TAG_FORCING = 0x464F5243u;

template <class T> __device__ __forceinline__ T u01(uint32_t x) { return (T(x) + T(0.5)) * T(2.3283064365386963e-10); }
__device__ __forceinline__ void sincospi_t(double x, double* s, double* c) { sincospi(x, s, c); }
__device__ __forceinline__ void sincospi_t(float x, float* s, float* c) { sincospif(x, s, c); }
__device__ __forceinline__ double log_t(double x) { return log(x); }
__device__ __forceinline__ float log_t(float x) { return logf(x); }
__device__ __forceinline__ double sqrt_t(double x) { return sqrt(x); }
__device__ __forceinline__ float sqrt_t(float x) { return sqrtf(x); }

// complex normal with E|z|^2 = 1 (Box-Muller), or a unit random phase
template <class T>
__device__ __forceinline__ cplx<T> draw(uint64_t e, uint64_t step, uint64_t seed, int phase) {
  uint32_t c[4] = {(uint32_t)e, (uint32_t)step, (uint32_t)(step >> 32), TAG_FORCING};
  philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  T s, co;
  if (phase) {
    sincospi_t(T(2) * u01<T>(c[0]), &s, &co);
    return mk<T>(co, s);
  }
  const T r = sqrt_t(T(-2) * log_t(u01<T>(c[0]))) * T(0.70710678118654752440);
  sincospi_t(T(2) * u01<T>(c[1]), &s, &co);
  return mk<T>(r * co, r * s);
}

// psi-hat of one layer from the layer values X[0..nl) at one wavenumber (K2 = |k|^2).
template <class T>
__device__ __forceinline__ void psi_all(const ModArgs& m, int nl, double K2, const cplx<T>* X, cplx<T>* psi,
                                        size_t tidx) {
  if (m.psi_kind == PSI_EIGEN) {
    if (K2 == 0.0) {
      for (int a = 0; a < nl; ++a) psi[a] = czero<T>();
      return;
    }
    cplx<T> y[MAXL];
    for (int a = 0; a < nl; ++a) {
      cplx<T> s = czero<T>();
      for (int b = 0; b < nl; ++b) s = s + T(m.Vinv[a * MAXL + b]) * X[b];
      y[a] = T(1.0 / (m.lam[a] - K2)) * s;
    }
    for (int a = 0; a < nl; ++a) {
      cplx<T> s = czero<T>();
      for (int b = 0; b < nl; ++b) s = s + T(m.V[a * MAXL + b]) * y[b];
      psi[a] = s;
    }
    return;
  }
  T f;
  if (m.psi_kind == PSI_INVK2) f = K2 == 0.0 ? T(0) : T(-1.0 / K2);
  else if (m.psi_kind == PSI_HELMHOLTZ) f = T(-1.0 / (K2 + m.ell_inv2));
  else f = -static_cast<const T*>(m.mult)[tidx];
  for (int a = 0; a < nl; ++a) psi[a] = f * X[a];
}

// ------------------------------------------------------------------------ column kernel
// Block: C adjacent kr columns x (NY/R) threads per column; thread (c, t) = (tid % C, tid / C)
// owns rows j = t + i (NY/R), i < R.  Shared memory: F (C x NY work column, interleaved
// [j][c]) and, for more than one layer, Xs and Ps (nl x C x NY each).
template <class T, int NY, int R>
__global__ void __launch_bounds__(512) col_stage_kernel(Geom g, ModArgs m, StepArgs s, Bufs b, int C) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int TPF = NY / R;
  cplx<T>* F = reinterpret_cast<cplx<T>*>(smem_raw);
  const int nl = g.nl;
  cplx<T>* Xs = F + C * NY;
  cplx<T>* Ps = Xs + nl * C * NY;
  const int tid = threadIdx.x, c = tid % C, t = tid / C;
  const int kr = blockIdx.x * C + c;
  const bool kin = kr < g.nkr;
  const double krv = kr * g.dkx;
  const cplx<T>* tw = static_cast<const cplx<T>*>(b.twid);
  const size_t lstride = (size_t)g.ny * g.ldk;

  if (s.do_fwd) {
    cplx<T>* P = static_cast<cplx<T>*>(b.P);
    const int nslot = 1 + m.hasB + m.hasC;
    for (int L = 0; L < nl; ++L) {
      cplx<T> nacc[R];
#pragma unroll
      for (int i = 0; i < R; ++i) nacc[i] = czero<T>();
      for (int f = 0; f < nslot; ++f) {
        const cplx<T>* Pf = P + ((size_t)f * nl + L) * lstride;
#pragma unroll
        for (int i = 0; i < R; ++i) {
          const int j = t + i * TPF;
          F[j * C + c] = kin ? Pf[(size_t)j * g.ldk + kr] : czero<T>();
        }
        __syncthreads();
        fft_smem<T, NY, R, -1>(F + c, C, t, tw);
        const int slot = (f == 0) ? 0 : (f == 1 && m.hasB) ? 1 : 2;
#pragma unroll
        for (int i = 0; i < R; ++i) {
          const int j = t + i * TPF;
          const cplx<T> v = F[j * C + c];
          if (slot == 0) nacc[i] = nacc[i] + T(krv) * mul_mi(v);               // -i kr A
          else if (slot == 1) nacc[i] = nacc[i] + T(lval(g, j)) * mul_mi(v);   // -i l B
          else nacc[i] = nacc[i] - v;                                         // -C
        }
        __syncthreads();
      }
      // epilogue: forcing, drag, stage combination
#pragma unroll
      for (int i = 0; i < R; ++i) {
        const int j = t + i * TPF;
        cplx<T> xn = czero<T>();
        if (kin) {
          const size_t ti = (size_t)j * g.ldk + kr;       // table index
          const size_t si = (size_t)L * lstride + ti;     // state index
          const T mk_ = kept(g, kr, j) ? T(1) : T(0);
          cplx<T> N = nacc[i];
          if (m.etah && m.U0 != 0.0) N = N - T(m.U0 * krv) * mul_i(static_cast<const cplx<T>*>(m.etah)[ti]);
          if (m.drag && L == nl - 1) N = N + static_cast<const cplx<T>*>(m.D)[ti];
          cplx<T>* sol = static_cast<cplx<T>*>(s.sol);
          const cplx<T> solm = mk_ * sol[si];
          // forcing
          if (s.fkind == FK_STATIC) {
            N = N + static_cast<const cplx<T>*>(s.Fh)[si];
          } else if (s.fkind == FK_HARMONIC) {
            N = N + T(s.fscale) * static_cast<const cplx<T>*>(s.Fh)[si];
          } else if (s.fkind == FK_STOCH || s.fkind == FK_STOCH_PHASE) {
            cplx<T> Fv;
            if (s.draw) {
              const T sp = static_cast<const T*>(s.fspec)[ti];
              const uint64_t e = (uint64_t)kr + (uint64_t)g.nkr * ((uint64_t)j + (uint64_t)g.ny * L);
              Fv = czero<T>();
              const bool zero_mean = (s.fkind == FK_STOCH_PHASE) && kr == 0 && j == 0;
              if (sp != T(0) && !zero_mean) Fv = sp * draw<T>(e, s.step, s.seed, s.fkind == FK_STOCH_PHASE);
              static_cast<cplx<T>*>(s.Fstore)[si] = Fv;
              static_cast<cplx<T>*>(s.prevsol)[si] = solm;
            } else {
              Fv = static_cast<const cplx<T>*>(s.Fh)[si];
            }
            N = N + Fv;
          }
          const T dt = T(s.dt);
          auto Lmul = [&](cplx<T> x) { return mulc(ldc<T>(s.Ltab, ti, s.cplxL), x, s.cplxL); };
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
            if (s.hasL) Rv = Rv + Lmul(s.stage == 1 ? solm : mk_ * X[si]);
            if (s.stage == 1) {
              acc[si] = T(1.0 / 6.0) * Rv;
              xn = solm + T(0.5) * dt * Rv;
            } else if (s.stage < 4) {
              acc[si] = acc[si] + T(1.0 / 3.0) * Rv;
              xn = solm + (s.stage == 2 ? T(0.5) * dt : dt) * Rv;
            } else {
              xn = finish(solm + dt * (acc[si] + T(1.0 / 6.0) * Rv));
            }
            if (s.hasL && s.stage < 4) X[si] = mk_ * xn;
          } else if (s.kind == SK_ETDRK4) {
            const int cx = s.cplxL;
            cplx<T>* acc = static_cast<cplx<T>*>(s.acc);
            if (s.stage == 1) {
              xn = mulc(ldc<T>(s.e2, ti, cx), solm, cx) + mulc(ldc<T>(s.zeta, ti, cx), N, cx);
              static_cast<cplx<T>*>(s.s1)[si] = mk_ * xn;
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
            if (s.ab3_euler) {
              upd = Rv;
            } else {
              const cplx<T> r1 = static_cast<const cplx<T>*>(s.Rm1)[si];
              const cplx<T> r2 = static_cast<const cplx<T>*>(s.Rm2)[si];
              upd = T(23.0 / 12.0) * Rv - T(16.0 / 12.0) * r1 + T(5.0 / 12.0) * r2;
            }
            static_cast<cplx<T>*>(s.Rout)[si] = Rv;
            xn = finish(solm + dt * upd);
          }
          xn = (kept(g, kr, j) ? T(1) : T(0)) * xn;
        }
        Xs[(L * NY + j) * C + c] = xn;
      }
    }
  } else {
    const cplx<T>* sol = static_cast<const cplx<T>*>(s.sol);
    for (int L = 0; L < nl; ++L) {
#pragma unroll
      for (int i = 0; i < R; ++i) {
        const int j = t + i * TPF;
        cplx<T> xn = czero<T>();
        if (kin && kept(g, kr, j)) xn = sol[(size_t)L * lstride + (size_t)j * g.ldk + kr];
        Xs[(L * NY + j) * C + c] = xn;
      }
    }
  }
  if (!s.do_inv) return;
  if ((int)blockIdx.x * C >= g.kcut) return;  // whole block aliased: W is never read there

  // PV inversion for every owned element (each thread reads back only what it wrote)
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const int j = t + i * TPF;
    const double lv = lval(g, j);
    const double K2 = krv * krv + lv * lv;
    const size_t ti = (size_t)j * g.ldk + (kin ? kr : 0);
    if (nl == 1) {
      cplx<T> x = Xs[j * C + c], p;
      psi_all<T>(m, 1, K2, &x, &p, ti);
      Ps[j * C + c] = p;
      if (m.drag && kin) static_cast<cplx<T>*>(m.D)[ti] = T(m.mu * K2) * p;
    } else {
      cplx<T> X[MAXL], ps[MAXL];
      for (int L = 0; L < nl; ++L) X[L] = Xs[(L * NY + j) * C + c];
      psi_all<T>(m, nl, K2, X, ps, ti);
      for (int L = 0; L < nl; ++L) Ps[(L * NY + j) * C + c] = ps[L];
      if (m.drag && kin) static_cast<cplx<T>*>(m.D)[ti] = T(m.mu * K2) * ps[nl - 1];
    }
  }
  // y-direction inverse FFT of (q, u, v) for every layer
  cplx<T>* W = static_cast<cplx<T>*>(b.W);
  const T sc = T(g.inv_nxny);
  for (int L = 0; L < nl; ++L) {
    for (int f = 0; f < 3; ++f) {
      __syncthreads();
#pragma unroll
      for (int i = 0; i < R; ++i) {
        const int j = t + i * TPF;
        const cplx<T> x = Xs[(L * NY + j) * C + c];
        const cplx<T> p = Ps[(L * NY + j) * C + c];
        cplx<T> v;
        if (f == 0) v = x;
        else if (f == 1) v = T(lval(g, j)) * mul_mi(p);  // u = -i l psi
        else v = T(krv) * mul_i(p);                        // v =  i kr psi
        F[j * C + c] = sc * v;
      }
      __syncthreads();
      fft_smem<T, NY, R, +1>(F + c, C, t, tw);
      if (kr < g.kcut) {
        cplx<T>* Wf = W + ((size_t)f * nl + L) * g.ny * g.ldw;
#pragma unroll
        for (int i = 0; i < R; ++i) {
          const int j = t + i * TPF;
          Wf[(size_t)j * g.ldw + kr] = F[j * C + c];
        }
      }
    }
  }
}

// --------------------------------------------------------------------------- row kernel
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

template <class T>
__device__ __forceinline__ void unpack_store(const cplx<T>* buf, int k, int NX, cplx<T>* Pa, cplx<T>* Pb) {
  const cplx<T> z = buf[k], w = buf[(NX - k) & (NX - 1)];
  Pa[k] = mk<T>(T(0.5) * (z.x + w.x), T(0.5) * (z.y - w.y));
  Pb[k] = mk<T>(T(0.5) * (z.y + w.y), T(0.5) * (w.x - z.x));
}

template <class T, int NX, int R>
__global__ void __launch_bounds__(512) row_nl_kernel(Geom g, ModArgs m, Bufs b, int B) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int TPF = NX / R;
  constexpr int M = NX / 2;
  const int tid = threadIdx.x, bp = tid / TPF, t = tid % TPF;
  const int j0 = 2 * (blockIdx.x * B + bp);
  cplx<T>* buf = reinterpret_cast<cplx<T>*>(smem_raw) + (size_t)bp * 3 * NX;
  const cplx<T>* tw = static_cast<const cplx<T>*>(b.twid);
  const cplx<T>* W = static_cast<const cplx<T>*>(b.W);
  cplx<T>* P = static_cast<cplx<T>*>(b.P);
  const int nl = g.nl;
  const T* eta = static_cast<const T*>(m.eta);
  const T* U1D = static_cast<const T*>(m.U1D);
  const T* Qy1D = static_cast<const T*>(m.Qy1D);
  const T* Qx2D = static_cast<const T*>(m.Qx2D);
  const T* Qy2D = static_cast<const T*>(m.Qy2D);
  const int nslot = 1 + m.hasB + m.hasC;
  for (int L = 0; L < nl; ++L) {
    for (int f = 0; f < 3; ++f) {
      const cplx<T>* Wf = W + ((size_t)f * nl + L) * g.ny * g.ldw;
      const cplx<T>* Wa = Wf + (size_t)j0 * g.ldw;
      const cplx<T>* Wb = Wa + g.ldw;
#pragma unroll
      for (int i = 0; i < R; ++i) {
        const int k = t + i * TPF;
        buf[f * NX + k] = packed_spec<T>(Wa, Wb, k, NX, g.kcut);
      }
    }
    __syncthreads();
    for (int f = 0; f < 3; ++f) fft_smem<T, NX, R, +1>(buf + f * NX, 1, t, tw);
    // physical-space products on the packed pairs
    const T Ua = U1D ? U1D[L * g.ny + j0] : T(0), Ub = U1D ? U1D[L * g.ny + j0 + 1] : T(0);
    const T Qa = Qy1D ? Qy1D[L * g.ny + j0] : T(0), Qb = Qy1D ? Qy1D[L * g.ny + j0 + 1] : T(0);
    const bool last = (L == nl - 1);
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int x = t + i * TPF;
      cplx<T> q = buf[x], u = buf[NX + x], v = buf[2 * NX + x];
      const cplx<T> Up = mk<T>(Ua, Ub);
      u = u + Up;
      if (eta) q = q + mk<T>(eta[(size_t)j0 * NX + x], eta[(size_t)(j0 + 1) * NX + x]);
      const cplx<T> au = m.linear ? Up : u;
      const cplx<T> A = mk<T>(au.x * q.x, au.y * q.y);
      const cplx<T> Bv = mk<T>(v.x * q.x, v.y * q.y);
      cplx<T> Cv = czero<T>();
      if (m.hasC) {
        cplx<T> Qy = mk<T>(Qa, Qb), Qx = czero<T>();
        if (last && Qy2D) Qy = Qy + mk<T>(Qy2D[(size_t)j0 * NX + x], Qy2D[(size_t)(j0 + 1) * NX + x]);
        if (last && Qx2D) Qx = mk<T>(Qx2D[(size_t)j0 * NX + x], Qx2D[(size_t)(j0 + 1) * NX + x]);
        Cv = mk<T>(u.x * Qx.x + v.x * Qy.x, u.y * Qx.y + v.y * Qy.y);
      }
      buf[x] = A;
      if (m.hasB) { buf[NX + x] = Bv; if (m.hasC) buf[2 * NX + x] = Cv; }
      else buf[NX + x] = Cv;
    }
    __syncthreads();
    for (int f = 0; f < nslot; ++f) fft_smem<T, NX, R, -1>(buf + f * NX, 1, t, tw);
    for (int f = 0; f < nslot; ++f) {
      cplx<T>* Pa = P + ((size_t)f * nl + L) * g.ny * g.ldk + (size_t)j0 * g.ldk;
#pragma unroll
      for (int i = 0; i < R; ++i) {
        const int k = t + i * TPF;
        if (k <= M) unpack_store<T>(buf + f * NX, k, NX, Pa, Pa + g.ldk);
      }
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------ generic transforms
// y-direction inverse FFT of a derived spectral field of every layer into W (full kr
// range, row stride ldk): kind selects X, psi, u, v, du/dy or the raw array.
template <class T, int NY, int R>
__global__ void __launch_bounds__(512) col_inv_generic(Geom g, ModArgs m, const void* src, int kind, int mask,
                                                        Bufs b, int C) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int TPF = NY / R;
  cplx<T>* F = reinterpret_cast<cplx<T>*>(smem_raw);
  const int tid = threadIdx.x, c = tid % C, t = tid / C;
  const int kr = blockIdx.x * C + c;
  const bool kin = kr < g.nkr;
  const double krv = kr * g.dkx;
  const cplx<T>* S = static_cast<const cplx<T>*>(src);
  const cplx<T>* tw = static_cast<const cplx<T>*>(b.twid);
  cplx<T>* W = static_cast<cplx<T>*>(b.W);
  const size_t lstride = (size_t)g.ny * g.ldk;
  const int nl = g.nl;
  for (int L = 0; L < nl; ++L) {
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int j = t + i * TPF;
      cplx<T> v = czero<T>();
      if (kin) {
        const size_t ti = (size_t)j * g.ldk + kr;
        cplx<T> X[MAXL], ps[MAXL];
        for (int a = 0; a < nl; ++a) X[a] = S[a * lstride + ti];
        if (mask && !kept(g, kr, j)) for (int a = 0; a < nl; ++a) X[a] = czero<T>();
        const double lv = lval(g, j);
        if (kind == SF_X || kind == SF_RAW) {
          v = X[L];
        } else if (kind == SF_DX) {
          v = T(krv) * mul_i(X[L]);
        } else if (kind == SF_DY) {
          v = T(lv) * mul_i(X[L]);
        } else {
          psi_all<T>(m, nl, krv * krv + lv * lv, X, ps, ti);
          const cplx<T> p = ps[L];
          if (kind == SF_PSI) v = p;
          else if (kind == SF_U) v = T(lv) * mul_mi(p);   // u = -i l psi
          else if (kind == SF_V) v = T(krv) * mul_i(p);   // v =  i kr psi
          else v = T(lv * lv) * p;                        // du/dy = i l u = l^2 psi
        }
      }
      F[j * C + c] = T(g.inv_nxny) * v;
    }
    __syncthreads();
    fft_smem<T, NY, R, +1>(F + c, C, t, tw);
    if (kin) {
#pragma unroll
      for (int i = 0; i < R; ++i) {
        const int j = t + i * TPF;
        W[(size_t)L * lstride + (size_t)j * g.ldk + kr] = F[j * C + c];
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
  cplx<T>* buf = reinterpret_cast<cplx<T>*>(smem_raw) + (size_t)bp * NX;
  const cplx<T>* tw = static_cast<const cplx<T>*>(b.twid);
  const cplx<T>* W = static_cast<const cplx<T>*>(b.W);
  for (int f = 0; f < nf; ++f) {
    const cplx<T>* Wa = W + (size_t)f * g.ny * g.ldk + (size_t)j0 * g.ldk;
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int k = t + i * TPF;
      buf[k] = packed_spec<T>(Wa, Wa + g.ldk, k, NX, g.nkr);
    }
    __syncthreads();
    fft_smem<T, NX, R, +1>(buf, 1, t, tw);
    T* o = out + (size_t)f * g.ny * NX + (size_t)j0 * NX;
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int x = t + i * TPF;
      const cplx<T> z = buf[x];
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
  cplx<T>* buf = reinterpret_cast<cplx<T>*>(smem_raw) + (size_t)bp * NX;
  const cplx<T>* tw = static_cast<const cplx<T>*>(b.twid);
  cplx<T>* P = static_cast<cplx<T>*>(b.P);
  for (int f = 0; f < nf; ++f) {
    const T* src = in + (size_t)f * g.ny * NX + (size_t)j0 * NX;
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int x = t + i * TPF;
      buf[x] = mk<T>(src[x], src[NX + x]);
    }
    __syncthreads();
    fft_smem<T, NX, R, -1>(buf, 1, t, tw);
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
  cplx<T>* F = reinterpret_cast<cplx<T>*>(smem_raw);
  const int tid = threadIdx.x, c = tid % C, t = tid / C;
  const int kr = blockIdx.x * C + c;
  const bool kin = kr < g.nkr;
  const cplx<T>* tw = static_cast<const cplx<T>*>(b.twid);
  const cplx<T>* P = static_cast<const cplx<T>*>(b.P);
  const size_t lstride = (size_t)g.ny * g.ldk;
  for (int f = 0; f < nf; ++f) {
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int j = t + i * TPF;
      F[j * C + c] = kin ? P[(size_t)f * lstride + (size_t)j * g.ldk + kr] : czero<T>();
    }
    __syncthreads();
    fft_smem<T, NY, R, -1>(F + c, C, t, tw);
    if (kin) {
#pragma unroll
      for (int i = 0; i < R; ++i) {
        const int j = t + i * TPF;
        cplx<T> v = F[j * C + c];
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
  const size_t n = (size_t)g.nl * g.ny * g.nkr;
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
  const size_t n = (size_t)g.ny * g.nkr;
  const int nl = g.nl;
  const size_t lstride = (size_t)g.ny * g.ldk;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int kr = e % g.nkr, j = e / g.nkr;
    const size_t ti = (size_t)j * g.ldk + kr;
    const double krv = kr * g.dkx, lv = lval(g, j), K2 = krv * krv + lv * lv;
    cplx<T> X[MAXL], Y[MAXL];
    for (int a = 0; a < nl; ++a) X[a] = in[a * lstride + ti];
    if (op == 1) {
      psi_all<T>(m, nl, K2, X, Y, ti);
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
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int kr = e % g.nkr, j = e / g.nkr;
    const size_t ti = (size_t)j * g.ldk + kr;
    const double w = (kr == 0 || (g.nx % 2 == 0 && kr == g.nkr - 1)) ? 1.0 : 2.0;
    const double krv = kr * g.dkx, lv = lval(g, j), K2 = krv * krv + lv * lv;
    const double iK2 = K2 == 0.0 ? 0.0 : 1.0 / K2;
    const bool k0 = (kr == 0 && j == 0);
    cplx<T> Xt[MAXL], Pt[MAXL];
    for (int a = 0; a < nl; ++a) Xt[a] = sol[a * lstride + ti];
    if (m.module == MOD_MLQG) {
      psi_all<T>(m, nl, K2, Xt, Pt, ti);
      for (int a = 0; a < nl; ++a) {
        const double pr = Pt[a].x, pi = Pt[a].y;
        if (mask & (1u << a)) acc[a].add(w * K2 * (pr * pr + pi * pi));
        if (a + 1 < nl && (mask & (1u << (nl + a)))) {
          const double dr = pr - (double)Pt[a + 1].x, di = pi - (double)Pt[a + 1].y;
          acc[nl + a].add(w * (dr * dr + di * di));
        }
      }
      continue;
    }
    const double sr = Xt[0].x, si = Xt[0].y, s2 = sr * sr + si * si;
    // forcing work term Re(S conj(F)), S = sol or (prevsol + sol)/2
    double wr = 0;
    if (Fh) {
      double ar = sr, ai = si;
      if (prevsol) { ar = 0.5 * (sr + (double)prevsol[ti].x); ai = 0.5 * (si + (double)prevsol[ti].y); }
      const double fr = Fh[ti].x, fi = Fh[ti].y;
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
      psi_all<T>(m, 1, K2, Xt, Pt, ti);
      const double p2 = (double)Pt[0].x * Pt[0].x + (double)Pt[0].y * Pt[0].y;
      v[0] = 0.5 * K2 * p2;
      v[1] = 0.5 * m.ell_inv2 * p2;
      double er = sr, ei = si;
      if (m.etah) { er += (double)static_cast<const cplx<T>*>(m.etah)[ti].x; ei += (double)static_cast<const cplx<T>*>(m.etah)[ti].y; }
      v[2] = 0.5 * (er * er + ei * ei);
      v[3] = k0 ? 0.0 : nu * powi(K2, nnu - 1) * s2;
      v[4] = k0 ? 0.0 : nu * powi(K2, nnu) * s2;
      v[5] = iK2 * wr;
      v[6] = wr;
      v[7] = k0 ? 0.0 : mu * iK2 * s2;
      v[8] = k0 ? 0.0 : mu * s2;
    } else {  // SQG
      const double M = static_cast<const T*>(m.mult)[ti];
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
    if (threadIdx.x == 0) partial[(size_t)q * gridDim.x + blockIdx.x] = red[0];
    __syncthreads();
  }
}

// final reduction of the block partials (one block, compensated)
__global__ void diag_finish_kernel(const double* partial, int nblocks, uint32_t mask, double* out);

}  // namespace gf
