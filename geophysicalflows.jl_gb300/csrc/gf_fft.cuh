// Shared-memory Stockham FFT building blocks for the fused pseudospectral step.
//
// The FFT here replaces the FFTW/CUFFT plans that FourierFlows builds for every
// TwoDGrid (`grid.rfftplan`, called through `mul!`/`ldiv!` at e.g.
// src/twodnavierstokes.jl:258-270 and src/multilayerqg.jl:471,478).  A length-N complex
// transform is executed by N/R threads as a sequence of radix-R Stockham passes
// (Govindaraju et al., "High performance discrete Fourier transforms on graphics
// processors", SC'08): every pass reads R elements strided by N/R, applies the twiddles
// w^(r*(j mod Ns)), does an in-register R-point DFT and writes the results to their
// expanded positions, so input and output are both in natural order.  The in-register
// DFT is a fully unrolled radix-2 decimation-in-time network; its constant twiddles are
// the 16th roots of unity, special-cased where they are 1, -i, or (1-i)/sqrt(2).
//
// Twiddles between passes come from one table of TWN = 4096 entries exp(-2 pi i k / TWN)
// computed in double precision on the host, so every FFT length N <= TWN indexes it with
// a stride of TWN / N.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>
#include <utility>

namespace gf {

constexpr int TWN = 4096;  // twiddle table length (largest supported transform)
__host__ __device__ constexpr int ilog2(int n) { return n <= 1 ? 0 : 1 + ilog2(n / 2); }

// FP64 / df64 FFTs: full radix passes from one run-time loop body (1) or each inlined at its
// stride (0).
#ifndef GF_FFT_LOOP
#define GF_FFT_LOOP 1
#endif

// ---------------------------------------------------------------------------------------
// df64: a double-word ("double-float") number hi + lo with |lo| <= ulp(hi)/2, giving a
// 48-bit significand with FP32 arithmetic.  GB300 runs FP64 at a small fraction of its FP32
// rate; the FP64-plain mode of this library computes in df64 instead.  Algorithms: Knuth's
// TwoSum and Dekker's FastTwoSum, FMA-based TwoProd, and the double-word sum (TwoSum of the
// high parts plus the low parts, renormalised -- its error is bounded relative to
// |a| + |b|, which is what a normwise FFT error bound needs) and product (TwoProd plus the
// cross terms) analysed by Joldes, Muller & Popescu, "Tight and rigorous error bounds for
// basic building blocks of double-word arithmetic" (ACM TOMS 2017).
// ---------------------------------------------------------------------------------------
struct __align__(8) df64 {
  float hi, lo;
  df64() = default;
  __host__ __device__ constexpr df64(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ constexpr df64(int i) : hi((float)i), lo(0.0f) {}  // exact for |i| < 2^24
  // from a double: constant-folded for compile-time constants; FP64 work otherwise
  __host__ __device__ constexpr df64(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
};
__host__ __device__ __forceinline__ double to_double(df64 a) { return (double)a.hi + (double)a.lo; }
__host__ __device__ __forceinline__ double to_double(double a) { return a; }
__host__ __device__ __forceinline__ double to_double(float a) { return (double)a; }

__device__ __forceinline__ df64 fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return df64(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ df64 operator+(df64 a, df64 b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float bb = __fsub_rn(s, a.hi);
  const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));  // TwoSum error
  return fast_two_sum(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}
// The same sum without its final renormalisation: (s, e + a.lo + b.lo) is a double-word value
// whose low word may exceed ulp(s)/2.  The sums, products and dot products of this file accept
// such a pair (TwoSum and TwoProd of the high words stay exact whatever the low words are, and
// the low words only enter FP32 sums), so an FFT butterfly level whose outputs feed only
// further butterflies skips the renormalisation: 8 instead of 11 FP32 operations.  The added
// error stays u |lo| = O(u^2 (|a| + |b|)), the order of the renormalised sum's normwise bound.
// The division takes normalised operands only (its first quotient is that of the high words);
// unnormalised pairs never leave a transform, whose last pass renormalises.
__device__ __forceinline__ df64 add_unnorm(df64 a, df64 b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float bb = __fsub_rn(s, a.hi);
  const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
  return df64(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}
// the double-word product below without its renormalisation (for the same consumers)
__device__ __forceinline__ df64 mul_unnorm(df64 a, df64 b) {
  const float p = __fmul_rn(a.hi, b.hi);
  const float e = __fmaf_rn(a.hi, b.hi, -p);  // TwoProd error
  return df64(p, __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e)));
}
__device__ __forceinline__ df64 operator-(df64 a) { return df64(-a.hi, -a.lo); }
__device__ __forceinline__ df64 operator-(df64 a, df64 b) { return a + (-b); }
__device__ __forceinline__ df64 operator*(df64 a, df64 b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);  // TwoProd error
  e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e));
  return fast_two_sum(p, e);
}
__device__ __forceinline__ df64 operator/(df64 a, df64 b) {
  const float q1 = __fdiv_rn(a.hi, b.hi);
  const df64 r = a - b * df64(q1, 0.0f);
  const float q2 = __fdiv_rn(r.hi, b.hi);
  return fast_two_sum(q1, q2);
}
__device__ __forceinline__ bool operator==(df64 a, df64 b) { return a.hi == b.hi && a.lo == b.lo; }
__device__ __forceinline__ bool operator!=(df64 a, df64 b) { return !(a == b); }

template <class T> struct cplx;
template <> struct __align__(8) cplx<float> { float x, y; };
template <> struct __align__(16) cplx<double> { double x, y; };
template <> struct __align__(16) cplx<df64> { df64 x, y; };

template <class T> __host__ __device__ __forceinline__ cplx<T> mk(T a, T b) { cplx<T> r; r.x = a; r.y = b; return r; }
template <class T> __device__ __forceinline__ cplx<T> operator+(cplx<T> a, cplx<T> b) { return mk<T>(a.x + b.x, a.y + b.y); }
template <class T> __device__ __forceinline__ cplx<T> operator-(cplx<T> a, cplx<T> b) { return mk<T>(a.x - b.x, a.y - b.y); }
template <class T> __device__ __forceinline__ cplx<T> operator*(cplx<T> a, cplx<T> b) {
  return mk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <class T> __device__ __forceinline__ cplx<T> operator*(T s, cplx<T> a) { return mk<T>(s * a.x, s * a.y); }

// a b + c d in double-word arithmetic as one two-term dot product: the two high-part products
// exactly (FMA TwoProd), their sum exactly (TwoSum), the cross terms a.hi b.lo + a.lo b.hi and
// c.hi d.lo + c.lo d.hi and the three exact errors summed into the low word, one
// renormalisation.  About 19 FP32 operations instead of 25 for two double-word products and a
// double-word sum; the error stays a few u^2 (|a b| + |c d|), u = 2^-24, as for that sequence
// (the dropped a.lo b.lo terms are below u^2 |a b|).
// NORM = false leaves the result unnormalised (add_unnorm above) for a caller that only feeds
// it to further sums.
template <bool NORM = true>
__device__ __forceinline__ df64 dw_dot2(df64 a, df64 b, df64 c, df64 d) {
  const float p = __fmul_rn(a.hi, b.hi);
  const float ep = __fmaf_rn(a.hi, b.hi, -p);
  const float q = __fmul_rn(c.hi, d.hi);
  const float eq = __fmaf_rn(c.hi, d.hi, -q);
  const float s = __fadd_rn(p, q);
  const float bb = __fsub_rn(s, p);
  const float es = __fadd_rn(__fsub_rn(p, __fsub_rn(s, bb)), __fsub_rn(q, bb));  // TwoSum error
  float lo = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, ep));
  lo = __fmaf_rn(c.hi, d.lo, __fmaf_rn(c.lo, d.hi, __fadd_rn(lo, eq)));
  if constexpr (NORM) return fast_two_sum(s, __fadd_rn(lo, es));
  else return df64(s, __fadd_rn(lo, es));
}
// complex double-word product through dw_dot2 (real and imaginary parts)
template <> __device__ __forceinline__ cplx<df64> operator*(cplx<df64> a, cplx<df64> b) {
  return mk<df64>(dw_dot2(a.x, b.x, -a.y, b.y), dw_dot2(a.x, b.y, a.y, b.x));
}
// Butterfly sums and twiddle products: renormalised (NORM) or, in df64, left unnormalised for
// a consumer that is another butterfly level.  FP32 and FP64 ignore NORM.
template <bool NORM, class T> __device__ __forceinline__ cplx<T> bf_add(cplx<T> a, cplx<T> b) {
  if constexpr (!NORM && std::is_same<T, df64>::value) return mk<T>(add_unnorm(a.x, b.x), add_unnorm(a.y, b.y));
  else return a + b;
}
template <bool NORM, class T> __device__ __forceinline__ cplx<T> bf_sub(cplx<T> a, cplx<T> b) {
  if constexpr (!NORM && std::is_same<T, df64>::value) return mk<T>(add_unnorm(a.x, -b.x), add_unnorm(a.y, -b.y));
  else return a - b;
}
template <bool NORM, class T> __device__ __forceinline__ cplx<T> tw_mul(cplx<T> a, cplx<T> w) {
  if constexpr (!NORM && std::is_same<T, df64>::value)
    return mk<T>(dw_dot2<false>(a.x, w.x, -a.y, w.y), dw_dot2<false>(a.x, w.y, a.y, w.x));
  else return a * w;
}
// renormalises an unnormalised df64 complex value (identity for FP32 and FP64)
template <class T> __device__ __forceinline__ cplx<T> renorm(cplx<T> a) {
  if constexpr (std::is_same<T, df64>::value) return mk<T>(fast_two_sum(a.x.hi, a.x.lo), fast_two_sum(a.y.hi, a.y.lo));
  else return a;
}
template <class T> __device__ __forceinline__ cplx<T> conj(cplx<T> a) { return mk<T>(a.x, -a.y); }
template <class T> __device__ __forceinline__ cplx<T> mul_i(cplx<T> a) { return mk<T>(-a.y, a.x); }   //  i*a
template <class T> __device__ __forceinline__ cplx<T> mul_mi(cplx<T> a) { return mk<T>(a.y, -a.x); }  // -i*a
template <class T> __device__ __forceinline__ cplx<T> czero() { return mk<T>(T(0), T(0)); }

// cos and sin of pi*m/8 for m = 1, 3 (exact decimal expansions of the algebraic numbers)
constexpr double kC1 = 0.92387953251128675612818318939678828682241662586364;  // cos(pi/8)
constexpr double kS1 = 0.38268343236508977172845998403039886676134456248563;  // sin(pi/8)
constexpr double kH = 0.70710678118654752440084436210484903928483593768847;   // sqrt(1/2)

// x * exp(DIR * 2 pi i * m / 16) with DIR = -1 (forward) or +1 (inverse), 0 <= m < 8.  NORM =
// false: a df64 result may be left unnormalised (for a butterfly sum, see add_unnorm).
template <int m, int DIR, class T, bool NORM = true>
__device__ __forceinline__ cplx<T> rot16(cplx<T> a) {
  if constexpr (m == 0) {
    return a;
  } else if constexpr (m == 4) {
    return DIR < 0 ? mul_mi(a) : mul_i(a);
  } else if constexpr (m == 2 || m == 6) {
    const T h = T(kH);
    // exp(-i pi/4) = h(1 - i); exp(-3 i pi/4) = h(-1 - i)
    if constexpr (std::is_same<T, df64>::value) {
      // the sums unnormalised (the product's TwoProd of the high words is exact on any pair)
      const df64 sp = add_unnorm(a.x, a.y), sm = add_unnorm(a.x, -a.y);
      const df64 hp = NORM ? h * sp : mul_unnorm(h, sp), hm = NORM ? h * sm : mul_unnorm(h, sm);  // h (x +- y)
      if constexpr (m == 2) return DIR < 0 ? mk<T>(hp, -hm) : mk<T>(hm, hp);
      else return DIR < 0 ? mk<T>(-hm, -hp) : mk<T>(-hp, hm);
    } else if constexpr (m == 2) {
      return DIR < 0 ? mk<T>(h * (a.x + a.y), h * (a.y - a.x)) : mk<T>(h * (a.x - a.y), h * (a.y + a.x));
    } else {
      return DIR < 0 ? mk<T>(h * (a.y - a.x), -h * (a.x + a.y)) : mk<T>(-h * (a.x + a.y), h * (a.x - a.y));
    }
  } else {
    // general angle theta = pi m / 8 with (c, s) = (cos theta, sin theta)
    constexpr double c = (m == 1) ? kC1 : (m == 3) ? kS1 : (m == 5) ? -kS1 : -kC1;
    constexpr double s = (m == 1 || m == 7) ? kS1 : kC1;
    const T cc = T(c), ss = T(s);
    if constexpr (std::is_same<T, df64>::value) {  // two-term double-word dot products
      if constexpr (DIR < 0) return mk<T>(dw_dot2<NORM>(a.x, cc, a.y, ss), dw_dot2<NORM>(a.y, cc, -a.x, ss));
      else return mk<T>(dw_dot2<NORM>(a.x, cc, -a.y, ss), dw_dot2<NORM>(a.y, cc, a.x, ss));
    } else {
      if constexpr (DIR < 0) return mk<T>(a.x * cc + a.y * ss, a.y * cc - a.x * ss);
      else return mk<T>(a.x * cc - a.y * ss, a.y * cc + a.x * ss);
    }
  }
}

// In-register R-point DFT (R = 1,2,4,8,16), natural order in and out.
// In df64 only the top level (TOP) renormalises: the inner levels' sums and rotations feed
// further butterflies and stay unnormalised (add_unnorm).
template <int R, int DIR, class T, bool TOP = true>
__device__ __forceinline__ void dft(cplx<T>* v) {
  if constexpr (R == 1) {
    return;
  } else if constexpr (R == 2) {
    cplx<T> a = v[0], b = v[1];
    v[0] = bf_add<TOP>(a, b);
    v[1] = bf_sub<TOP>(a, b);
  } else {
    constexpr int H = R / 2;
    cplx<T> e[H], o[H];
#pragma unroll
    for (int i = 0; i < H; ++i) { e[i] = v[2 * i]; o[i] = v[2 * i + 1]; }
    dft<H, DIR, T, false>(e);
    dft<H, DIR, T, false>(o);
    auto step = [&](auto kk) {
      constexpr int k = decltype(kk)::value;
      cplx<T> t = rot16<k * (16 / R), DIR, T, false>(o[k]);
      v[k] = bf_add<TOP>(e[k], t);
      v[k + H] = bf_sub<TOP>(e[k], t);
    };
    // unrolled over k = 0..H-1 with k a compile-time constant
    [&]<int... ks>(std::integer_sequence<int, ks...>) {
      (step(std::integral_constant<int, ks>{}), ...);
    }(std::make_integer_sequence<int, H>{});
  }
}

// Asynchronous global -> shared copies (cp.async, sm_80+): 8- or 16-byte elements.
template <class T>
__device__ __forceinline__ void cp_async_elem(cplx<T>* smem, const cplx<T>* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  if constexpr (sizeof(cplx<T>) == 16) asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
  else asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

template <int DIR, class T>
__device__ __forceinline__ cplx<T> twiddle(const cplx<T>* __restrict__ tw, int idx) {
  cplx<T> w = tw[idx];
  return DIR < 0 ? w : conj(w);
}

// Shared-memory slot of logical element a of an FFT buffer: an XOR swizzle inside each
// aligned block of 16 (8-byte elements) or 8 (16-byte elements) slots.  With it, every
// access pattern of the radix-8 Stockham passes -- consecutive reads, the stride-8 writes
// of the first pass, the (j/8)*64 + j%8 writes of the second -- hits distinct banks
// within a 128-byte shared-memory wavefront, without padding.
template <class T>
__device__ __forceinline__ int swz(int a) {
  if constexpr (sizeof(cplx<T>) == 8) return a ^ (((a >> 4) & 7) | ((a >> 3) & 8));
  else return a ^ ((a >> 3) & 7);
}
// Threads per 128-byte shared-memory wavefront for T's complex element.
template <class T> __host__ __device__ constexpr int wave_threads() { return 128 / (int)sizeof(cplx<T>); }

// One radix pass of a length-N Stockham FFT on a swizzled shared-memory buffer.  Threads t in
// [0, N/R) each do R/Rp butterflies of radix Rp = min(R, N/Ns).  The caller must have
// synchronised before the first pass.
template <class T, int N, int R, int DIR, int Ns>
__device__ __forceinline__ void fft_passes(cplx<T>* buf, int t, const cplx<T>* __restrict__ tw) {
  if constexpr (Ns < N) {
    constexpr int Rp = (N / Ns < R) ? (N / Ns) : R;
    constexpr int NB = R / Rp;
    constexpr int TPF = N / R;
    constexpr int TWS = TWN / (Ns * Rp);
    cplx<T> v[NB][Rp];
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      const int j = t + b * TPF;
#pragma unroll
      for (int r = 0; r < Rp; ++r) v[b][r] = buf[swz<T>(j + r * (N / Rp))];
      if constexpr (Ns > 1) {
        const int k = j & (Ns - 1);
        if constexpr (sizeof(T) == 4) {
          // FP32: one table load, the other powers by complex multiplication
          // (w^r error ~ r ulp, far below the FP32 path's tolerance); fewer L1 requests
          const cplx<T> w1 = twiddle<DIR>(tw, k * TWS);
          cplx<T> wr = w1;
#pragma unroll
          for (int r = 1; r < Rp; ++r) {
            v[b][r] = v[b][r] * wr;
            if (r + 1 < Rp) wr = wr * w1;
          }
        } else {
#pragma unroll
          for (int r = 1; r < Rp; ++r) v[b][r] = tw_mul<false>(v[b][r], twiddle<DIR>(tw, r * k * TWS));
        }
      }
      dft<Rp, DIR, T, (Ns * Rp >= N)>(v[b]);  // df64: normalised only by the last pass
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      const int j = t + b * TPF;
      const int idxD = (j / Ns) * Ns * Rp + (j & (Ns - 1));
#pragma unroll
      for (int r = 0; r < Rp; ++r) buf[swz<T>(idxD + r * Ns)] = v[b][r];
    }
    __syncthreads();
    fft_passes<T, N, R, DIR, Ns * Rp>(buf, t, tw);
  }
}

// Number of full radix-R passes of a length-N transform (R^p <= N) and the stride after them.
template <int N, int R> __host__ __device__ constexpr int full_passes() { int p = 0; for (int s = R; s <= N; s *= R) ++p; return p; }
template <int N, int R> __host__ __device__ constexpr int full_stride() { int s = 1; for (int p = 0; p < full_passes<N, R>(); ++p) s *= R; return s; }

// One full radix-R pass at a run-time stride Ns = R^p (2^lg): the same arithmetic as
// fft_passes at that Ns, but one body serves every full pass (code size: the step kernels
// are bound by instruction fetch when every pass is inlined separately).
// In df64 the pass's outputs are renormalised only when it is the transform's last pass (last);
// the next pass's twiddle products and butterflies accept unnormalised values.
template <class T, int N, int R, int DIR, int NF>
__device__ __forceinline__ void fft_pass_dyn(cplx<T>* buf, int stride, int t, const cplx<T>* __restrict__ tw,
                                             int Ns, int lg, bool last) {
  constexpr int TWR = TWN / R;  // TWS = TWN / (Ns R) = TWR >> lg
  cplx<T> v[NF][R];
#pragma unroll
  for (int f = 0; f < NF; ++f)
#pragma unroll
    for (int r = 0; r < R; ++r) v[f][r] = buf[f * stride + swz<T>(t + r * (N / R))];
  const int k = t & (Ns - 1);
  if (Ns > 1) {
    const int tws = TWR >> lg;
    cplx<T> w[R];
    if constexpr (sizeof(T) == 4) {
      const cplx<T> w1 = twiddle<DIR>(tw, k * tws);
      w[1] = w1;
#pragma unroll
      for (int r = 2; r < R; ++r) w[r] = w[r - 1] * w1;
    } else {
#pragma unroll
      for (int r = 1; r < R; ++r) w[r] = twiddle<DIR>(tw, r * k * tws);
    }
#pragma unroll
    for (int f = 0; f < NF; ++f)
#pragma unroll
      for (int r = 1; r < R; ++r) v[f][r] = tw_mul<false>(v[f][r], w[r]);
  }
#pragma unroll
  for (int f = 0; f < NF; ++f) dft<R, DIR, T, false>(v[f]);
  if constexpr (std::is_same<T, df64>::value) {
    if (last) {
#pragma unroll
      for (int f = 0; f < NF; ++f)
#pragma unroll
        for (int r = 0; r < R; ++r) v[f][r] = renorm(v[f][r]);
    }
  }
  __syncthreads();
  const int idxD = ((t >> lg) << lg) * R + k;
#pragma unroll
  for (int f = 0; f < NF; ++f)
#pragma unroll
    for (int r = 0; r < R; ++r) buf[f * stride + swz<T>(idxD + r * Ns)] = v[f][r];
  __syncthreads();
}

// NF independent length-N Stockham FFTs in lockstep on buffers buf + f * stride: one pair of
// block barriers per pass for all of them, NF x R independent shared-memory loads in flight
// per thread, and one twiddle computation shared by the NF butterflies of a thread.
template <class T, int N, int R, int DIR, int Ns, int NF>
__device__ __forceinline__ void fft_passes_multi(cplx<T>* buf, int stride, int t, const cplx<T>* __restrict__ tw) {
  if constexpr (Ns < N) {
    constexpr int Rp = (N / Ns < R) ? (N / Ns) : R;
    constexpr int NB = R / Rp;
    constexpr int TPF = N / R;
    constexpr int TWS = TWN / (Ns * Rp);
    cplx<T> v[NF][NB][Rp];
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      const int j = t + b * TPF;
#pragma unroll
      for (int f = 0; f < NF; ++f)
#pragma unroll
        for (int r = 0; r < Rp; ++r) v[f][b][r] = buf[f * stride + swz<T>(j + r * (N / Rp))];
    }
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      const int j = t + b * TPF;
      if constexpr (Ns > 1) {
        const int k = j & (Ns - 1);
        cplx<T> w[Rp];
        if constexpr (sizeof(T) == 4) {
          const cplx<T> w1 = twiddle<DIR>(tw, k * TWS);
          w[1] = w1;
#pragma unroll
          for (int r = 2; r < Rp; ++r) w[r] = w[r - 1] * w1;
        } else {
#pragma unroll
          for (int r = 1; r < Rp; ++r) w[r] = twiddle<DIR>(tw, r * k * TWS);
        }
#pragma unroll
        for (int f = 0; f < NF; ++f)
#pragma unroll
          for (int r = 1; r < Rp; ++r) v[f][b][r] = tw_mul<false>(v[f][b][r], w[r]);
      }
#pragma unroll
      for (int f = 0; f < NF; ++f) dft<Rp, DIR, T, (Ns * Rp >= N)>(v[f][b]);
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      const int j = t + b * TPF;
      const int idxD = (j / Ns) * Ns * Rp + (j & (Ns - 1));
#pragma unroll
      for (int f = 0; f < NF; ++f)
#pragma unroll
        for (int r = 0; r < Rp; ++r) buf[f * stride + swz<T>(idxD + r * Ns)] = v[f][b][r];
    }
    __syncthreads();
    fft_passes_multi<T, N, R, DIR, Ns * Rp, NF>(buf, stride, t, tw);
  }
}

// NF in-place FFTs of buffers buf + f * stride (same layout as fft_smem), in lockstep.
template <class T, int N, int R, int DIR, int NF>
__device__ __forceinline__ void fft_smem_multi(cplx<T>* buf, int stride, int t, const cplx<T>* __restrict__ tw) {
  if constexpr (GF_FFT_LOOP && sizeof(T) == 8) {
    int lg = 0;
#pragma unroll 1
    for (int Ns = 1; Ns < full_stride<N, R>(); Ns *= R, lg += ilog2(R))
      fft_pass_dyn<T, N, R, DIR, NF>(buf, stride, t, tw, Ns, lg, Ns * R == N);
    fft_passes_multi<T, N, R, DIR, full_stride<N, R>(), NF>(buf, stride, t, tw);
  } else {
    fft_passes_multi<T, N, R, DIR, 1, NF>(buf, stride, t, tw);
  }
}

// NF FFTs of buffers buf + f * stride: in lockstep when the registers allow (FP32, NF x R <=
// 24 values per thread), otherwise one after the other.
template <class T, int N, int R, int DIR, int NF>
__device__ __forceinline__ void fft_smem_group(cplx<T>* buf, int stride, int t, const cplx<T>* __restrict__ tw);

// In-place length-N FFT (DIR = -1 forward, +1 inverse; both unnormalised) of the swizzled
// buffer buf (logical element a at buf[swz<T>(a)]) by threads t in [0, N/R).  Every thread
// of the block must call it (it synchronises the block).  In FP64 and df64 the full radix-R
// passes run from one loop body and the remaining smaller-radix pass after them (their
// butterflies are long code); FP32 inlines every pass at its stride (measured faster).
template <class T, int N, int R, int DIR>
__device__ __forceinline__ void fft_smem(cplx<T>* buf, int t, const cplx<T>* __restrict__ tw) {
  if constexpr (GF_FFT_LOOP && sizeof(T) == 8) {
    int lg = 0;
#pragma unroll 1
    for (int Ns = 1; Ns < full_stride<N, R>(); Ns *= R, lg += ilog2(R)) fft_pass_dyn<T, N, R, DIR, 1>(buf, 0, t, tw, Ns, lg, Ns * R == N);
    fft_passes<T, N, R, DIR, full_stride<N, R>()>(buf, t, tw);
  } else {
    fft_passes<T, N, R, DIR, 1>(buf, t, tw);
  }
}

#ifndef GF_FFT_MULTI
#define GF_FFT_MULTI 1
#endif
template <class T, int N, int R, int DIR, int NF>
__device__ __forceinline__ void fft_smem_group(cplx<T>* buf, int stride, int t, const cplx<T>* __restrict__ tw) {
  if constexpr (GF_FFT_MULTI && sizeof(T) == 4 && NF * R <= 24 && NF > 1) {
    fft_smem_multi<T, N, R, DIR, NF>(buf, stride, t, tw);
  } else {
#pragma unroll 1
    for (int f = 0; f < NF; ++f) fft_smem<T, N, R, DIR>(buf + f * stride, t, tw);
  }
}

}  // namespace gf
