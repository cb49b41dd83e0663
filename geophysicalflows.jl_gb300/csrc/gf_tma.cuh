// Column stage with TMA tile copies (cp.async.bulk.tensor) for one layer without bottom drag
// and at most two product fields: TwoDNavierStokes, SingleLayerQG without a PV-gradient
// product, SurfaceQG -- the one-layer branch of col_stage_kernel (gf_kernels.cuh), with its
// global traffic moved to the tensor-memory-access engine.
//
// One elected thread issues the loads of the block's product tile -- C adjacent kr columns x
// NY rows of each product field, as boxes of min(NY, 256) rows -- onto one mbarrier, so the
// whole tile is in flight at once with no per-element instructions; the other threads wait on
// the barrier with a time limit.  TMA writes a box densely ([j][C], element (c, j) at
// j * C + c).  The first FFT pass reads that dense tile with the lanes of a warp running
// column-fastest (conflict-free: consecutive lanes read consecutive 8- or 16-byte elements)
// and writes the swizzled column layout of gf_fft.cuh (c * cs + swz(j)) in place; the middle
// passes are the usual column-major Stockham passes.  The inverse transforms end the same
// way in reverse: their last pass writes the dense layout, which the elected thread stores to
// the pruned inverse fields W with TMA tile stores (clipped at kr = kcut by the tensor map).
// The stage epilogue (stepper combination, forcing, dealias) is the shared stage_epilogue.
//
// Tensor maps (built on the host per context, see tma_maps in gf_api.cu) view P and W as 3-D
// arrays of 32-bit words: x = the complex element's words along a row (kr), y = field * ny + j,
// z = instance.
#pragma once
#include <cuda.h>

#include "gf_kernels.cuh"

namespace gf {

// ---------------------------------------------------------------- PTX: mbarrier and TMA
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
// makes the initialised barrier visible to the asynchronous (TMA) proxy
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Waits for the barrier phase with the given parity; false once `limit_ns` nanoseconds have
// passed without it completing (the caller then reports an error instead of hanging).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity, uint64_t limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  while (!mbar_try_wait(bar, parity))
    if (global_ns() - t0 > limit_ns) return false;
  return true;
}
// 3-D tile load global -> shared, completion counted in bytes on `bar`
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
      ::"r"(smem_u32(dst)), "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}
// 3-D tile store shared -> global (bulk group of the issuing thread)
__device__ __forceinline__ void tma_store_3d(const CUtensorMap* map, int x, int y, int z, const void* src) {
  asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%1, %2, %3}], [%4];"
               ::"l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(src))
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// the issuing thread's bulk stores have finished reading shared memory
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// ... and have completed
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
// orders this thread's shared-memory writes before later asynchronous-proxy (TMA) reads
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// time limit of a wait for a tile load (a load of a few hundred KB takes microseconds)
constexpr uint64_t kTmaWaitNs = 1000000000ull;
// rows per TMA box (the hardware limit is 256 per dimension)
template <int NY> __host__ __device__ constexpr int tma_box_rows() { return NY < 256 ? NY : 256; }

// ------------------------------------------------------------------- FFT passes
// One Stockham pass of NF length-N FFTs in lockstep (field f at F + f * fstride) at stride Ns
// (radix Rp = min(R, N / Ns)).  SRCD / DSTD: the pass reads / writes the dense [j][C] tile
// layout (element (c, j) at j * C + c) instead of the swizzled column layout (c * cs +
// swz(j)); a pass touching the dense layout maps the lanes column-fastest (c = tid % C, the
// butterfly index tid / C), the others column-major (column tid / TPF, butterfly tid % TPF).
// Both mappings are bank-conflict free for C = 2, 4 (8-byte elements) and C = 1, 2 (16-byte
// elements) at radix 8 and 16 from NY = 128 on.
template <class T, int N, int R, int DIR, int NF, int C, int Ns, bool SRCD, bool DSTD>
__device__ __forceinline__ void tma_pass(cplx<T>* F, int fstride, int cs, int tid, const cplx<T>* __restrict__ tw) {
  constexpr int TPF = N / R;
  constexpr int Rp = (N / Ns < R) ? (N / Ns) : R;
  constexpr int NB = R / Rp;
  constexpr int TWS = TWN / (Ns * Rp);
  constexpr bool dense_map = SRCD || DSTD;
  const int col = dense_map ? tid % C : tid / TPF;
  const int tt = dense_map ? tid / C : tid % TPF;
  cplx<T> v[NF][NB][Rp];
#pragma unroll
  for (int b = 0; b < NB; ++b) {
    const int j = tt + b * TPF;
#pragma unroll
    for (int f = 0; f < NF; ++f)
#pragma unroll
      for (int r = 0; r < Rp; ++r) {
        const int src = j + r * (N / Rp);
        v[f][b][r] = SRCD ? F[f * fstride + src * C + col] : F[f * fstride + col * cs + swz<T>(src)];
      }
  }
#pragma unroll
  for (int b = 0; b < NB; ++b) {
    const int j = tt + b * TPF;
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
    for (int f = 0; f < NF; ++f) dft<Rp, DIR, T, (Ns * Rp >= N)>(v[f][b]);  // df64: last pass normalises
  }
  __syncthreads();
#pragma unroll
  for (int b = 0; b < NB; ++b) {
    const int j = tt + b * TPF;
    const int idxD = (j / Ns) * Ns * Rp + (j & (Ns - 1));
#pragma unroll
    for (int f = 0; f < NF; ++f)
#pragma unroll
      for (int r = 0; r < Rp; ++r) {
        const int dst = idxD + r * Ns;
        if constexpr (DSTD) F[f * fstride + dst * C + col] = v[f][b][r];
        else F[f * fstride + col * cs + swz<T>(dst)] = v[f][b][r];
      }
  }
  __syncthreads();
}

// All passes of NF lockstep length-N FFTs from stride Ns on; the first pass (Ns = 1) reads
// the dense layout when SRCD, the last one writes it when DSTD.  The caller synchronises the
// block before the first pass; every pass ends with a block barrier.
template <class T, int N, int R, int DIR, int NF, int C, int Ns, bool SRCD, bool DSTD>
__device__ __forceinline__ void tma_passes(cplx<T>* F, int fstride, int cs, int tid, const cplx<T>* __restrict__ tw) {
  if constexpr (Ns < N) {
    constexpr int Rp = (N / Ns < R) ? (N / Ns) : R;
    tma_pass<T, N, R, DIR, NF, C, Ns, SRCD && Ns == 1, DSTD && Ns * Rp >= N>(F, fstride, cs, tid, tw);
    tma_passes<T, N, R, DIR, NF, C, Ns * Rp, SRCD, DSTD>(F, fstride, cs, tid, tw);
  }
}

// Stride of the last pass of a length-N transform at radix R (the largest R^p below N).
template <int N, int R> __host__ __device__ constexpr int last_stride() {
  int s = 1;
  while (s * ((N / s < R) ? N / s : R) < N) s *= R;
  return s;
}

// The same passes for 8-byte types (FP64, df64), whose butterflies are long code: the first
// and last passes inlined (they touch the dense layout), the full radix-R passes between them
// from one run-time loop body (fft_pass_dyn, column-major mapping) for the instruction cache.
template <class T, int N, int R, int DIR, int NF, int C, bool SRCD, bool DSTD>
__device__ __forceinline__ void tma_passes_looped(cplx<T>* F, int fstride, int cs, int tid,
                                                  const cplx<T>* __restrict__ tw) {
  constexpr int NL = last_stride<N, R>();
  if constexpr (NL == 1) {
    tma_pass<T, N, R, DIR, NF, C, 1, SRCD, DSTD>(F, fstride, cs, tid, tw);
  } else {
    constexpr int TPF = N / R;
    tma_pass<T, N, R, DIR, NF, C, 1, SRCD, false>(F, fstride, cs, tid, tw);
    int lg = ilog2(R);
#pragma unroll 1
    for (int Ns = R; Ns < NL; Ns *= R, lg += ilog2(R))
      fft_pass_dyn<T, N, R, DIR, NF>(F + (tid / TPF) * cs, fstride, tid % TPF, tw, Ns, lg, false);
    tma_pass<T, N, R, DIR, NF, C, NL, false, DSTD>(F, fstride, cs, tid, tw);
  }
}

// NF FFTs of fields F + f * fstride: in lockstep when the registers allow (FP32, NF x R <= 24
// values per thread), otherwise one after the other.
template <class T, int N, int R, int DIR, int NF, int C, bool SRCD, bool DSTD>
__device__ __forceinline__ void tma_fft(cplx<T>* F, int fstride, int cs, int tid, const cplx<T>* __restrict__ tw) {
  if constexpr (sizeof(T) == 8 && GF_FFT_LOOP) {
#pragma unroll 1
    for (int f = 0; f < NF; ++f) tma_passes_looped<T, N, R, DIR, 1, C, SRCD, DSTD>(F + f * fstride, 0, cs, tid, tw);
  } else if constexpr (NF == 1 || (sizeof(T) == 4 && NF * R <= 24)) {
    tma_passes<T, N, R, DIR, NF, C, 1, SRCD, DSTD>(F, fstride, cs, tid, tw);
  } else {
#pragma unroll 1
    for (int f = 0; f < NF; ++f) tma_passes<T, N, R, DIR, 1, C, 1, SRCD, DSTD>(F + f * fstride, 0, cs, tid, tw);
  }
}

// ------------------------------------------------------------------------ the kernel
// Block: C adjacent kr columns x NY / R threads per column; two shared buffers of C columns
// (column stride cs) and the mbarrier after them.  Tensor copies need a 128-byte aligned
// shared address: the kernel has no static shared memory, rounds the dynamic base up to 128
// bytes (the launch asks for 128 bytes more), and every field and box offset is a multiple of
// 128 bytes (col_stride pads to multiples of 4 columns' worth); a block that still finds its
// buffers misaligned reports it (err |= 2) and copies nothing.  `err` |= 1: a tile load did
// not complete within kTmaWaitNs.  Three blocks per SM at up to 256 threads (register budget
// 85), one above.
template <class T, int NY, int R, int C>
__global__ void __launch_bounds__(C*(NY / R), (C * (NY / R) <= 256) ? 3 : 1)
    col_tma_kernel(Geom g, ModArgs m, StepArgs s, Bufs b, const __grid_constant__ CUtensorMap tmP,
                   const __grid_constant__ CUtensorMap tmW, int* err) {
  extern __shared__ __align__(16) unsigned char smem_dyn[];
  constexpr int TPF = NY / R;
  constexpr int WPC = (int)(sizeof(cplx<T>) / 4);  // 32-bit words per complex element
  constexpr int BR = tma_box_rows<NY>();
  const int cs = g.cs;
  const int fstride = C * cs;
  unsigned char* smem_raw = smem_dyn + ((128u - (smem_u32(smem_dyn) & 127u)) & 127u);
  cplx<T>* F0 = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* F1 = F0 + fstride;
  uint64_t& bar = *reinterpret_cast<uint64_t*>(F0 + 2 * fstride);
  const int tid = threadIdx.x, c = tid % C, t = tid / C;
  const int kr0 = blockIdx.x * C, kr = kr0 + c;
  const int z = blockIdx.y;  // ensemble instance
  // unobserved step (kout set): products only for kr < kout = kcut, the state updated only at
  // kept modes (as in col_stage_kernel)
  const bool prune = g.kout > 0;
  const bool kin = kr < (prune ? g.kout : g.nkr);
  const cplx<T>* tw = static_cast<const cplx<T>*>(b.twid);
  const EpiCtx<T> ec = epi_ctx<T>(g, m, s, kr, (size_t)z);
  const T ell2 = sel<T>(m.ell_inv2, m.ell_inv2_f, m.ell_inv2_l);
  const T sc = sel<T>(g.inv_nxny, g.inv_nxny_f, g.inv_nxny_l);
  const int nslot = 1 + m.hasB + m.hasC;  // <= 2 (the host launches this kernel only then)

  if (__syncthreads_or(tid == 0 && ((smem_u32(F0) | smem_u32(F1)) & 127u) != 0)) {
    if (tid == 0) atomicOr(err, 2);
    return;
  }
  // The next stage's X at element (c, j) goes straight into the slots of that element: q = X
  // into F0 and v = i kr psi into F1 (scaled by 1 / (nx ny)), so no per-thread array of X is
  // kept (with the shared-memory carve-out L1 is small, and such an array would live in local
  // memory backed by L2).  Each thread reads and writes only its own elements' slots.
  const T dky = ec.dky, krT = ec.krT;
  auto fill_qv = [&](int j, cplx<T> x) {
    const T lv = T(lidx(g, j)) * dky;
    const T K2 = krT * krT + lv * lv;
    const cplx<T> p = psi_factor<T>(m.psi_kind, K2, ell2, m.mult, (size_t)j * g.ldk + (kin ? kr : 0)) * x;
    F0[c * cs + swz<T>(j)] = sc * x;
    F1[c * cs + swz<T>(j)] = sc * (krT * mul_i(p));   // v = i kr psi
  };
  if (s.do_fwd) {
    if (tid == 0) {
      mbar_init(&bar, 1);
      mbar_fence_init();
    }
    __syncthreads();
    if (tid == 0) {
      mbar_arrive_expect_tx(&bar, (unsigned)(nslot * NY * C * sizeof(cplx<T>)));
      for (int f = 0; f < nslot; ++f)
        for (int r0 = 0; r0 < NY; r0 += BR)
          tma_load_3d(F0 + f * fstride + r0 * C, &tmP, kr0 * WPC, f * g.ny + r0, z, &bar);
    }
    const bool ok = mbar_wait_bounded(&bar, 0, kTmaWaitNs);
    if (__syncthreads_or(!ok)) {
      // the tile did not arrive in time: report it, give the copies a second period to land
      // in this block's shared memory, and leave
      if (tid == 0) atomicOr(err, 1);
      mbar_wait_bounded(&bar, 0, kTmaWaitNs);
      return;
    }
    if (nslot == 2) tma_fft<T, NY, R, -1, 2, C, true, false>(F0, fstride, cs, tid, tw);
    else tma_fft<T, NY, R, -1, 1, C, true, false>(F0, fstride, cs, tid, tw);
#pragma unroll 1
    for (int i = 0; i < R; ++i) {
      const int j = t + i * TPF;
      cplx<T> xn = czero<T>();
      if (kin && !(prune && !kept(g, kr, j))) {
        cplx<T> N = czero<T>();
        for (int f = 0; f < nslot; ++f) {
          const int slot = (f == 0) ? 0 : m.hasB ? 1 : 2;
          N = N + product_term<T>(ec, g, m, slot, j, F0[f * fstride + c * cs + swz<T>(j)]);
        }
        xn = stage_epilogue<T>(ec, g, m, s, 0, j, N);
      }
      fill_qv(j, xn);
    }
  } else {
    const cplx<T>* sol = static_cast<const cplx<T>*>(s.sol);
#pragma unroll 1
    for (int i = 0; i < R; ++i) {
      const int j = t + i * TPF;
      fill_qv(j, (kin && kept(g, kr, j)) ? sol[ec.ioff + (size_t)j * g.ldk + kr] : czero<T>());
    }
  }
  if (!s.do_inv) return;
  if (kr0 >= g.kcut) return;  // whole block aliased: W is never read there
  __syncthreads();

  // y-inverse FFTs of the next stage's (q, u, v): v (F1) first, stored by TMA; then u = -i l
  // psi formed from the untransformed q in F0 (psi = f q / sc) into F1, and q and u
  // transformed and stored together.
  tma_fft<T, NY, R, +1, 1, C, false, true>(F1, fstride, cs, tid, tw);
  fence_proxy_async_smem();
  __syncthreads();
  if (tid == 0) {
    for (int r0 = 0; r0 < NY; r0 += BR) tma_store_3d(&tmW, kr0 * WPC, 2 * g.ny + r0, z, F1 + r0 * C);
    bulk_commit();
    bulk_wait_read();  // F1 is refilled with u below
  }
  __syncthreads();
#pragma unroll 1
  for (int i = 0; i < R; ++i) {
    const int j = t + i * TPF;
    const T lv = T(lidx(g, j)) * dky;
    const T K2 = krT * krT + lv * lv;
    const cplx<T> p =
        psi_factor<T>(m.psi_kind, K2, ell2, m.mult, (size_t)j * g.ldk + (kin ? kr : 0)) * F0[c * cs + swz<T>(j)];
    F1[c * cs + swz<T>(j)] = lv * mul_mi(p);   // u = -i l psi
  }
  __syncthreads();
  tma_fft<T, NY, R, +1, 2, C, false, true>(F0, fstride, cs, tid, tw);
  fence_proxy_async_smem();
  __syncthreads();
  if (tid == 0) {
    for (int f = 0; f < 2; ++f)
      for (int r0 = 0; r0 < NY; r0 += BR) tma_store_3d(&tmW, kr0 * WPC, f * g.ny + r0, z, F0 + f * fstride + r0 * C);
    bulk_commit();
    bulk_wait_all();
  }
}

// Shared-memory bytes of col_tma_kernel: two buffers of C columns with column stride cs, the
// mbarrier, and 128 bytes to align the base.
__host__ __forceinline__ size_t col_tma_smem(int C, int cs, size_t elem) { return (size_t)2 * C * cs * elem + 16 + 128; }

}  // namespace gf
