// Persistent ensemble kernels: the row and column stage kernels of several size classes in one
// launch each.  An ensemble of independent runs with uneven grid sizes (e.g. 1024 x 64^2 +
// 384 x 128^2 + 128 x 256^2) steps with one row launch and one column launch per stage for
// all of them, instead of one pair per size class on concurrent streams.  The grid is sized
// to the blocks that fit on the GPU at once; every block walks the work list -- the tiles of
// class 0 (instance-major), then class 1, ... -- with a stride of the grid size and runs
// each tile with the size's body (row_nl_body / col_stage_body, gf_kernels.cuh), so the
// physics is that of the per-class kernels.
//
// All sizes share one block of ENS_THREADS threads: length 32 at radix 4, 64 and 128 at radix
// 8 and 256 at radix 8, with ens_per_block(n) = ENS_THREADS / (n / radix) row pairs or kr
// columns per block.  The merged bodies need 128 registers (below that the column kernel
// spills heavily), so four blocks of 128 threads fit on an SM; measured on the 1536-run
// benchmark ensemble this is slower than one tuned launch pair per size class on concurrent
// streams (2.07 vs 1.38 ms per step), which therefore stays the default (gf_set_ensemble_mode).
#include <algorithm>

#include "gf_kernels.cuh"
#include "gf_launch.cuh"

namespace gf {

bool ens_size_ok(int n) { return n == 32 || n == 64 || n == 128 || n == 256; }
static int ens_radix(int n) { return n == 32 ? 4 : 8; }
int ens_per_block(int n) { return ENS_THREADS / (n / ens_radix(n)); }
template <class T> size_t ens_col_stride(int n) { return (size_t)col_stride<T>(n, ens_per_block(n)); }

// class and tile of work item `item`
__device__ __forceinline__ int ens_find(const EnsArgs& a, int item, int* bx, int* by) {
  int c = 0, base = 0;
  while (c + 1 < a.ncls && item >= base + a.c[c].nbx * a.c[c].nby) {
    base += a.c[c].nbx * a.c[c].nby;
    ++c;
  }
  const int local = item - base;
  *bx = local % a.c[c].nbx;
  *by = local / a.c[c].nbx;
  return c;
}

template <class T>
__global__ void __launch_bounds__(ENS_THREADS, 4) ens_row_kernel(const __grid_constant__ EnsArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
#pragma unroll 1
  for (int item = blockIdx.x; item < a.total; item += gridDim.x) {
    int bx, by;
    const EnsClass& k = a.c[ens_find(a, item, &bx, &by)];
    switch (k.n) {
      case 32: row_nl_body<T, 32, 4, false>(k.g, k.m, k.b, k.per, bx, by, smem_raw); break;
      case 64: row_nl_body<T, 64, 8, false>(k.g, k.m, k.b, k.per, bx, by, smem_raw); break;
      case 128: row_nl_body<T, 128, 8, false>(k.g, k.m, k.b, k.per, bx, by, smem_raw); break;
      default: row_nl_body<T, 256, 8, false>(k.g, k.m, k.b, k.per, bx, by, smem_raw); break;
    }
    __syncthreads();  // the next tile refills the shared buffers
  }
}

template <class T>
__global__ void __launch_bounds__(ENS_THREADS, 4) ens_col_kernel(const __grid_constant__ EnsArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ T eig[MAXL + 2 * MAXL * MAXL];
#pragma unroll 1
  for (int item = blockIdx.x; item < a.total; item += gridDim.x) {
    int bx, by;
    const EnsClass& k = a.c[ens_find(a, item, &bx, &by)];
    switch (k.n) {
      case 32: col_stage_body<T, 32, 4, 512, true>(k.g, k.m, k.s, k.b, k.per, bx, by, smem_raw, eig); break;
      case 64: col_stage_body<T, 64, 8, 512, true>(k.g, k.m, k.s, k.b, k.per, bx, by, smem_raw, eig); break;
      case 128: col_stage_body<T, 128, 8, 512, true>(k.g, k.m, k.s, k.b, k.per, bx, by, smem_raw, eig); break;
      default: col_stage_body<T, 256, 8, 512, true>(k.g, k.m, k.s, k.b, k.per, bx, by, smem_raw, eig); break;
    }
    __syncthreads();
  }
}

// dynamic shared memory of a launch: the largest tile of its classes
template <class T>
static size_t ens_smem(const EnsArgs& a, bool row) {
  size_t sm = 0;
  for (int c = 0; c < a.ncls; ++c) {
    const int n = a.c[c].n, per = a.c[c].per, tpf = n / ens_radix(n);
    const size_t e = sizeof(cplx<T>);
    sm = std::max(sm, row ? (size_t)per * 3 * row_stride<T>(n, tpf) * e : (size_t)3 * per * ens_col_stride<T>(n) * e);
  }
  return sm;
}

// blocks of the persistent grid: as many as fit on the GPU at once, at most one per item
template <class K>
static int ens_grid(K kernel, size_t sm, int total) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, ENS_THREADS, sm) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  return std::max(1, std::min(total, per_sm * num_sms()));
}

template <class T>
cudaError_t launch_ens_row(const EnsArgs& a, cudaStream_t st) {
  const size_t sm = ens_smem<T>(a, true);
  cudaError_t err = set_smem(ens_row_kernel<T>, sm);
  if (err != cudaSuccess) return err;
  ens_row_kernel<T><<<ens_grid(ens_row_kernel<T>, sm, a.total), ENS_THREADS, sm, st>>>(a);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_ens_col(const EnsArgs& a, cudaStream_t st) {
  const size_t sm = ens_smem<T>(a, false);
  cudaError_t err = set_smem(ens_col_kernel<T>, sm);
  if (err != cudaSuccess) return err;
  ens_col_kernel<T><<<ens_grid(ens_col_kernel<T>, sm, a.total), ENS_THREADS, sm, st>>>(a);
  return cudaGetLastError();
}

#define GF_INST_ENS(T)                                                              \
  template cudaError_t launch_ens_row<T>(const EnsArgs&, cudaStream_t);             \
  template cudaError_t launch_ens_col<T>(const EnsArgs&, cudaStream_t);             \
  template size_t ens_col_stride<T>(int);

GF_INST_ENS(float)
GF_INST_ENS(double)
GF_INST_ENS(df64)

}  // namespace gf
