// Allocation-free forward 2-D real FFT.
//
// Some callers cannot allocate device memory: code running inside another runtime that owns
// the device's memory (a Julia session whose CUDA.jl pool holds the GPU and enforces a
// memory limit, a host framework with its own caching allocator), or a latency-critical
// loop in which cudaMalloc/cudaFree, which can synchronise the device, are not acceptable.
// For them gf_rfft2_noalloc transforms a caller-owned device field into a caller-owned
// device spectrum without allocating: its intermediate (the x-transformed rows) and its
// twiddle tables live in file-scope __device__ arrays of fixed size that every GPU loading
// the library keeps until the process exits.
//
// Limits and rules (also in include/gfcuda.h):
//   * nx, ny powers of two in [32, GF_NOALLOC_MAX_N]; larger sizes are rejected.
//   * The first call on a device does the set-up for that device (symbol addresses, twiddle
//     tables copied in, then a device synchronisation so that the tables are complete for a
//     kernel on any stream); make that first call before any stream capture.
//   * At most 64 devices.  A device reset is not supported: the set-up is not redone, so
//     the reset device's tables would stay unwritten.
//   * All calls share the scratch array: calls that overlap on the GPU (different streams,
//     or different host threads without ordering) race and give wrong results.  Every
//     scratch element a call reads is written earlier in the same call, so nothing has to
//     be cleared between calls.
#include <cmath>
#include <mutex>
#include <string>

#include "gf_fft.cuh"
#include "gf_internal.h"
#include "gfcuda.h"

namespace {

constexpr int kMaxN = GF_NOALLOC_MAX_N;
constexpr int kMaxDevices = 64;
// x-transformed rows: ny rows of nx/2+1 complex values, largest case in double precision
static __device__ __align__(256) unsigned char g_noalloc_scratch[(size_t)kMaxN * (kMaxN / 2 + 1) * 16];
static __device__ __align__(256) unsigned char g_noalloc_tw64[gf::TWN * 16];
static __device__ __align__(256) unsigned char g_noalloc_tw32[gf::TWN * 8];

struct DeviceSlot {
  bool ready = false;
  void* scratch = nullptr;
  void* tw64 = nullptr;
  void* tw32 = nullptr;
};
DeviceSlot g_slots[kMaxDevices];
std::mutex g_mutex;

int fail(int code, const std::string& msg) {
  gf::set_global_error(msg);  // readable through gf_last_error(NULL)
  return code;
}

// Per-device set-up, done once with that device current.
int setup(int dev, DeviceSlot** out) {
  std::lock_guard<std::mutex> lk(g_mutex);
  DeviceSlot& s = g_slots[dev];
  if (!s.ready) {
    void *scratch = nullptr, *tw64 = nullptr, *tw32 = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&scratch, g_noalloc_scratch);
    if (e == cudaSuccess) e = cudaGetSymbolAddress(&tw64, g_noalloc_tw64);
    if (e == cudaSuccess) e = cudaGetSymbolAddress(&tw32, g_noalloc_tw32);
    if (e != cudaSuccess) return fail(GF_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    static double t64[2 * gf::TWN];
    static float t32[2 * gf::TWN];
    for (int i = 0; i < gf::TWN; ++i) {
      t64[2 * i] = std::cos(2 * M_PI * i / gf::TWN);
      t64[2 * i + 1] = -std::sin(2 * M_PI * i / gf::TWN);
      t32[2 * i] = (float)t64[2 * i];
      t32[2 * i + 1] = (float)t64[2 * i + 1];
    }
    e = cudaMemcpyToSymbol(g_noalloc_tw64, t64, sizeof(t64));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_noalloc_tw32, t32, sizeof(t32));
    if (e != cudaSuccess) return fail(GF_ERR_CUDA, std::string("cudaMemcpyToSymbol: ") + cudaGetErrorString(e));
    // A copy from pageable host memory may return before the data reaches the device, and it
    // is ordered only against the legacy default stream; the kernels go to the caller's
    // stream, which may be non-blocking.  Wait for the device once here so that no kernel of
    // any stream can read a partly written table.
    e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return fail(GF_ERR_CUDA, std::string("cudaDeviceSynchronize: ") + cudaGetErrorString(e));
    s.scratch = scratch;
    s.tw64 = tw64;
    s.tw32 = tw32;
    s.ready = true;
  }
  *out = &s;
  return GF_OK;
}

bool pow2_in_range(int n) { return n >= 32 && n <= kMaxN && (n & (n - 1)) == 0; }

}  // namespace

extern "C" int gf_rfft2_noalloc(const void* field, void* fieldh, int32_t nx, int32_t ny, int32_t precision,
                                void* stream) {
  if (!field || !fieldh) return fail(GF_ERR_ARG, "gf_rfft2_noalloc: null field or fieldh");
  if (precision != GF_F32 && precision != GF_F64) return fail(GF_ERR_ARG, "gf_rfft2_noalloc: unknown precision");
  if (!pow2_in_range(nx) || !pow2_in_range(ny))
    return fail(GF_ERR_UNSUPPORTED, "gf_rfft2_noalloc: nx and ny must be powers of two in [32, GF_NOALLOC_MAX_N = 512]");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0) return fail(GF_ERR_CUDA, "gf_rfft2_noalloc: no current device");
  if (dev >= kMaxDevices)
    return fail(GF_ERR_UNSUPPORTED, "gf_rfft2_noalloc: device ordinal " + std::to_string(dev) +
                                        " is beyond the supported 64 devices (ordinals 0..63)");
  DeviceSlot* s = nullptr;
  if (int r = setup(dev, &s)) return r;
  gf::Geom g{};
  g.nx = nx; g.ny = ny; g.nkr = nx / 2 + 1; g.ldk = g.nkr; g.ldw = g.nkr; g.nl = 1;
  g.kcut = g.nkr; g.lA = 1; g.lB = 0;
  g.nb = 1;  // one field: a single instance (the per-instance strides are never used)
  g.dkx = 1; g.dky = 1; g.inv_nxny = 1.0 / ((double)nx * ny);
  g.dkx_f = 1.0f; g.dky_f = 1.0f; g.inv_nxny_f = (float)g.inv_nxny;
  cudaStream_t st = (cudaStream_t)stream;
  gf::Bufs b{precision == GF_F64 ? s->tw64 : s->tw32, nullptr, s->scratch};
  // consume a pending non-sticky error of an earlier runtime call in this thread, which the
  // launch checks below (cudaGetLastError) would otherwise report as theirs
  (void)cudaGetLastError();
  if (precision == GF_F64) {
    e = gf::launch_row_r2c<double>(g, b, 1, field, st);
    if (e == cudaSuccess) e = gf::launch_col_fwd<double>(g, b, 1, fieldh, 0, st);
  } else {
    e = gf::launch_row_r2c<float>(g, b, 1, field, st);
    if (e == cudaSuccess) e = gf::launch_col_fwd<float>(g, b, 1, fieldh, 0, st);
  }
  if (e != cudaSuccess) return fail(GF_ERR_CUDA, cudaGetErrorString(e));
  return GF_OK;
}
