// C ABI of libgfcuda: problem construction, state transfer, the time-step loop and the
// diagnostics.  The kernels live in gf_kernels.cuh (instantiated by gf_f32.cu/gf_f64.cu);
// this file holds the host-side orchestration and the FP64 setup kernels.
#include <cuda.h>

#include <atomic>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "gf_fft.cuh"
#include "gf_internal.h"
#include "gf_launch.cuh"
#include "gf_philox.cuh"
#include "gfcuda.h"

using namespace gf;

static std::string g_create_error;

void gf::set_global_error(const std::string& msg) { g_create_error = msg; }

struct gf_ctx {
  gf_config cfg;
  int prec = GF_F32;
  size_t rb = 4, cb = 8;  // real / complex element bytes
  cudaStream_t stream = nullptr;
  int dev = 0;  // the device current at gf_create; every call runs on it (DevGuard)
  Geom g{};
  ModArgs m{};
  int kind = SK_RK4, filtered = 0, hasL = 0, cplxL = 0, nstages = 4;
  double t = 0;
  int64_t step = 0;
  bool W_valid = false;
  double last_fscale = 0;  // forcing scale of the last calcN! (deterministic forcing)
  double Hsum = 1, f0 = 1;
  std::vector<double> gprime, Hl;
  std::vector<double> filt_host;  // the Filtered steppers' filter, [ny][nx/2+1]
  double* Ud = nullptr;           // MultiLayerQG U(y) per layer [nl][ny], FP64 (fluxes)
  // device buffers
  std::vector<void*> allocs;
  void *sol = nullptr, *X = nullptr, *acc = nullptr, *s1 = nullptr, *N1 = nullptr, *R3[3] = {nullptr, nullptr, nullptr};
  void* Xg = nullptr;       // several layers: the next stage's X between the two column launches
  void *W = nullptr, *P = nullptr, *D = nullptr, *twid = nullptr;
  void *Ltab = nullptr, *filt = nullptr, *etd[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  void *mult = nullptr, *eta = nullptr, *U1D = nullptr, *Qy1D = nullptr, *Qx2D = nullptr, *Qy2D = nullptr,
       *etah = nullptr;
  void *Fh = nullptr, *fspec = nullptr, *Fstore = nullptr, *prevsol = nullptr;
  void *phys = nullptr;     // [4][nl][ny][nx] physical fields from updatevars!
  void *tmp_spec = nullptr; // [nl][ny][ldk] scratch spectral array
  void *tmp_spec2 = nullptr;
  void *stage = nullptr;    // staging for host transfers (contiguous copy, re-pitched / df64-converted on the device)
  double *dpart = nullptr, *dout = nullptr;
  int diag_blocks = 0;
  int ab3_out = 0, ab3_m1 = 1, ab3_m2 = 2;
  // kernel timing (gf_profile_enable): CUDA events around every row / column launch
  bool profiling = false;
  std::vector<cudaEvent_t> ev_free;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev_used;
  double prof_ms[2] = {0, 0};
  int64_t prof_n[2] = {0, 0};
  int64_t launches = 0;
  // device clock and graph replay of multi-step sequences
  DevClock* dclk = nullptr;
  int graph_steps = 4;
  // captured step sequences [AB3 ring phase][0: every step unobserved, 1: the last observed]
  cudaGraphExec_t gexec[3][2] = {{nullptr, nullptr}, {nullptr, nullptr}, {nullptr, nullptr}};
  bool own_stream = false;
  // adjoint (gf_adjoint_setup): checkpoints, the recomputed forward fields of one segment,
  // and the cotangent arrays; freed by gf_destroy or a new set-up
  struct Adjoint {
    bool ready = false, forward_done = false;
    int64_t nsteps = 0;
    int every = 1, nseg = 0;   // recomputation unit (steps whose forward fields are kept at once), units
    int snaps = 0;             // state snapshot slots (slot 0: the initial state)
    std::vector<void*> mem;
    void *ckpt = nullptr, *phys = nullptr, *ub = nullptr, *n1acc = nullptr, *xaacc = nullptr, *x1acc = nullptr;
    void *ubar_in = nullptr, *ubar_out = nullptr, *Wb = nullptr, *Pb = nullptr, *etab = nullptr;
    void *final_state = nullptr, *tmp = nullptr;
    void *qxb = nullptr, *qyb = nullptr;  // U(y): cotangents of Qx, Qy (physical)
    void* nbar = nullptr;               // several layers / bottom drag: the current stage's Nbar
    int nwb = 2;                        // cotangent fields in Wb (3 with the U(y) product)
    std::vector<double> ck_t;           // per slot
    std::vector<int64_t> ck_step;
    std::vector<int> split;             // binomial schedule: split[n * snaps + s]
    std::vector<std::pair<int, int>> spine;  // (unit, slot) snapshots taken by the forward pass
    int64_t forward_units = 0;          // unit advances the last reverse sweep added (recomputation)
    double t_end = 0;
    int64_t step_end = 0;
    // pipelined reverse sweep: the transposed stages of one unit run on `ts` while the
    // context stream recomputes the next unit into the other half of `phys` (two units of
    // forward fields); ev_rec[k] / ev_adj[k] mark the recomputation into / the last read of
    // half k, ev_sync orders the two streams at the start and end of a sweep
    cudaStream_t ts = nullptr;
    cudaEvent_t ev_rec[2] = {nullptr, nullptr}, ev_adj[2] = {nullptr, nullptr}, ev_sync = nullptr;
    size_t unit_phys = 0;               // bytes of one unit's forward fields
    int half = 0;                       // half of `phys` the next recomputation writes
  } adj;
  void* row_phys = nullptr;  // forward row kernels also store (q + eta, u, v) here when set
  TmaMaps tma;               // tensor maps of the TMA column stage (one layer)
  int* derr = nullptr;       // device error flag: a tile-load wait ran out of time
  void *twx = nullptr, *twy = nullptr;  // generic-length twiddle tables (nx and ny entries)
  // identity and graph generation (an ensemble graph records the members it was built for)
  uint64_t uid = 0, gen = 0;
  cudaGraphExec_t egraph[2] = {nullptr, nullptr};      // ensemble graphs held by the first member (as gexec)
  std::vector<std::pair<uint64_t, uint64_t>> emembers;  // (uid, gen) of its members
  int eG = 0;
  // ensemble execution when this context leads gf_ensemble_step: 1 the persistent ensemble
  // kernels where the members allow them, 0 (default, faster on the benchmark ensemble) one
  // batched context per stream; eMode: the execution the held ensemble graphs were captured with
  int ens_mode = 0, eMode = -1;
  cudaEvent_t order_ev = nullptr;  // orders this context's stream with an ensemble graph launch
  std::string err;
};

// ------------------------------------------------------------------------ FP64 setup kernels
template <class T>
__global__ void etd_coeffs_kernel(int n, const double* __restrict__ Lre, const double* __restrict__ Lim, double dt,
                                  int ncirc, double rcirc, int cplx_out, T* e, T* e2, T* zeta, T* alpha, T* beta,
                                  T* gamma, int nkr, int ldk) {
  typedef std::complex<double> Z;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
    const double lr = Lre[idx], li = Lim ? Lim[idx] : 0.0;
    double zr = 0, zi = 0, ar = 0, ai = 0, br = 0, bi = 0, gr = 0, gi = 0;
    for (int q = 0; q < ncirc; ++q) {
      double s, c;
      sincospi(2.0 * (q + 0.5) / ncirc, &s, &c);
      // z = dt L + r e^{i theta}
      const double xr = dt * lr + rcirc * c, xi = dt * li + rcirc * s;
      double es, ec;
      sincos(xi, &es, &ec);
      const double ea = exp(xr);
      const double ezr = ea * ec, ezi = ea * es;  // e^z
      sincos(0.5 * xi, &es, &ec);
      const double eh = exp(0.5 * xr);
      const double ehr = eh * ec, ehi = eh * es;  // e^{z/2}
      // complex helpers
      auto mul = [](double a, double b, double c_, double d, double* r, double* i) { *r = a * c_ - b * d; *i = a * d + b * c_; };
      double z2r, z2i, z3r, z3i;
      mul(xr, xi, xr, xi, &z2r, &z2i);
      mul(z2r, z2i, xr, xi, &z3r, &z3i);
      const double den1 = xr * xr + xi * xi, den3 = z3r * z3r + z3i * z3i;
      double nr, ni, tr, ti;
      // zeta: (e^{z/2} - 1) / z
      nr = ehr - 1; ni = ehi;
      zr += (nr * xr + ni * xi) / den1; zi += (ni * xr - nr * xi) / den1;
      // alpha: (-4 - z + e^z (4 - 3z + z^2)) / z^3
      mul(ezr, ezi, 4 - 3 * xr + z2r, -3 * xi + z2i, &tr, &ti);
      nr = -4 - xr + tr; ni = -xi + ti;
      ar += (nr * z3r + ni * z3i) / den3; ai += (ni * z3r - nr * z3i) / den3;
      // beta: (2 + z + e^z (-2 + z)) / z^3
      mul(ezr, ezi, -2 + xr, xi, &tr, &ti);
      nr = 2 + xr + tr; ni = xi + ti;
      br += (nr * z3r + ni * z3i) / den3; bi += (ni * z3r - nr * z3i) / den3;
      // gamma: (-4 - 3z - z^2 + e^z (4 - z)) / z^3
      mul(ezr, ezi, 4 - xr, -xi, &tr, &ti);
      nr = -4 - 3 * xr - z2r + tr; ni = -3 * xi - z2i + ti;
      gr += (nr * z3r + ni * z3i) / den3; gi += (ni * z3r - nr * z3i) / den3;
    }
    const double sc = dt / ncirc;
    double s_, c_;
    sincos(dt * li, &s_, &c_);
    const double ea = exp(dt * lr);
    sincos(0.5 * dt * li, &s_, &c_);
    double s2, c2;
    sincos(dt * li, &s2, &c2);
    const double er = ea * c2, ei = ea * s2;
    const double eh = exp(0.5 * dt * lr);
    const double e2r = eh * c_, e2i = eh * s_;
    const int kr = idx % nkr, j = idx / nkr;
    const size_t o = (size_t)j * ldk + kr;
    const double vals[12] = {er, ei, e2r, e2i, zr * sc, zi * sc, ar * sc, ai * sc, br * sc, bi * sc, gr * sc, gi * sc};
    T* outs[6] = {e, e2, zeta, alpha, beta, gamma};
    for (int q = 0; q < 6; ++q) {
      if (cplx_out) { outs[q][2 * o] = (T)vals[2 * q]; outs[q][2 * o + 1] = (T)vals[2 * q + 1]; }
      else outs[q][o] = (T)vals[2 * q];
    }
  }
}

__global__ void diag_finish(const double* __restrict__ partial, int nblocks, uint32_t mask, double* out) {
  __shared__ double red[256];
  const int nb = gridDim.x, ib = blockIdx.x;  // one block per ensemble instance
  for (int q = 0; q < NDIAG; ++q) {
    if (!(mask & (1u << q))) { if (threadIdx.x == 0) out[(size_t)q * nb + ib] = 0; continue; }
    double s = 0, c = 0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
      const double x = partial[((size_t)q * nb + ib) * nblocks + b];
      const double t = s + x;
      c += (fabs(s) >= fabs(x)) ? (s - t) + x : (x - t) + s;
      s = t;
    }
    red[threadIdx.x] = s + c;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
      if ((int)threadIdx.x < st) red[threadIdx.x] += red[threadIdx.x + st];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[(size_t)q * nb + ib] = red[0];
    __syncthreads();
  }
}

// clock advance after a step, and the harmonic forcing scales of the next step's stages
__global__ void advance_clock_kernel(DevClock* clk, double dt, double omega, double phase, int harmonic, int nst) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  clk->t += dt;
  clk->step += 1;
  if (harmonic) {
    for (int k = 0; k < 4; ++k) {
      const double off = (nst == 4) ? (k == 0 ? 0.0 : k == 3 ? 1.0 : 0.5) : 0.0;
      const double v = cos(omega * (clk->t + off * dt) + phase);
      clk->fs[k] = v;
      clk->fs_f[k] = (float)v;
      clk->fs_l[k] = (float)(v - (double)clk->fs_f[k]);
    }
  }
}

template <class T>
__global__ void add_scalar_kernel(T* a, size_t n, double v) {
  const T tv = T(v);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    a[i] = a[i] + tv;
}

// `rows` rows of `w` 8-byte words from one row stride to another (in words): the pitch
// conversion between a contiguous host-transfer staging buffer and the padded layout
__global__ void repack_kernel(const uint64_t* __restrict__ src, size_t ss, uint64_t* __restrict__ dst, size_t ds,
                              size_t rows, size_t w) {
  const size_t n = rows * w;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const size_t r = e / w, k = e - r * w;
    dst[r * ds + k] = src[r * ss + k];
  }
}

// double <-> df64 copies of `rows` rows of `w` reals with their own row strides (in reals)
__global__ void to_df64_kernel(const double* __restrict__ src, size_t ss, df64* __restrict__ dst, size_t ds,
                               size_t rows, size_t w) {
  const size_t n = rows * w;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const size_t r = e / w, k = e - r * w;
    const double d = src[r * ss + k];
    const float h = (float)d;
    dst[r * ds + k] = df64(h, (float)(d - (double)h));
  }
}
__global__ void from_df64_kernel(const df64* __restrict__ src, size_t ss, double* __restrict__ dst, size_t ds,
                                 size_t rows, size_t w) {
  const size_t n = rows * w;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const size_t r = e / w, k = e - r * w;
    dst[r * ds + k] = to_double(src[r * ss + k]);
  }
}

// ------------------------------------------------------------------------------- helpers
#define GF_CUDA(ctx, call)                                                           \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess) {                                                         \
      (ctx)->err = std::string(#call) + ": " + cudaGetErrorString(e_);              \
      return GF_ERR_CUDA;                                                            \
    }                                                                                \
  } while (0)

// A pending non-sticky error of an earlier runtime call in the caller's thread (the caller's
// own, or another library's -- a refused cudaHostRegister, say) would be read back by this
// library's launch checks (cudaGetLastError after a launch) as if one of its launches had
// failed; every entry point that launches work consumes it first.  Sticky errors (a lost
// context) still surface through the calls that follow.
static inline void clear_stale_error() { (void)cudaGetLastError(); }

// A context's buffers, stream and graphs live on the device that was current at gf_create.
// Each entry point that works on a context makes that device current for the call and puts
// the caller's current device back when it returns, so a caller that switched devices (a
// CUDA.jl task on another GPU, say) does not launch this context's kernels on the wrong one.
struct DevGuard {
  int prev = -1;
  explicit DevGuard(int dev) {
    int cur = -1;
    if (cudaGetDevice(&cur) == cudaSuccess && cur != dev && cudaSetDevice(dev) == cudaSuccess) prev = cur;
  }
  ~DevGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
  DevGuard(const DevGuard&) = delete;
  DevGuard& operator=(const DevGuard&) = delete;
};

static int fail(gf_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg; else g_create_error = msg;
  return code;
}

static void* dalloc(gf_ctx* c, size_t bytes) {
  void* p = nullptr;
  if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
  cudaMemsetAsync(p, 0, bytes, c->stream);
  c->allocs.push_back(p);
  return p;
}

static bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

// FFT lengths with compiled-in kernels; every other even length runs the generic-length path
static bool fixed_length(int n) { return is_pow2(n) && n >= 32 && n <= 2048; }

// Radix plan of a generic length n (product of the radices = n): 16s, then 8, 4, 2 for the
// power of two, then the odd primes in increasing order.  False if a prime factor exceeds
// MAXPRIME or the plan has more than MAXP passes.
static bool radix_plan(int n, int* plan, int* np) {
  *np = 0;
  auto push = [&](int r) {
    if (*np >= MAXP) return false;
    plan[(*np)++] = r;
    return true;
  };
  while (n % 16 == 0) { if (!push(16)) return false; n /= 16; }
  for (int r : {8, 4, 2})
    if (n % r == 0) { if (!push(r)) return false; n /= r; }
  for (int p = 3; p <= MAXPRIME && n > 1; p += 2)
    while (n % p == 0) { if (!push(p)) return false; n /= p; }
  return n == 1;
}

// Largest generic length: five shared buffers of the length per column block.
static int max_generic_length(int precision) { return precision == GF_F32 ? 4096 : 2048; }

static size_t nspec(const gf_ctx* c) { return (size_t)c->g.nl * c->g.ny * c->g.ldk; }

// upload a host double array of n values as the context's real type
static int upload_real(gf_ctx* c, void* dst, const double* src, size_t n) {
  if (c->prec == GF_F64) {
    GF_CUDA(c, cudaMemcpyAsync(dst, src, n * 8, cudaMemcpyHostToDevice, c->stream));
  } else if (c->prec == GF_DF64) {
    std::vector<float> f(2 * n);
    for (size_t i = 0; i < n; ++i) split_hl(src[i], &f[2 * i], &f[2 * i + 1]);
    GF_CUDA(c, cudaMemcpyAsync(dst, f.data(), n * 8, cudaMemcpyHostToDevice, c->stream));
    GF_CUDA(c, cudaStreamSynchronize(c->stream));
  } else {
    std::vector<float> f(n);
    for (size_t i = 0; i < n; ++i) f[i] = (float)src[i];
    GF_CUDA(c, cudaMemcpyAsync(dst, f.data(), n * 4, cudaMemcpyHostToDevice, c->stream));
    GF_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  return GF_OK;
}
// upload a host double table defined on [j][kr] (nkr x ny) into [j][ldk]
static int upload_table(gf_ctx* c, void* dst, const std::vector<double>& v, int cplx) {
  const Geom& g = c->g;
  const int w = cplx ? 2 : 1;
  std::vector<double> pad((size_t)g.ny * g.ldk * w, 0.0);
  for (int j = 0; j < g.ny; ++j)
    for (int k = 0; k < g.nkr * w; ++k) pad[(size_t)j * g.ldk * w + k] = v[((size_t)j * g.nkr) * w + k];
  int r = upload_real(c, dst, pad.data(), pad.size());
  if (r) return r;
  GF_CUDA(c, cudaStreamSynchronize(c->stream));
  return GF_OK;
}

static Bufs bufs(gf_ctx* c) { return Bufs{c->twid, c->W, c->P, c->row_phys, &c->tma, c->derr, c->twx, c->twy}; }
static Geom full_geom(const gf_ctx* c) {
  Geom g = c->g;
  g.kcut = g.nkr; g.lA = 1; g.lB = 0; g.ldw = g.ldk;
  return g;
}

// host copy of the device clock for the step starting at c->t (stage forcing scales)
static int upload_clock(gf_ctx* c) {
  DevClock h{};
  h.t = c->t;
  h.step = c->step;
  for (int k = 0; k < 4; ++k) {
    const double off = (c->nstages == 4) ? (k == 0 ? 0.0 : k == 3 ? 1.0 : 0.5) : 0.0;
    h.fs[k] = c->cfg.forcing_kind == GF_FORCING_HARMONIC
                  ? std::cos(c->cfg.forcing_omega * (c->t + off * c->cfg.dt) + c->cfg.forcing_phase)
                  : 1.0;
    split_hl(h.fs[k], &h.fs_f[k], &h.fs_l[k]);
  }
  GF_CUDA(c, cudaMemcpyAsync(c->dclk, &h, sizeof(h), cudaMemcpyHostToDevice, c->stream));
  GF_CUDA(c, cudaStreamSynchronize(c->stream));
  return GF_OK;
}

#define DISPATCH(c, fn, ...)                                      \
  ((c)->prec == GF_F64 ? fn<double>(__VA_ARGS__)                  \
                       : (c)->prec == GF_DF64 ? fn<df64>(__VA_ARGS__) : fn<float>(__VA_ARGS__))

// symmetric Jacobi eigen-decomposition (small n), A overwritten, Q columns = eigenvectors
static void jacobi_eig(int n, std::vector<double>& A, std::vector<double>& Q, std::vector<double>& lam) {
  Q.assign(n * n, 0.0);
  for (int i = 0; i < n; ++i) Q[i * n + i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0;
    for (int p = 0; p < n; ++p) for (int q = p + 1; q < n; ++q) off += A[p * n + q] * A[p * n + q];
    if (off < 1e-30) break;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = A[p * n + q];
        if (std::fabs(apq) < 1e-300) continue;
        const double th = (A[q * n + q] - A[p * n + p]) / (2 * apq);
        const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1));
        const double cs = 1 / std::sqrt(t * t + 1), sn = t * cs;
        for (int k = 0; k < n; ++k) {  // A = J^T A J
          const double akp = A[k * n + p], akq = A[k * n + q];
          A[k * n + p] = cs * akp - sn * akq;
          A[k * n + q] = sn * akp + cs * akq;
        }
        for (int k = 0; k < n; ++k) {
          const double apk = A[p * n + k], aqk = A[q * n + k];
          A[p * n + k] = cs * apk - sn * aqk;
          A[q * n + k] = sn * apk + cs * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double qkp = Q[k * n + p], qkq = Q[k * n + q];
          Q[k * n + p] = cs * qkp - sn * qkq;
          Q[k * n + q] = sn * qkp + cs * qkq;
        }
      }
  }
  lam.resize(n);
  for (int i = 0; i < n; ++i) lam[i] = A[i * n + i];
}

// second y-derivative of a periodic 1-D profile by an exact DFT (setup only)
static std::vector<double> d2dy2(const std::vector<double>& u, double Ly) {
  const int n = (int)u.size();
  std::vector<std::complex<double>> uh(n);
  for (int k = 0; k < n; ++k) {
    std::complex<double> s = 0;
    for (int j = 0; j < n; ++j) s += u[j] * std::polar(1.0, -2 * M_PI * (double)((long long)k * j % n) / n);
    const double l = 2 * M_PI / Ly * (k < n / 2 ? k : k - n);
    uh[k] = -l * l * s;
  }
  std::vector<double> r(n);
  for (int j = 0; j < n; ++j) {
    std::complex<double> s = 0;
    for (int k = 0; k < n; ++k) s += uh[k] * std::polar(1.0, 2 * M_PI * (double)((long long)k * j % n) / n);
    r[j] = s.real() / n;
  }
  return r;
}

static double powi_h(double x, int n) {
  if (n == 0) return 1.0;
  double r = 1.0, b = n > 0 ? x : 1.0 / x;
  for (int e = n > 0 ? n : -n; e; e >>= 1) { if (e & 1) r *= b; b *= b; }
  return r;
}

// forward transform of nl physical fields (device, context type) into out (internal layout)
static int fwd_transform(gf_ctx* c, const void* phys_dev, void* out, int zero_mean) {
  Geom g = full_geom(c);
  GF_CUDA(c, DISPATCH(c, launch_row_r2c, g, bufs(c), g.nl, phys_dev, c->stream));
  GF_CUDA(c, DISPATCH(c, launch_col_fwd, g, bufs(c), g.nl, out, zero_mean, c->stream));
  return GF_OK;
}
// inverse transform of kind(src) for all layers into physical out[nl][ny][nx]
static int inv_transform(gf_ctx* c, const void* src, int kind, int mask, void* out) {
  Geom g = full_geom(c);
  GF_CUDA(c, DISPATCH(c, launch_col_inv, g, c->m, src, kind, mask, bufs(c), c->stream));
  GF_CUDA(c, DISPATCH(c, launch_row_c2r, g, bufs(c), g.nl, out, c->stream));
  return GF_OK;
}

// ------------------------------------------------------------------------------- create
extern "C" int gf_abi_version(void) { return GFCUDA_ABI_VERSION; }

extern "C" const char* gf_last_error(const gf_ctx* c) { return c ? c->err.c_str() : g_create_error.c_str(); }

// cuTensorMapEncodeTiled from the driver (through the runtime's entry-point query, so the
// library links libcudart only); null if the driver does not provide it.
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
// A driver entry point by name, resolved once per process (the static's initialisation is
// thread-safe); null if the driver does not provide it.
static void* driver_entry(const char* name) {
  void* p = nullptr;
  cudaDriverEntryPointQueryResult q{};
  if (cudaGetDriverEntryPointByVersion(name, &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return p;
}
static EncodeTiledFn encode_tiled() {
  static const EncodeTiledFn fn = reinterpret_cast<EncodeTiledFn>(driver_entry("cuTensorMapEncodeTiled"));
  return fn;
}

// Device address of the caller's host buffer [p, p + bytes) when the whole range lies in one
// page-locked allocation that the current device addresses (cudaMallocHost, cudaHostAlloc,
// cudaHostRegister): both ends are page-locked host memory with device addresses bytes - 1
// apart, and the driver reports one buffer id for both (one allocation, hence contiguous).
// The host transfers then run as one kernel pass that reads or writes the buffer over the
// host link and re-pitches on the way, instead of a copy-engine transfer through the staging
// buffer followed by a device pass.  The driver must also report that the device may read the
// range, and with write (the kernel stores into it) read and write it: a
// cudaHostRegisterReadOnly range is only read directly.  Null for pageable memory, or when any
// check cannot be made: the staged path is used.
typedef CUresult (*PtrAttrFn)(void*, CUpointer_attribute, CUdeviceptr);
static PtrAttrFn ptr_attr_fn() {
  static const PtrAttrFn fn = reinterpret_cast<PtrAttrFn>(driver_entry("cuPointerGetAttribute"));
  return fn;
}
static void* host_mapped(const void* p, size_t bytes, bool write) {
  const PtrAttrFn fn = ptr_attr_fn();
  if (!fn || !p || bytes == 0) return nullptr;
  const char* a = static_cast<const char*>(p);
  const char* z = a + (bytes - 1);
  cudaPointerAttributes pa{}, pz{};
  if (cudaPointerGetAttributes(&pa, a) != cudaSuccess || cudaPointerGetAttributes(&pz, z) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (pa.type != cudaMemoryTypeHost || pz.type != cudaMemoryTypeHost || !pa.devicePointer || !pz.devicePointer)
    return nullptr;
  if (static_cast<const char*>(pz.devicePointer) - static_cast<const char*>(pa.devicePointer) != (ptrdiff_t)(bytes - 1))
    return nullptr;
  unsigned long long ia = 0, iz = 0;
  if (fn(&ia, CU_POINTER_ATTRIBUTE_BUFFER_ID, (CUdeviceptr)(uintptr_t)a) != CUDA_SUCCESS ||
      fn(&iz, CU_POINTER_ATTRIBUTE_BUFFER_ID, (CUdeviceptr)(uintptr_t)z) != CUDA_SUCCESS || ia != iz)
    return nullptr;
  unsigned int acc = 0;  // the device's access to the range: read for gf_set_state, read-write for gf_get_state
  if (fn(&acc, CU_POINTER_ATTRIBUTE_ACCESS_FLAGS, (CUdeviceptr)(uintptr_t)a) != CUDA_SUCCESS ||
      (write ? acc != CU_POINTER_ATTRIBUTE_ACCESS_FLAG_READWRITE : !(acc & CU_POINTER_ATTRIBUTE_ACCESS_FLAG_READ)))
    return nullptr;
  return pa.devicePointer;
}

// Tensor maps of the TMA column stage (one layer): P and W as 3-D arrays of 32-bit words
// (x: the words of a row's complex elements; y: field * ny + j; z: instance), boxes of C
// columns x min(ny, 256) rows for the two candidate column counts (2 and 4 columns of
// 8-byte elements, 1 and 2 of 16-byte ones: box rows of 16 or 32 bytes).  P's rows span the
// padded width ldk (loads of columns past nkr read padding the kernel ignores); W's rows are
// clipped at kcut, so tile stores drop the aliased columns.  Leaves c->tma.ok false if the
// driver cannot encode them (the cp.async column kernel is used then).
static void tma_maps(gf_ctx* c) {
  const EncodeTiledFn fn = encode_tiled();
  c->tma.ok = false;
  if (!fn) return;
  const Geom& g = c->g;
  const cuuint32_t wpc = (cuuint32_t)(c->cb / 4);
  const cuuint32_t rows = (cuuint32_t)std::min(g.ny, 256);
  const cuuint64_t dP[3] = {(cuuint64_t)g.ldk * wpc, (cuuint64_t)3 * g.ny, (cuuint64_t)g.nb};
  const cuuint64_t sP[2] = {(cuuint64_t)g.ldk * c->cb, (cuuint64_t)g.bs_p * c->cb};
  const cuuint64_t dW[3] = {(cuuint64_t)g.kcut * wpc, (cuuint64_t)3 * g.ny, (cuuint64_t)g.nb};
  const cuuint64_t sW[2] = {(cuuint64_t)g.ldw * c->cb, (cuuint64_t)g.bs_w * c->cb};
  const cuuint32_t es[3] = {1, 1, 1};
  for (int i = 0; i < 2; ++i) {
    const int C = (c->cb == 8 ? 2 : 1) << i;
    c->tma.Cs[i] = C;
    const cuuint32_t box[3] = {(cuuint32_t)C * wpc, rows, 1};
    if (fn(reinterpret_cast<CUtensorMap*>(c->tma.p[i]), CU_TENSOR_MAP_DATA_TYPE_UINT32, 3, c->P, dP, sP, box, es,
           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return;
    if (fn(reinterpret_cast<CUtensorMap*>(c->tma.w[i]), CU_TENSOR_MAP_DATA_TYPE_UINT32, 3, c->W, dW, sW, box, es,
           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return;
  }
  c->tma.ok = true;
}

static bool fp_ctx_ok(const gf_ctx* c);
static void set_fp(gf_ctx* c, int Rr, int Rc, int C);

static int build(gf_ctx* c, const gf_config* cfg) {
  const gf_config& k = *cfg;
  Geom& g = c->g;
  g.nx = k.nx; g.ny = k.ny; g.nkr = k.nx / 2 + 1;
  g.nl = (k.module == GF_MULTILAYERQG) ? k.nlayers : 1;
  g.ldk = (g.nkr + 15) / 16 * 16;
  // dealias ranges (FourierFlows TwoDGrid with aliased_fraction)
  const double af = k.aliased_fraction;
  if (af > 0) {
    const double L = (1 - af) / 2, R = (1 + af) / 2;
    const int iLx = (int)std::floor(L * k.nx) + 1;
    const int iLy = (int)std::floor(L * k.ny) + 1, iRy = (int)std::ceil(R * k.ny);
    g.kcut = std::min(iLx - 1, g.nkr);
    g.lA = iLy - 1; g.lB = iRy - 1;
  } else {
    g.kcut = g.nkr; g.lA = 1; g.lB = 0;
  }
  g.ldw = (g.kcut + 15) / 16 * 16;
  g.dkx = 2 * M_PI / k.Lx; g.dky = 2 * M_PI / k.Ly;
  g.inv_nxny = 1.0 / ((double)k.nx * k.ny);
  split_hl(g.dkx, &g.dkx_f, &g.dkx_l);
  split_hl(g.dky, &g.dky_f, &g.dky_l);
  split_hl(g.inv_nxny, &g.inv_nxny_f, &g.inv_nxny_l);
  c->prec = k.precision;
  c->rb = k.precision == GF_F32 ? 4 : 8;
  c->cb = 2 * c->rb;
  const int st = k.stepper;
  c->filtered = (st == GF_FILTEREDFORWARDEULER || st == GF_FILTEREDRK4 || st == GF_FILTEREDETDRK4 || st == GF_FILTEREDAB3);
  c->kind = (st <= 1) ? SK_FE : (st <= 3) ? SK_RK4 : (st <= 5) ? SK_ETDRK4 : SK_AB3;
  c->nstages = (c->kind == SK_RK4 || c->kind == SK_ETDRK4) ? 4 : 1;

  const size_t nsp = nspec(c), tsz = (size_t)g.ny * g.ldk;
  const size_t cb = c->cb, rb = c->rb;
  g.nb = k.batch > 1 ? k.batch : 1;
  const size_t NB = g.nb;
  // ----- twiddles
  {
    std::vector<double> tw(2 * TWN);
    for (int i = 0; i < TWN; ++i) {
      tw[2 * i] = std::cos(2 * M_PI * i / TWN);
      tw[2 * i + 1] = -std::sin(2 * M_PI * i / TWN);
    }
    if (!(c->twid = dalloc(c, 2 * TWN * rb))) return fail(c, GF_ERR_NOMEM, "twiddles");
    if (int r = upload_real(c, c->twid, tw.data(), tw.size())) return r;
  }
  // ----- generic-length transforms: radix plans and exp(-2 pi i k / n) tables
  g.rtx = !fixed_length(k.nx);
  g.rty = !fixed_length(k.ny);
  if (g.rtx && !radix_plan(k.nx, g.plx, &g.npx)) return fail(c, GF_ERR_UNSUPPORTED, "nx has no radix plan");
  if (g.rty && !radix_plan(k.ny, g.ply, &g.npy)) return fail(c, GF_ERR_UNSUPPORTED, "ny has no radix plan");
  for (int d = 0; d < 2; ++d) {
    const int n = d == 0 ? k.nx : k.ny;
    if (!(d == 0 ? g.rtx : g.rty)) continue;
    std::vector<double> tw(2 * (size_t)n);
    for (int i = 0; i < n; ++i) {
      tw[2 * i] = std::cos(2 * M_PI * i / n);
      tw[2 * i + 1] = -std::sin(2 * M_PI * i / n);
    }
    void*& dst = d == 0 ? c->twx : c->twy;
    if (!(dst = dalloc(c, 2 * (size_t)n * rb))) return fail(c, GF_ERR_NOMEM, "twiddles");
    if (int r = upload_real(c, dst, tw.data(), tw.size())) return r;
  }
  // ----- wavenumber tables on the host (double)
  std::vector<double> K2((size_t)g.ny * g.nkr), krv(g.nkr), lv(g.ny);
  for (int i = 0; i < g.nkr; ++i) krv[i] = g.dkx * i;
  for (int j = 0; j < g.ny; ++j) lv[j] = g.dky * (j < g.ny / 2 ? j : j - g.ny);
  for (int j = 0; j < g.ny; ++j)
    for (int i = 0; i < g.nkr; ++i) K2[(size_t)j * g.nkr + i] = krv[i] * krv[i] + lv[j] * lv[j];

  // ----- module parameters and the linear operator L (real or complex)
  ModArgs& m = c->m;
  std::memset(&m, 0, sizeof(m));
  m.module = k.module;
  m.hasB = 1;
  m.nu = k.nu; m.nnu = k.nnu; m.mu_visc = k.mu; m.nmu = k.nmu;
  std::vector<double> Lre((size_t)g.ny * g.nkr, 0.0), Lim;
  auto K2pow = [&](size_t e, int n) { return powi_h(K2[e], n); };
  const size_t nt = (size_t)g.ny * g.nkr;
  if (k.module == GF_TWODNAVIERSTOKES) {
    m.psi_kind = PSI_INVK2;
    for (size_t e = 1; e < nt; ++e) Lre[e] = -k.nu * K2pow(e, k.nnu) - k.mu * K2pow(e, k.nmu);
  } else if (k.module == GF_SURFACEQG) {
    m.psi_kind = PSI_TABLE;
    const double H = (k.H_sqg > 0) ? k.H_sqg : INFINITY;
    std::vector<double> M(nt, 0.0);
    for (size_t e = 1; e < nt; ++e) {
      const double Kk = std::sqrt(K2[e]);
      M[e] = (std::isinf(H) ? 1.0 : 1.0 / std::tanh(H * Kk)) / Kk;
      Lre[e] = -k.nu * K2pow(e, k.nnu);
    }
    if (!(c->mult = dalloc(c, tsz * rb))) return fail(c, GF_ERR_NOMEM, "mult");
    if (int r = upload_table(c, c->mult, M, 0)) return r;
    m.mult = c->mult;
  } else if (k.module == GF_BAROTROPICQGQL) {
    // L = -mu - nu K^(2 nnu) + i beta kr / K^2 (src/barotropicqgql.jl:168-173)
    m.psi_kind = PSI_INVK2;
    m.hasC = 1;
    m.ql = 1;
    m.nmu = 0;
    Lim.assign(nt, 0.0);
    for (size_t e = 1; e < nt; ++e) {
      Lre[e] = -k.mu - k.nu * K2pow(e, k.nnu);
      Lim[e] = k.beta * krv[e % g.nkr] / K2[e];
    }
  } else if (k.module == GF_SINGLELAYERQG) {
    const bool barotropic = !(k.deformation_radius > 0) || std::isinf(k.deformation_radius);
    m.psi_kind = barotropic ? PSI_INVK2 : PSI_HELMHOLTZ;
    m.ell_inv2 = barotropic ? 0.0 : 1.0 / (k.deformation_radius * k.deformation_radius);
    Lim.assign(nt, 0.0);
    const bool Uconst = (k.U_y == nullptr);
    for (size_t e = 1; e < nt; ++e) {
      const int kr = e % g.nkr;
      Lre[e] = -k.mu - k.nu * K2pow(e, k.nnu);
      Lim[e] = barotropic ? k.beta * krv[kr] / K2[e] : k.beta * krv[kr] / (K2[e] + m.ell_inv2);
      if (Uconst) Lim[e] -= k.U * krv[kr];
    }
    m.U0 = Uconst ? k.U : 0.0;
  } else {  // MultiLayerQG
    const int n = g.nl;
    for (size_t e = 1; e < nt; ++e) Lre[e] = -k.nu * K2pow(e, k.nnu);
    m.hasB = k.linear ? 0 : 1;
    m.hasC = 1;
    m.linear = k.linear;
    m.drag = (k.mu != 0);
    m.mu = k.mu;
    c->f0 = k.f0;
    c->Hl.assign(k.H, k.H + n);
    c->Hsum = 0;
    for (int j = 0; j < n; ++j) c->Hsum += k.H[j];
    std::vector<double> Fp(n > 1 ? n - 1 : 0), Fm(n > 1 ? n - 1 : 0);
    if (n == 1) {
      m.psi_kind = PSI_INVK2;
    } else {
      m.psi_kind = PSI_EIGEN;
      c->gprime.resize(n - 1);
      for (int j = 0; j < n - 1; ++j) {
        c->gprime[j] = k.b[j] - k.b[j + 1];
        Fm[j] = k.f0 * k.f0 / (c->gprime[j] * k.H[j + 1]);
        Fp[j] = k.f0 * k.f0 / (c->gprime[j] * k.H[j]);
      }
      std::vector<double> F(n * n, 0.0);
      for (int j = 0; j < n - 1; ++j) { F[j * n + j + 1] = Fp[j]; F[(j + 1) * n + j] = Fm[j]; }
      for (int j = 0; j < n; ++j) F[j * n + j] = -((j < n - 1 ? Fp[j] : 0) + (j > 0 ? Fm[j - 1] : 0));
      // diag(sqrt H) F diag(1/sqrt H) is symmetric: F = D^-1 Q Lam Q^T D
      std::vector<double> A(n * n), Q, lam;
      for (int a = 0; a < n; ++a)
        for (int b = 0; b < n; ++b) A[a * n + b] = std::sqrt(k.H[a]) * F[a * n + b] / std::sqrt(k.H[b]);
      for (int a = 0; a < n; ++a)
        for (int b = a + 1; b < n; ++b) { const double s = 0.5 * (A[a * n + b] + A[b * n + a]); A[a * n + b] = A[b * n + a] = s; }
      jacobi_eig(n, A, Q, lam);
      for (int a = 0; a < n; ++a) {
        m.lam[a] = lam[a];
        for (int b = 0; b < n; ++b) {
          m.V[a * MAXL + b] = Q[a * n + b] / std::sqrt(k.H[a]);      // D^-1 Q
          m.Vinv[a * MAXL + b] = Q[b * n + a] * std::sqrt(k.H[b]);   // Q^T D
        }
      }
    }
    // U(y) per layer, Qy1D = beta - Uyy - (F dU terms)
    std::vector<double> U((size_t)n * g.ny, 0.0), Qy((size_t)n * g.ny, 0.0);
    if (k.U_y) for (size_t i = 0; i < U.size(); ++i) U[i] = k.U_y[i];
    for (int L = 0; L < n; ++L) {
      std::vector<double> u(U.begin() + (size_t)L * g.ny, U.begin() + (size_t)(L + 1) * g.ny);
      auto uyy = d2dy2(u, k.Ly);
      for (int j = 0; j < g.ny; ++j) Qy[(size_t)L * g.ny + j] = k.beta - uyy[j];
    }
    if (n >= 2) {
      for (int j = 0; j < g.ny; ++j) {
        auto Uv = [&](int L) { return U[(size_t)L * g.ny + j]; };
        Qy[j] -= Fp[0] * (Uv(1) - Uv(0));
        for (int L = 1; L < n - 1; ++L) Qy[(size_t)L * g.ny + j] -= Fp[L] * (Uv(L + 1) - Uv(L)) + Fm[L - 1] * (Uv(L - 1) - Uv(L));
        Qy[(size_t)(n - 1) * g.ny + j] -= Fm[n - 2] * (Uv(n - 2) - Uv(n - 1));
      }
    }
    if (!(c->U1D = dalloc(c, U.size() * rb)) || !(c->Qy1D = dalloc(c, Qy.size() * rb))) return fail(c, GF_ERR_NOMEM, "U");
    if (int r = upload_real(c, c->U1D, U.data(), U.size())) return r;
    if (int r = upload_real(c, c->Qy1D, Qy.data(), Qy.size())) return r;
    if (k.module == GF_MULTILAYERQG) {
      if (!(c->Ud = (double*)dalloc(c, U.size() * 8))) return fail(c, GF_ERR_NOMEM, "U");
      GF_CUDA(c, cudaMemcpyAsync(c->Ud, U.data(), U.size() * 8, cudaMemcpyHostToDevice, c->stream));
      GF_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    m.U1D = c->U1D; m.Qy1D = c->Qy1D;
  }
  c->hasL = 0;
  for (size_t e = 0; e < nt; ++e) if (Lre[e] != 0 || (!Lim.empty() && Lim[e] != 0)) { c->hasL = 1; break; }
  c->cplxL = !Lim.empty();

  // ----- buffers
  const size_t Wn = std::max((size_t)3 * g.nl * g.ny * g.ldw, nsp);
  g.bs_spec = nsp; g.bs_w = Wn; g.bs_p = 3 * nsp; g.bs_d = tsz; g.bs_phys = (size_t)g.nl * g.ny * g.nx;
  if (!(c->sol = dalloc(c, NB * nsp * cb)) || !(c->W = dalloc(c, NB * Wn * cb)) ||
      !(c->P = dalloc(c, NB * 3 * nsp * cb)) || !(c->D = dalloc(c, NB * tsz * cb)) ||
      !(c->tmp_spec = dalloc(c, NB * nsp * cb)) || !(c->tmp_spec2 = dalloc(c, NB * nsp * cb)) ||
      !(c->phys = dalloc(c, NB * (k.module == GF_BAROTROPICQGQL ? 7 : 4) * g.bs_phys * rb)) || !(c->dclk = (DevClock*)dalloc(c, sizeof(DevClock))))
    return fail(c, GF_ERR_NOMEM, "state buffers");
  m.D = c->D;
  if (!(c->stage = dalloc(c, NB * std::max(nsp * cb, g.bs_phys * rb))))  // host-transfer staging
    return fail(c, GF_ERR_NOMEM, "staging");
  if (g.nl > 1 && !(c->Xg = dalloc(c, NB * nsp * cb))) return fail(c, GF_ERR_NOMEM, "layer X");
  if (!(c->derr = (int*)dalloc(c, sizeof(int)))) return fail(c, GF_ERR_NOMEM, "error flag");
  GF_CUDA(c, cudaMemsetAsync(c->derr, 0, sizeof(int), c->stream));
  if (g.nl == 1) tma_maps(c);
  // grids whose row pairs (of all instances) do not cover the SMs: the field-parallel kernels
  if (fp_ctx_ok(c) && (size_t)NB * (g.ny / 2) < (size_t)num_sms()) 
    set_fp(c, fp_default_row_radix(g.nx), fp_default_col_radix(g.ny), 1);
  if (c->kind == SK_RK4) {
    if (!(c->acc = dalloc(c, NB * nsp * cb))) return fail(c, GF_ERR_NOMEM, "acc");
    if (c->hasL && !(c->X = dalloc(c, NB * nsp * cb))) return fail(c, GF_ERR_NOMEM, "X");
  } else if (c->kind == SK_ETDRK4) {
    if (!(c->acc = dalloc(c, NB * nsp * cb)) || !(c->s1 = dalloc(c, NB * nsp * cb)) ||
        !(c->N1 = dalloc(c, NB * nsp * cb)))
      return fail(c, GF_ERR_NOMEM, "etdrk4 state");
  } else if (c->kind == SK_AB3) {
    for (int i = 0; i < 3; ++i) if (!(c->R3[i] = dalloc(c, NB * nsp * cb))) return fail(c, GF_ERR_NOMEM, "ab3 state");
  }
  // ----- L, filter, ETDRK4 coefficients
  const int w = c->cplxL ? 2 : 1;
  if (c->hasL && c->kind != SK_ETDRK4) {
    std::vector<double> Lt(nt * w);
    for (size_t e = 0; e < nt; ++e) {
      if (c->cplxL) { Lt[2 * e] = Lre[e]; Lt[2 * e + 1] = Lim[e]; } else Lt[e] = Lre[e];
    }
    if (!(c->Ltab = dalloc(c, tsz * w * rb))) return fail(c, GF_ERR_NOMEM, "L");
    if (int r = upload_table(c, c->Ltab, Lt, c->cplxL)) return r;
  }
  if (c->filtered) {
    const double order = k.filter_order > 0 ? k.filter_order : 4.0;
    const double inner = k.filter_innerK > 0 ? k.filter_innerK : 0.65;
    const double outer = k.filter_outerK > 0 ? k.filter_outerK : 1.0;
    const double decay = 15 * std::log(10.0) / std::pow(outer - inner, order);
    const double dx = k.Lx / k.nx, dy = k.Ly / k.ny;
    std::vector<double> f(nt);
    for (int j = 0; j < g.ny; ++j)
      for (int i = 0; i < g.nkr; ++i) {
        const double a = krv[i] * dx / M_PI, b = lv[j] * dy / M_PI;
        const double Kf = std::sqrt(a * a + b * b);
        f[(size_t)j * g.nkr + i] = Kf < inner ? 1.0 : std::exp(-decay * std::pow(Kf - inner, order));
      }
    if (!(c->filt = dalloc(c, tsz * rb))) return fail(c, GF_ERR_NOMEM, "filter");
    if (int r = upload_table(c, c->filt, f, 0)) return r;
    c->filt_host = f;
  }
  if (c->kind == SK_ETDRK4) {
    for (int q = 0; q < 6; ++q) if (!(c->etd[q] = dalloc(c, tsz * w * rb))) return fail(c, GF_ERR_NOMEM, "etdrk4 coefficients");
    double *dLr = nullptr, *dLi = nullptr;
    GF_CUDA(c, cudaMalloc(&dLr, nt * 8));
    if (c->cplxL) GF_CUDA(c, cudaMalloc(&dLi, nt * 8));
    GF_CUDA(c, cudaMemcpyAsync(dLr, Lre.data(), nt * 8, cudaMemcpyHostToDevice, c->stream));
    if (dLi) GF_CUDA(c, cudaMemcpyAsync(dLi, Lim.data(), nt * 8, cudaMemcpyHostToDevice, c->stream));
    const int ncirc = k.etdrk4_ncirc > 0 ? k.etdrk4_ncirc : 32;
    const double rcirc = k.etdrk4_rcirc > 0 ? k.etdrk4_rcirc : 1.0;
    const int nb = (int)std::min<size_t>((nt + 255) / 256, 4096);
    if (c->prec == GF_F64)
      etd_coeffs_kernel<double><<<nb, 256, 0, c->stream>>>((int)nt, dLr, dLi, k.dt, ncirc, rcirc, c->cplxL,
          (double*)c->etd[0], (double*)c->etd[1], (double*)c->etd[2], (double*)c->etd[3], (double*)c->etd[4],
          (double*)c->etd[5], g.nkr, g.ldk);
    else if (c->prec == GF_DF64)
      etd_coeffs_kernel<df64><<<nb, 256, 0, c->stream>>>((int)nt, dLr, dLi, k.dt, ncirc, rcirc, c->cplxL,
          (df64*)c->etd[0], (df64*)c->etd[1], (df64*)c->etd[2], (df64*)c->etd[3], (df64*)c->etd[4],
          (df64*)c->etd[5], g.nkr, g.ldk);
    else
      etd_coeffs_kernel<float><<<nb, 256, 0, c->stream>>>((int)nt, dLr, dLi, k.dt, ncirc, rcirc, c->cplxL,
          (float*)c->etd[0], (float*)c->etd[1], (float*)c->etd[2], (float*)c->etd[3], (float*)c->etd[4],
          (float*)c->etd[5], g.nkr, g.ldk);
    GF_CUDA(c, cudaGetLastError());
    GF_CUDA(c, cudaStreamSynchronize(c->stream));
    cudaFree(dLr);
    if (dLi) cudaFree(dLi);
  }
  // ----- topography (eta) derived fields
  if (k.eta && (k.module == GF_SINGLELAYERQG || k.module == GF_MULTILAYERQG)) {
    const size_t np = (size_t)g.ny * g.nx;
    void* eta_d = dalloc(c, np * rb);
    if (!eta_d || !(c->etah = dalloc(c, nsp * cb))) return fail(c, GF_ERR_NOMEM, "eta");
    if (int r = upload_real(c, eta_d, k.eta, np)) return r;
    // etah = rfft(eta) (one layer)
    Geom g1 = full_geom(c); g1.nl = 1; g1.nb = 1;
    GF_CUDA(c, DISPATCH(c, launch_row_r2c, g1, bufs(c), 1, eta_d, c->stream));
    GF_CUDA(c, DISPATCH(c, launch_col_fwd, g1, bufs(c), 1, c->etah, 0, c->stream));
    // Qx = irfft(i kr etah), Qy = irfft(i l etah) (src/singlelayerqg.jl:185-186,
    // src/multilayerqg.jl:262-264), plus the large-scale topographic PV gradient
    const bool needQ = (k.module == GF_MULTILAYERQG) || (k.U_y != nullptr);
    if (needQ) {
      if (!(c->Qx2D = dalloc(c, np * rb)) || !(c->Qy2D = dalloc(c, np * rb))) return fail(c, GF_ERR_NOMEM, "Q");
      GF_CUDA(c, DISPATCH(c, launch_col_inv, g1, m, c->etah, (int)SF_DX, 0, bufs(c), c->stream));
      GF_CUDA(c, DISPATCH(c, launch_row_c2r, g1, bufs(c), 1, c->Qx2D, c->stream));
      GF_CUDA(c, DISPATCH(c, launch_col_inv, g1, m, c->etah, (int)SF_DY, 0, bufs(c), c->stream));
      GF_CUDA(c, DISPATCH(c, launch_row_c2r, g1, bufs(c), 1, c->Qy2D, c->stream));
      if (k.module == GF_MULTILAYERQG) {
        const int nb = 256;
        if (c->prec == GF_F64) {
          add_scalar_kernel<double><<<nb, 256, 0, c->stream>>>((double*)c->Qx2D, np, k.topographic_pv_gradient[0]);
          add_scalar_kernel<double><<<nb, 256, 0, c->stream>>>((double*)c->Qy2D, np, k.topographic_pv_gradient[1]);
        } else if (c->prec == GF_DF64) {
          add_scalar_kernel<df64><<<nb, 256, 0, c->stream>>>((df64*)c->Qx2D, np, k.topographic_pv_gradient[0]);
          add_scalar_kernel<df64><<<nb, 256, 0, c->stream>>>((df64*)c->Qy2D, np, k.topographic_pv_gradient[1]);
        } else {
          add_scalar_kernel<float><<<nb, 256, 0, c->stream>>>((float*)c->Qx2D, np, k.topographic_pv_gradient[0]);
          add_scalar_kernel<float><<<nb, 256, 0, c->stream>>>((float*)c->Qy2D, np, k.topographic_pv_gradient[1]);
        }
        GF_CUDA(c, cudaGetLastError());
      }
      m.Qx2D = c->Qx2D; m.Qy2D = c->Qy2D;
    }
    if (k.module == GF_SINGLELAYERQG) {
      if (k.U_y == nullptr) m.eta = eta_d;  // q + eta in the products (constant-U path)
      m.etah = c->etah;                     // -i kr U etah term and the enstrophy diagnostic
    }
    GF_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  if (k.module == GF_MULTILAYERQG && !k.eta &&
      (k.topographic_pv_gradient[0] != 0 || k.topographic_pv_gradient[1] != 0)) {
    const size_t np = (size_t)g.ny * g.nx;
    std::vector<double> gx(np, k.topographic_pv_gradient[0]), gy(np, k.topographic_pv_gradient[1]);
    if (!(c->Qx2D = dalloc(c, np * rb)) || !(c->Qy2D = dalloc(c, np * rb))) return fail(c, GF_ERR_NOMEM, "Q");
    if (int r = upload_real(c, c->Qx2D, gx.data(), np)) return r;
    if (int r = upload_real(c, c->Qy2D, gy.data(), np)) return r;
    m.Qx2D = c->Qx2D; m.Qy2D = c->Qy2D;
  }
  if (k.module == GF_SINGLELAYERQG && k.U_y != nullptr) {
    // U(y) path: u' = u + U, C = u' Qx + v Qy with Qy = d(eta)/dy - Uyy
    std::vector<double> U(k.U_y, k.U_y + g.ny);
    auto uyy = d2dy2(U, k.Ly);
    std::vector<double> Qy(g.ny);
    for (int j = 0; j < g.ny; ++j) Qy[j] = -uyy[j];
    if (!(c->U1D = dalloc(c, g.ny * rb)) || !(c->Qy1D = dalloc(c, g.ny * rb))) return fail(c, GF_ERR_NOMEM, "U");
    if (int r = upload_real(c, c->U1D, U.data(), g.ny)) return r;
    if (int r = upload_real(c, c->Qy1D, Qy.data(), g.ny)) return r;
    m.U1D = c->U1D; m.Qy1D = c->Qy1D; m.hasC = 1;
  }
  // float mirrors of the per-element scalars
  m.Ueta = (m.etah != nullptr && m.U0 != 0.0);
  split_hl(m.ell_inv2, &m.ell_inv2_f, &m.ell_inv2_l);
  split_hl(m.U0, &m.U0_f, &m.U0_l);
  split_hl(m.mu, &m.mu_f, &m.mu_l);
  for (int a = 0; a < MAXL; ++a) split_hl(m.lam[a], &m.lam_f[a], &m.lam_l[a]);
  for (int a = 0; a < MAXL * MAXL; ++a) {
    split_hl(m.V[a], &m.V_f[a], &m.V_l[a]);
    split_hl(m.Vinv[a], &m.Vinv_f[a], &m.Vinv_l[a]);
  }
  // ----- forcing buffers
  if (k.forcing_kind != GF_FORCING_NONE) {
    if (!(c->Fh = dalloc(c, NB * nsp * cb))) return fail(c, GF_ERR_NOMEM, "forcing");
    if (k.forcing_kind >= GF_FORCING_STOCHASTIC) {
      if (!(c->fspec = dalloc(c, tsz * rb)) || !(c->prevsol = dalloc(c, NB * nsp * cb)))
        return fail(c, GF_ERR_NOMEM, "stochastic forcing");
      c->Fstore = c->Fh;
    }
  }
  c->diag_blocks = (int)std::min<size_t>((nt + DIAG_BLOCK - 1) / DIAG_BLOCK, 1024);
  if (!(c->dpart = (double*)dalloc(c, (size_t)NDIAG * NB * c->diag_blocks * 8)) ||
      !(c->dout = (double*)dalloc(c, (size_t)NDIAG * NB * 8)))
    return fail(c, GF_ERR_NOMEM, "diagnostics");
  if (int r = upload_clock(c)) return r;
  GF_CUDA(c, cudaStreamSynchronize(c->stream));
  return GF_OK;
}

extern "C" int gf_create(const gf_config* cfg, void* stream, gf_ctx** out) {
  if (!cfg || !out) return fail(nullptr, GF_ERR_ARG, "null argument");
  clear_stale_error();
  *out = nullptr;
  const gf_config& k = *cfg;
  if (k.module < 0 || k.module > 4) return fail(nullptr, GF_ERR_ARG, "unknown module");
  if (k.precision != GF_F32 && k.precision != GF_F64 && k.precision != GF_DF64)
    return fail(nullptr, GF_ERR_ARG, "unknown precision");
  if (k.stepper < 0 || k.stepper > 7) return fail(nullptr, GF_ERR_ARG, "unknown stepper");
  if (k.nx <= 0 || k.ny <= 0 || !(k.Lx > 0) || !(k.Ly > 0) || !(k.dt > 0))
    return fail(nullptr, GF_ERR_ARG, "nx, ny, Lx, Ly and dt must be positive");
  for (int n : {k.nx, k.ny}) {
    if (fixed_length(n)) continue;
    int plan[MAXP], np = 0;
    if (n % 2 != 0 || n < 4 || n > max_generic_length(k.precision) || !radix_plan(n, plan, &np))
      return fail(nullptr, GF_ERR_UNSUPPORTED,
                  "nx and ny must be even, at least 4, at most 4096 (FP32) or 2048 (FP64, df64), with prime factors "
                  "no larger than 61");
  }
  if (!(k.aliased_fraction >= 0) || !(k.aliased_fraction < 1))
    return fail(nullptr, GF_ERR_ARG, "`aliased_fraction` must be less than 1");
  if (k.module == GF_MULTILAYERQG) {
    if (k.nlayers < 1) return fail(nullptr, GF_ERR_ARG, "nlayers must be >= 1");
    if (k.nlayers > MAXL) return fail(nullptr, GF_ERR_UNSUPPORTED, "at most 8 layers");
    if (k.nlayers > 1 && (!k.H || !k.b)) return fail(nullptr, GF_ERR_ARG, "MultiLayerQG needs H and b");
    if (k.nlayers > 1)
      for (int j = 0; j + 1 < k.nlayers; ++j)
        if (k.b[j] == k.b[j + 1]) return fail(nullptr, GF_ERR_ARG, "equal buoyancies give zero reduced gravity");
  } else if (k.nlayers > 1) {
    return fail(nullptr, GF_ERR_ARG, "nlayers > 1 is only valid for MultiLayerQG");
  }
  if (k.forcing_kind < 0 || k.forcing_kind > 4) return fail(nullptr, GF_ERR_ARG, "unknown forcing kind");
  if (k.batch < 0 || k.batch > 65535) return fail(nullptr, GF_ERR_ARG, "batch must be in [0, 65535]");
  gf_ctx* c = new gf_ctx();
  if (cudaGetDevice(&c->dev) != cudaSuccess) {
    delete c;
    return fail(nullptr, GF_ERR_CUDA, "no current CUDA device");
  }
  static std::atomic<uint64_t> next_uid{1};
  c->uid = next_uid++;
  c->cfg = k;
  c->stream = (cudaStream_t)stream;
  if (!c->stream) {
    // a stream of our own (graph capture needs one); blocking, so it orders with the legacy
    // default stream like the caller's other work
    if (cudaStreamCreate(&c->stream) != cudaSuccess) {
      delete c;
      return fail(nullptr, GF_ERR_CUDA, "cudaStreamCreate failed");
    }
    c->own_stream = true;
  }
  const int r = build(c, cfg);
  if (r != GF_OK) {
    g_create_error = c->err.empty() ? g_create_error : c->err;
    gf_destroy(c);
    return r;
  }
  *out = c;
  return GF_OK;
}

// Frees the adjoint's buffers, its second stream and its events (after both streams finish).
static void adj_release(gf_ctx* c) {
  auto& a = c->adj;
  if (a.ts) cudaStreamSynchronize(a.ts);
  for (void* p : a.mem) cudaFree(p);
  for (cudaEvent_t e : {a.ev_rec[0], a.ev_rec[1], a.ev_adj[0], a.ev_adj[1], a.ev_sync})
    if (e) cudaEventDestroy(e);
  if (a.ts) cudaStreamDestroy(a.ts);
  a = gf_ctx::Adjoint{};
}

extern "C" int gf_destroy(gf_ctx* c) {
  if (!c) return GF_OK;
  DevGuard dg_(c->dev);
  if (c->stream) cudaStreamSynchronize(c->stream); else cudaDeviceSynchronize();
  for (void* p : c->allocs) cudaFree(p);
  for (auto e : c->ev_free) cudaEventDestroy(e);
  for (auto& u : c->ev_used) { cudaEventDestroy(u.second.first); cudaEventDestroy(u.second.second); }
  for (auto& ph : c->gexec)
    for (auto& gx : ph) if (gx) cudaGraphExecDestroy(gx);
  for (auto& gx : c->egraph) if (gx) cudaGraphExecDestroy(gx);
  if (c->order_ev) cudaEventDestroy(c->order_ev);
  adj_release(c);
  if (c->own_stream) cudaStreamDestroy(c->stream);
  delete c;
  return GF_OK;
}

extern "C" int gf_get_dims(const gf_ctx* c, int32_t* nkr, int32_t* ny, int32_t* nl, int32_t* rbytes) {
  if (!c) return GF_ERR_ARG;
  if (nkr) *nkr = c->g.nkr;
  if (ny) *ny = c->g.ny;
  if (nl) *nl = c->g.nl;
  if (rbytes) *rbytes = (int32_t)c->rb;
  return GF_OK;
}

// ------------------------------------------------------------------------------- state
static int convert_launch(gf_ctx* c, bool to_df, const void* src, size_t ss, void* dst, size_t ds, size_t rows,
                          size_t w) {
  const int nb = (int)std::min<size_t>((rows * w + 255) / 256, 4096);
  if (to_df) to_df64_kernel<<<nb, 256, 0, c->stream>>>((const double*)src, ss, (df64*)dst, ds, rows, w);
  else from_df64_kernel<<<nb, 256, 0, c->stream>>>((const df64*)src, ss, (double*)dst, ds, rows, w);
  GF_CUDA(c, cudaGetLastError());
  return GF_OK;
}

static int repack_launch(gf_ctx* c, const void* src, size_t ss, void* dst, size_t ds, size_t rows, size_t w) {
  const int nb = (int)std::min<size_t>((rows * w + 255) / 256, 4096);
  repack_kernel<<<nb, 256, 0, c->stream>>>((const uint64_t*)src, ss, (uint64_t*)dst, ds, rows, w);
  GF_CUDA(c, cudaGetLastError());
  return GF_OK;
}

// caller spectral array (Julia layout, row stride nkr) -> internal array (row stride ldk).
// Pageable host arrays travel as one contiguous copy through the staging buffer and are
// re-pitched on the device (a pitched host copy of thousands of short rows is several times
// slower); page-locked ones are read or written by the re-pitch kernel itself.
static int copy_spec_in(gf_ctx* c, void* dst, const void* src, int where) {
  const Geom& g = c->g;
  const cudaMemcpyKind kind = where == GF_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  const size_t rows = (size_t)g.ny * g.nl * g.nb;
  // page-locked host buffer: read by the re-pitch kernel directly (see host_mapped)
  const void* hm = where == GF_HOST ? host_mapped(src, rows * g.nkr * (c->prec == GF_DF64 ? 16 : c->cb), false) : nullptr;
  if (c->prec == GF_DF64) {
    if (!hm) GF_CUDA(c, cudaMemcpyAsync(c->stage, src, (size_t)g.nkr * g.ny * g.nl * g.nb * 16, kind, c->stream));
    if (int r = convert_launch(c, true, hm ? hm : c->stage, 2 * (size_t)g.nkr, dst, 2 * (size_t)g.ldk,
                               (size_t)g.ny * g.nl * g.nb, 2 * (size_t)g.nkr)) return r;
  } else if (where == GF_HOST) {
    const size_t wpe = c->cb / 8;  // 8-byte words per complex element
    if (!hm) GF_CUDA(c, cudaMemcpyAsync(c->stage, src, rows * g.nkr * c->cb, kind, c->stream));
    if (int r = repack_launch(c, hm ? hm : c->stage, wpe * g.nkr, dst, wpe * g.ldk, rows, wpe * g.nkr)) return r;
  } else {
    GF_CUDA(c, cudaMemcpy2DAsync(dst, g.ldk * c->cb, src, g.nkr * c->cb, g.nkr * c->cb, (size_t)g.ny * g.nl * g.nb,
                                 kind, c->stream));
  }
  if (where == GF_HOST) GF_CUDA(c, cudaStreamSynchronize(c->stream));
  return GF_OK;
}
static int copy_spec_out(gf_ctx* c, void* dst, const void* src, int where) {
  const Geom& g = c->g;
  const cudaMemcpyKind kind = where == GF_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  const size_t rows = (size_t)g.ny * g.nl * g.nb;
  // page-locked host buffer: written by the re-pitch kernel directly (see host_mapped)
  void* hm = where == GF_HOST ? host_mapped(dst, rows * g.nkr * (c->prec == GF_DF64 ? 16 : c->cb), true) : nullptr;
  if (c->prec == GF_DF64) {
    if (int r = convert_launch(c, false, src, 2 * (size_t)g.ldk, hm ? hm : c->stage, 2 * (size_t)g.nkr,
                               (size_t)g.ny * g.nl * g.nb, 2 * (size_t)g.nkr)) return r;
    if (!hm) GF_CUDA(c, cudaMemcpyAsync(dst, c->stage, (size_t)g.nkr * g.ny * g.nl * g.nb * 16, kind, c->stream));
  } else if (where == GF_HOST) {
    const size_t wpe = c->cb / 8;
    if (int r = repack_launch(c, src, wpe * g.ldk, hm ? hm : c->stage, wpe * g.nkr, rows, wpe * g.nkr)) return r;
    if (!hm) GF_CUDA(c, cudaMemcpyAsync(dst, c->stage, rows * g.nkr * c->cb, kind, c->stream));
  } else {
    GF_CUDA(c, cudaMemcpy2DAsync(dst, g.nkr * c->cb, src, g.ldk * c->cb, g.nkr * c->cb, (size_t)g.ny * g.nl * g.nb,
                                 kind, c->stream));
  }
  if (where == GF_HOST) GF_CUDA(c, cudaStreamSynchronize(c->stream));
  return GF_OK;
}
// caller physical array (nl x ny x nx reals) <-> internal physical array
static int copy_phys_in(gf_ctx* c, void* dst, const void* src, int where) {
  const size_t n = (size_t)c->g.nl * c->g.ny * c->g.nx * c->g.nb;
  const cudaMemcpyKind kind = where == GF_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  if (c->prec == GF_DF64) {
    GF_CUDA(c, cudaMemcpyAsync(c->stage, src, n * 8, kind, c->stream));
    return convert_launch(c, true, c->stage, n, dst, n, 1, n);
  }
  GF_CUDA(c, cudaMemcpyAsync(dst, src, n * c->rb, kind, c->stream));
  return GF_OK;
}
// nplanes: the number of [ny][nx] planes (0: every layer of every instance)
static int copy_phys_out(gf_ctx* c, void* dst, const void* src, int where, int nplanes = 0) {
  const size_t n = (size_t)(nplanes > 0 ? nplanes : c->g.nl * c->g.nb) * c->g.ny * c->g.nx;
  const cudaMemcpyKind kind = where == GF_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  if (c->prec == GF_DF64) {
    if (int r = convert_launch(c, false, src, n, c->stage, n, 1, n)) return r;
    GF_CUDA(c, cudaMemcpyAsync(dst, c->stage, n * 8, kind, c->stream));
  } else {
    GF_CUDA(c, cudaMemcpyAsync(dst, src, n * c->rb, kind, c->stream));
  }
  if (where == GF_HOST) GF_CUDA(c, cudaStreamSynchronize(c->stream));
  return GF_OK;
}

extern "C" int gf_set_state(gf_ctx* c, const void* sol, int where) {
  if (!c || !sol) return GF_ERR_ARG;
  DevGuard dg_(c->dev);
  clear_stale_error();
  c->W_valid = false;
  return copy_spec_in(c, c->sol, sol, where);
}
extern "C" int gf_get_state(gf_ctx* c, void* sol, int where) {
  if (!c || !sol) return GF_ERR_ARG;
  DevGuard dg_(c->dev);
  clear_stale_error();
  return copy_spec_out(c, sol, c->sol, where);
}
extern "C" int gf_get_clock(const gf_ctx* c, double* t, int64_t* step) {
  if (!c) return GF_ERR_ARG;
  if (t) *t = c->t;
  if (step) *step = c->step;
  return GF_OK;
}
extern "C" int gf_set_clock(gf_ctx* c, double t, int64_t step) {
  if (!c) return GF_ERR_ARG;
  DevGuard dg_(c->dev);
  c->t = t; c->step = step;
  return upload_clock(c);
}
extern "C" int gf_synchronize(gf_ctx* c) {
  if (!c) return GF_ERR_ARG;
  DevGuard dg_(c->dev);
  clear_stale_error();
  GF_CUDA(c, cudaStreamSynchronize(c->stream));
  int flag = 0;
  GF_CUDA(c, cudaMemcpy(&flag, c->derr, sizeof(int), cudaMemcpyDeviceToHost));
  if (flag) return fail(c, GF_ERR_CUDA, "a column-stage tile load did not complete within its time limit");
  return GF_OK;
}

// BarotropicQGQL: sol[0,0] = 0, then the eddy (kr > 0) and zonal-mean (kr = 0) parts
__global__ void ql_split_kernel(const char* sol, char* eddy, char* mean, int cb, int nkr, int ny, int ldk,
                                size_t bs, int nb) {
  const size_t n = (size_t)nb * ny * nkr;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int kr = (int)(e % nkr);
    const size_t r = e / nkr;
    const int j = (int)(r % ny);
    const size_t ib = r / ny;
    const size_t off = (ib * bs + (size_t)j * ldk + kr) * cb;
    const bool k0 = (kr == 0 && j == 0);
    for (int b = 0; b < cb; ++b) {
      const char v = k0 ? 0 : sol[off + b];
      eddy[off + b] = kr == 0 ? 0 : v;
      mean[off + b] = kr == 0 ? v : 0;
    }
  }
}

// sol[0, 0] = 0 of every instance
__global__ void zero_k0_kernel(char* sol, int cb, size_t bs, int nb) {
  const int ib = blockIdx.x * blockDim.x + threadIdx.x;
  if (ib >= nb) return;
  for (int b = 0; b < cb; ++b) sol[ib * bs * cb + b] = 0;
}

extern "C" int gf_updatevars(gf_ctx* c) {
  if (!c) return GF_ERR_ARG;
  DevGuard dg_(c->dev);
  clear_stale_error();
  const size_t pf = (size_t)c->g.nl * c->g.ny * c->g.nx * c->g.nb * c->rb;
  GF_CUDA(c, DISPATCH(c, launch_mask_inplace, c->g, c->sol, c->stream));
  c->W_valid = false;
  if (c->cfg.module == GF_BAROTROPICQGQL) {  // src/barotropicqgql.jl:380-407
    const Geom& g = c->g;
    ql_split_kernel<<<256, 256, 0, c->stream>>>((const char*)c->sol, (char*)c->tmp_spec, (char*)c->tmp_spec2,
                                                (int)c->cb, g.nkr, g.ny, g.ldk, g.bs_spec, g.nb);
    GF_CUDA(c, cudaGetLastError());
    zero_k0_kernel<<<(g.nb + 255) / 256, 256, 0, c->stream>>>((char*)c->sol, (int)c->cb, g.bs_spec, g.nb);
    GF_CUDA(c, cudaGetLastError());
    const int kinds[4] = {SF_X, SF_PSI, SF_U, SF_V};
    for (int f = 0; f < 4; ++f)
      if (int r = inv_transform(c, c->tmp_spec, kinds[f], 0, (char*)c->phys + f * pf)) return r;
    for (int f = 0; f < 3; ++f)
      if (int r = inv_transform(c, c->tmp_spec2, kinds[f], 0, (char*)c->phys + (4 + f) * pf)) return r;
    return GF_OK;
  }
  const int kinds[4] = {SF_X, SF_PSI, SF_U, SF_V};
  for (int f = 0; f < 4; ++f)
    if (int r = inv_transform(c, c->sol, kinds[f], 0, (char*)c->phys + f * pf)) return r;
  return GF_OK;
}

extern "C" int gf_get_field(gf_ctx* c, int which, void* out, int where) {
  if (!c || !out) return GF_ERR_ARG;
  DevGuard dg_(c->dev);
  clear_stale_error();
  const int maxf = c->cfg.module == GF_BAROTROPICQGQL ? 6 : 3;
  if (which < 0 || which > maxf) return fail(c, GF_ERR_ARG, "unknown field");
  const size_t pf = (size_t)c->g.nl * c->g.ny * c->g.nx * c->g.nb * c->rb;
  return copy_phys_out(c, out, (char*)c->phys + which * pf, where);
}

extern "C" int gf_fwdtransform(gf_ctx* c, void* fieldh, const void* field, int where) {
  if (!c || !fieldh || !field) return GF_ERR_ARG;
  DevGuard dg_(c->dev);
  clear_stale_error();
  const size_t pf = (size_t)c->g.nl * c->g.ny * c->g.nx * c->g.nb * c->rb;
  void* ph = (char*)c->phys + 3 * pf;
  if (int r = copy_phys_in(c, ph, field, where)) return r;
  if (int r = fwd_transform(c, ph, c->tmp_spec, 0)) return r;
  return copy_spec_out(c, fieldh, c->tmp_spec, where);
}

extern "C" int gf_invtransform(gf_ctx* c, void* field, const void* fieldh, int where) {
  if (!c || !fieldh || !field) return GF_ERR_ARG;
  DevGuard dg_(c->dev);
  clear_stale_error();
  const size_t pf = (size_t)c->g.nl * c->g.ny * c->g.nx * c->g.nb * c->rb;
  if (int r = copy_spec_in(c, c->tmp_spec, fieldh, where)) return r;
  void* ph = (char*)c->phys + 3 * pf;
  if (int r = inv_transform(c, c->tmp_spec, SF_RAW, 0, ph)) return r;
  return copy_phys_out(c, field, ph, where);
}

// ------------------------------------------------------------ peakedisotropicspectrum
// src/utils.jl:29-54: psi_hat = mask * z * (K^2 (1 + (K/k0)^4))^(-1/2) with z complex normal
// (allones: z = 1), energy e0 = sum over the HALF spectrum of K^2 |psi_hat|^2 / (nx ny)^2
// (the reference's :50), zeta_hat = -K^2 psi_hat sqrt(E0 / e0), zeta = irfft(zeta_hat).
// Draws: element e = j (nx/2+1) + ik, counter (e, 0, 0, TAG_INITIAL), key seed + instance.
__device__ __forceinline__ double peaked_amp(const Geom& g, int ik, int j, double k0, double* K2out) {
  const double kr = g.dkx * ik, l = g.dky * (j < g.ny / 2 ? j : j - g.ny);
  const double K2 = kr * kr + l * l;
  *K2out = K2;
  if (K2 == 0.0) return 0.0;
  const double r = sqrt(K2) / k0;
  return 1.0 / sqrt(K2 * (1.0 + r * r * r * r));
}

__device__ __forceinline__ cplx<double> peaked_psih(const Geom& g, int ik, int j, double k0, int allones,
                                                    const double* mask, uint64_t seed, double* K2) {
  double a = peaked_amp(g, ik, j, k0, K2);
  const size_t e = (size_t)j * g.nkr + ik;
  if (mask) a *= mask[e];
  if (allones) return mk<double>(a, 0.0);
  const cplx<double> z = draw<double>(e, 0, seed, 0, TAG_INITIAL);
  return mk<double>(a * z.x, a * z.y);
}

// per-block compensated partial sums of K^2 |psi_hat|^2, instance blockIdx.y
__global__ void peaked_energy_kernel(Geom g, double k0, int allones, const double* mask, uint64_t seed,
                                     double* partial) {
  __shared__ double red[256];
  const int ib = blockIdx.y;
  const size_t n = (size_t)g.nkr * g.ny;
  double s = 0, c = 0;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    double K2;
    const cplx<double> p = peaked_psih(g, (int)(e % g.nkr), (int)(e / g.nkr), k0, allones, mask, seed + ib, &K2);
    const double x = K2 * (p.x * p.x + p.y * p.y), t = s + x;
    c += (fabs(s) >= fabs(x)) ? (s - t) + x : (x - t) + s;
    s = t;
  }
  red[threadIdx.x] = s + c;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if ((int)threadIdx.x < st) red[threadIdx.x] += red[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[(size_t)ib * gridDim.x + blockIdx.x] = red[0];
}

template <class T> __device__ __forceinline__ T from_d(double x) { return T(x); }
template <> __device__ __forceinline__ df64 from_d<df64>(double x) { return df64(x); }

template <class T>
__global__ void peaked_zetah_kernel(Geom g, double k0, double E0, int allones, const double* mask, uint64_t seed,
                                    const double* esum, cplx<T>* out) {
  const int ib = blockIdx.y;
  const size_t n = (size_t)g.nkr * g.ny;
  const double e0 = esum[ib] / ((double)g.nx * g.ny * (double)g.nx * g.ny);
  const double sc = e0 > 0 ? sqrt(E0 / e0) : 0.0;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int ik = (int)(e % g.nkr), j = (int)(e / g.nkr);
    double K2;
    const cplx<double> p = peaked_psih(g, ik, j, k0, allones, mask, seed + ib, &K2);
    out[(size_t)ib * g.bs_spec + (size_t)j * g.ldk + ik] = mk<T>(from_d<T>(-K2 * sc * p.x), from_d<T>(-K2 * sc * p.y));
  }
}

extern "C" int gf_peakedisotropicspectrum(gf_ctx* c, double kpeak, double E0, const double* mask, int32_t allones,
                                          uint64_t seed, void* zeta, int where) {
  if (!c || !zeta) return GF_ERR_ARG;
  DevGuard dg_(c->dev);
  clear_stale_error();
  if (c->g.nl != 1) return fail(c, GF_ERR_UNSUPPORTED, "peakedisotropicspectrum makes one 2-D field (nlayers = 1)");
  if (c->cfg.Lx != c->cfg.Ly) return fail(c, GF_ERR_ARG, "the domain is not square");  // src/utils.jl:30
  if (!(kpeak > 0) || !(E0 >= 0)) return fail(c, GF_ERR_ARG, "peakedisotropicspectrum: kpeak > 0 and E0 >= 0");
  const Geom& g = c->g;
  const size_t n = (size_t)g.nkr * g.ny;
  double* dmask = nullptr;
  if (mask) {
    if (where == GF_DEVICE) {
      dmask = const_cast<double*>(mask);
    } else {
      GF_CUDA(c, cudaMallocAsync((void**)&dmask, n * 8, c->stream));
      GF_CUDA(c, cudaMemcpyAsync(dmask, mask, n * 8, cudaMemcpyHostToDevice, c->stream));
    }
  }
  const double k0 = kpeak * 2 * M_PI / c->cfg.Lx;
  const int nbk = c->diag_blocks;
  dim3 grid(nbk, g.nb);
  peaked_energy_kernel<<<grid, 256, 0, c->stream>>>(g, k0, allones, dmask, seed, c->dpart);
  diag_finish<<<g.nb, 256, 0, c->stream>>>(c->dpart, nbk, 1u, c->dout);
  if (c->prec == GF_F64)
    peaked_zetah_kernel<double><<<grid, 256, 0, c->stream>>>(g, k0, E0, allones, dmask, seed, c->dout,
                                                            (cplx<double>*)c->tmp_spec);
  else if (c->prec == GF_DF64)
    peaked_zetah_kernel<df64><<<grid, 256, 0, c->stream>>>(g, k0, E0, allones, dmask, seed, c->dout,
                                                          (cplx<df64>*)c->tmp_spec);
  else
    peaked_zetah_kernel<float><<<grid, 256, 0, c->stream>>>(g, k0, E0, allones, dmask, seed, c->dout,
                                                           (cplx<float>*)c->tmp_spec);
  GF_CUDA(c, cudaGetLastError());
  if (mask && where != GF_DEVICE) GF_CUDA(c, cudaFreeAsync(dmask, c->stream));
  void* ph = (char*)c->phys + 3 * (size_t)g.bs_phys * g.nb * c->rb;
  if (int r = inv_transform(c, c->tmp_spec, SF_RAW, 0, ph)) return r;
  return copy_phys_out(c, zeta, ph, where);
}

extern "C" int gf_get_filter(const gf_ctx* c, double* out) {
  if (!c || !out) return GF_ERR_ARG;
  if (c->filt_host.empty()) return GF_ERR_STATE;
  std::memcpy(out, c->filt_host.data(), c->filt_host.size() * sizeof(double));
  return GF_OK;
}

extern "C" int gf_set_physical(gf_ctx* c, int which, const void* field, int where) {
  if (!c || !field) return GF_ERR_ARG;
  DevGuard dg_(c->dev);
  clear_stale_error();
  const int mod = c->cfg.module;
  if (which != GF_FIELD_Q && !(which == GF_FIELD_PSI && mod == GF_MULTILAYERQG))
    return fail(c, GF_ERR_ARG, "set_physical supports q/zeta/b, and psi for MultiLayerQG");
  const size_t pf = (size_t)c->g.nl * c->g.ny * c->g.nx * c->g.nb * c->rb;
  void* ph = (char*)c->phys + 3 * pf;
  if (int r = copy_phys_in(c, ph, field, where)) return r;
  if (which == GF_FIELD_PSI) {
    // q = irfft(S rfft(psi)), then set_q!
    if (int r = fwd_transform(c, ph, c->tmp_spec, 0)) return r;
    GF_CUDA(c, DISPATCH(c, launch_spec_apply, c->g, c->m, c->tmp_spec, c->tmp_spec2, 0, c->stream));
    if (int r = inv_transform(c, c->tmp_spec2, SF_RAW, 0, ph)) return r;
  }
  const int zero_mean = (mod != GF_SINGLELAYERQG);  // SingleLayerQG set_q! keeps the mean
  if (int r = fwd_transform(c, ph, c->sol, zero_mean)) return r;
  c->W_valid = false;
  if (where == GF_HOST) GF_CUDA(c, cudaStreamSynchronize(c->stream));
  return gf_updatevars(c);
}

extern "C" int gf_set_forcing(gf_ctx* c, const void* data, int where) {
  if (!c || !data) return GF_ERR_ARG;
  DevGuard dg_(c->dev);
  clear_stale_error();
  const int fk = c->cfg.forcing_kind;
  if (fk == GF_FORCING_NONE) return fail(c, GF_ERR_STATE, "problem was created without forcing");
  if (fk == GF_FORCING_STATIC || fk == GF_FORCING_HARMONIC) return copy_spec_in(c, c->Fh, data, where);
  // stochastic: spectrum (real, nkr x ny) -> sqrt(spectrum / dt), one table for all layers
  const Geom& g = c->g;
  const size_t nt = (size_t)g.ny * g.nkr;
  std::vector<double> spec(nt);
  if (where == GF_DEVICE) {
    std::vector<char> tmp(nt * c->rb);
    GF_CUDA(c, cudaMemcpy(tmp.data(), data, nt * c->rb, cudaMemcpyDeviceToHost));
    for (size_t e = 0; e < nt; ++e) spec[e] = c->rb == 8 ? ((double*)tmp.data())[e] : ((float*)tmp.data())[e];
  } else {
    for (size_t e = 0; e < nt; ++e) spec[e] = c->rb == 8 ? ((const double*)data)[e] : ((const float*)data)[e];
  }
  for (size_t e = 0; e < nt; ++e) {
    if (spec[e] < 0) return fail(c, GF_ERR_ARG, "forcing spectrum must be non-negative");
    spec[e] = std::sqrt(spec[e] / c->cfg.dt);
  }
  return upload_table(c, c->fspec, spec, 0);
}

// ------------------------------------------------------------------------------- stepping
static StepArgs stage_args(gf_ctx* c, int stage, double tstage) {
  StepArgs s{};
  s.kind = c->kind; s.stage = stage; s.filtered = c->filtered; s.hasL = c->hasL; s.cplxL = c->cplxL;
  s.ab3_euler = c->step < 3;
  s.do_fwd = 1; s.do_inv = 1;
  s.dt = c->cfg.dt;
  s.Ltab = c->Ltab; s.filt = c->filt;
  s.e = c->etd[0]; s.e2 = c->etd[1]; s.zeta = c->etd[2]; s.alpha = c->etd[3]; s.beta = c->etd[4]; s.gamma = c->etd[5];
  s.sol = c->sol; s.X = c->X; s.acc = c->acc; s.s1 = c->s1; s.N1 = c->N1; s.Xg = c->Xg;
  if (c->kind == SK_AB3) { s.Rout = c->R3[c->ab3_out]; s.Rm1 = c->R3[c->ab3_m1]; s.Rm2 = c->R3[c->ab3_m2]; }
  s.fkind = c->cfg.forcing_kind;
  s.Fh = c->Fh;
  s.fspec = c->fspec; s.Fstore = c->Fstore; s.prevsol = c->prevsol;
  s.seed = c->cfg.seed; s.step = (uint64_t)c->step;
  s.draw = (stage == 1);
  if (s.fkind == FK_HARMONIC) s.fscale = std::cos(c->cfg.forcing_omega * tstage + c->cfg.forcing_phase);
  else s.fscale = 1.0;
  split_hl(s.dt, &s.dt_f, &s.dt_l);
  split_hl(s.fscale, &s.fscale_f, &s.fscale_l);
  return s;
}

static cudaEvent_t take_event(gf_ctx* c) {
  if (!c->ev_free.empty()) { cudaEvent_t e = c->ev_free.back(); c->ev_free.pop_back(); return e; }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}

// one row (products) and/or column (stage) launch, timed when profiling is on; `prune`:
// a stage of an unobserved step (products only for kr < kcut, state only at kept modes)
static int launch_stage(gf_ctx* c, const StepArgs& s, int with_row, bool prune = false) {
  Geom g = c->g;
  if (prune) g.kout = g.kcut;
  for (int which = with_row ? 0 : 1; which < 2; ++which) {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (c->profiling) { e0 = take_event(c); e1 = take_event(c); GF_CUDA(c, cudaEventRecord(e0, c->stream)); }
    if (which == 0) GF_CUDA(c, DISPATCH(c, launch_row, g, c->m, bufs(c), c->stream));
    else GF_CUDA(c, DISPATCH(c, launch_col, g, c->m, s, bufs(c), c->stream));
    c->launches++;
    if (c->profiling) { GF_CUDA(c, cudaEventRecord(e1, c->stream)); c->ev_used.push_back({which, {e0, e1}}); }
  }
  return GF_OK;
}

extern "C" int gf_profile_enable(gf_ctx* c, int on) {
  if (!c) return GF_ERR_ARG;
  c->profiling = on != 0;
  return GF_OK;
}

extern "C" int gf_profile_read(gf_ctx* c, double* ms, int64_t* n, int64_t* launches) {
  if (!c) return GF_ERR_ARG;
  DevGuard dg_(c->dev);
  clear_stale_error();
  GF_CUDA(c, cudaStreamSynchronize(c->stream));
  for (auto& u : c->ev_used) {
    float t = 0;
    GF_CUDA(c, cudaEventElapsedTime(&t, u.second.first, u.second.second));
    c->prof_ms[u.first] += t;
    c->prof_n[u.first] += 1;
    c->ev_free.push_back(u.second.first);
    c->ev_free.push_back(u.second.second);
  }
  c->ev_used.clear();
  if (ms) { ms[0] = c->prof_ms[0]; ms[1] = c->prof_ms[1]; }
  if (n) { n[0] = c->prof_n[0]; n[1] = c->prof_n[1]; }
  if (launches) *launches = c->launches;
  c->prof_ms[0] = c->prof_ms[1] = 0;
  c->prof_n[0] = c->prof_n[1] = 0;
  c->launches = 0;
  return GF_OK;
}

static int ensure_W(gf_ctx* c) {
  if (c->W_valid) return GF_OK;
  StepArgs s = stage_args(c, 0, c->t);
  s.do_fwd = 0; s.do_inv = 1;
  if (int r = launch_stage(c, s, 0)) return r;
  c->W_valid = true;
  return GF_OK;
}

// Host bookkeeping of one step (clock, AB3 ring, forcing scale of the last calcN!).
static void host_advance(gf_ctx* c) {
  const double dt = c->cfg.dt;
  if (c->cfg.forcing_kind == GF_FORCING_HARMONIC) {
    const double tl = c->t + (c->nstages == 4 ? dt : 0.0);  // time of the step's last calcN!
    c->last_fscale = std::cos(c->cfg.forcing_omega * tl + c->cfg.forcing_phase);
  } else if (c->cfg.forcing_kind != GF_FORCING_NONE) {
    c->last_fscale = 1.0;
  }
  if (c->kind == SK_AB3) {  // RHS_{-2} <- RHS_{-1} <- RHS
    const int o = c->ab3_out, m1 = c->ab3_m1, m2 = c->ab3_m2;
    c->ab3_m1 = o; c->ab3_m2 = m1; c->ab3_out = m2;
  }
  c->t += dt;
  c->step += 1;
}

// Observed and unobserved steps.  Every calcN! starts with dealias!(sol), so the aliased
// modes of a step's result are never read by a later step: they matter only when the state
// is looked at (the end of a stepforward! call, diagnostics, output).  A step whose result
// nobody looks at skips them -- the products' aliased columns and the stage combination at
// aliased modes -- and leaves exactly the same kept modes.  AB3's aliased modes of a step
// also use the RHS of the two steps before, so the last three steps of a call are observed.
static int observed_tail(const gf_ctx* c) { return c->kind == SK_AB3 ? 3 : 1; }

// Launches of one step: the stages (row + column kernels each) and the device-clock advance.
// W must be valid (the first half of the step's first calcN! done).
static int enqueue_step(gf_ctx* c, bool observed = true) {
  const double dt = c->cfg.dt;
  const bool prune = !observed && c->g.kcut < c->g.nkr;
  for (int stg = 1; stg <= c->nstages; ++stg) {
    const double ts = c->t + (c->nstages == 4 ? (stg == 1 ? 0.0 : stg == 4 ? dt : 0.5 * dt) : 0.0);
    StepArgs s = stage_args(c, stg, ts);
    s.clk = c->dclk;
    if (int r = launch_stage(c, s, 1, prune)) return r;
  }
  advance_clock_kernel<<<1, 32, 0, c->stream>>>(c->dclk, dt, c->cfg.forcing_omega, c->cfg.forcing_phase,
                                                c->cfg.forcing_kind == GF_FORCING_HARMONIC, c->nstages);
  GF_CUDA(c, cudaGetLastError());
  c->launches++;
  return GF_OK;
}

static int one_step(gf_ctx* c, bool observed = true) {
  if (int r = ensure_W(c)) return r;
  if (int r = enqueue_step(c, observed)) return r;
  host_advance(c);
  return GF_OK;
}

static void drop_ensemble_graphs(gf_ctx* c) {
  for (auto& gx : c->egraph)
    if (gx) { cudaGraphExecDestroy(gx); gx = nullptr; }
}

static void drop_graphs(gf_ctx* c) {
  for (auto& ph : c->gexec)
    for (auto& gx : ph)
      if (gx) { cudaGraphExecDestroy(gx); gx = nullptr; }
  drop_ensemble_graphs(c);
  c->gen++;
}

// Capture G steps (starting from the current AB3 ring phase) into an executable graph; with
// last_observed the last step (AB3: three) computes the aliased modes, otherwise none does
// (a replay followed by further steps of the same call).
static int capture_steps(gf_ctx* c, int G, cudaGraphExec_t* out, bool last_observed) {
  const double t0 = c->t;
  const int64_t s0 = c->step, l0 = c->launches;
  const int r0 = c->ab3_out, r1 = c->ab3_m1, r2 = c->ab3_m2;
  const double f0 = c->last_fscale;
  GF_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  int rc = GF_OK;
  for (int i = 0; i < G && rc == GF_OK; ++i) {
    rc = enqueue_step(c, last_observed && i >= G - observed_tail(c));
    host_advance(c);
  }
  cudaGraph_t graph = nullptr;
  const cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
  c->t = t0; c->step = s0; c->launches = l0;
  c->ab3_out = r0; c->ab3_m1 = r1; c->ab3_m2 = r2;
  c->last_fscale = f0;
  if (rc != GF_OK) { if (graph) cudaGraphDestroy(graph); return rc; }
  if (e != cudaSuccess) return fail(c, GF_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  const cudaError_t e2 = cudaGraphInstantiate(out, graph, 0);
  cudaGraphDestroy(graph);
  if (e2 != cudaSuccess) return fail(c, GF_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e2));
  return GF_OK;
}

extern "C" int gf_set_graph_steps(gf_ctx* c, int32_t steps) {
  if (!c || steps < 0) return GF_ERR_ARG;
  DevGuard dg_(c->dev);
  drop_graphs(c);
  c->graph_steps = steps;
  return GF_OK;
}

extern "C" int gf_step(gf_ctx* c, int64_t nsteps) {
  if (!c || nsteps < 0) return GF_ERR_ARG;
  DevGuard dg_(c->dev);
  clear_stale_error();
  if (c->cfg.forcing_kind >= GF_FORCING_STOCHASTIC && !c->fspec) return fail(c, GF_ERR_STATE, "no forcing spectrum");
  // AB3 rotates three RHS buffers: a graph covers three steps so that it can be replayed
  const int G = c->graph_steps <= 0 ? 0 : (c->kind == SK_AB3 ? 3 : c->graph_steps);
  while (nsteps > 0) {
    if (G > 0 && nsteps >= G && !c->profiling) {
      if (int r = ensure_W(c)) return r;
      const int phase = (c->kind == SK_AB3) ? c->ab3_out : 0;
      const int obs = nsteps - G < observed_tail(c);  // replay holds some of the call's last steps
      if (!c->gexec[phase][obs])
        if (int r = capture_steps(c, G, &c->gexec[phase][obs], obs)) return r;
      GF_CUDA(c, cudaGraphLaunch(c->gexec[phase][obs], c->stream));
      for (int i = 0; i < G; ++i) host_advance(c);
      c->launches += (int64_t)G * (2 * c->nstages + 1);
      nsteps -= G;
    } else {
      if (int r = one_step(c, nsteps <= observed_tail(c))) return r;
      nsteps -= 1;
    }
  }
  return GF_OK;
}

// stepforward! with an arbitrary host calcF!: before every stage the callback fills F-hat
// (user layout, the context's element type) for that stage's time, and the library uploads
// it and runs the stage; each stage waits for the host, so this is the slow, general path.
extern "C" int gf_step_callback(gf_ctx* c, int64_t nsteps, gf_forcing_fn fn, void* user) {
  if (!c || nsteps < 0 || !fn) return GF_ERR_ARG;
  DevGuard dg_(c->dev);
  clear_stale_error();
  if (c->cfg.forcing_kind != GF_FORCING_STATIC)
    return fail(c, GF_ERR_STATE, "gf_step_callback needs a context created with forcing_kind = GF_FORCING_STATIC");
  const Geom& g = c->g;
  const size_t elems = (size_t)g.nl * g.ny * g.nkr * g.nb;
  std::vector<char> host(elems * (c->prec == GF_DF64 ? 16 : c->cb));
  const double dt = c->cfg.dt;
  for (int64_t k = 0; k < nsteps; ++k) {
    if (int r = ensure_W(c)) return r;
    for (int stg = 1; stg <= c->nstages; ++stg) {
      const double ts = c->t + (c->nstages == 4 ? (stg == 1 ? 0.0 : stg == 4 ? dt : 0.5 * dt) : 0.0);
      std::memset(host.data(), 0, host.size());
      if (int r = fn(ts, c->step, stg, host.data(), user)) return fail(c, GF_ERR_ARG, "forcing callback returned " + std::to_string(r));
      if (int r = copy_spec_in(c, c->Fh, host.data(), GF_HOST)) return r;
      StepArgs s = stage_args(c, stg, ts);
      s.clk = c->dclk;
      if (int r = launch_stage(c, s, 1)) return r;
    }
    advance_clock_kernel<<<1, 32, 0, c->stream>>>(c->dclk, dt, c->cfg.forcing_omega, c->cfg.forcing_phase, 0, c->nstages);
    GF_CUDA(c, cudaGetLastError());
    c->launches++;
    host_advance(c);
  }
  return GF_OK;
}

// Several independent problems (e.g. the size classes of an ensemble) stepped together.
// When every context replays captured graphs of the same length G (not AB3, profiling off),
// G steps of all of them are captured as ONE graph on the first context's stream -- the
// other contexts' streams fork from it and join back, so their kernels run concurrently --
// and replayed with one launch; otherwise each context steps on its own stream.
// Whether the members can step through the persistent ensemble kernels: at most ENS_MAXCLS
// contexts of one precision and stage count, each one layer without bottom drag on a square
// grid of 32, 64, 128 or 256 points, no AB3 (its buffer ring rotates per context).
static bool ens_fusable(gf_ctx* const* ctxs, int32_t n) {
  if (n < 1 || n > ENS_MAXCLS || ctxs[0]->ens_mode != 1) return false;
  for (int32_t i = 0; i < n; ++i) {
    const gf_ctx* c = ctxs[i];
    if (c->prec != ctxs[0]->prec || c->nstages != ctxs[0]->nstages || c->kind == SK_AB3 || c->g.nl != 1 ||
        c->m.drag || c->g.nx != c->g.ny || !ens_size_ok(c->g.nx) || c->g.rtx || c->g.rty || c->profiling)
      return false;
  }
  return true;
}

static size_t ens_cs(const gf_ctx* c, int n) {
  return c->prec == GF_F32 ? ens_col_stride<float>(n) : c->prec == GF_F64 ? ens_col_stride<double>(n)
                                                                          : ens_col_stride<df64>(n);
}

// G steps of every member with one persistent row launch and one persistent column launch per
// stage on the first member's stream (inside a capture), then the members' clock advances.
// Steps k >= G - 1 of a replay that ends the call are observed (every column and mode).
static int enqueue_ens_steps(gf_ctx* const* ctxs, int32_t n, int G, int obs) {
  gf_ctx* o = ctxs[0];
  const int nst = o->nstages;
  for (int k = 0; k < G; ++k) {
    for (int stg = 1; stg <= nst; ++stg) {
      EnsArgs ra{}, ca{};
      ra.ncls = ca.ncls = n;
      for (int32_t i = 0; i < n; ++i) {
        gf_ctx* c = ctxs[i];
        const bool observed = obs && k >= G - observed_tail(c);
        Geom g = c->g;
        if (!observed && g.kcut < g.nkr) g.kout = g.kcut;
        const double dt = c->cfg.dt;
        const double ts = c->t + (nst == 4 ? (stg == 1 ? 0.0 : stg == 4 ? dt : 0.5 * dt) : 0.0);
        StepArgs s = stage_args(c, stg, ts);
        s.clk = c->dclk;
        const int per = ens_per_block(g.nx);
        EnsClass& r = ra.c[i];
        r.g = g; r.m = c->m; r.s = s; r.b = bufs(c); r.n = g.nx; r.per = per;
        r.nbx = (g.ny / 2) / per; r.nby = g.nb;
        EnsClass& q = ca.c[i];
        q = r;
        q.g.cs = (int)ens_cs(c, g.ny);
        q.nbx = ((g.kout > 0 ? g.kout : g.nkr) + per - 1) / per;
        ra.total += r.nbx * r.nby;
        ca.total += q.nbx * q.nby;
      }
      GF_CUDA(o, DISPATCH(o, launch_ens_row, ra, o->stream));
      GF_CUDA(o, DISPATCH(o, launch_ens_col, ca, o->stream));
    }
    for (int32_t i = 0; i < n; ++i) {
      gf_ctx* c = ctxs[i];
      advance_clock_kernel<<<1, 32, 0, o->stream>>>(c->dclk, c->cfg.dt, c->cfg.forcing_omega, c->cfg.forcing_phase,
                                                    c->cfg.forcing_kind == GF_FORCING_HARMONIC, c->nstages);
      GF_CUDA(o, cudaGetLastError());
      host_advance(c);
    }
  }
  return GF_OK;
}

extern "C" int gf_set_ensemble_mode(gf_ctx* c, int32_t mode) {
  if (!c || (mode != 0 && mode != 1)) return GF_ERR_ARG;
  DevGuard dg_(c->dev);
  c->ens_mode = mode;
  return GF_OK;
}

static int ensemble_capture(gf_ctx* const* ctxs, int32_t n, int G, int obs) {
  gf_ctx* o = ctxs[0];
  const bool fused = ens_fusable(ctxs, n);
  std::vector<cudaEvent_t> ev;
  auto cleanup = [&]() { for (auto e : ev) cudaEventDestroy(e); };
  for (int32_t i = 0; i < 2 * n; ++i) {
    cudaEvent_t e;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) { cleanup(); return fail(o, GF_ERR_CUDA, "event"); }
    ev.push_back(e);
  }
  struct Saved { double t, fs; int64_t step, launches; };
  std::vector<Saved> sv(n);
  for (int32_t i = 0; i < n; ++i) sv[i] = {ctxs[i]->t, ctxs[i]->last_fscale, ctxs[i]->step, ctxs[i]->launches};
  cudaError_t e = cudaStreamBeginCapture(o->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) { cleanup(); return fail(o, GF_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e)); }
  int rc = GF_OK;
  if (fused) {
    rc = enqueue_ens_steps(ctxs, n, G, obs);
  } else {
    cudaEventRecord(ev[0], o->stream);
    for (int32_t i = 1; i < n; ++i) cudaStreamWaitEvent(ctxs[i]->stream, ev[0], 0);   // fork
    for (int32_t i = 0; i < n && rc == GF_OK; ++i)
      for (int k = 0; k < G && rc == GF_OK; ++k) {
        rc = enqueue_step(ctxs[i], obs && k >= G - observed_tail(ctxs[i]));
        host_advance(ctxs[i]);
      }
    for (int32_t i = 1; i < n; ++i) {                                                 // join
      cudaEventRecord(ev[n + i], ctxs[i]->stream);
      cudaStreamWaitEvent(o->stream, ev[n + i], 0);
    }
  }
  cudaGraph_t graph = nullptr;
  e = cudaStreamEndCapture(o->stream, &graph);
  for (int32_t i = 0; i < n; ++i) {
    ctxs[i]->t = sv[i].t; ctxs[i]->last_fscale = sv[i].fs; ctxs[i]->step = sv[i].step; ctxs[i]->launches = sv[i].launches;
  }
  cleanup();
  if (rc != GF_OK) { if (graph) cudaGraphDestroy(graph); return rc; }
  if (e != cudaSuccess) return fail(o, GF_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  // a new membership, graph length or execution invalidates both kinds
  bool same = o->eG == G && o->eMode == (int)fused && (int32_t)o->emembers.size() == n;
  for (int32_t i = 0; same && i < n; ++i)
    same = o->emembers[i].first == ctxs[i]->uid && o->emembers[i].second == ctxs[i]->gen;
  if (!same) drop_ensemble_graphs(o);
  if (o->egraph[obs]) { cudaGraphExecDestroy(o->egraph[obs]); o->egraph[obs] = nullptr; }
  e = cudaGraphInstantiate(&o->egraph[obs], graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) { o->egraph[obs] = nullptr; return fail(o, GF_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e)); }
  o->emembers.clear();
  for (int32_t i = 0; i < n; ++i) o->emembers.push_back({ctxs[i]->uid, ctxs[i]->gen});
  o->eG = G;
  o->eMode = (int)fused;
  return GF_OK;
}

extern "C" int gf_ensemble_step(gf_ctx* const* ctxs, int32_t n, int64_t nsteps) {
  if (!ctxs || n <= 0 || nsteps < 0) return fail(nullptr, GF_ERR_ARG, "gf_ensemble_step: bad arguments");
  clear_stale_error();
  for (int32_t i = 0; i < n; ++i) {
    if (!ctxs[i]) return fail(nullptr, GF_ERR_ARG, "gf_ensemble_step: null context");
    for (int32_t k = 0; k < i; ++k)
      if (ctxs[k] == ctxs[i]) return fail(nullptr, GF_ERR_ARG, "gf_ensemble_step: a context appears twice");
    if (ctxs[i]->cfg.forcing_kind >= GF_FORCING_STOCHASTIC && !ctxs[i]->fspec)
      return fail(ctxs[i], GF_ERR_STATE, "no forcing spectrum");
    if (ctxs[i]->dev != ctxs[0]->dev)
      return fail(nullptr, GF_ERR_ARG, "gf_ensemble_step: the contexts belong to different devices");
  }
  DevGuard dg_(ctxs[0]->dev);
  int G = ctxs[0]->graph_steps;
  bool one_graph = n > 1 && G > 0;
  for (int32_t i = 0; i < n; ++i)
    one_graph = one_graph && ctxs[i]->graph_steps == G && ctxs[i]->kind != SK_AB3 && !ctxs[i]->profiling;
  gf_ctx* o = ctxs[0];
  while (one_graph && nsteps >= G) {
    for (int32_t i = 0; i < n; ++i)
      if (int r = ensure_W(ctxs[i])) { g_create_error = ctxs[i]->err; return r; }
    const int obs = nsteps - G < 1;  // the replay holds the call's last step
    bool same = o->egraph[obs] && o->eG == G && o->eMode == (int)ens_fusable(ctxs, n) &&
                (int32_t)o->emembers.size() == n;
    for (int32_t i = 0; same && i < n; ++i)
      same = o->emembers[i].first == ctxs[i]->uid && o->emembers[i].second == ctxs[i]->gen;
    if (!same)
      if (int r = ensemble_capture(ctxs, n, G, obs)) { g_create_error = o->err; return r; }
    // the graph (on the first stream) waits for the members' earlier work and their streams
    // wait for the graph, so that later calls on any member are ordered after it
    for (int32_t i = 0; i < n; ++i)
      if (!ctxs[i]->order_ev) GF_CUDA(ctxs[i], cudaEventCreateWithFlags(&ctxs[i]->order_ev, cudaEventDisableTiming));
    for (int32_t i = 1; i < n; ++i) {
      GF_CUDA(ctxs[i], cudaEventRecord(ctxs[i]->order_ev, ctxs[i]->stream));
      GF_CUDA(o, cudaStreamWaitEvent(o->stream, ctxs[i]->order_ev, 0));
    }
    const cudaError_t e = cudaGraphLaunch(o->egraph[obs], o->stream);
    if (e != cudaSuccess) return fail(o, GF_ERR_CUDA, std::string("graph launch: ") + cudaGetErrorString(e));
    GF_CUDA(o, cudaEventRecord(o->order_ev, o->stream));
    for (int32_t i = 1; i < n; ++i) GF_CUDA(ctxs[i], cudaStreamWaitEvent(ctxs[i]->stream, o->order_ev, 0));
    for (int32_t i = 0; i < n; ++i) {
      for (int k = 0; k < G; ++k) host_advance(ctxs[i]);
      ctxs[i]->launches += (int64_t)G * (2 * ctxs[i]->nstages + 1);
    }
    nsteps -= G;
  }
  for (int32_t i = 0; i < n; ++i)
    if (int r = gf_step(ctxs[i], nsteps)) {
      g_create_error = ctxs[i]->err;
      return r;
    }
  return GF_OK;
}

extern "C" int gf_get_batch(const gf_ctx* c, int32_t* nb) {
  if (!c || !nb) return GF_ERR_ARG;
  *nb = c->g.nb;
  return GF_OK;
}


extern "C" int gf_calcN(gf_ctx* c, void* N, void* sol, double t, int where) {
  if (!c || !N || !sol) return GF_ERR_ARG;
  DevGuard dg_(c->dev);
  clear_stale_error();
  if (c->cfg.forcing_kind >= GF_FORCING_STOCHASTIC && !c->fspec) return fail(c, GF_ERR_STATE, "no forcing spectrum");
  if (int r = copy_spec_in(c, c->tmp_spec, sol, where)) return r;
  // first half of calcN! (dealias + inversion + inverse y-FFTs) on the caller's sol
  StepArgs s = stage_args(c, 1, t);
  s.sol = c->tmp_spec;
  s.do_fwd = 0; s.do_inv = 1;
  if (int r = launch_stage(c, s, 0)) return r;
  // products, forward FFTs, N = -i kr A - i l B - C + extras + forcing, written to tmp_spec2
  s = stage_args(c, 1, t);
  s.kind = SK_NOUT; s.sol = c->tmp_spec; s.acc = c->tmp_spec2; s.do_fwd = 1; s.do_inv = 0;
  s.draw = (t == c->t);  // stochastic forcing is redrawn only when t == clock.t
  if (s.fkind >= FK_STOCH && !s.draw) s.Fh = c->Fstore;
  if (int r = launch_stage(c, s, 1)) return r;
  if (s.fkind == FK_HARMONIC) c->last_fscale = s.fscale;
  else if (s.fkind != FK_NONE) c->last_fscale = 1.0;
  // like the reference, calcN! leaves sol dealiased
  GF_CUDA(c, DISPATCH(c, launch_mask_inplace, c->g, c->tmp_spec, c->stream));
  c->W_valid = false;
  if (int r = copy_spec_out(c, N, c->tmp_spec2, where)) return r;
  return copy_spec_out(c, sol, c->tmp_spec, where);
}

// ------------------------------------------------------------------------------- diagnostics
// Which reduction slots the diagnostics `which` need (validation of the ids).
static int diag_mask(gf_ctx* c, const int32_t* which, int32_t nd, uint32_t* maskp) {
  const int mod = c->cfg.module;
  const bool finite_ell = (mod == GF_SINGLELAYERQG) && c->m.psi_kind == PSI_HELMHOLTZ;
  uint32_t mask = 0;
  for (int i = 0; i < nd; ++i) {
    const int d = which[i];
    if (mod == GF_MULTILAYERQG) {
      const int n = c->g.nl;
      if (d >= 0 && d < n) mask |= 1u << d;
      else if (d >= GF_D_MLQG_PE0 && d < GF_D_MLQG_PE0 + n - 1) mask |= 1u << (n + d - GF_D_MLQG_PE0);
      else return fail(c, GF_ERR_ARG, "unknown MultiLayerQG diagnostic");
      continue;
    }
    const int maxd = mod == GF_TWODNAVIERSTOKES ? 8 : mod == GF_SINGLELAYERQG ? 9 : 4;  // SQG, QGQL: 4
    if (d < 0 || d > maxd) return fail(c, GF_ERR_ARG, "unknown diagnostic");
    if (mod == GF_SINGLELAYERQG && d == GF_D_SLQG_ENERGY) { mask |= 3u; continue; }
    if (finite_ell && d >= 3) return fail(c, GF_ERR_NOT_IMPLEMENTED, "not implemented for finite deformation radius");
    mask |= 1u << d;
  }
  *maskp = mask;
  return GF_OK;
}

// The reductions of the current state into dst[NDIAG][batch] (device), no host wait.
static int diag_launch(gf_ctx* c, uint32_t mask, double* dst) {
  const void* Fh = (c->cfg.forcing_kind != GF_FORCING_NONE) ? c->Fh : nullptr;
  const void* prev = (c->cfg.forcing_kind >= GF_FORCING_STOCHASTIC) ? c->prevsol : nullptr;
  GF_CUDA(c, DISPATCH(c, launch_diag, c->g, c->m, c->sol, prev, Fh, mask, c->dpart, c->diag_blocks, c->stream));
  diag_finish<<<c->g.nb, 256, 0, c->stream>>>(c->dpart, c->diag_blocks, mask, dst);
  GF_CUDA(c, cudaGetLastError());
  c->launches += 2;
  return GF_OK;
}

// Host normalisation of the raw sums hv[NDIAG][batch] into out[batch][nd]; fs is the
// forcing scale of the last calcN! (harmonic / static forcing work terms).
static void diag_post(const gf_ctx* c, const int32_t* which, int32_t nd, const double* hv, double fs, double* out) {
  const int mod = c->cfg.module, NB = c->g.nb;
  const double nn = (double)c->g.nx * c->g.ny, norm = 1.0 / (nn * nn);
  for (int ib = 0; ib < NB; ++ib) {
    auto h = [&](int q) { return hv[(size_t)q * NB + ib]; };
    for (int i = 0; i < nd; ++i) {
      const int d = which[i];
      double v;
      if (mod == GF_MULTILAYERQG) {
        const int n = c->g.nl;
        if (n == 1) v = h(0) * norm / 2;
        else if (d < n) v = h(d) * norm * c->Hl[d] / (2 * c->Hsum);
        else { const int j = d - GF_D_MLQG_PE0; v = h(n + j) * norm * c->f0 * c->f0 / (c->gprime[j] * 2 * c->Hsum); }
      } else if (mod == GF_SINGLELAYERQG && d == GF_D_SLQG_ENERGY) {
        v = (h(0) + h(1)) * norm;
      } else {
        v = h(d) * norm;
        const bool work = (mod == GF_TWODNAVIERSTOKES && (d == 7 || d == 8)) || (mod == GF_SINGLELAYERQG && (d == 5 || d == 6)) ||
                          (mod == GF_SURFACEQG && d == 4) || (mod == GF_BAROTROPICQGQL && d == 3);
        if (work) v *= fs;
      }
      out[(size_t)ib * nd + i] = v;
    }
  }
}

static double diag_fscale(const gf_ctx* c) {
  return (c->cfg.forcing_kind == GF_FORCING_HARMONIC || c->cfg.forcing_kind == GF_FORCING_STATIC) ? c->last_fscale : 1.0;
}

extern "C" int gf_diagnostics(gf_ctx* c, const int32_t* which, int32_t nd, double* out) {
  if (!c || (nd > 0 && (!which || !out))) return GF_ERR_ARG;
  DevGuard dg_(c->dev);
  clear_stale_error();
  uint32_t mask = 0;
  if (int r = diag_mask(c, which, nd, &mask)) return r;
  if (int r = diag_launch(c, mask, c->dout)) return r;
  std::vector<double> hv((size_t)NDIAG * c->g.nb);
  GF_CUDA(c, cudaMemcpyAsync(hv.data(), c->dout, hv.size() * 8, cudaMemcpyDeviceToHost, c->stream));
  GF_CUDA(c, cudaStreamSynchronize(c->stream));
  diag_post(c, which, nd, hv.data(), diag_fscale(c), out);
  return GF_OK;
}

// stepforward!(prob, diags, nsteps) with the diagnostics of every step reduced into a
// device ring buffer: the host waits once per ring fill (up to 64 MB of raw sums), not once
// per step; out[step][instance][nd].
extern "C" int gf_step_diags(gf_ctx* c, int64_t nsteps, const int32_t* which, int32_t nd, double* out) {
  if (!c || nsteps < 0 || (nd > 0 && (!which || !out))) return GF_ERR_ARG;
  DevGuard dg_(c->dev);
  clear_stale_error();
  if (nd == 0) return gf_step(c, nsteps);
  uint32_t mask = 0;
  if (int r = diag_mask(c, which, nd, &mask)) return r;
  const size_t slot = (size_t)NDIAG * c->g.nb;
  const int64_t cap = std::max<int64_t>(1, std::min<int64_t>(nsteps, (int64_t)((64u << 20) / (slot * 8))));
  double* ring = nullptr;
  GF_CUDA(c, cudaMallocAsync((void**)&ring, (size_t)cap * slot * 8, c->stream));
  std::vector<double> hv((size_t)cap * slot), fs((size_t)cap);
  int rc = GF_OK;
  for (int64_t i0 = 0; i0 < nsteps && rc == GF_OK; i0 += cap) {
    const int64_t n = std::min<int64_t>(cap, nsteps - i0);
    for (int64_t k = 0; k < n && rc == GF_OK; ++k) {
      rc = one_step(c);
      if (rc == GF_OK) rc = diag_launch(c, mask, ring + k * slot);
      fs[k] = diag_fscale(c);
    }
    if (rc != GF_OK) break;
    if (cudaMemcpyAsync(hv.data(), ring, (size_t)n * slot * 8, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess) {
      rc = fail(c, GF_ERR_CUDA, "diagnostics ring copy");
      break;
    }
    for (int64_t k = 0; k < n; ++k)
      diag_post(c, which, nd, hv.data() + k * slot, fs[k], out + (i0 + k) * nd * c->g.nb);
  }
  cudaFreeAsync(ring, c->stream);
  return rc;
}

// ---------------------------------------------------------------------------- fluxes
// MultiLayerQG.fluxes (src/multilayerqg.jl:977-1022): lateral_j = H_j / V sum U_j v_j du_j/dy
// dx dy and vertical_{j+1/2} = f0^2 / (g'_j V) sum (U_j - U_{j+1}) v_{j+1} psi_j dx dy,
// V = Lx Ly sum(H) (one layer: V = Lx Ly, no H factor), after updatevars!; FP64 sums.
extern "C" int gf_fluxes(gf_ctx* c, double* lateral, double* vertical) {
  if (!c || !lateral) return GF_ERR_ARG;
  DevGuard dg_(c->dev);
  clear_stale_error();
  if (c->cfg.module != GF_MULTILAYERQG) return fail(c, GF_ERR_ARG, "fluxes is a MultiLayerQG diagnostic");
  const Geom& g = c->g;
  const int nl = g.nl, NB = g.nb;
  if (nl > 1 && !vertical) return GF_ERR_ARG;
  if (int r = gf_updatevars(c)) return r;
  const size_t pf = (size_t)nl * g.ny * g.nx * NB * c->rb;
  void* uy = nullptr;
  GF_CUDA(c, cudaMallocAsync(&uy, pf, c->stream));
  int rc = inv_transform(c, c->sol, SF_UY, 0, uy);
  if (rc == GF_OK) {
    const cudaError_t e = DISPATCH(c, launch_flux, g, (const char*)c->phys + 3 * pf, uy, (const char*)c->phys + pf,
                                   c->Ud, c->dpart, c->diag_blocks, c->stream);
    if (e != cudaSuccess) rc = fail(c, GF_ERR_CUDA, cudaGetErrorString(e));
  }
  if (rc == GF_OK) {
    diag_finish<<<NB, 256, 0, c->stream>>>(c->dpart, c->diag_blocks, (1u << (2 * nl - 1)) - 1, c->dout);
    c->launches += 2;
  }
  cudaFreeAsync(uy, c->stream);
  if (rc != GF_OK) return rc;
  std::vector<double> hv((size_t)NDIAG * NB);
  GF_CUDA(c, cudaMemcpyAsync(hv.data(), c->dout, hv.size() * 8, cudaMemcpyDeviceToHost, c->stream));
  GF_CUDA(c, cudaStreamSynchronize(c->stream));
  const double dxdy = (c->cfg.Lx / g.nx) * (c->cfg.Ly / g.ny);
  const double V = c->cfg.Lx * c->cfg.Ly * (nl > 1 ? c->Hsum : 1.0);
  for (int ib = 0; ib < NB; ++ib) {
    auto h = [&](int q) { return hv[(size_t)q * NB + ib]; };
    for (int L = 0; L < nl; ++L) lateral[(size_t)ib * nl + L] = (nl > 1 ? c->Hl[L] : 1.0) * h(L) * dxdy / V;
    for (int L = 0; L < nl - 1; ++L)
      vertical[(size_t)ib * (nl - 1) + L] = c->f0 * c->f0 / c->gprime[L] * h(nl + L) * dxdy / V;
  }
  return GF_OK;
}

// ------------------------------------------------------------------------------ autotune
// Launch-shape autotuner: times the step of this context at every candidate shape
// -- column kernel: FFT radix (FP32: 4, 8, 16; FP64/df64: 8) x columns per block C, the TMA
// column stage, and on small grids the field-parallel kernel (radix 2, 4, 8 x C); row
// kernel: radix x row pairs per block B (threads per row = length / radix) and the
// field-parallel kernel (radix 2, 4, 8) -- by the GPU time of a graph-replayed step, and
// keeps the fastest.  The state, clock, AB3 history and stochastic-forcing record are
// restored afterwards; captured graphs are dropped (they are re-captured with the new
// shapes).
static int set_shape(gf_ctx* c, int Rr, int B, int Rc, int C, int tmaC = 0) {
  c->g.tuneRr = Rr; c->g.tuneB = B; c->g.tuneRc = Rc; c->g.tuneC = C; c->g.tmaC = tmaC;
  drop_graphs(c);
  return GF_OK;
}

// whether the TMA column stage can run this context, and with C columns per block
static bool tma_eligible(const gf_ctx* c, int C) {
  return c->tma.ok && !c->g.rty && c->g.nl == 1 && !c->m.drag && 1 + c->m.hasB + c->m.hasC <= 2 &&
         (C == c->tma.Cs[0] || C == c->tma.Cs[1]);
}

extern "C" int gf_set_tma_columns(gf_ctx* c, int32_t C) {
  if (!c) return GF_ERR_ARG;
  DevGuard dg_(c->dev);
  if (C != 0 && !tma_eligible(c, C))
    return fail(c, GF_ERR_UNSUPPORTED, "no TMA column stage with this column count for this context");
  c->g.tmaC = C;
  if (C) { c->g.fpRc = 0; c->g.fpC = 0; }  // the TMA stage is a form of the classic column kernel
  drop_graphs(c);
  return GF_OK;
}

extern "C" int gf_get_tma_columns(const gf_ctx* c, int32_t* C) {
  if (!c || !C) return GF_ERR_ARG;
  *C = c->g.tmaC;
  return GF_OK;
}

// whether the field-parallel small-grid kernels can run this context
static bool fp_ctx_ok(const gf_ctx* c) {
  return !c->g.rtx && !c->g.rty && fp_len_ok(c->g.nx) && fp_len_ok(c->g.ny) && c->g.nl == 1 && !c->m.drag;
}

static void set_fp(gf_ctx* c, int Rr, int Rc, int C) {
  c->g.fpR = Rr; c->g.fpRc = Rc; c->g.fpC = Rc ? std::max(C, 1) : 0;
  drop_graphs(c);
}

extern "C" int gf_set_field_parallel(gf_ctx* c, int32_t row_radix, int32_t col_radix, int32_t columns) {
  if (!c || row_radix < 0 || col_radix < 0 || columns < 0) return GF_ERR_ARG;
  DevGuard dg_(c->dev);
  if ((row_radix || col_radix) && !fp_ctx_ok(c))
    return fail(c, GF_ERR_UNSUPPORTED, "field-parallel kernels: one layer without bottom drag, power-of-two lengths 32 ... 512");
  if (row_radix && !fp_radix_ok(c->g.nx, row_radix)) return fail(c, GF_ERR_ARG, "field-parallel row radix must be 2, 4 or 8");
  if (col_radix && (!fp_radix_ok(c->g.ny, col_radix) || !fp_cols_ok(c->g.ny, col_radix, columns ? columns : 1)))
    return fail(c, GF_ERR_ARG, "field-parallel column radix must be 2, 4 or 8, with 3 x columns x ny / radix <= 384");
  set_fp(c, row_radix, col_radix, columns);
  return GF_OK;
}

extern "C" int gf_get_field_parallel(const gf_ctx* c, int32_t* out) {
  if (!c || !out) return GF_ERR_ARG;
  out[0] = c->g.fpR; out[1] = c->g.fpRc; out[2] = c->g.fpC;
  return GF_OK;
}

extern "C" int gf_set_launch_shape(gf_ctx* c, const int32_t* shape) {
  if (!c || !shape) return GF_ERR_ARG;
  DevGuard dg_(c->dev);
  for (int k = 0; k < 4; ++k) if (shape[k] < 0) return fail(c, GF_ERR_ARG, "launch shape entries must be >= 0");
  const bool f32 = c->prec == GF_F32;
  for (int k : {0, 2}) {
    const int R = shape[k], N = k == 0 ? c->g.nx : c->g.ny;
    if (R != 0 && R != 8 && !(f32 && f32_radix_built(N, R))) return fail(c, GF_ERR_ARG, "radix not built for this size");
  }
  set_fp(c, 0, 0, 0);  // an explicit launch shape runs the classic kernels
  return set_shape(c, shape[0], shape[1], shape[2], shape[3], c->g.tmaC);
}

extern "C" int gf_get_launch_shape(const gf_ctx* c, int32_t* shape) {
  if (!c || !shape) return GF_ERR_ARG;
  shape[0] = c->g.tuneRr; shape[1] = c->g.tuneB; shape[2] = c->g.tuneRc; shape[3] = c->g.tuneC;
  return GF_OK;
}

extern "C" int gf_autotune(gf_ctx* c, int32_t reps, int32_t* shape) {
  if (!c) return GF_ERR_ARG;
  DevGuard dg_(c->dev);
  clear_stale_error();
  if (c->g.rtx || c->g.rty) {  // generic lengths: one launch shape, nothing to tune
    if (shape) for (int q = 0; q < 4; ++q) shape[q] = 0;
    return GF_OK;
  }
  if (c->cfg.forcing_kind >= GF_FORCING_STOCHASTIC && !c->fspec) return fail(c, GF_ERR_STATE, "no forcing spectrum");
  if (reps <= 0) reps = 4;
  const Geom g0 = c->g;
  const size_t spec = g0.bs_spec * g0.nb * c->cb;
  // snapshot of what a step changes
  std::vector<std::pair<void*, void*>> saved;  // (buffer, copy)
  auto keep = [&](void* p) -> int {
    if (!p) return GF_OK;
    void* q = nullptr;
    GF_CUDA(c, cudaMallocAsync(&q, spec, c->stream));
    GF_CUDA(c, cudaMemcpyAsync(q, p, spec, cudaMemcpyDeviceToDevice, c->stream));
    saved.push_back({p, q});
    return GF_OK;
  };
  int rc = keep(c->sol);
  if (c->kind == SK_AB3) for (int i = 0; i < 3 && rc == GF_OK; ++i) rc = keep(c->R3[i]);
  if (c->cfg.forcing_kind >= GF_FORCING_STOCHASTIC && rc == GF_OK) { rc = keep(c->Fh); if (rc == GF_OK) rc = keep(c->prevsol); }
  const double t0 = c->t, fs0 = c->last_fscale;
  const int64_t s0 = c->step;
  const int a0 = c->ab3_out, a1 = c->ab3_m1, a2 = c->ab3_m2;
  const bool prof0 = c->profiling;
  auto restore = [&]() {
    for (auto& pq : saved) cudaMemcpyAsync(pq.first, pq.second, spec, cudaMemcpyDeviceToDevice, c->stream);
    c->t = t0; c->step = s0; c->last_fscale = fs0;
    c->ab3_out = a0; c->ab3_m1 = a1; c->ab3_m2 = a2;
    c->W_valid = false;
  };
  // average time of the row (which = 0) or column (1) kernel at the current shape
  // time of one unobserved step (the bulk of a stepforward! call) at the current shape: a few
  // steps captured as one CUDA graph, as gf_step replays them, replayed twice and the second
  // replay timed with events -- GPU time only (per-launch events around small kernels also
  // count the host's launch gaps).  The column candidates are compared with the row shape
  // fixed, then the row candidates with the chosen column shape.
  auto measure = [&](int, double* ms) -> int {
    restore();
    if (int r = upload_clock(c)) return r;
    c->profiling = false;
    if (int r = one_step(c, false)) return r;  // warm-up (kernel attributes, W)
    if (int r = ensure_W(c)) return r;
    const int G = (c->kind == SK_AB3) ? 3 : std::max(reps, 2);
    cudaGraphExec_t gx = nullptr;
    if (int r = capture_steps(c, G, &gx, false)) return r;
    cudaEvent_t e0 = take_event(c), e1 = take_event(c);
    cudaError_t err = cudaGraphLaunch(gx, c->stream);
    if (err == cudaSuccess) err = cudaEventRecord(e0, c->stream);
    if (err == cudaSuccess) err = cudaGraphLaunch(gx, c->stream);
    if (err == cudaSuccess) err = cudaEventRecord(e1, c->stream);
    if (err == cudaSuccess) err = cudaEventSynchronize(e1);
    float t = 0;
    if (err == cudaSuccess) err = cudaEventElapsedTime(&t, e0, e1);
    cudaGraphExecDestroy(gx);
    c->ev_free.push_back(e0);
    c->ev_free.push_back(e1);
    c->profiling = prof0;
    if (err != cudaSuccess) return fail(c, GF_ERR_CUDA, std::string("autotune timing: ") + cudaGetErrorString(err));
    *ms = t / G;
    return GF_OK;
  };
  const bool f32 = c->prec == GF_F32;
  const int radii[3] = {8, 16, 4};
  const int unit = 128 / (int)c->cb;  // elements per 128-byte wavefront
  int bestRc = 0, bestC = 0, bestRr = 0, bestB = 0, bestT = 0;
  int bestFc = 0, bestFC = 0, bestFr = 0;  // field-parallel kernels (radix 0: not chosen)
  const bool fpok = fp_ctx_ok(c);
  set_fp(c, 0, 0, 0);
  double best = 1e30;
  for (int ri = 0; ri < (f32 ? 3 : 1) && rc == GF_OK; ++ri) {
    const int R = radii[ri], TPF = g0.ny / R;
    if (!f32_radix_built(g0.ny, R) || TPF < 1) continue;
    for (const int C : {1, 2, 3, 4, 5, 6, 7, 8, 10, 12, 16}) {
      if (rc != GF_OK) break;
      const int cs = C > 1 ? g0.ny + std::max(unit / C, 1) : g0.ny;
      const size_t sm = col_stage_smem(g0.ny, C, cs, c->m, g0.nl, c->cb, C * TPF, c->prec == GF_DF64);
      if (C * TPF > col_max_threads(c->rb, g0.ny, c->m, g0.nl) || sm > (size_t)SMEM_CAP) continue;
      set_shape(c, 0, 0, R, C);
      double ms = 0;
      rc = measure(1, &ms);
      if (rc == GF_OK && ms < best) { best = ms; bestRc = R; bestC = C; bestT = 0; }
    }
    // the TMA column stage at this radix
    for (int k = 0; k < 2 && rc == GF_OK; ++k) {
      const int C = c->tma.Cs[k];
      if (!tma_eligible(c, C) || C * TPF > 1024) continue;
      set_shape(c, 0, 0, R, 0, C);
      double ms = 0;
      rc = measure(1, &ms);
      if (rc == GF_OK && ms < best) { best = ms; bestRc = R; bestC = 0; bestT = C; }
    }
  }
  // the field-parallel column kernel (small grids)
  for (const int R : {2, 4, 8}) {
    if (!fpok || rc != GF_OK || !fp_radix_ok(g0.ny, R)) continue;
    for (const int C : {1, 2, 4}) {
      if (rc != GF_OK || !fp_cols_ok(g0.ny, R, C)) continue;
      set_shape(c, 0, 0, 0, 0, 0);
      set_fp(c, 0, R, C);
      double ms = 0;
      rc = measure(1, &ms);
      if (rc == GF_OK && ms < best) { best = ms; bestFc = R; bestFC = C; }
    }
  }
  set_fp(c, 0, bestFc, bestFC);
  best = 1e30;
  for (int ri = 0; ri < (f32 ? 3 : 1) && rc == GF_OK; ++ri) {
    const int R = radii[ri], TPF = g0.nx / R;
    if (!f32_radix_built(g0.nx, R) || TPF < 1 || TPF > 256) continue;
    for (int B = 1; B * TPF <= 256 && rc == GF_OK; B *= 2) {
      if (!row_shape_ok(g0.nx, R, c->cb, 3, g0.ny / 2, B)) continue;
      set_shape(c, R, B, bestRc, bestC, bestT);
      double ms = 0;
      rc = measure(0, &ms);
      if (rc == GF_OK && ms < best) { best = ms; bestRr = R; bestB = B; }
    }
  }
  for (const int R : {2, 4, 8}) {  // the field-parallel row kernel
    if (!fpok || rc != GF_OK || !fp_radix_ok(g0.nx, R)) continue;
    set_shape(c, 0, 0, bestRc, bestC, bestT);
    set_fp(c, R, bestFc, bestFC);
    double ms = 0;
    rc = measure(0, &ms);
    if (rc == GF_OK && ms < best) { best = ms; bestFr = R; }
  }
  c->profiling = prof0;
  restore();
  for (auto& pq : saved) cudaFreeAsync(pq.second, c->stream);
  if (rc != GF_OK) {
    set_shape(c, g0.tuneRr, g0.tuneB, g0.tuneRc, g0.tuneC, g0.tmaC);
    set_fp(c, g0.fpR, g0.fpRc, g0.fpC);
    upload_clock(c);
    return rc;
  }
  set_shape(c, bestRr, bestB, bestRc, bestC, bestT);
  set_fp(c, bestFr, bestFc, bestFC);
  if (int r = upload_clock(c)) return r;
  if (shape) { shape[0] = bestRr; shape[1] = bestB; shape[2] = bestRc; shape[3] = bestC; }
  return GF_OK;
}

// Output streaming: every `every` steps the diagnostics `which_diag` are reduced into a
// device ring and the physical fields `which_field` (updatevars!) are copied into a device
// ring; the host waits once per ring fill (<= 256 MB of fields), not once per output.
// diag_out[k][instance][nd]; field_out[k][f][instance][layer][ny][nx] (context real type;
// FP64 for df64).  Steps after the last output are stepped too.
extern "C" int gf_step_output(gf_ctx* c, int64_t nsteps, int32_t every, const int32_t* which_diag, int32_t nd,
                              double* diag_out, const int32_t* which_field, int32_t nf, void* field_out) {
  if (!c || nsteps < 0 || every < 1 || nd < 0 || nf < 0 || (nd > 0 && (!which_diag || !diag_out)) ||
      (nf > 0 && (!which_field || !field_out)))
    return GF_ERR_ARG;
  DevGuard dg_(c->dev);
  clear_stale_error();
  uint32_t mask = 0;
  if (nd > 0)
    if (int r = diag_mask(c, which_diag, nd, &mask)) return r;
  const int maxf = c->cfg.module == GF_BAROTROPICQGQL ? 6 : 3;
  for (int32_t f = 0; f < nf; ++f)
    if (which_field[f] < 0 || which_field[f] > maxf) return fail(c, GF_ERR_ARG, "unknown field");
  const int64_t nout = nsteps / every;
  const Geom& g = c->g;
  const size_t pf = (size_t)g.nl * g.ny * g.nx * g.nb * c->rb;      // one field, all instances (device)
  const size_t pfo = (size_t)g.nl * g.ny * g.nx * g.nb * (c->prec == GF_DF64 ? 8 : c->rb);  // at the ABI
  const size_t dslot = (size_t)NDIAG * g.nb;
  int64_t cap = nout > 0 ? nout : 1;
  if (nf > 0) cap = std::max<int64_t>(1, std::min<int64_t>(cap, (int64_t)((256u << 20) / (nf * pf))));
  double* dring = nullptr;
  char* fring = nullptr;
  if (nd > 0) GF_CUDA(c, cudaMallocAsync((void**)&dring, (size_t)cap * dslot * 8, c->stream));
  if (nf > 0) GF_CUDA(c, cudaMallocAsync((void**)&fring, (size_t)cap * nf * pf, c->stream));
  std::vector<double> hv(nd > 0 ? (size_t)cap * dslot : 0), fs(cap);
  int rc = GF_OK;
  for (int64_t k0 = 0; k0 < nout && rc == GF_OK; k0 += cap) {
    const int64_t n = std::min<int64_t>(cap, nout - k0);
    for (int64_t k = 0; k < n && rc == GF_OK; ++k) {
      rc = gf_step(c, every);
      if (rc == GF_OK && nd > 0) rc = diag_launch(c, mask, dring + k * dslot);
      fs[k] = diag_fscale(c);
      if (rc == GF_OK && nf > 0) {
        rc = gf_updatevars(c);
        for (int32_t f = 0; f < nf && rc == GF_OK; ++f)
          if (cudaMemcpyAsync(fring + ((size_t)k * nf + f) * pf, (char*)c->phys + (size_t)which_field[f] * pf, pf,
                              cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess)
            rc = fail(c, GF_ERR_CUDA, "output field copy");
      }
    }
    if (rc != GF_OK) break;
    if (nd > 0) {
      if (cudaMemcpyAsync(hv.data(), dring, (size_t)n * dslot * 8, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess) {
        rc = fail(c, GF_ERR_CUDA, "output diagnostics copy");
        break;
      }
    }
    for (int64_t k = 0; k < n && nf > 0 && rc == GF_OK; ++k)
      for (int32_t f = 0; f < nf && rc == GF_OK; ++f)
        rc = copy_phys_out(c, (char*)field_out + ((size_t)(k0 + k) * nf + f) * pfo, fring + ((size_t)k * nf + f) * pf,
                           GF_HOST);
    if (rc == GF_OK && cudaStreamSynchronize(c->stream) != cudaSuccess) rc = fail(c, GF_ERR_CUDA, "output sync");
    for (int64_t k = 0; k < n && nd > 0 && rc == GF_OK; ++k)
      diag_post(c, which_diag, nd, hv.data() + k * dslot, fs[k], diag_out + (size_t)(k0 + k) * nd * g.nb);
  }
  if (dring) cudaFreeAsync(dring, c->stream);
  if (fring) cudaFreeAsync(fring, c->stream);
  if (rc == GF_OK && nsteps - nout * every > 0) rc = gf_step(c, nsteps - nout * every);
  return rc;
}

// ------------------------------------------------------------------------------- adjoint
// Reverse-mode derivative of stepforward!(prob, nsteps) for TwoDNavierStokes and
// SingleLayerQG (constant U or U(y)) with ETDRK4 / FilteredETDRK4 or RK4 / FilteredRK4 (the
// kernels are in gf_adjoint.cuh).
// Checkpointing: the forward pass stores the state every `every` steps; the reverse pass
// recomputes one segment at a time from its checkpoint with the fused forward kernels,
// keeping the physical fields (q + eta, u, v) of all its stages, then runs the transposed
// stages of the segment's steps in reverse.  Work: one forward pass + one recomputation +
// the transposed stages; memory: nsteps / every states + every x 4 x 3 physical fields.
static int adj_check(gf_ctx* c) {
  const int mod = c->cfg.module;
  if (c->g.rtx || c->g.rty) return fail(c, GF_ERR_UNSUPPORTED, "the adjoint needs power-of-two nx, ny in [32, 2048]");
  if (mod != GF_TWODNAVIERSTOKES && mod != GF_SINGLELAYERQG && mod != GF_MULTILAYERQG && mod != GF_SURFACEQG)
    return fail(c, GF_ERR_UNSUPPORTED,
                "the adjoint covers TwoDNavierStokes, SingleLayerQG, MultiLayerQG and SurfaceQG");
  if ((c->g.nl > 1 || c->m.drag) && (size_t)3 * c->g.nl * c->g.ny * c->cb > (size_t)SMEM_CAP)
    return fail(c, GF_ERR_UNSUPPORTED, "the several-layer adjoint holds every layer of a column: 3 x nlayers x ny "
                                       "complex values must fit in 200 KB of shared memory");
  if (c->kind != SK_ETDRK4 && c->kind != SK_RK4)
    return fail(c, GF_ERR_UNSUPPORTED, "the adjoint follows the ETDRK4 / FilteredETDRK4 and RK4 / FilteredRK4 stages");
  if (c->g.nb != 1) return fail(c, GF_ERR_UNSUPPORTED, "the adjoint runs one instance (batch = 1)");
  if (c->m.linear) return fail(c, GF_ERR_UNSUPPORTED, "the adjoint covers the nonlinear step");
  return GF_OK;
}

static void* adj_alloc(gf_ctx* c, size_t bytes) {
  void* p = nullptr;
  if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
  c->adj.mem.push_back(p);
  return p;
}

// Binomial (Griewank) checkpoint schedule over units of `every` steps: reversing n units whose
// first state is stored, with s free snapshot slots, costs
//   C(n, s) = min_{1<=m<n} [ m + C(n - m, s - 1) + C(m, s) ],  C(1, s) = 0,
//   C(n, 0) = n (n - 1) / 2 (advance from the start for each unit, last first),
// in unit advances (every unit is also recomputed once with its forward fields kept).  The
// minimising splits are the binomial schedule; with n - 1 free slots it stores every unit
// boundary in one forward pass (cost n - 1).
static int adj_schedule(gf_ctx* c) {
  auto& a = c->adj;
  const int U = a.nseg, S = a.snaps;  // s ranges over 0 .. S - 1 free slots
  a.split.assign((size_t)(U + 1) * S, 0);
  std::vector<int64_t> cost((size_t)(U + 1) * S, 0);
  auto C = [&](int n, int sf) -> int64_t& { return cost[(size_t)n * S + sf]; };
  for (int n = 1; n <= U; ++n)
    for (int sf = 0; sf < S; ++sf) {
      if (n == 1) { C(n, sf) = 0; continue; }
      if (sf == 0) { C(n, sf) = (int64_t)n * (n - 1) / 2; continue; }
      if (sf >= n - 1) { C(n, sf) = n - 1; a.split[(size_t)n * S + sf] = 1; continue; }
      int64_t best = -1; int bm = 1;
      for (int m = 1; m < n; ++m) {
        const int64_t v = m + C(n - m, sf - 1) + C(m, sf);
        if (best < 0 || v < best) { best = v; bm = m; }
      }
      C(n, sf) = best;
      a.split[(size_t)n * S + sf] = bm;
    }
  return GF_OK;
}

extern "C" int gf_adjoint_setup(gf_ctx* c, int64_t nsteps, int32_t checkpoint_every) {
  if (!c || nsteps < 1 || checkpoint_every < 1) return GF_ERR_ARG;
  DevGuard dg_(c->dev);
  clear_stale_error();
  if (int r = adj_check(c)) return r;
  if ((nsteps + checkpoint_every - 1) / checkpoint_every > 4096)
    return fail(c, GF_ERR_ARG, "more than 4096 recomputation units: raise checkpoint_every");
  GF_CUDA(c, cudaStreamSynchronize(c->stream));
  auto& a = c->adj;
  adj_release(c);
  const Geom& g = c->g;
  a.nsteps = nsteps;
  a.every = (int)std::min<int64_t>(checkpoint_every, nsteps);
  a.nseg = (int)((nsteps + a.every - 1) / a.every);
  a.snaps = a.nseg;  // one slot per unit boundary: a single forward pass, no recomputation of advances
  const size_t spec = g.bs_spec * c->cb, plane = (size_t)g.ny * g.nx * c->rb;
  const size_t wide = (size_t)g.nl * g.ny * g.ldk * c->cb;  // one field, every layer
  a.unit_phys = (size_t)a.every * 4 * 3 * g.nl * plane;
  // the second stream is non-blocking: it is ordered with the context stream by events only,
  // never implicitly with the legacy default stream
  if (cudaStreamCreateWithFlags(&a.ts, cudaStreamNonBlocking) != cudaSuccess) {
    a.ts = nullptr;
    return fail(c, GF_ERR_CUDA, "adjoint stream");
  }
  for (cudaEvent_t* e : {&a.ev_rec[0], &a.ev_rec[1], &a.ev_adj[0], &a.ev_adj[1], &a.ev_sync})
    if (cudaEventCreateWithFlags(e, cudaEventDisableTiming) != cudaSuccess) {
      *e = nullptr;
      adj_release(c);
      return fail(c, GF_ERR_CUDA, "adjoint events");
    }
  a.nwb = c->m.hasC ? 3 : 2;
  if (!(a.ckpt = adj_alloc(c, a.snaps * spec)) || !(a.phys = adj_alloc(c, 2 * a.unit_phys)) ||
      !(a.ub = adj_alloc(c, spec)) || !(a.n1acc = adj_alloc(c, spec)) || !(a.xaacc = adj_alloc(c, spec)) ||
      !(a.x1acc = adj_alloc(c, spec)) || !(a.ubar_in = adj_alloc(c, spec)) || !(a.ubar_out = adj_alloc(c, spec)) ||
      !(a.final_state = adj_alloc(c, spec)) || !(a.tmp = adj_alloc(c, spec)) || !(a.Wb = adj_alloc(c, a.nwb * wide)) ||
      !(a.Pb = adj_alloc(c, 3 * wide)) || !(a.etab = adj_alloc(c, plane)) ||
      (((c->cfg.module == GF_SINGLELAYERQG && c->m.hasC) || c->cfg.module == GF_MULTILAYERQG) &&
       (!(a.qxb = adj_alloc(c, plane)) || !(a.qyb = adj_alloc(c, plane)))) ||
      ((g.nl > 1 || c->m.drag) && !(a.nbar = adj_alloc(c, spec)))) {
    adj_release(c);
    return fail(c, GF_ERR_NOMEM, "adjoint buffers");
  }
  // unused padding columns of the accumulators stay zero
  for (void* p : {a.ub, a.n1acc, a.xaacc, a.x1acc, a.ubar_in, a.ubar_out, a.tmp})
    GF_CUDA(c, cudaMemsetAsync(p, 0, spec, c->stream));
  GF_CUDA(c, cudaMemsetAsync(a.Wb, 0, a.nwb * wide, c->stream));
  GF_CUDA(c, cudaMemsetAsync(a.Pb, 0, 3 * wide, c->stream));
  a.ck_t.assign(a.snaps, 0.0);
  a.ck_step.assign(a.snaps, 0);
  adj_schedule(c);
  a.ready = true;
  return GF_OK;
}

extern "C" int gf_adjoint_set_snapshots(gf_ctx* c, int32_t snapshots) {
  if (!c) return GF_ERR_ARG;
  DevGuard dg_(c->dev);
  auto& a = c->adj;
  if (!a.ready) return fail(c, GF_ERR_STATE, "call gf_adjoint_setup first");
  if (snapshots < 1) return fail(c, GF_ERR_ARG, "at least one snapshot (the initial state)");
  snapshots = std::min(snapshots, a.nseg);
  const size_t spec = c->g.bs_spec * c->cb;
  void* p = nullptr;
  if (cudaMalloc(&p, (size_t)snapshots * spec) != cudaSuccess) return fail(c, GF_ERR_NOMEM, "snapshots");
  GF_CUDA(c, cudaStreamSynchronize(c->stream));
  for (auto& q : a.mem) if (q == a.ckpt) { cudaFree(q); q = p; }
  a.ckpt = p;
  a.snaps = snapshots;
  a.ck_t.assign(a.snaps, 0.0);
  a.ck_step.assign(a.snaps, 0);
  a.forward_done = false;
  return adj_schedule(c);
}

extern "C" int gf_adjoint_info(const gf_ctx* c, int32_t* units, int32_t* snapshots, int64_t* unit_advances) {
  if (!c) return GF_ERR_ARG;
  if (units) *units = c->adj.nseg;
  if (snapshots) *snapshots = c->adj.snaps;
  if (unit_advances) *unit_advances = c->adj.forward_units;
  return GF_OK;
}

static int adj_store(gf_ctx* c, int slot) {
  auto& a = c->adj;
  const size_t spec = c->g.bs_spec * c->cb;
  GF_CUDA(c, cudaMemcpyAsync((char*)a.ckpt + slot * spec, c->sol, spec, cudaMemcpyDeviceToDevice, c->stream));
  a.ck_t[slot] = c->t;
  a.ck_step[slot] = c->step;
  return GF_OK;
}

static int adj_restore(gf_ctx* c, int slot) {
  auto& a = c->adj;
  const size_t spec = c->g.bs_spec * c->cb;
  GF_CUDA(c, cudaMemcpyAsync(c->sol, (char*)a.ckpt + slot * spec, spec, cudaMemcpyDeviceToDevice, c->stream));
  c->t = a.ck_t[slot];
  c->step = a.ck_step[slot];
  c->W_valid = false;
  return upload_clock(c);
}

// steps of units [u0, u0 + n)
static int64_t adj_unit_steps(const gf_ctx* c, int u0, int n) {
  const auto& a = c->adj;
  return std::min<int64_t>((int64_t)(u0 + n) * a.every, a.nsteps) - (int64_t)u0 * a.every;
}

// stepforward!(prob, nsteps) keeping the initial state and the snapshots of the schedule's
// first descent (the "spine"), so that the reverse sweep starts without recomputation.
extern "C" int gf_adjoint_forward(gf_ctx* c) {
  if (!c) return GF_ERR_ARG;
  DevGuard dg_(c->dev);
  clear_stale_error();
  auto& a = c->adj;
  if (!a.ready) return fail(c, GF_ERR_STATE, "call gf_adjoint_setup first");
  const size_t spec = c->g.bs_spec * c->cb;
  a.spine.clear();
  if (int r = adj_store(c, 0)) return r;
  int p = 0, n = a.nseg, sf = a.snaps - 1, slot = 1;
  while (n > 1 && sf > 0) {
    const int m = a.split[(size_t)n * a.snaps + sf];
    if (int r = gf_step(c, adj_unit_steps(c, p, m))) return r;
    p += m; n -= m; sf -= 1;
    if (int r = adj_store(c, slot)) return r;
    a.spine.push_back({p, slot++});
  }
  if (int r = gf_step(c, adj_unit_steps(c, p, n))) return r;
  GF_CUDA(c, cudaMemcpyAsync(a.final_state, c->sol, spec, cudaMemcpyDeviceToDevice, c->stream));
  a.t_end = c->t;
  a.step_end = c->step;
  a.forward_done = true;
  return GF_OK;
}

static AdjArgs adj_args(gf_ctx* c) {
  auto& d = c->adj;
  AdjArgs a{};
  a.filtered = c->filtered;
  a.cplx = c->cplxL;
  a.e = c->etd[0]; a.e2 = c->etd[1]; a.zeta = c->etd[2]; a.alpha = c->etd[3]; a.beta = c->etd[4]; a.gamma = c->etd[5];
  a.filt = c->filt;
  a.ub = d.ub; a.n1acc = d.n1acc; a.xaacc = d.xaacc; a.x1acc = d.x1acc;
  a.ubar_in = d.ubar_in; a.ubar_out = d.ubar_out; a.Wb = d.Wb; a.Pb = d.Pb; a.etab = d.etab;
  a.U = (c->cfg.module == GF_SINGLELAYERQG) ? c->cfg.U : 0.0;
  split_hl(a.U, &a.U_f, &a.U_l);
  a.rk4 = c->kind == SK_RK4;
  a.L = (c->kind == SK_RK4 && c->hasL) ? c->Ltab : nullptr;
  a.dt = c->cfg.dt;
  split_hl(a.dt, &a.dt_f, &a.dt_l);
  a.hasC = c->m.hasC;
  a.Qy1D = c->m.Qy1D; a.Qx2D = c->m.Qx2D; a.Qy2D = c->m.Qy2D;
  a.qxb = d.qxb; a.qyb = d.qyb;
  a.nbar = d.nbar;
  return a;
}

// The reverse sweep from the cotangent in adj.ubar_in (internal layout) to adj.ubar_out
// and adj.etab; the state and clock are the forward pass's result again afterwards.
// Recompute unit u from the current state with its forward fields kept, then run its
// transposed stages, last step first.  The recomputed steps skip the aliased modes: the
// transposed stages read only the kept forward fields (q + eta, u, v), and the state after
// the sweep is the stored forward result.
//
// Two streams: the recomputation (and every restore and advance before it) runs on the
// context stream into one half of d.phys, the transposed stages on d.ts from that half.  So
// the recomputation of the next unit of the sweep overlaps the transposed stages of this
// one -- they share only read-only tables -- and a recomputation into a half waits for the
// transposed stages that last read it.
static int adj_unit(gf_ctx* c, AdjArgs& a, int u) {
  auto& d = c->adj;
  const Geom& g = c->g;
  const size_t plane = (size_t)g.ny * g.nx * c->rb;
  const double dt = c->cfg.dt;
  const Bufs b = Bufs{c->twid, nullptr, nullptr};
  const int cnt = (int)adj_unit_steps(c, u, 1);
  const int k = d.half;
  d.half ^= 1;
  char* ph = (char*)d.phys + k * d.unit_phys;
  GF_CUDA(c, cudaStreamWaitEvent(c->stream, d.ev_adj[k], 0));  // no-op before the half's first use
  for (int i = 0; i < cnt; ++i) {
    if (int r = ensure_W(c)) return r;
    for (int stg = 1; stg <= 4; ++stg) {
      const double ts = c->t + (stg == 1 ? 0.0 : stg == 4 ? dt : 0.5 * dt);
      StepArgs s = stage_args(c, stg, ts);
      s.clk = c->dclk;
      c->row_phys = ph + ((size_t)i * 4 + stg - 1) * 3 * g.nl * plane;
      const int r = launch_stage(c, s, 1, c->g.kcut < c->g.nkr);
      c->row_phys = nullptr;
      if (r) return r;
    }
    advance_clock_kernel<<<1, 32, 0, c->stream>>>(c->dclk, dt, c->cfg.forcing_omega, c->cfg.forcing_phase,
                                                  c->cfg.forcing_kind == GF_FORCING_HARMONIC, c->nstages);
    GF_CUDA(c, cudaGetLastError());
    c->launches++;
    host_advance(c);
  }
  GF_CUDA(c, cudaEventRecord(d.ev_rec[k], c->stream));
  GF_CUDA(c, cudaStreamWaitEvent(d.ts, d.ev_rec[k], 0));
  for (int i = cnt - 1; i >= 0; --i) {
    for (int r = 4; r >= 1; --r) {
      a.stage = r;
      a.head = (r == 1) && !(u == 0 && i == 0);
      a.phys = ph + ((size_t)i * 4 + r - 1) * 3 * g.nl * plane;
      GF_CUDA(c, DISPATCH(c, launch_adj_row, g, a, b, d.ts));
      GF_CUDA(c, DISPATCH(c, launch_adj_col, g, c->m, a, b, d.ts));
      c->launches += 2;
    }
  }
  GF_CUDA(c, cudaEventRecord(d.ev_adj[k], d.ts));
  return GF_OK;
}

// Reverse units [p, p + n): the state at unit p is in slot sp, sf slots are free.
static int adj_rev(gf_ctx* c, AdjArgs& a, int p, int n, int sp, int sf, bool spine, std::vector<int>& freeslots,
                   size_t& spine_i) {
  auto& d = c->adj;
  if (n == 1) {
    if (int r = adj_restore(c, sp)) return r;
    return adj_unit(c, a, p);
  }
  if (sf == 0) {  // no slot left: advance from the start for each unit, last first
    for (int k = n - 1; k >= 0; --k) {
      if (int r = adj_restore(c, sp)) return r;
      if (k > 0) {
        if (int r = gf_step(c, adj_unit_steps(c, p, k))) return r;
        d.forward_units += k;
      }
      if (int r = adj_unit(c, a, p + k)) return r;
    }
    return GF_OK;
  }
  const int m = d.split[(size_t)n * d.snaps + sf];
  int q;
  if (spine && spine_i < d.spine.size() && d.spine[spine_i].first == p + m) {
    q = d.spine[spine_i++].second;  // stored by the forward pass
  } else {
    if (freeslots.empty()) return fail(c, GF_ERR_STATE, "adjoint schedule ran out of snapshot slots");
    q = freeslots.back();
    freeslots.pop_back();
    if (int r = adj_restore(c, sp)) return r;
    if (int r = gf_step(c, adj_unit_steps(c, p, m))) return r;
    d.forward_units += m;
    if (int r = adj_store(c, q)) return r;
  }
  if (int r = adj_rev(c, a, p + m, n - m, q, sf - 1, spine, freeslots, spine_i)) return r;
  freeslots.push_back(q);
  return adj_rev(c, a, p, m, sp, sf, false, freeslots, spine_i);
}

// The reverse sweep from the cotangent in adj.ubar_in (internal layout) to adj.ubar_out
// and adj.etab; the state and clock are the forward pass's result again afterwards.
static int adjoint_reverse(gf_ctx* c) {
  auto& d = c->adj;
  const Geom& g = c->g;
  const size_t spec = g.bs_spec * c->cb, plane = (size_t)g.ny * g.nx * c->rb;
  GF_CUDA(c, cudaMemsetAsync(d.etab, 0, plane, c->stream));
  if (d.qxb) {
    GF_CUDA(c, cudaMemsetAsync(d.qxb, 0, plane, c->stream));
    GF_CUDA(c, cudaMemsetAsync(d.qyb, 0, plane, c->stream));
  }
  AdjArgs a = adj_args(c);
  const Bufs b = Bufs{c->twid, nullptr, nullptr};
  // the transposed stages (stream d.ts) start after everything the context stream did so far
  // (the cotangent of the result, the cleared etab)
  GF_CUDA(c, cudaEventRecord(d.ev_sync, c->stream));
  GF_CUDA(c, cudaStreamWaitEvent(d.ts, d.ev_sync, 0));
  a.stage = 5;
  GF_CUDA(c, DISPATCH(c, launch_adj_col, g, c->m, a, b, d.ts));
  c->launches++;
  std::vector<int> freeslots;
  for (int k = d.snaps - 1; k >= 1 + (int)d.spine.size(); --k) freeslots.push_back(k);
  size_t spine_i = 0;
  d.forward_units = 0;  // unit advances the reverse sweep adds to the forward pass
  d.half = 0;
  if (int r = adj_rev(c, a, 0, d.nseg, 0, d.snaps - 1, true, freeslots, spine_i)) return r;
  // the context stream continues after the last transposed stage (ubar_out, etab)
  GF_CUDA(c, cudaEventRecord(d.ev_sync, d.ts));
  GF_CUDA(c, cudaStreamWaitEvent(c->stream, d.ev_sync, 0));
  if (d.qxb) {  // U(y), MultiLayerQG: Qx = d(eta)/dx + ..., Qy = ... + d(eta)/dy (bottom layer),
                //   so etabar -= d(Qxbar)/dx + d(Qybar)/dy (one-layer transforms)
    const size_t pf = (size_t)g.ny * g.nx * c->rb;
    char* ph = (char*)c->phys;
    Geom g1 = full_geom(c);
    g1.nl = 1;
    g1.nb = 1;
    const void* src[2] = {d.qxb, d.qyb};
    for (int k = 0; k < 2; ++k) {
      GF_CUDA(c, DISPATCH(c, launch_row_r2c, g1, bufs(c), 1, src[k], c->stream));
      GF_CUDA(c, DISPATCH(c, launch_col_fwd, g1, bufs(c), 1, d.tmp, 0, c->stream));
      GF_CUDA(c, DISPATCH(c, launch_col_inv, g1, c->m, d.tmp, (int)(k == 0 ? SF_DX : SF_DY), 0, bufs(c), c->stream));
      GF_CUDA(c, DISPATCH(c, launch_row_c2r, g1, bufs(c), 1, ph + k * pf, c->stream));
    }
    GF_CUDA(c, DISPATCH(c, launch_sub2, (size_t)g.ny * g.nx, d.etab, ph, ph + pf, c->stream));
  }
  GF_CUDA(c, cudaMemcpyAsync(c->sol, d.final_state, spec, cudaMemcpyDeviceToDevice, c->stream));
  c->t = d.t_end;
  c->step = d.step_end;
  c->W_valid = false;
  return upload_clock(c);
}

extern "C" int gf_adjoint_backward(gf_ctx* c, const void* sol_bar, void* sol0_bar, void* eta_bar, int where) {
  if (!c || !sol_bar) return GF_ERR_ARG;
  DevGuard dg_(c->dev);
  clear_stale_error();
  auto& d = c->adj;
  if (!d.forward_done) return fail(c, GF_ERR_STATE, "run gf_adjoint_forward first");
  if (eta_bar && c->cfg.module != GF_SINGLELAYERQG && c->cfg.module != GF_MULTILAYERQG)
    return fail(c, GF_ERR_ARG, "the topography gradient covers SingleLayerQG and MultiLayerQG");
  if (int r = copy_spec_in(c, d.ubar_in, sol_bar, where)) return r;
  if (int r = adjoint_reverse(c)) return r;
  if (sol0_bar)
    if (int r = copy_spec_out(c, sol0_bar, d.ubar_out, where)) return r;
  if (eta_bar)
    if (int r = copy_phys_out(c, eta_bar, d.etab, where, 1)) return r;
  if (where == GF_HOST) GF_CUDA(c, cudaStreamSynchronize(c->stream));
  return GF_OK;
}

extern "C" int gf_grad(gf_ctx* c, int loss_kind, void* dq0, void* deta, double* loss, int where) {
  if (!c) return GF_ERR_ARG;
  DevGuard dg_(c->dev);
  clear_stale_error();
  if (loss_kind != GF_LOSS_KINETIC_ENERGY) return fail(c, GF_ERR_ARG, "unknown loss");
  auto& d = c->adj;
  if (!d.ready) return fail(c, GF_ERR_STATE, "call gf_adjoint_setup first");
  if (deta && c->cfg.module != GF_SINGLELAYERQG && c->cfg.module != GF_MULTILAYERQG)
    return fail(c, GF_ERR_ARG, "the topography gradient covers SingleLayerQG and MultiLayerQG");
  if (int r = gf_adjoint_forward(c)) return r;
  // loss: SingleLayerQG.kinetic_energy / TwoDNavierStokes.energy / the total kinetic energy of
  // MultiLayerQG.energies of the final state
  const bool ml = c->cfg.module == GF_MULTILAYERQG;
  LayerWeights hw{};
  for (int L = 0; L < c->g.nl; ++L) hw.w[L] = (ml && c->g.nl > 1) ? c->Hl[L] / c->Hsum : 1.0;
  if (loss) {
    std::vector<int32_t> ids(ml ? c->g.nl : 1);
    for (size_t q = 0; q < ids.size(); ++q) ids[q] = (int32_t)q;
    std::vector<double> v(ids.size());
    if (int r = gf_diagnostics(c, ids.data(), (int32_t)ids.size(), v.data())) return r;
    *loss = 0;
    for (double x : v) *loss += x;
  }
  if (ml) GF_CUDA(c, DISPATCH(c, launch_adj_spec_ml, c->g, c->m, hw, c->sol, d.ubar_in, 0, c->stream));
  else GF_CUDA(c, DISPATCH(c, launch_adj_spec, c->g, c->m, c->sol, d.ubar_in, 0, c->stream));
  if (int r = adjoint_reverse(c)) return r;
  if (dq0) {  // gradient with respect to q0 in set_q!(prob, q0): rfft^T of the dealiased cotangent
    // (MultiLayerQG set_q! and SurfaceQG set_b! remove the k = 0 mode: so does its cotangent)
    if (ml || c->cfg.module == GF_SURFACEQG)
      GF_CUDA(c, DISPATCH(c, launch_adj_spec_ml, c->g, c->m, hw, d.ubar_out, d.tmp, 1, c->stream));
    else GF_CUDA(c, DISPATCH(c, launch_adj_spec, c->g, c->m, d.ubar_out, d.tmp, 1, c->stream));
    const size_t pf = (size_t)c->g.nl * c->g.ny * c->g.nx * c->rb;
    void* ph = (char*)c->phys + 3 * pf;
    if (int r = inv_transform(c, d.tmp, SF_RAW, 0, ph)) return r;
    if (int r = copy_phys_out(c, dq0, ph, where)) return r;
  }
  if (deta)
    if (int r = copy_phys_out(c, deta, d.etab, where, 1)) return r;
  if (where == GF_HOST) GF_CUDA(c, cudaStreamSynchronize(c->stream));
  return GF_OK;
}
