// Internal (non-ABI) declarations shared by the C-ABI layer and the kernel translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

namespace gf {

struct df64;
template <class T> struct cplx;

enum Module { MOD_TWODNS = 0, MOD_SLQG = 1, MOD_MLQG = 2, MOD_SQG = 3, MOD_QGQL = 4 };
enum StepKind { SK_FE = 0, SK_RK4 = 1, SK_ETDRK4 = 2, SK_AB3 = 3, SK_NOUT = 4 /* write N to acc (calcN!) */ };
enum PsiKind { PSI_INVK2 = 0, PSI_HELMHOLTZ = 1, PSI_TABLE = 2, PSI_EIGEN = 3 };
enum ForceKind { FK_NONE = 0, FK_STATIC = 1, FK_HARMONIC = 2, FK_STOCH = 3, FK_STOCH_PHASE = 4 };
constexpr int MAXL = 8;  // largest number of layers
constexpr int MAXP = 16; // passes of a generic-length FFT plan
constexpr int MAXPRIME = 61;  // largest prime factor of a generic length

// Grid geometry in the internal layout: spectral arrays are [layer][j][kr] with row stride
// ldk (>= nkr); the pruned inverse intermediates are [field][layer][j][kr < kcut] with row
// stride ldw; physical arrays are [layer][j][i] with row stride nx.
struct Geom {
  int nx, ny, nkr, ldk, ldw, nl;
  int kcut;    // kr indices >= kcut are aliased
  int lA, lB;  // l indices in [lA, lB] are aliased (empty when lA > lB)
  double dkx, dky, inv_nxny;
  float dkx_f, dky_f, inv_nxny_f;  // float copies (the FP32 kernels never touch FP64)
  float dkx_l, dky_l, inv_nxny_l;  // low words: (x_f, x_l) is the df64 value
  int cs;                          // column stride (elements) of the column kernels' buffers
  // step-kernel launches of an unobserved step: only columns kr < kout of the products are
  // formed and only the kept modes of the state are updated (0: every column, every mode)
  int kout;
  // batch of independent instances (an ensemble): instance blockIdx.y of every kernel works
  // on its own slice; strides (elements) of the per-instance arrays
  int nb;
  size_t bs_spec, bs_w, bs_p, bs_d, bs_phys;
  // launch shape chosen by gf_autotune (0: the block-shape heuristic): column-kernel columns
  // per block and FFT radix, row-kernel row pairs per block and FFT radix
  int tuneC, tuneRc, tuneB, tuneRr;
  // columns per block of the TMA column stage (0: the cp.async column kernel)
  int tmaC;
  // field-parallel small-grid kernels (gf_fpar.cuh): row-kernel radix, column-kernel radix
  // and columns per block (radix 0: the classic kernel)
  int fpR, fpRc, fpC;
  // generic-length transforms (lengths other than the powers of two 32 ... 2048 that have
  // their own kernels): rtx for the x direction (rows, length nx), rty for y (columns, ny),
  // with their radix plans (product = the length)
  int rtx, rty, npx, npy;
  int plx[MAXP], ply[MAXP];
};

// Device-resident clock, advanced on the GPU after every step so that a captured graph of
// several steps can be replayed: stage forcing scales for the harmonic forcing of the step
// about to run, and the step number used by the stochastic draws and AB3's start-up.
struct DevClock {
  double t;
  long long step;
  double fs[4];
  float fs_f[4], fs_l[4];
};

// How psi-hat follows from the layer PV/vorticity/buoyancy X, and what the physical-space
// products are.  The inverse fields of every layer are (X, -i l psi, i kr psi) = (q, u, v).
struct ModArgs {
  int module, psi_kind;
  double ell_inv2;       // 1/ell^2 for PSI_HELMHOLTZ
  const void* mult;      // PSI_TABLE: real [j][kr] table, psi = -mult * X
  // PSI_EIGEN: S_k^-1 = V diag(1/(lam - K^2)) Vinv (K = 0 -> 0)
  double lam[MAXL], V[MAXL * MAXL], Vinv[MAXL * MAXL];
  // physical-space products
  int hasB, hasC, linear;
  int ql;  // BarotropicQGQL: products (U z' + u' Z, v' Z, v' z'), N by kr column (zonal mean / eddies)
  const void* eta;       // real [j][i] or null: q' = q + eta
  const void* U1D;       // real [layer][j] or null: u' = u + U
  const void* Qy1D;      // real [layer][j] or null
  const void* Qx2D;      // real [j][i] or null (last layer)
  const void* Qy2D;      // real [j][i] or null (last layer)
  // spectral-side extras
  const void* etah;      // complex [j][kr] or null: N -= i kr U0 etah
  double U0;
  int drag; double mu;   // N_last += mu K^2 psi_last (MultiLayerQG bottom drag)
  // dissipation parameters used by the diagnostics (nu, nnu; mu_visc, nmu)
  double nu, mu_visc; int nnu, nmu;
  void* D;               // complex [j][kr] buffer carrying mu K^2 psi_last between kernels
  int Ueta;              // U0 != 0 and etah present
  float ell_inv2_f, U0_f, mu_f;
  float lam_f[MAXL], V_f[MAXL * MAXL], Vinv_f[MAXL * MAXL];
  float ell_inv2_l, U0_l, mu_l;
  float lam_l[MAXL], V_l[MAXL * MAXL], Vinv_l[MAXL * MAXL];
};

struct StepArgs {
  int kind, stage, filtered, hasL, cplxL, ab3_euler, do_fwd, do_inv;
  double dt;
  const void *Ltab, *filt, *e, *e2, *zeta, *alpha, *beta, *gamma;  // [j][kr]
  void *sol, *X, *acc, *s1, *N1, *Rm1, *Rm2, *Rout;                // [layer][j][kr]
  // forcing
  int fkind, draw;
  double fscale;
  const void* Fh;      // static / harmonic F-hat, or the stored stochastic draw
  const void* fspec;   // real [j][kr]: sqrt(spectrum / dt) (stochastic)
  void* Fstore;        // stochastic draw written at the first stage
  void* prevsol;       // sol at the first stage (stochastic budgets)
  uint64_t seed, step;
  float dt_f, fscale_f, dt_l, fscale_l;
  const DevClock* clk;  // if set, step / fscale / AB3 start-up come from the device clock
  // several layers: column stage as two launches over (column block, layer) -- see the
  // column kernel; Xg holds the next stage's X of every layer between them
  int layer_split;
  void* Xg;
};

// value of a host-prepared scalar (double d, its float rounding h and the remainder l) in
// the arithmetic type T; the kernels never convert doubles at run time
template <class T> __host__ __device__ __forceinline__ T sel(double d, float h, float l);
template <> __host__ __device__ __forceinline__ double sel<double>(double d, float, float) { return d; }
template <> __host__ __device__ __forceinline__ float sel<float>(double, float h, float) { return h; }
template <> __host__ __device__ __forceinline__ df64 sel<df64>(double, float h, float l) { return df64(h, l); }
// split a double into the (h, l) pair used by sel
inline void split_hl(double d, float* h, float* l) {
  *h = (float)d;
  *l = (float)(d - (double)*h);
}

// Tensor maps (CUtensorMap, 128 bytes each) of P (tile loads) and W (tile stores) for the TMA
// column stage, one pair per candidate column count Cs[i] of a block.
struct TmaMaps {
  alignas(64) unsigned char p[2][128];
  alignas(64) unsigned char w[2][128];
  int Cs[2] = {0, 0};
  bool ok = false;
};

struct Bufs {
  const void* twid;       // TWN twiddles
  void* W;                // [3][layer][j][ldw]
  void* P;                // [3][layer][j][ldk]
  void* phys = nullptr;   // row kernel: also store (q + eta, u, v) [3][layer][j][nx] (adjoint recompute)
  const TmaMaps* tma = nullptr;  // host copy of the context's tensor maps (null: no TMA column stage)
  int* derr = nullptr;           // device error flag (a TMA wait that ran out of time sets it)
  const void* twx = nullptr;     // generic-length path: exp(-2 pi i k / nx), k < nx
  const void* twy = nullptr;     //                      exp(-2 pi i k / ny), k < ny
};

// Arguments of the adjoint kernels (gf_adjoint.cuh).
struct AdjArgs {
  int stage;      // 4..1: the forward stage whose calcN! is transposed; 5: start a step from ubar_in
  int head;       // stage 1: also start the previous step from the result
  int filtered, cplx;
  const void *e, *e2, *zeta, *alpha, *beta, *gamma, *filt;
  void *ub, *n1acc, *xaacc, *x1acc;   // [j][ldk] cotangent accumulators
  const void* ubar_in;                // stage 5: cotangent of the step's result
  void* ubar_out;                     // stage 1: cotangent of the step's initial state
  void *Wb, *Pb;                      // [2][j][ldk] y-inverse (abar, bbar) spectra; [3][j][ldk] products
  const void* phys;                   // forward (q + eta, u, v) of the stage, [3][j][nx]
  void* etab;                         // [j][nx] cotangent of eta
  double U; float U_f, U_l;
  // RK4 / FilteredRK4: the linear operator L ([j][kr], null when the step has none) and dt
  int rk4;
  const void* L;
  double dt; float dt_f, dt_l;
  // U(y) (SingleLayerQG): the third product C = (U + u) Qx + v Qy, its cotangent field in Wb,
  // the PV gradients (Qy1D [j], Qx2D / Qy2D [j][nx] or null) and the physical accumulators of
  // the cotangents of Qx and Qy ([j][nx]) from which the topography gradient follows
  int hasC;
  const void *Qy1D, *Qx2D, *Qy2D;
  void *qxb, *qyb;
  // several layers or bottom drag (MultiLayerQG): Nbar of the current stage of every layer,
  // [layer][j][ldk], written by each column launch for the next (the drag term reads it)
  void* nbar;
};

// Generic transforms (updatevars!, set_*!, fwdtransform!/invtransform!).
enum SpecField { SF_X = 0, SF_PSI = 1, SF_U = 2, SF_V = 3, SF_UY = 4, SF_RAW = 5, SF_DX = 6, SF_DY = 7 };

// Persistent ensemble launch (gf_ens.cu): one row launch and one column launch per stage for
// several size classes (contexts) at once; each block walks the work list of every class's
// tiles (class, instance, row-pair block or column block).  Square classes of 32, 64, 128 or
// 256 points, one layer, no bottom drag.
constexpr int ENS_MAXCLS = 4;
constexpr int ENS_THREADS = 128;
struct EnsClass {
  Geom g;
  ModArgs m;
  StepArgs s;   // column launches
  Bufs b;
  int n;        // FFT length (nx = ny)
  int per;      // row pairs (row launch) or columns (column launch) per block
  int nbx, nby; // blocks per instance, instances
};
struct EnsArgs {
  int ncls, total;  // classes, work items (sum of nbx * nby)
  EnsClass c[ENS_MAXCLS];
};
bool ens_size_ok(int n);
int ens_per_block(int n);  // row pairs and columns per block of ENS_THREADS threads
template <class T> cudaError_t launch_ens_row(const EnsArgs&, cudaStream_t);
template <class T> cudaError_t launch_ens_col(const EnsArgs&, cudaStream_t);
template <class T> size_t ens_col_stride(int n);

// field-parallel small-grid launchers (gf_fpar.cuh, gf_fp_<type>.cu), used by the dispatchers
// when Geom::fpR / fpRc is set: one layer without bottom drag, power-of-two lengths 32 ... 512,
// radix 2, 4 or 8, blocks of 3 x (columns) x length / radix <= FP_MAXT threads
constexpr int FP_MAXT = 384;
// the radices a small-grid context starts with (gf_autotune may change them): rows 4, columns
// 2 up to 128 points and 4 above (measured on TwoDNavierStokes 64^2 ... 256^2, FP32/FP64/df64)
inline int fp_default_row_radix(int) { return 4; }
inline int fp_default_col_radix(int ny) { return ny <= 128 ? 2 : 4; }
inline bool fp_len_ok(int n) { return n == 32 || n == 64 || n == 128 || n == 256 || n == 512; }
inline bool fp_radix_ok(int n, int R) { return (R == 2 || R == 4 || R == 8) && 3 * (n / R) <= FP_MAXT; }
inline bool fp_cols_ok(int n, int R, int C) { return C >= 1 && C <= 8 && 3 * C * (n / R) <= FP_MAXT; }
template <class T> cudaError_t launch_row_fp(const Geom&, const ModArgs&, const Bufs&, cudaStream_t);
template <class T> cudaError_t launch_col_fp(const Geom&, const ModArgs&, const StepArgs&, const Bufs&, cudaStream_t);
template <class T> cudaError_t launch_adj_row_fp(const Geom&, const AdjArgs&, const Bufs&, cudaStream_t);
template <class T>
cudaError_t launch_adj_col_fp(const Geom&, const ModArgs&, const AdjArgs&, const Bufs&, cudaStream_t);

// generic-length launchers (gf_rt.cu), used by the dispatchers when Geom::rtx / rty is set
template <class T> cudaError_t launch_row_rt(const Geom&, const ModArgs&, const Bufs&, cudaStream_t);
template <class T> cudaError_t launch_col_rt(const Geom&, const ModArgs&, const StepArgs&, const Bufs&, cudaStream_t);
template <class T> cudaError_t launch_col_inv_rt(const Geom&, const ModArgs&, const void* src, int kind, int mask,
                                                 const Bufs&, cudaStream_t);
template <class T> cudaError_t launch_row_c2r_rt(const Geom&, const Bufs&, int nf, void* out, cudaStream_t);
template <class T> cudaError_t launch_row_r2c_rt(const Geom&, const Bufs&, int nf, const void* in, cudaStream_t);
template <class T> cudaError_t launch_col_fwd_rt(const Geom&, const Bufs&, int nf, void* out, int zero_mean,
                                                 cudaStream_t);

template <class T> cudaError_t launch_row(const Geom&, const ModArgs&, const Bufs&, cudaStream_t);
template <class T> cudaError_t launch_col(const Geom&, const ModArgs&, const StepArgs&, const Bufs&, cudaStream_t);
template <class T> cudaError_t launch_col_inv(const Geom&, const ModArgs&, const void* src, int kind, int mask,
                                              const Bufs&, cudaStream_t);
template <class T> cudaError_t launch_row_c2r(const Geom&, const Bufs&, int nf, void* out, cudaStream_t);
template <class T> cudaError_t launch_row_r2c(const Geom&, const Bufs&, int nf, const void* in, cudaStream_t);
template <class T> cudaError_t launch_col_fwd(const Geom&, const Bufs&, int nf, void* out, int zero_mean,
                                              cudaStream_t);
template <class T> cudaError_t launch_diag(const Geom&, const ModArgs&, const void* sol, const void* prevsol,
                                           const void* Fh, uint32_t mask, double* partial, int nblocks,
                                           cudaStream_t);
template <class T> cudaError_t launch_mask_inplace(const Geom&, void* sol, cudaStream_t);
template <class T> cudaError_t launch_spec_apply(const Geom&, const ModArgs&, const void* in, void* out, int op,
                                                 cudaStream_t);

template <class T> cudaError_t launch_adj_row(const Geom&, const AdjArgs&, const Bufs&, cudaStream_t);
template <class T> cudaError_t launch_adj_col(const Geom&, const ModArgs&, const AdjArgs&, const Bufs&, cudaStream_t);
// element-wise adjoint helpers: op 0 kinetic-energy gradient, op 1 rfft^T preparation (see gf_dispatch.cu)
template <class T> cudaError_t launch_adj_spec(const Geom&, const ModArgs&, const void* in, void* out, int op,
                                               cudaStream_t);

// per-layer weights (H_j / sum H) of the MultiLayerQG kinetic-energy loss
struct LayerWeights { double w[MAXL]; };
template <class T> cudaError_t launch_adj_spec_ml(const Geom&, const ModArgs&, const LayerWeights&, const void* in,
                                                  void* out, int op, cudaStream_t);

// out -= a + b over n physical elements (gf_dispatch.cu)
template <class T> cudaError_t launch_sub2(size_t n, void* out, const void* a, const void* b, cudaStream_t);

// MultiLayerQG fluxes: per-block partial sums (gf_dispatch.cu)
template <class T> cudaError_t launch_flux(const Geom&, const void* v, const void* uy, const void* psi, const double* U,
                                           double* partial, int nblocks, cudaStream_t);

// message returned by gf_last_error(NULL)
void set_global_error(const std::string& msg);

constexpr int DIAG_BLOCK = 256;
constexpr int NDIAG = 24;  // number of reduction slots
}  // namespace gf
