/* libgfcuda -- C ABI of the GB300 (sm_103a) pseudospectral time step.
 *
 * Drop-in boundary for the hot path of GeophysicalFlows.jl v0.16.5 / FourierFlows.jl 0.10.5:
 * Problem construction, stepforward!, calcN!, updatevars!, set_*! and the Parseval-sum
 * diagnostics of TwoDNavierStokes, SingleLayerQG, MultiLayerQG and SurfaceQG.  Every call
 * returns GF_OK (0) or a negative gf_status; gf_last_error() gives the message.  A call that
 * launches GPU work first consumes a non-sticky CUDA runtime error that earlier calls of the
 * caller's thread left pending (cudaGetLastError), so that it is not reported as the call's
 * own; check your own runtime calls before calling into the library.
 *
 * Array conventions (identical to the reference's Julia arrays, column-major):
 *   spectral  (nkr, ny[, nlayers]) complex, nkr = nx/2 + 1, element (ik, j, L) at
 *             ik + nkr*(j + ny*L);   physical (nx, ny[, nlayers]) real, (i, j, L) at
 *             i + nx*(j + ny*L).
 *   Element type: float/complex-float for GF_F32 contexts, double/complex-double otherwise
 *   (GF_F64 and GF_DF64).
 *   `where` = GF_HOST (pageable or pinned host memory) or GF_DEVICE (device pointer on the
 *   context's GPU, e.g. from a CuArray).
 * One context = one problem on one stream; a context is not thread-safe, separate
 * contexts are independent.  A context belongs to the device that was current at gf_create:
 * every call on it runs there and gives the caller back its own current device on return.
 * Grid sizes: nx and ny even, at least 4, with no prime factor above 61 and at most 4096
 * (GF_F32) or 2048 (GF_F64, GF_DF64) -- the sizes FourierFlows' TwoDGrid accepts in practice,
 * e.g. the reference tests' 128 x 126, 64 x 66, 32 x 34 and 16 x 16 (FourierFlows also takes
 * odd sizes and larger primes; those return GF_ERR_UNSUPPORTED here).  The powers of two 32
 * ... 2048 run compiled-in FFT lengths (fastest; the TMA column stage, the autotuner and the
 * adjoint need them); every other length runs a mixed-radix FFT over a run-time radix plan.
 */
#ifndef GFCUDA_H
#define GFCUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GFCUDA_ABI_VERSION 1

typedef struct gf_ctx gf_ctx;

typedef enum {
  GF_OK = 0,
  GF_ERR_ARG = -1,          /* invalid argument / configuration */
  GF_ERR_UNSUPPORTED = -2,  /* valid for the reference but not supported here (e.g. nx not 2^k) */
  GF_ERR_CUDA = -3,         /* CUDA runtime error */
  GF_ERR_NOMEM = -4,        /* device allocation failed */
  GF_ERR_STATE = -5,        /* call not valid in the current state */
  GF_ERR_NOT_IMPLEMENTED = -6 /* the reference raises for this case (e.g. finite deformation radius budgets) */
} gf_status;

/* GF_BAROTROPICQGQL: the quasi-linear barotropic QG module (src/barotropicqgql.jl): zonal mean
 * (kr = 0) and eddies (kr > 0) advected quasi-linearly; parameters beta, nu, nnu, mu (linear
 * drag), eta (kept, unused by the advection as in the reference). */
typedef enum { GF_TWODNAVIERSTOKES = 0, GF_SINGLELAYERQG = 1, GF_MULTILAYERQG = 2, GF_SURFACEQG = 3,
               GF_BAROTROPICQGQL = 4 } gf_module;

/* GF_F64: IEEE double throughout.  GF_F32: float bulk (FFTs, products, stage combination);
 * FP64 stays in the setup (ETDRK4 coefficients, inversion factorisation) and in the
 * diagnostics reductions.  GF_DF64: the FP64-plain mode computed in double-float
 * arithmetic (48-bit significand from pairs of floats; GB300's FP64 units are a small
 * fraction of its FP32 throughput); arrays at the ABI are double/complex-double as for
 * GF_F64, and setup and diagnostics are FP64. */
typedef enum { GF_F32 = 0, GF_F64 = 1, GF_DF64 = 2 } gf_precision;

/* FourierFlows timestepper names (test/runtests.jl:58) */
typedef enum {
  GF_FORWARDEULER = 0, GF_FILTEREDFORWARDEULER = 1, GF_RK4 = 2, GF_FILTEREDRK4 = 3,
  GF_ETDRK4 = 4, GF_FILTEREDETDRK4 = 5, GF_AB3 = 6, GF_FILTEREDAB3 = 7
} gf_stepper;

/* Forcing kinds: the device-side forms of the reference's calcF! callbacks.
 *   STATIC:     F-hat fixed (set with gf_set_forcing; e.g. test/test_twodnavierstokes.jl:237-241)
 *   HARMONIC:   F-hat * cos(omega t + phase), evaluated at every stage time
 *               (test/test_twodnavierstokes.jl:136-141)
 *   STOCHASTIC: randn(complex) * sqrt(spectrum / dt), drawn once per step at the first stage
 *               with Philox4x32-10 (examples/singlelayerqg_betaforced.jl:86-90); `stochastic=true`
 *               semantics (prevsol kept, Stratonovich budgets)
 *   STOCHASTIC_PHASE: exp(2 pi i u) * sqrt(spectrum / dt), [0,0] = 0 (test/test_twodnavierstokes.jl:41-46) */
typedef enum {
  GF_FORCING_NONE = 0, GF_FORCING_STATIC = 1, GF_FORCING_HARMONIC = 2,
  GF_FORCING_STOCHASTIC = 3, GF_FORCING_STOCHASTIC_PHASE = 4
} gf_forcing_kind;

typedef enum { GF_HOST = 0, GF_DEVICE = 1 } gf_where;

/* Problem configuration: the keyword arguments of the four modules' Problem() constructors
 * (src/twodnavierstokes.jl:71-89, src/singlelayerqg.jl:91-112, src/multilayerqg.jl:87-114,
 * src/surfaceqg.jl:76-90).  Zero-initialise, then set what the module needs. */
typedef struct gf_config {
  int32_t module, precision, stepper;
  int32_t nx, ny, nlayers;          /* nlayers: MultiLayerQG only (1..8); others use 1 */
  double Lx, Ly, dt, aliased_fraction;
  /* (hyper)viscosity: TwoDNavierStokes nu, nnu, mu, nmu; SingleLayerQG nu, nnu, mu (drag);
   * MultiLayerQG nu, nnu, mu (bottom drag); SurfaceQG nu, nnu */
  double nu, mu;
  int32_t nnu, nmu;
  /* SingleLayerQG / MultiLayerQG */
  double beta;
  double deformation_radius;        /* SingleLayerQG; <= 0 or inf = barotropic */
  double U;                         /* SingleLayerQG constant U (used when U_y is NULL) */
  const double* U_y;                /* SingleLayerQG U(y) [ny] or NULL; MultiLayerQG U [nlayers*ny]
                                       (layer-major, U_y[L*ny + j]) or NULL for zero */
  const double* eta;                /* topographic PV (nx, ny) physical, or NULL for flat */
  double f0;                        /* MultiLayerQG */
  const double* H;                  /* MultiLayerQG rest layer depths [nlayers] */
  const double* b;                  /* MultiLayerQG layer buoyancies [nlayers] */
  double topographic_pv_gradient[2];/* MultiLayerQG */
  int32_t linear;                   /* MultiLayerQG linear=true */
  double H_sqg;                     /* SurfaceQG layer depth; <= 0 or inf = infinite depth */
  /* forcing */
  int32_t forcing_kind;
  uint64_t seed;
  double forcing_omega, forcing_phase;
  /* spectral filter of the Filtered* steppers (FourierFlows makefilter); 0 = defaults
   * order=4, innerK=0.65, outerK=1 */
  double filter_order, filter_innerK, filter_outerK;
  /* ETDRK4 contour (FourierFlows getetdcoeffs); 0 = defaults ncirc=32, rcirc=1 */
  int32_t etdrk4_ncirc;
  double etdrk4_rcirc;
  /* ensemble: number of independent instances of this problem in the context (0 or 1 =
   * one).  Instances share grid, parameters and stepper; each has its own state, forcing
   * draws (Philox key seed + instance) and diagnostics.  Arrays at the ABI gain a leading
   * (slowest) instance dimension. */
  int32_t batch;
} gf_config;

/* Field selectors for gf_get_field / gf_set_physical */
typedef enum {
  GF_FIELD_Q = 0,     /* TwoDNavierStokes zeta / SingleLayerQG, MultiLayerQG q / SurfaceQG b */
  GF_FIELD_PSI = 1,
  GF_FIELD_U = 2,
  GF_FIELD_V = 3,
  /* BarotropicQGQL (src/barotropicqgql.jl:380-407): Q/PSI/U/V are the eddy (kr > 0) zeta, psi,
   * u, v; these are the zonal-mean Zeta, Psi and U */
  GF_FIELD_ZETA_MEAN = 4, GF_FIELD_PSI_MEAN = 5, GF_FIELD_U_MEAN = 6
} gf_field;

/* Diagnostic selectors (gf_diagnostics).  Values are the reference functions' values. */
typedef enum {
  /* TwoDNavierStokes (src/twodnavierstokes.jl:374-535) */
  GF_D_2DNS_ENERGY = 0, GF_D_2DNS_ENSTROPHY = 1, GF_D_2DNS_PALINSTROPHY = 2,
  GF_D_2DNS_ENERGY_DISSIPATION_HYPERVISCOSITY = 3, GF_D_2DNS_ENERGY_DISSIPATION_HYPOVISCOSITY = 4,
  GF_D_2DNS_ENSTROPHY_DISSIPATION_HYPERVISCOSITY = 5, GF_D_2DNS_ENSTROPHY_DISSIPATION_HYPOVISCOSITY = 6,
  GF_D_2DNS_ENERGY_WORK = 7, GF_D_2DNS_ENSTROPHY_WORK = 8,
  /* SingleLayerQG (src/singlelayerqg.jl:546-715) */
  GF_D_SLQG_KINETIC_ENERGY = 0, GF_D_SLQG_POTENTIAL_ENERGY = 1, GF_D_SLQG_ENSTROPHY = 2,
  GF_D_SLQG_ENERGY_DISSIPATION = 3, GF_D_SLQG_ENSTROPHY_DISSIPATION = 4, GF_D_SLQG_ENERGY_WORK = 5,
  GF_D_SLQG_ENSTROPHY_WORK = 6, GF_D_SLQG_ENERGY_DRAG = 7, GF_D_SLQG_ENSTROPHY_DRAG = 8,
  GF_D_SLQG_ENERGY = 9,
  /* SurfaceQG (src/surfaceqg.jl:390-483) */
  GF_D_SQG_KINETIC_ENERGY = 0, GF_D_SQG_BUOYANCY_VARIANCE = 1, GF_D_SQG_TOTAL_3D_ENERGY = 2,
  GF_D_SQG_BUOYANCY_DISSIPATION = 3, GF_D_SQG_BUOYANCY_WORK = 4,
  /* MultiLayerQG energies (src/multilayerqg.jl:918-951): KE_j = j, PE_{j+1/2} = nlayers + j */
  GF_D_MLQG_KE0 = 0, GF_D_MLQG_PE0 = 8,
  /* BarotropicQGQL (src/barotropicqgql.jl:433-510) */
  GF_D_QGQL_ENERGY = 0, GF_D_QGQL_ENSTROPHY = 1, GF_D_QGQL_DISSIPATION = 2, GF_D_QGQL_WORK = 3,
  GF_D_QGQL_DRAG = 4
} gf_diag;

/* ---- lifetime ------------------------------------------------------------------------- */
/* Replaces Problem(dev; kw...) (e.g. src/twodnavierstokes.jl:71-100,
 * src/multilayerqg.jl:87-135): grid, params, vars, equation (L) and timestepper state
 * (ETDRK4 coefficients, filter) are built on the GPU.  `stream` is a cudaStream_t or NULL. */
int gf_create(const gf_config* cfg, void* stream, gf_ctx** out);
int gf_destroy(gf_ctx* ctx);
/* Message of the last failed call on ctx (or of the last failed gf_create when ctx is NULL). */
const char* gf_last_error(const gf_ctx* ctx);
int gf_abi_version(void);
/* Sizes: nkr, nl(=ny), nlayers, element size in bytes of a real value */
int gf_get_dims(const gf_ctx* ctx, int32_t* nkr, int32_t* ny, int32_t* nlayers, int32_t* real_bytes);

/* ---- state (prob.sol, prob.clock) ----------------------------------------------------- */
/* prob.sol as a (ny, nkr) complex array per layer and instance (nkr fastest, Julia's memory
 * order), in the context's arithmetic type (complex128 for GF_DF64).  where = GF_HOST: the call
 * returns when the copy is complete, so the caller may reuse its buffer; a page-locked buffer
 * (cudaMallocHost, cudaHostAlloc, cudaHostRegister; CUDA.jl's pinned arrays) lying in one
 * allocation is read or written by the library's re-pitch kernel directly, a pageable one goes
 * through a copy into a staging buffer.  where = GF_DEVICE: stream-ordered device copies. */
int gf_set_state(gf_ctx* ctx, const void* sol, int where);
int gf_get_state(gf_ctx* ctx, void* sol, int where);
int gf_get_clock(const gf_ctx* ctx, double* t, int64_t* step);
int gf_set_clock(gf_ctx* ctx, double t, int64_t step);

/* set_zeta!/set_q!/set_b! (src/twodnavierstokes.jl:352-360, src/singlelayerqg.jl:525-534,
 * src/surfaceqg.jl:356-364, src/multilayerqg.jl:842-870) with which = GF_FIELD_Q, and
 * MultiLayerQG set_psi! (src/multilayerqg.jl:872-894) with which = GF_FIELD_PSI: forward
 * transform of a physical field into sol (domain mean zeroed where the reference does),
 * then updatevars!. */
int gf_set_physical(gf_ctx* ctx, int which, const void* field, int where);

/* ---- the hot path ----------------------------------------------------------------------- */
/* stepforward!(prob, nsteps) (FourierFlows; calls calcN! 4x per ETDRK4/RK4 step).  Every
 * calcN! starts with dealias!(sol), so the aliased modes of a step's result are read by no
 * later step: only the last step of the call (AB3: the last three) computes them; the others
 * form the products for the kept kr columns only and update the kept modes only.  The state
 * the call leaves (every mode), and the clock, are bit for bit those of nsteps calls of one
 * step each (to FP32 rounding where the autotuner gave the inner steps wider column blocks
 * than the last step's, see gf_autotune). */
int gf_step(gf_ctx* ctx, int64_t nsteps);
/* stepforward!(prob, diags, nsteps): also records the diagnostics `which[0..nd)` after
 * every step into out[step*nd + d] (host memory, nsteps*nd doubles). */
int gf_step_diags(gf_ctx* ctx, int64_t nsteps, const int32_t* which, int32_t nd, double* out);
/* One calcN!(N, sol, t, ...) evaluation (e.g. src/twodnavierstokes.jl:286-294) on
 * caller arrays; like the reference it dealiases `sol` in place. */
int gf_calcN(gf_ctx* ctx, void* N, void* sol, double t, int where);

/* updatevars!(prob) (src/twodnavierstokes.jl:331-345 and siblings): dealias sol in place and
 * compute the physical fields; gf_get_field copies one of them out. */
int gf_updatevars(gf_ctx* ctx);
int gf_get_field(gf_ctx* ctx, int which, void* out, int where);

/* MultiLayerQG.fluxes(prob) (src/multilayerqg.jl:977-1022), after updatevars!: the lateral eddy
 * fluxes H_j / V sum U_j v_j du_j/dy dx dy per layer (lateral[batch][nlayers]) and the vertical
 * eddy fluxes f0^2 / (g'_{j+1/2} V) sum (U_j - U_{j+1}) v_{j+1} psi_j dx dy per interface
 * (vertical[batch][nlayers-1], may be NULL for one layer), V = Lx Ly sum(H); FP64 sums. */
int gf_fluxes(gf_ctx* ctx, double* lateral, double* vertical);

/* GeophysicalFlows.peakedisotropicspectrum(grid, kpeak, E0; mask, allones) (src/utils.jl:29-54)
 * on the context's grid (nlayers = 1, Lx = Ly): writes the physical field zeta = irfft(-K^2 psi_hat)
 * for every ensemble instance ([batch][ny][nx], the context's real type; FP64 for GF_DF64).
 * psi_hat = mask * z * (K^2 (1 + (K/k0)^4))^(-1/2), k0 = kpeak 2 pi / Lx, z complex normal
 * (allones: z = 1) drawn with Philox4x32-10, counter (j (nx/2+1) + ik, 0, 0, 0x494E4954) and key
 * seed + instance; normalised so that sum over the half spectrum of K^2 |psi_hat|^2 / (nx ny)^2 = E0
 * (the reference's :50).  mask: NULL (ones) or a [ny][nx/2+1] FP64 array in `where` memory.
 * Julia's randn stream is replaced by Philox; the amplitudes and the normalisation are the
 * reference's. */
int gf_peakedisotropicspectrum(gf_ctx* ctx, double kpeak, double E0, const double* mask, int32_t allones,
                               uint64_t seed, void* zeta, int where);
/* prob.timestepper.filter of the Filtered steppers (FourierFlows makefilter, order 4, inner 0.65,
 * outer 1 unless set in gf_config) as [ny][nx/2+1] FP64; GF_ERR_STATE for unfiltered steppers. */
int gf_get_filter(const gf_ctx* ctx, double* out);

/* MultiLayerQG fwdtransform!/invtransform! (src/multilayerqg.jl:483-493) and the plain
 * rfft/irfft of FourierFlows' rfftplan, applied to nlayers fields at once. */
int gf_fwdtransform(gf_ctx* ctx, void* fieldh, const void* field, int where);
int gf_invtransform(gf_ctx* ctx, void* field, const void* fieldh, int where);

/* Parseval-sum diagnostics (reductions in FP64 with compensated sums on the GPU);
 * out[instance * nd + i] for a batched context. */
int gf_diagnostics(gf_ctx* ctx, const int32_t* which, int32_t nd, double* out);
int gf_get_batch(const gf_ctx* ctx, int32_t* batch);

/* ---- graphs and ensembles -------------------------------------------------------------
 * gf_step replays a CUDA graph of `steps` captured time steps (the step counter, time and
 * harmonic-forcing phases live on the GPU, so one graph serves every later step); AB3
 * problems always use graphs of 3 steps (their right-hand-side ring has period 3).
 * steps = 0 launches kernel by kernel.  Default 4.  Two sequences are captured per ring
 * phase: every step unobserved (replayed while more steps of the call follow) and the last
 * step (AB3: three) computing the aliased modes (the replay that ends the call), so a long
 * call pays for one observed step.  No counterpart in the reference (its steps are
 * launched broadcast by broadcast). */
int gf_set_graph_steps(gf_ctx* ctx, int32_t steps);
/* Steps n contexts (e.g. one batched context per grid size of an ensemble of independent runs
 * with uneven grid sizes) by nsteps each.  No counterpart in the reference (its ensembles are
 * a host loop over Problems).  With graphs on (gf_set_graph_steps > 0) the steps are replayed
 * from one CUDA graph for all contexts, in one of two executions (gf_set_ensemble_mode on the
 * first context): 0 (default) each context runs its own tuned launches on its own stream and
 * the size classes execute concurrently; 1, when the contexts allow it -- at most 4 contexts
 * of one precision and stepper family (not AB3), each one layer without bottom drag on a
 * square grid of 32, 64, 128 or 256 points -- every stage of every context runs in ONE
 * persistent row launch and ONE persistent column launch whose blocks walk the work list of
 * all contexts' tiles (otherwise mode 0).  Errors: gf_last_error(NULL). */
int gf_ensemble_step(gf_ctx* const* ctxs, int32_t n, int64_t nsteps);
/* Ensemble execution when ctx is the first context of gf_ensemble_step: 0 (default) one
 * context per stream, 1 the persistent ensemble launches.  No counterpart in the reference. */
int gf_set_ensemble_mode(gf_ctx* ctx, int32_t mode);

/* F-hat for GF_FORCING_STATIC / HARMONIC (same layout as sol), or the forcing spectrum
 * (real, (nkr, ny), the reference's `forcing_spectrum`) for the stochastic kinds.  This is
 * also the per-step escape hatch for an arbitrary Julia calcF!: call it before each step. */
int gf_set_forcing(gf_ctx* ctx, const void* data, int where);

/* Block until the context's stream has finished. */
int gf_synchronize(gf_ctx* ctx);

/* Output streaming (the reference's Diagnostic with freq = every and Output snapshots,
 * e.g. examples/twodnavierstokes_decaying.jl:90-115): nsteps steps; after every `every` steps
 * the diagnostics which_diag (gf_diagnostics ids) go to diag_out[k][instance][nd] and the
 * physical fields which_field (gf_field selectors, after updatevars!) to
 * field_out[k][f][instance][layer][ny][nx] (host memory, the context's real type; FP64 for
 * GF_DF64), k = 0 .. nsteps/every - 1.  Diagnostics and fields collect in device rings; the
 * host waits once per ring fill (<= 256 MB of fields), not once per output.  nd or nf may be 0. */
int gf_step_output(gf_ctx* ctx, int64_t nsteps, int32_t every, const int32_t* which_diag, int32_t nd,
                   double* diag_out, const int32_t* which_field, int32_t nf, void* field_out);

/* stepforward!(prob, nsteps) with an arbitrary host calcF! (calcF!(Fh, sol, t, clock, vars, params,
 * grid), e.g. examples/singlelayerqg_betaforced.jl:86-90): before every stage the library calls
 * fn(t_stage, clock.step, stage (1-based), Fh, user); fn fills Fh in the layout of gf_set_forcing
 * (host memory, the context's element type, zeroed before the call) and returns 0; the library
 * uploads it and runs the stage with N += Fh.  Each stage waits for the host: this is the slow,
 * general escape hatch beside the device forcing kinds.  The context must have been created with
 * forcing_kind = GF_FORCING_STATIC.  A non-zero return from fn stops the call with GF_ERR_ARG. */
typedef int (*gf_forcing_fn)(double t, int64_t step, int32_t stage, void* Fh, void* user);
int gf_step_callback(gf_ctx* ctx, int64_t nsteps, gf_forcing_fn fn, void* user);

/* ---- launch-shape autotuner (no reference counterpart) ----------------------------------
 * gf_autotune times the step kernels of this context at every candidate launch shape --
 * column kernel: FFT radix (FP32: 4, 8, 16; otherwise 8) x kr columns per block; row kernel:
 * radix x row pairs per block (threads per row = length / radix) -- by the GPU time of
 * `reps` steps (<= 0: 4) replayed from a CUDA graph, and keeps the fastest.  The state,
 * clock, AB3 history and stochastic-forcing record are restored; captured graphs are
 * re-captured.
 * shape (may be NULL) receives {row radix, row pairs per block, column radix, columns per
 * block}; 0 entries mean the built-in block-shape rule.  The candidates are timed on the
 * steps inside a gf_step call (those that skip the aliased modes); FP32 one-layer problems
 * without bottom drag with columns of >= 1024 may get blocks of up to 640 threads there,
 * while the last step of a call keeps blocks of <= 512 threads (the column count capped).
 * gf_set_launch_shape applies a shape found earlier (e.g. for another context of the same
 * size) and selects the classic kernels for both halves of the stage (the field-parallel
 * kernels below off).  The autotuner also times the TMA column stage (below) at each column radix where
 * it applies, and selects it (gf_get_tma_columns) when it is the fastest, and likewise the
 * field-parallel kernels (below) on grids where they apply (gf_get_field_parallel). */
int gf_autotune(gf_ctx* ctx, int32_t reps, int32_t* shape);
int gf_set_launch_shape(gf_ctx* ctx, const int32_t* shape);
int gf_get_launch_shape(const gf_ctx* ctx, int32_t* shape);

/* TMA column stage (no reference counterpart): for one layer without bottom drag and with at
 * most two nonlinear product fields (TwoDNavierStokes, SurfaceQG, SingleLayerQG without a PV
 * gradient product), the column half of each stage can load its product tiles and store the
 * inverse fields with tensor-memory-access tile copies (cp.async.bulk.tensor) instead of
 * per-thread copies.  C = columns per block: 2 or 4 (GF_F32), 1 or 2 (GF_F64, GF_DF64);
 * 0 selects the per-thread-copy column kernel; C > 0 also turns the field-parallel column
 * kernel (below) off.  GF_ERR_UNSUPPORTED if the context cannot use it with C.  The column radix stays that of the launch shape.  If a tile load does not
 * arrive within one second the kernel sets an error flag that gf_synchronize reports. */
int gf_set_tma_columns(gf_ctx* ctx, int32_t C);
int gf_get_tma_columns(const gf_ctx* ctx, int32_t* C);

/* Field-parallel small-grid kernels (no reference counterpart): for one layer without bottom
 * drag and power-of-two nx, ny in 32 ... 512, the row and column halves of each stage can run
 * with one thread group per field (the three inverse transforms, and the product transforms,
 * concurrently inside a block) at FFT radix 2, 4 or 8 (512: 4 or 8) -- the fast form when the grid has too
 * few row pairs and columns to occupy the GPU (e.g. one 128^2 run).  row_radix / col_radix 0
 * select the classic kernel for that half; columns = kr columns per column block (3 x columns
 * x ny / col_radix <= 384 threads; 0 means 1).  A context whose row pairs, over all instances,
 * are fewer than the GPU's SMs starts with them (row radix 4; column radix 2 up to ny = 128,
 * 4 above; one column per block);
 * gf_autotune times them against the classic kernels.  GF_ERR_UNSUPPORTED for contexts they
 * cannot run.  gf_get_field_parallel writes {row_radix, col_radix, columns}. */
int gf_set_field_parallel(gf_ctx* ctx, int32_t row_radix, int32_t col_radix, int32_t columns);
int gf_get_field_parallel(const gf_ctx* ctx, int32_t* out);

/* ---- adjoint ----------------------------------------------------------------------------
 * Reverse-mode derivative of stepforward!(prob, nsteps), the counterpart of a
 * ChainRulesCore.rrule on stepforward! (the reference has no derivative; its step is
 * src/singlelayerqg.jl:356-382 / src/twodnavierstokes.jl:253-294 under FourierFlows' ETDRK4
 * or RK4).
 * Supported: TwoDNavierStokes, SingleLayerQG (constant U or U(y)), MultiLayerQG (nonlinear)
 * and SurfaceQG, stepper ETDRK4, FilteredETDRK4, RK4 or FilteredRK4, batch = 1.  The loss
 * GF_LOSS_KINETIC_ENERGY is the module's kinetic energy (MultiLayerQG: summed over the layers);
 * the topography gradient is SingleLayerQG's and MultiLayerQG's.  It is the exact transpose of the discrete step the library
 * computes (dealiasing, PV inversion, stage combinations), in the context's precision.
 * Checkpointing: see gf_adjoint_set_snapshots (binomial schedule over units of
 * checkpoint_every steps; each unit is recomputed once with its forward fields kept).
 *
 * gf_adjoint_setup: allocate for nsteps steps (call again to change them).
 * gf_adjoint_forward: stepforward!(prob, nsteps) from the current state, keeping checkpoints.
 * gf_adjoint_backward: given the cotangent sol_bar of the final state (layout of
 *   gf_get_state), the cotangent of the initial state (sol0_bar, may be NULL) and of the
 *   topographic PV eta (eta_bar, [ny][nx] physical, SingleLayerQG only, may be NULL).  The
 *   state and clock are left at the forward pass's result.  Spectral arrays are taken as
 *   real vectors of (Re, Im) pairs over the stored half spectrum.
 * gf_grad: gf_adjoint_forward, the loss of the final state (loss_kind
 *   GF_LOSS_KINETIC_ENERGY: SingleLayerQG.kinetic_energy, src/singlelayerqg.jl:546-553,
 *   TwoDNavierStokes.energy, src/twodnavierstokes.jl:374-380, the sum of MultiLayerQG's
 *   per-layer kinetic energies, src/multilayerqg.jl:918-951, or SurfaceQG.kinetic_energy,
 *   src/surfaceqg.jl:380-400) into *loss, and its gradients with respect to the physical
 *   initial field q0 of set_q!/set_zeta!/set_b! (dq0, [nlayers][ny][nx]) and to the
 *   topography eta (deta, [ny][nx]: SingleLayerQG, MultiLayerQG), either may be NULL. */
enum { GF_LOSS_KINETIC_ENERGY = 0 };
int gf_adjoint_setup(gf_ctx* ctx, int64_t nsteps, int32_t checkpoint_every);
/* Binomial checkpointing (Griewank's schedule) over units of checkpoint_every steps: the
 * reverse sweep recomputes each unit once with its forward fields kept and reaches unit
 * starts from at most `snapshots` stored states (slot 0 = the initial state), choosing the
 * snapshot positions that minimise the unit advances C(n, s) = min_m [m + C(n-m, s-1) + C(m, s)].
 * The default (one snapshot per unit) needs no advance beyond the forward pass; fewer
 * snapshots trade memory for recomputation.  Call after gf_adjoint_setup.  gf_adjoint_info
 * reports the units, the snapshot slots and the unit advances the last reverse sweep added
 * to the forward pass (0 with one snapshot per unit). */
int gf_adjoint_set_snapshots(gf_ctx* ctx, int32_t snapshots);
int gf_adjoint_info(const gf_ctx* ctx, int32_t* units, int32_t* snapshots, int64_t* unit_advances);
int gf_adjoint_forward(gf_ctx* ctx);
int gf_adjoint_backward(gf_ctx* ctx, const void* sol_bar, void* sol0_bar, void* eta_bar, int where);
int gf_grad(gf_ctx* ctx, int loss_kind, void* dq0, void* deta, double* loss, int where);

/* Kernel timing for benchmarks: while enabled, CUDA events are recorded on the context's
 * stream around every row-pass and column-pass kernel launch.  gf_profile_read waits for the
 * stream, returns the summed milliseconds ms[0] (row pass) and ms[1] (column pass), the
 * launch counts n[0], n[1], and the number of kernels libgfcuda launched since the last
 * read, then resets the counters.  No counterpart in the reference (which has no timing). */
int gf_profile_enable(gf_ctx* ctx, int on);
int gf_profile_read(gf_ctx* ctx, double* ms, int64_t* n, int64_t* launches);

/* ---- allocation-free forward transform ------------------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device memory (code
 * running inside another runtime that owns the GPU's memory, such as a Julia session whose
 * CUDA.jl pool holds the device and enforces a memory limit, or a latency-critical loop
 * where cudaMalloc/cudaFree and their device synchronisation are not acceptable).
 * Computes the unnormalised 2-D r2c transform of the device field (nx, ny) into the device
 * spectrum (nx/2+1, ny) (the same result as gf_fwdtransform) without allocating: its
 * intermediate rows and twiddle tables live in fixed __device__ arrays that every GPU
 * loading the library keeps until exit (about 2.2 MB of scratch plus 96 KB of tables).
 * nx, ny: powers of two in [32, GF_NOALLOC_MAX_N]; larger sizes return GF_ERR_UNSUPPORTED.
 * precision: GF_F32 (float in, complex-float out) or GF_F64.  stream: cudaStream_t or NULL.
 * The first call on a device sets that device up (it must be current): it copies the twiddle
 * tables in and waits for the device before it launches, so the tables are complete whatever
 * stream the call runs on; make that first call before any stream capture.  At most 64
 * devices (ordinals 0..63).  A device reset (cudaDeviceReset, CUDA.jl's device_reset!) is not
 * supported: the tables of the reset device are not copied in again.  All calls share the
 * scratch: calls that overlap on the GPU race.  Errors: gf_last_error(NULL). */
#define GF_NOALLOC_MAX_N 512
int gf_rfft2_noalloc(const void* field, void* fieldh, int32_t nx, int32_t ny, int32_t precision, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* GFCUDA_H */
