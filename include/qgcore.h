/*
 * qgcore.h - C ABI of the GB300-native multilayer quasi-geostrophic (QG) time step.
 *
 * The library (libqgcore.so) replaces somax's QG hot path below the model classes'
 * public API.  Each entry point names the reference symbol it stands in for:
 *
 *   qg_plan_create   BaroclinicQG.create / BarotropicQG.create + ModalTransform.from_physics
 *                    (somax/_src/models/qg/baroclinic.py:230-332,
 *                     somax/_src/models/qg/barotropic.py:186-248,
 *                     somax/_src/core/transforms.py:172-200)
 *   qg_invert        BaroclinicQG._invert_pv (baroclinic.py:135-159),
 *                    BarotropicQG._invert_pv (barotropic.py:113-121)
 *   qg_rhs           BaroclinicQG.vector_field (baroclinic.py:161-190),
 *                    BarotropicQG.vector_field (barotropic.py:123-152); with QG_RHS_APPLY_BC
 *                    it is SomaxModel.build_terms._rhs (somax/_src/core/model.py:47-49)
 *   qg_step          SomaxModel.integrate with ConstantStepSize (core/model.py:53-88)
 *   qg_diagnose      BaroclinicQG.diagnose KE / enstrophy (baroclinic.py:197-228)
 *   qg_rhs_vjp       reverse-mode derivative of vector_field / _rhs, and
 *   qg_invert_vjp    of _invert_pv, that the reference takes with JAX autodiff
 *                    (eqx.filter_grad through integrate: tests/models/test_qg_baroclinic.py:293-312)
 *   qg_status        non-finite check of the runner (somax/_src/cli/_run.py:671-686)
 *
 * Conventions: every field is float32, layout (n_layers, Ny, Nx) row-major per member with
 * Ny = ny + 2, Nx = nx + 2 (one ghost ring); members of an ensemble are concatenated in
 * the order given to qg_plan_create (qg_plan_member_offset gives each member's offset in
 * floats).  All device pointers are owned by the caller; the plan owns its constants and
 * workspace, and no entry point below allocates device memory after qg_plan_create.
 * Calls are asynchronous on the given stream; a plan must not be used from two streams
 * at the same time.  Every entry point returns QG_OK or a QG_ERR_* code; nothing throws
 * across the ABI.
 */
#ifndef QGCORE_H
#define QGCORE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QG_MAX_LAYERS 8

/* status codes */
#define QG_OK 0
#define QG_ERR_NULL 1         /* a required pointer is NULL */
#define QG_ERR_SHAPE 2        /* bad grid size / layer count / member count */
#define QG_ERR_CUDA 3         /* a CUDA runtime call failed */
#define QG_ERR_NONFINITE 4    /* a kernel saw a non-finite value (qg_status) */
#define QG_ERR_TIMEOUT 5      /* a bounded device-side wait gave up */
#define QG_ERR_ARG 6          /* bad enum / option value */
#define QG_ERR_UNSUPPORTED 7  /* option not available on this device */
#define QG_ERR_TOO_LARGE 8    /* member exceeds the fixed scratch of qg_invert_static, or has
                                  more than 28000 land boundary points */

/* dst_precision: arithmetic of the DST-I GEMMs of the PV inversion */
#define QG_DST_FP32 0    /* plain FP32 on the CUDA cores (the baseline path) */
#define QG_DST_TF32 1    /* tcgen05 kind::tf32, FP32 accumulate */
#define QG_DST_BF16X3 2  /* tcgen05 kind::f16, split bf16 hi/lo, 3 products, FP32 accumulate */

/* eigs_mode: where the Helmholtz eigenvalues come from (transforms.py:192-194) */
#define QG_EIGS_CONSISTENT 0 /* eig(A), paired with the modes */
#define QG_EIGS_REFERENCE 1  /* eigh((A + A^T) / 2), as jnp.linalg.eigh does */

/* time schemes for qg_step */
#define QG_SCHEME_EULER 0
#define QG_SCHEME_HEUN 1   /* diffrax.Heun */
#define QG_SCHEME_SSPRK3 2 /* Shu-Osher SSP-RK3 */
#define QG_SCHEME_TSIT5 3  /* diffrax.Tsit5 (the reference default) */

/* wind profile (baroclinic.py:313-318) */
#define QG_WIND_DOUBLEGYRE 0 /* -sin(2 pi y / Ly) */
#define QG_WIND_SINGLE 1     /* sin(pi y / Ly) */

/* flags for qg_rhs */
#define QG_RHS_APPLY_BC 1 /* zero the ghost ring of q first (core/model.py:47-49) */
/* flags for qg_step */
#define QG_STEP_APPLY_BC 1 /* zero the ring of the initial state in place (integrate() on a new
                              state0); without it the call continues an integration */

/* params layout: per member, QG_NPARAMS floats in device memory */
#define QG_NPARAMS 4
#define QG_P_NU 0    /* lateral_viscosity (m^2/s) */
#define QG_P_KAPPA 1 /* bottom_drag (1/s) */
#define QG_P_TAU0 2  /* wind_amplitude (wind-stress curl amplitude, 1/s^2) */
#define QG_P_NU4 3   /* biharmonic viscosity (m^4/s), extension; 0 = off */

typedef struct qg_member_desc {
    int nx, ny;         /* interior cells */
    int n_layers;       /* 1..QG_MAX_LAYERS */
    int barotropic;     /* 1: BarotropicQG semantics (Poisson, psi ring kept, wind not / H) */
    double Lx, Ly;      /* domain size (m) */
    double f0, beta;    /* Coriolis parameter (1/s), its meridional gradient (1/(m s)) */
    double H[QG_MAX_LAYERS];       /* layer thicknesses, top to bottom (m) */
    double g_prime[QG_MAX_LAYERS]; /* reduced gravities at each interface (m/s^2) */
    int wind_profile;   /* QG_WIND_* */
    int eigs_mode;      /* QG_EIGS_* */
    /* optional override of the modal matrices (row-major nl x nl) and the Helmholtz
       lambdas f0^2 * eig (nl); used when has_modes != 0 */
    int has_modes;
    double Cl2m[QG_MAX_LAYERS * QG_MAX_LAYERS];
    double Cm2l[QG_MAX_LAYERS * QG_MAX_LAYERS];
    double lambdas[QG_MAX_LAYERS];
    /* optional land mask (extension; host memory, (ny + 2) x (nx + 2) row-major, 1 = ocean,
       0 = land, read during qg_plan_create only; NULL = no land).  Interior land cells read
       q as 0, have psi = 0 and dq = 0; the inversion keeps psi = 0 on the land cells next to
       the ocean with an FP64 capacitance-matrix correction (a second DST solve).  The ring
       keeps the unmasked rules. */
    const unsigned char* mask;
} qg_member_desc;

typedef struct qg_options {
    int dst_precision;  /* QG_DST_* */
    int refine_sweeps;  /* FP32 residual-refinement sweeps of the Helmholtz solve (0 or 1) */
    int use_graphs;     /* 1: qg_step replays a captured CUDA graph per step */
    int persistent;     /* 1: qg_step advances all steps in one persistent cooperative launch
                           (tensor-core precisions without refinement) */
    int autotune;       /* 1: qg_plan_create times the stencil variants and keeps the fastest */
    int stencil;        /* 0: autotuner's choice; QG_STENCIL_* + 1: run that variant */
    int gemm_tile;      /* 0: autotuner's choice; 144, 80, 48, 32 or 16: that tensor-core tile width */
    int cluster;        /* cluster-resident stepping of small members (qg_step with Heun / SSP-RK3:
                           one thread-block cluster per member runs every stage of every step in
                           one launch, FP32 DST passes on the CUDA cores, state in shared memory):
                           0: used when the autotuner times it faster than the multi-launch path,
                           1: used whenever the members allow it, 2: never */
} qg_options;

typedef struct qg_plan qg_plan;

/* Build a plan for an ensemble of members (n_members >= 1). opts may be NULL (defaults:
   FP32, no refinement, graphs on).  Allocates the plan's device constants and workspace on
   the current device. */
int qg_plan_create(const qg_member_desc* members, int n_members, const qg_options* opts,
                   qg_plan** out);
void qg_plan_destroy(qg_plan* plan);

/* Number of floats in one packed field (all members), and member i's offset into it. */
int64_t qg_plan_state_size(const qg_plan* plan);
int64_t qg_plan_member_offset(const qg_plan* plan, int member);
/* Helmholtz lambdas f0^2 * eig (nl values) and the modal matrices the plan uses. */
int qg_plan_member_modes(const qg_plan* plan, int member, double* lambdas, double* Cl2m,
                         double* Cm2l);

/* psi = _invert_pv(q) for every member. q and psi: packed fields (device). */
int qg_invert(qg_plan* plan, const float* q, float* psi, void* stream);

/* dq = vector_field(q) for every member. params: n_members * QG_NPARAMS floats (device). */
int qg_rhs(qg_plan* plan, const float* q, float* dq, const float* params, int flags,
           void* stream);

/* Advance q in place by n_steps steps of size dt with the given scheme.  The BC is applied
   to every stage input (core/model.py:47-49); with QG_STEP_APPLY_BC the ghost ring of q is
   zeroed first, as SomaxModel.integrate does to state0 (model.py:74).  The returned state's
   ring is the stepped (not re-zeroed) ring, so consecutive calls without the flag give the
   same result as one call over all their steps. */
int qg_step(qg_plan* plan, float* q, const float* params, double dt, int n_steps, int scheme,
            int flags, void* stream);

/* Vector-Jacobian products (hand-written adjoints; device pointers, packed fields).
   qg_rhs_vjp: for the qg_rhs call with the same q, params and flags, and the cotangent
   dq_bar of its dq: q_bar = (d dq / d q)^T dq_bar and, when params_bar is not NULL,
   params_bar = (d dq / d params)^T dq_bar (n_members * QG_NPARAMS floats, overwritten).
   qg_invert_vjp: q_bar = (d psi / d q)^T psi_bar for qg_invert.  Both run one adjoint
   Helmholtz solve on the plan's DST-I GEMMs (the solve is self-adjoint) with the plan's
   precision and refinement. */
int qg_rhs_vjp(qg_plan* plan, const float* q, const float* params, const float* dq_bar, float* q_bar,
               float* params_bar, int flags, void* stream);
int qg_invert_vjp(qg_plan* plan, const float* psi_bar, float* q_bar, void* stream);

/* Adjoint of one qg_step step (any scheme, in Butcher form) from the state y0 (packed, ring as
   stepped): on entry y_bar is the cotangent of the step's result, on return the cotangent of
   y0; params_bar (may be NULL) receives the parameter cotangents of the step (overwritten).
   The step's stage inputs are recomputed with the fused right-hand side (keeping each stage's
   streamfunction), then the stages are reversed with qg_rhs_vjp's kernels and fused
   linear-combination kernels.  work: caller-owned
   device scratch of qg_step_vjp_workspace(plan, scheme) floats.  With graphs on (qg_options)
   the call's launches are captured once and replayed while y0, params, y_bar, params_bar,
   work, dt and scheme repeat; a change of any of them captures again.  The checkpointed adjoint of
   integrate (diffrax's recursive checkpointing under eqx.filter_grad,
   tests/models/test_qg_baroclinic.py:293-312) calls it once per step in reverse. */
int64_t qg_step_vjp_workspace(const qg_plan* plan, int scheme);
int qg_step_vjp(qg_plan* plan, const float* y0, const float* params, double dt, int scheme, float* y_bar,
                float* params_bar, float* work, void* stream);

/* Geostrophic projection P = G (Q G)^-1 Q of a multilayer shallow-water state (h, u, v), each a
   packed field like q (device pointers): ReparameterizedQG.project
   (somax/_src/models/qg/reparameterized.py:142-178).  Q: q = curl(u, v) - f0 (h - H) / H with
   the vorticity at the C-grid corner points; (Q G)^-1: the plan's modal Helmholtz inversion
   (as qg_invert); G: (u_g, v_g) = grad_perp(psi) at the u / v points and
   h_g = H (1 + f0 Cm2l diag(eig) Cl2m psi) with eig = lambda / f0^2.  psi (may be NULL)
   receives the streamfunction.  Baroclinic unmasked members (QG_ERR_UNSUPPORTED otherwise);
   the plan's stage planes serve as scratch, so calls on one plan are not concurrent. */
int qg_project(qg_plan* plan, const float* h, const float* u, const float* v, float* h_g, float* u_g,
               float* v_g, float* psi, void* stream);
/* The reverse mode of qg_project: (h_bar, u_bar, v_bar) = P^T (h_g_bar, u_g_bar, v_g_bar) for
   P = G (Q G)^-1 Q, the transposes of the reconstruction and PV kernels around one adjoint
   inversion (qg_invert_vjp).  The same members as qg_project. */
int qg_project_vjp(qg_plan* plan, const float* h_g_bar, const float* u_g_bar, const float* v_g_bar, float* h_bar,
                   float* u_bar, float* v_bar, void* stream);

/* Kinetic energy and enstrophy per layer: ke, ens each sum(n_layers) floats (device). */
int qg_diagnose(qg_plan* plan, const float* q, float* ke, float* ens, void* stream);
/* The whole diagnose record (baroclinic.py:197-228) with one inversion: psi, u = -d_y psi (V
   points), v = d_x psi (U points), zeta = lap psi (packed fields like q, ring 0 for u, v, zeta),
   and ke, ens as qg_diagnose. */
int qg_diagnose_fields(qg_plan* plan, const float* q, float* psi, float* u, float* v, float* zeta, float* ke,
                       float* ens, void* stream);

/* qg_invert for one member without a plan and without allocating device memory.
   No counterpart in the reference: this is for callers that may not allocate at the time
   they invert (code inside a framework's compiled program or memory pool, loops with an
   allocation ban).  Scratch is one fixed file-scope device array of about 14.9 MB that
   every GPU loading the library holds until exit.  Limits: nx, ny <= 512 and n_layers *
   (ny+2) * round_up(nx+2, 32) <= 2^20 (and the same with x and y swapped); larger members
   return QG_ERR_TOO_LARGE.  All calls on a device share that scratch, so calls that
   overlap on the GPU race; serialise them.  The first call on each device looks up the
   scratch address (cudaGetSymbolAddress), and so does the first call in a new context of
   that device (after cudaDeviceReset); make those calls before any stream capture. */
int qg_invert_static(const qg_member_desc* member, const float* q, float* psi, void* stream);

/* State statistics of the runner's chunk log (somax/_src/cli/_run.py:408-432,
   _state_diagnostics): stats[0..3] = min, mean and max over the finite entries of the packed
   field q and the number of non-finite entries (device pointer, 4 doubles; NaN for min /
   mean / max when no entry is finite).  Reduced on the device, no host scan. */
int qg_state_stats(qg_plan* plan, const float* q, double* stats, void* stream);

/* Device-side status: synchronises the stream, returns QG_OK or QG_ERR_NONFINITE /
   QG_ERR_TIMEOUT, writes the raw flag word to *flags (may be NULL) and clears it. */
int qg_status(qg_plan* plan, int* flags, void* stream);

const char* qg_strerror(int code);

/* Clock64 cycles that a CTA of the persistent step kernel waits at its grid barrier before it
   gives up (the launch then sets the time-out flag that qg_status reports as QG_ERR_TIMEOUT,
   and every CTA drains its copies in flight and returns).  0 restores the default of about
   2 s; the waits on TMA and tensor-core completions keep that default.  Counterpart of the
   runner's divergence guard (somax/_src/cli/_run.py:671-686): a wait that cannot end is
   reported, never left to hang the device.  Takes effect on the next qg_step. */
int qg_plan_set_wait_limit(qg_plan* plan, int64_t cycles);

/* The layer-per-warp sweep launches one kernel per (layer count, strip class) group; by
   default (on = 1) a stage forks them onto plan-owned side streams as parallel branches and
   joins them before the next DST pass.  on = 0 launches them one after another on the call's
   stream (same arithmetic, same result bit for bit).  Discards the captured step graphs.
   No reference counterpart: a switch of this library's launch schedule. */
int qg_plan_set_parallel_sweep(qg_plan* plan, int on);

/* Per-kernel-class timing with CUDA events recorded on the launch stream around every
   launch while profiling is on (graphs are bypassed then).  Used by the benchmark to turn
   algorithmic bytes / flops into achieved bandwidth / throughput per kernel. */
#define QG_K_PREP 0    /* layer -> mode prologue (BC, Cl2m, operand format) */
#define QG_K_GEMM 1    /* DST-I GEMMs of the inversion */
#define QG_K_STENCIL 2 /* fused RHS stencil (+ RK stage update, + next-stage prologue) */
#define QG_K_OTHER 3   /* mode -> layer epilogue, residual, diagnostics, packing */
#define QG_K_PERSISTENT 4 /* the persistent step kernel (all phases of all steps) */
#define QG_K_COUNT 5
int qg_set_profiling(qg_plan* plan, int enable); /* resets the counters */
int qg_kernel_stats(qg_plan* plan, int kclass, double* total_ms, int64_t* launches);

/* Stencil variants the autotuner times (one RK stage each: the four DST passes and the
   step-mode stencil, on the plan's own planes):
   the tile stencil with 32 x 8 or 64 x 16 tiles (TMA halo boxes; also the persistent kernel's
   stencil phase) and the column-sweep stencil with 16-, 32- or 64-row strips. */
#define QG_STENCIL_TILE_32X8 0
#define QG_STENCIL_TILE_64X16 1
#define QG_STENCIL_SWEEP_16 2
#define QG_STENCIL_SWEEP_32 3
#define QG_STENCIL_SWEEP_64 4
#define QG_STENCIL_LSWEEP_16 5 /* layer-per-warp column sweep, two columns per lane */
#define QG_STENCIL_LSWEEP_32 6
#define QG_STENCIL_LSWEEP_64 7
#define QG_STENCIL_VARIANTS 8
/* The plan's tuned choice: *variant = the stencil the multi-launch path runs; ms[k] (k < n)
   the autotuner's time of one stage with variant k in ms (-1 when not measured). */
int qg_plan_tuning(const qg_plan* plan, int* variant, float* ms, int n);
/* The tensor-core DST passes' output tile width the autotuner kept (144, 80, 48, 32 or 16
   columns; 64 for the FP32 CUDA-core passes) and the time of the four passes it measured
   with each width in ms (ms[0..4] in that order; -1 when not measured). */
int qg_plan_gemm_tuning(const qg_plan* plan, int* tile_n, float* ms, int n);
/* The stepping engine qg_step uses for Heun / SSP-RK3: *cluster_ctas = the CTAs of one
   member's cluster when the cluster-resident engine runs (all members alike in layers and
   grid, unmasked, small enough for one cluster's shared memory), else 0; ms[0], ms[1] (n >= 2)
   the autotuner's time of four SSP-RK3 steps with the multi-launch path and with the cluster
   engine (-1 when not measured). */
int qg_plan_engine(const qg_plan* plan, int* cluster_ctas, float* ms, int n);

/* ---------------------------------------------------------------------------------------
   Multilayer shallow-water right-hand side: MultilayerShallowWater2D
   (somax/_src/models/swm/multilayer.py:150-200 vector_field, :202-219 apply_boundary_conditions,
   :259-363 create).  The state is one packed float32 array (3, n_layers, ny + 2, nx + 2): layer
   thickness h (T points), then u (U points, east faces), then v (V points, north faces).
   params: 3 floats in device memory, QG_SWM_P_* below.
   --------------------------------------------------------------------------------------- */
#define QG_SWM_PERIODIC 0 /* bc = "periodic": every field wraps */
#define QG_SWM_WALL 1     /* bc = "wall": no normal flow, free slip, zero-gradient h */
#define QG_SWM_NPARAMS 3
#define QG_SWM_P_NU 0    /* lateral_viscosity (m^2/s) */
#define QG_SWM_P_KAPPA 1 /* bottom_drag (1/s) */
#define QG_SWM_P_TAU0 2  /* wind_amplitude (m/s^2); the top layer gets tau0 * tau_x(y) / H[0] */

typedef struct qg_swm_desc {
    int nx, ny;         /* interior cells */
    int n_layers;       /* 1..QG_MAX_LAYERS */
    double Lx, Ly;      /* domain size (m) */
    double f0, beta;    /* f(y) = f0 + beta (y - Ly / 2), y_j = j * Ly / ny */
    double H[QG_MAX_LAYERS];       /* layer thicknesses, top to bottom (m) */
    double g_prime[QG_MAX_LAYERS]; /* g'_0 = g, then the reduced gravities (m/s^2) */
    int wind_profile;   /* QG_WIND_DOUBLEGYRE: tau_x = -cos(2 pi y / Ly); QG_WIND_SINGLE: -cos(pi y / Ly) */
    int bc;             /* QG_SWM_PERIODIC or QG_SWM_WALL */
} qg_swm_desc;

typedef struct qg_swm_plan qg_swm_plan;

/* MultilayerShallowWater2D.create: device constants and the stepper's stage buffers. */
int qg_swm_create(const qg_swm_desc* desc, qg_swm_plan** out);
void qg_swm_destroy(qg_swm_plan* plan);
/* Floats of one packed state (3 * n_layers * (ny + 2) * (nx + 2)). */
int64_t qg_swm_state_size(const qg_swm_plan* plan);
/* tend = vector_field(state) (dh, du, dv packed like the state); with QG_RHS_APPLY_BC the
   boundary rules are applied to the state as it is read (the _rhs wrapper, core/model.py:47-49). */
int qg_swm_rhs(qg_swm_plan* plan, const float* state, float* tend, const float* params, int flags, void* stream);
/* apply_boundary_conditions in place. */
int qg_swm_apply_bc(qg_swm_plan* plan, float* state, void* stream);
/* Advance the state in place by n_steps constant steps (QG_SCHEME_*; Tsit5 is the reference's
   default solver): BC on every stage input, QG_STEP_APPLY_BC applies it to the initial state
   first (integrate() on a new state0), the returned state is as stepped.  The params are
   copied into the plan on the stream first; each stage is one fused launch (stage input,
   right-hand side, and on the last stage the next state, written alternately into the state
   and a plan buffer); the steps run as captured CUDA graphs of 8 and of 1 steps, replayed
   while the state pointer, dt and the scheme repeat (recaptured otherwise). */
int qg_swm_step(qg_swm_plan* plan, float* state, const float* params, double dt, int n_steps, int scheme,
                int flags, void* stream);
/* Per-kernel-class timing of qg_swm_step: CUDA events on the launch stream around every
   launch while profiling is on (graphs are bypassed then); set_profiling resets the counters.
   No reference counterpart: the benchmark's per-kernel durations. */
#define QG_SWM_K_STAGE 0   /* k_swm_stage: stage input, right-hand side, (last stage) next state */
#define QG_SWM_K_COMBINE 1 /* k_swm_combine: a stage input of qg_reparam_step or its final combination */
#define QG_SWM_K_CLUSTER 2 /* k_swm_cluster: every step of a qg_swm_step call (cluster engine) */
#define QG_SWM_K_COUNT 3
int qg_swm_set_profiling(qg_swm_plan* plan, int enable);
int qg_swm_kernel_stats(qg_swm_plan* plan, int kclass, double* total_ms, int64_t* launches);
/* Stepping engine of qg_swm_step.  The cluster engine runs every step of a call in one launch
   of one thread-block cluster (16, 8, 4 or 2 CTAs, each holding a band of rows of the state,
   of the stage derivatives and of the stage inputs in shared memory; the halo rows come from
   the neighbouring CTAs' shared memory); it applies when the basin fits (small grids, e.g.
   2 layers of 64^2).  AUTO: the engine that ran 32 steps of a rest state faster, timed on the
   plan's own buffers at the first qg_swm_step / qg_swm_engine call of each scheme (that call
   synchronises the device; call qg_swm_engine before capturing qg_swm_step into a graph).
   No reference counterpart: a switch of this library's launch schedule. */
#define QG_SWM_ENGINE_AUTO 0
#define QG_SWM_ENGINE_STAGES 1  /* one k_swm_stage launch per stage, graph-replayed */
#define QG_SWM_ENGINE_CLUSTER 2 /* the cluster engine; qg_swm_step returns QG_ERR_UNSUPPORTED if it does not fit */
int qg_swm_set_engine(qg_swm_plan* plan, int engine);
/* The engine qg_swm_step uses for a scheme (QG_SWM_ENGINE_STAGES or _CLUSTER; a negative
   QG_ERR_* on bad arguments), the cluster's CTA count (0 without the cluster engine) and,
   when times_ms is not NULL, the tuning times of 32 steps (times_ms[0] the fastest cluster,
   times_ms[1] the stage engine; -1 where not timed).  Tunes the scheme if not yet done. */
int qg_swm_engine(qg_swm_plan* plan, int scheme, int* cluster_ctas, float* times_ms);
/* ReparameterizedQG (somax/_src/models/qg/reparameterized.py:65-228) stepped like qg_swm_step:
   every stage input gets the model's apply_boundary_conditions (the SWM wall rules, then the
   geostrophic projection of qg_project on qgplan, reparameterized.py:186-189) before the
   shallow-water vector_field (:180-184); QG_STEP_APPLY_BC does the same to the initial state.
   plan must have wall boundaries (QG_ERR_ARG) and qgplan one baroclinic member of the same
   grid and layers (QG_ERR_SHAPE).  Launched directly (no graph). */
int qg_reparam_step(qg_swm_plan* plan, qg_plan* qgplan, float* state, const float* params, double dt,
                    int n_steps, int scheme, int flags, void* stream);
/* Reverse mode of the shallow-water model (what the reference takes with JAX autodiff through
   vector_field and integrate: tests/models/test_swm_multilayer.py:239-252).
   qg_swm_rhs_vjp: state_bar = J^T tend_bar for tend = vector_field(state) (with
   QG_RHS_APPLY_BC: of the boundary rules applied on read, so state_bar is the cotangent of
   the raw state), params_bar[0..2] = the cotangents of nu, kappa, tau0 (overwritten).  The
   upwind switch is differentiated as a fixed choice of upwind cell.
   qg_swm_bc_vjp: the transpose of apply_boundary_conditions on a cotangent, in place.
   qg_swm_step_vjp: the adjoint of one qg_swm_step step from y0: y_bar holds the cotangent of
   the step's result on entry and that of y0 on return; params_bar receives the parameter
   cotangents (overwritten); work holds qg_swm_step_vjp_workspace(plan, scheme) floats.  The
   step's adjoint is captured as a CUDA graph and replayed while its five pointers, dt and the
   scheme repeat (recaptured otherwise). */
int qg_swm_rhs_vjp(qg_swm_plan* plan, const float* state, const float* params, const float* tend_bar,
                   float* state_bar, float* params_bar, int flags, void* stream);
int qg_swm_bc_vjp(qg_swm_plan* plan, float* state_bar, void* stream);
int64_t qg_swm_step_vjp_workspace(const qg_swm_plan* plan, int scheme);
/* The adjoint of k steps from the checkpoint y_start in one call: the segment's states are
   recomputed into work (qg_swm_segment_vjp_workspace(plan, scheme, k) floats), then every
   step's adjoint runs in reverse; y_bar holds the cotangent of the k-th state on entry and
   that of y_start on return, params_bar the parameter cotangents summed over the k steps.
   Replayed as one captured graph while its pointers, dt, k and the scheme repeat. */
int64_t qg_swm_segment_vjp_workspace(const qg_swm_plan* plan, int scheme, int k);
int qg_swm_segment_vjp(qg_swm_plan* plan, const float* y_start, const float* params, double dt, int k, int scheme,
                       float* y_bar, float* params_bar, float* work, void* stream);
int qg_swm_step_vjp(qg_swm_plan* plan, const float* y0, const float* params, double dt, int scheme, float* y_bar,
                    float* params_bar, float* work, void* stream);
/* The runner's state statistics (cli/_run.py:408-432) of n floats at x (one field of a state,
   or several): stats[0..3] = min, mean, max over the finite entries and the count of
   non-finite entries, as device doubles. */
int qg_swm_state_stats(qg_swm_plan* plan, const float* x, int64_t n, double* stats, void* stream);
/* Reverse mode of the reparameterised model (reparameterized.py's gradient test,
   tests/models/test_qg_reparameterized.py:193-206), the same plans as qg_reparam_step:
   qg_reparam_bc_vjp: y_bar <- B^T P^T y_bar, the transpose of its apply_boundary_conditions
   (wall rules B, then the projection P), in place;
   qg_reparam_step_vjp: the adjoint of one qg_reparam_step step from y0 (y_bar: the result's
   cotangent in, y0's out; params_bar: (nu, kappa, tau0), overwritten; work:
   qg_reparam_step_vjp_workspace(plan, scheme) floats). */
int qg_reparam_bc_vjp(qg_swm_plan* plan, qg_plan* qgplan, float* y_bar, void* stream);
int64_t qg_reparam_step_vjp_workspace(const qg_swm_plan* plan, int scheme);
int qg_reparam_step_vjp(qg_swm_plan* plan, qg_plan* qgplan, const float* y0, const float* params, double dt,
                        int scheme, float* y_bar, float* params_bar, float* work, void* stream);
/* QG_OK or QG_ERR_NONFINITE (a tendency was not finite since the last call); clears the flag. */
int qg_swm_status(qg_swm_plan* plan, int* flags, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* QGCORE_H */
