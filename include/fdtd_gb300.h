/*
 * fdtd_gb300.h -- C ABI of the GB300 (sm_103a) FDTD time-stepping library.
 *
 * The library replaces the per-step hot path of fdtdx (a JAX package):
 *
 *   fdtd_forward          one or more forward Yee steps: update_E, source E-injection,
 *                         PEC zeroing, update_H, source H-injection, PMC zeroing,
 *                         detector accumulation and PML-interface recording.
 *                         Replaces the body of the time loop in
 *                         fdtdx/fdtd/fdtd.py:482-493 (checkpointed_fdtd) and
 *                         fdtdx/fdtd/fdtd.py:157-163 (reversible forward), i.e.
 *                         fdtdx/fdtd/forward.py:83-156 with
 *                         fdtdx/fdtd/update.py:256-523, 689-853, 1040-1178.
 *   fdtd_reverse          one or more time-reversed steps (interface re-imposition,
 *                         reverse H, reverse E with frozen CPML psi).  Replaces
 *                         fdtdx/fdtd/backward.py:62-135 with
 *                         fdtdx/fdtd/update.py:526-686, 856-1007, 1181-1222.
 *   fdtd_adjoint          the backward loop of the reversible gradient: per step a
 *                         reverse step (the reconstruction) followed by the transposed
 *                         (vector-Jacobian) forward step.  Replaces body_fn of the
 *                         custom VJP, fdtdx/fdtd/fdtd.py:215-251 (backward() then
 *                         jax.vjp of forward_single_args_wrapper), accumulating
 *                         d/d inv_eps as fdtdx/fdtd/fdtd.py:324-333 returns it.
 *
 * Conventions
 *   - Every buffer is caller-owned device memory, float32, C order, z fastest.
 *     Fields are (3, nx, ny, nz).  Material arrays are (n, nx, ny, nz), n in {1, 3, 9}.
 *   - The plan copies the small host tables of FdtdDesc (PML coefficients,
 *     per-step source and detector tables, plane-source profiles) to device
 *     memory it owns, plus scratch for reductions.  It never touches caller buffers
 *     outside the calls below.
 *   - Errors are returned as FDTD_* status codes; fdtd_last_error(plan) gives a
 *     message.  No exception crosses the ABI.
 *   - Streams are passed as void* (a cudaStream_t); a plan must not be used from
 *     two host threads at once.  Independent plans are independent.
 */
#ifndef FDTD_GB300_H
#define FDTD_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FDTD_OK 0
#define FDTD_EINVAL 1
#define FDTD_ENOMEM 2
#define FDTD_ECUDA 3
#define FDTD_ETIMEOUT 4
#define FDTD_ENONFINITE 5

#define FDTD_MAX_SLABS 6
#define FDTD_MAX_SOURCES 16
#define FDTD_MAX_DETECTORS 32
#define FDTD_MAX_FREQS 16

#define FDTD_PROFILE_CW 0       /* SingleFrequencyProfile (fdtdx/objects/sources/profile.py:253-273) */
#define FDTD_PROFILE_GAUSSIAN 1 /* GaussianPulseProfile   (fdtdx/objects/sources/profile.py:276-345) */

#define FDTD_SRC_DIPOLE 0 /* PointDipoleSource  (fdtdx/objects/sources/dipole.py:195-277) */
#define FDTD_SRC_PLANE 1  /* TFSF plane source  (fdtdx/objects/sources/tfsf.py:193-409, 739-806) */

#define FDTD_DET_FIELD 0  /* FieldDetector        (fdtdx/objects/detectors/field.py:31-63) */
#define FDTD_DET_PHASOR 1 /* PhasorDetector       (fdtdx/objects/detectors/phasor.py:190-235) */
#define FDTD_DET_FLUX 2   /* PoyntingFluxDetector (fdtdx/objects/detectors/poynting_flux.py:171-195) */
#define FDTD_DET_ENERGY 3 /* EnergyDetector       (fdtdx/objects/detectors/energy.py) */

/* One CPML slab (fdtdx/objects/boundaries/perfectly_matched_layer.py:97-190).
 * The slab spans the whole domain transverse to `axis` and `thickness` cells along it. */
typedef struct {
    int32_t axis;          /* 0, 1, 2 */
    int32_t direction;     /* -1: min side ("-"), +1: max side ("+") */
    int32_t thickness;     /* L */
    int32_t kappa_is_one;  /* 1: corrections are psi alone (perfectly_matched_layer.py:184-185) */
    const float* coef;     /* host, 6*L floats: a_E, b_E, inv_kappa_E, a_H, b_H, inv_kappa_H */
} FdtdSlabDesc;

/* One source.  All per-step tables are host arrays of length n_table = T + 2,
 * entry (t + 1) for time step t in [-1, T]. */
typedef struct {
    int32_t kind;          /* FDTD_SRC_* */
    int32_t lo[3], hi[3];  /* cell box: one cell (dipole) or one plane (TFSF) */
    int32_t component;     /* dipole: polarization axis */
    int32_t magnetic;      /* dipole: 1 injects into H (source_type "magnetic") */
    int32_t normal_axis;   /* plane: propagation axis */
    float sign;            /* plane: +1 for direction "+", -1 for "-"; dipole: unused */
    float coef;            /* dipole: c*amplitude*static_factor*inv_material_local; plane: c*static_factor */
    const float* inc_E;    /* plane: host (3, face cells) incident E profile (energy-normalised) */
    const float* inc_H;    /* plane: host (3, face cells) incident H profile (impedance-divided) */
    const float* off_E;    /* plane: host (3, face cells) Yee time offsets of E, in steps */
    const float* off_H;    /* plane: host (3, face cells) Yee time offsets of H, in steps */
    int32_t profile;       /* FDTD_PROFILE_* */
    float omega_dt;        /* carrier phase advance per step, rad */
    float ramp_inv_steps;  /* CW: dt / (num_startup_periods * period) */
    float t0_steps;        /* Gaussian: envelope centre in steps */
    float inv_two_sigma2;  /* Gaussian: dt^2 / (2 sigma_t^2) */
    const float* phase_E;  /* (omega*dt*teff + phase0) mod 2 pi, E-side time */
    const float* phase_H;  /* same at teff + 0.5, H-side time */
    const float* teff;     /* on/off-adjusted time step (fdtdx/objects/sources/source.py:41-49) */
    const uint8_t* on;     /* 1 when the source is on */
    /* plane in a dispersive scene: host table of the E side's temporal profile (the H incident
     * field's profile) at every integer step 0 .. n_e_table - 1, read by linear interpolation at
     * the fractional time and 0 outside (fdtdx/objects/sources/tfsf.py:21-141, 256-261); NULL:
     * the analytic profile */
    const float* e_table;
    int32_t n_e_table;
} FdtdSourceDesc;

/* One detector.  Tables are host arrays of length n_table (entry t + 1). */
typedef struct {
    int32_t kind;           /* FDTD_DET_* */
    int32_t lo[3], hi[3];   /* region box */
    int32_t comp_mask;      /* bit c for component c of (Ex, Ey, Ez, Hx, Hy, Hz) */
    int32_t exact_interpolation;
    int32_t reduce_volume;
    int32_t inverse;        /* phasor: subtract instead of add */
    int32_t n_freq;         /* phasor */
    int32_t flux_axis;      /* flux: propagation axis */
    float flux_sign;        /* flux: -1 for direction "-" */
    int32_t keep_all;       /* flux: keep the three Poynting components */
    float cell_weight;      /* dx^3 (volume means, energy sums) or dx^2 (flux sums) */
    const int32_t* slot;    /* state slot for time step t, -1 when off */
    const float* weights;   /* phasor: (n_table, n_freq, 2) complex weight per step */
} FdtdDetectorDesc;

typedef struct {
    int32_t nx, ny, nz;
    int32_t n_steps_total;  /* T; tables hold T + 2 entries */
    float courant;          /* courant_factor / sqrt(3) */
    int32_t n_eps;          /* 1, 3 or 9 (a full tensor, row-major) */
    int32_t n_mu;           /* 0 (scalar inv_mu), 1, 3 or 9 */
    float inv_mu_scalar;
    int32_t n_sigma_E;      /* 0 (no conductivity), 1, 3 or 9 */
    int32_t n_sigma_H;
    int32_t periodic[3];
    int32_t pec_faces;      /* bit (2*axis + side), side 1 = max face */
    int32_t pmc_faces;
    int32_t n_slabs;
    FdtdSlabDesc slabs[FDTD_MAX_SLABS];
    int32_t n_sources;
    FdtdSourceDesc sources[FDTD_MAX_SOURCES];
    int32_t n_detectors;
    FdtdDetectorDesc detectors[FDTD_MAX_DETECTORS];
    int32_t record_interfaces; /* 1: record E, H on each slab's innermost layer after every step */
    int32_t recording_dtype;   /* 0: float32, 1: bfloat16, 2: float16 */
    /* Recorder time filter (fdtdx/interfaces/time_filter.py:140-257), or rec_slots = 0 for one
     * slot per step.  Tables of n_steps_total + 2 entries (entry t + 1 for step t): the slot
     * step t is stored in (-1: not stored), and the two slots and the weight a reverse step
     * restores from: v = v[rec_a] + rec_w (v[rec_b] - v[rec_a]).  Host pointers, copied. */
    int32_t rec_slots;
    const int32_t* rec_store;
    const int32_t* rec_a;
    const int32_t* rec_b;
    const float* rec_w;
    /* Bloch boundaries with a non-zero vector (fdtdx/objects/boundaries/bloch.py:13-155): bit a
     * set when the (periodic) axis a carries the phase exp(i k_a L_a) = bloch_cos[a] + i
     * bloch_sin[a] on its '+' ghost layer (its conjugate on the '-' one).  The fields are then
     * complex: E, H, every psi array, the H twin and the interface recording hold their real
     * parts followed by their imaginary parts (planar, a leading dimension of 2); detector states
     * keep their layouts (phasors complex, the rest real).  The cotangents of fdtd_adjoint are
     * planar the same way (dL/dRe, then dL/dIm). */
    int32_t bloch_axes;
    float bloch_cos[3];
    float bloch_sin[3];
    /* dispersive (ADE) materials (fdtdx/fdtd/update.py:316-350): n_poles > 0 poles per cell
     * with recurrence coefficients of n_disp (1 or 3) components; the buffers then carry the
     * polarisation pair and the coefficient arrays.  Forward steps only (the reference's
     * reversible path refuses dispersion as well). */
    int32_t n_poles;
    int32_t n_disp;
} FdtdDesc;

typedef struct {
    float* E;                   /* (3, nx, ny, nz) */
    float* H;                   /* (3, nx, ny, nz) */
    const float* inv_eps;       /* (n_eps, nx, ny, nz) */
    const float* inv_mu;        /* (n_mu, nx, ny, nz) or NULL */
    const float* sigma_E;       /* (n_sigma_E, ...) or NULL */
    const float* sigma_H;
    float* psi_E[FDTD_MAX_SLABS][2];  /* slab-shaped psi pairs (psi_1, psi_2) */
    float* psi_H[FDTD_MAX_SLABS][2];
    void* det_state[FDTD_MAX_DETECTORS];
    void* recording;            /* (T or rec_slots, fdtd_interface_floats(plan)) in recording_dtype, or NULL */
    float* disp_P_curr;         /* (n_poles, 3, nx, ny, nz) polarisation P^n (n_poles > 0) */
    float* disp_P_prev;         /* (n_poles, 3, nx, ny, nz) P^(n-1) */
    const float* disp_c1;       /* (n_poles, n_disp, nx, ny, nz) recurrence coefficients */
    const float* disp_c2;
    const float* disp_c3;
} FdtdBuffers;

/* Cotangent (adjoint) buffers of the reversible gradient. */
typedef struct {
    float* lam_E;               /* (3, nx, ny, nz) cotangent of E */
    float* lam_H;               /* (3, nx, ny, nz) cotangent of H */
    float* lam_psi_E[FDTD_MAX_SLABS][2];
    float* lam_psi_H[FDTD_MAX_SLABS][2];
    /* cotangent of each detector state (same layout; complex states interleaved re, im,
     * with torch's convention dL/dRe + i dL/dIm), or NULL for zero.  Entries the forward
     * step overwrote (field, flux, energy slots) are cleared as the loop passes them. */
    void* lam_det[FDTD_MAX_DETECTORS];
    float* grad_inv_eps;        /* (n_eps, nx, ny, nz), accumulated (+=), or NULL */
    /* (n_mu, nx, ny, nz), accumulated (+=), or NULL; needs an inv_mu array (n_mu 1 or 3).
     * The reference's custom VJP returns this cotangent as cot[6] (fdtdx/fdtd/fdtd.py:331). */
    float* grad_inv_mu;
    /* dispersive scenes (fdtd_adjoint_stored only): cotangents of the polarisation pair,
     * (n_poles, 3, nx, ny, nz) each, updated in place like lam_E */
    float* lam_P_curr;
    float* lam_P_prev;
} FdtdAdjointBuffers;

typedef struct FdtdPlan FdtdPlan;

/* Build a plan from a scene description.  Copies all host tables. */
int fdtd_plan_create(const FdtdDesc* desc, FdtdPlan** out);
void fdtd_plan_destroy(FdtdPlan* plan);
const char* fdtd_last_error(const FdtdPlan* plan);
/* Floats per time step in the interface recording (E and H on every slab interface). */
int64_t fdtd_interface_floats(const FdtdPlan* plan);
/* Device bytes the plan itself holds (tables + scratch). */
int64_t fdtd_plan_device_bytes(const FdtdPlan* plan);
/* Device bytes one simulation of this description needs (fields, materials, psi,
 * detector states, recording, plan tables and scratch; with record_interfaces also the
 * reversible gradient's cotangents, twins, reconstruction copy and material gradients):
 * serving admission.  Computed on the host; needs no GPU. */
int64_t fdtd_footprint_bytes(const FdtdDesc* desc);

/* Forward steps t0 .. t0+n_steps-1.  flags: FDTD_FWD_GRAPH replays the loop from a CUDA graph;
 * FDTD_FWD_CHECK_FINITE scans E and H once after the last step (one read of both fields) and
 * makes the next fdtd_plan_status return FDTD_ENONFINITE when either holds a NaN or an
 * infinity (n_steps = 0 with this flag runs the check alone).  The reference raises no such
 * error: a diverging JAX run returns the non-finite arrays (fdtdx/fdtd/fdtd.py:482-496). */
#define FDTD_FWD_GRAPH 1
#define FDTD_FWD_CHECK_FINITE 2
int fdtd_forward(FdtdPlan* plan, const FdtdBuffers* bufs, int32_t t0, int32_t n_steps, int32_t flags, void* stream);

/* Reverse steps: state at t_end is taken back to t_end - n_steps.  Uses the
 * recording (interfaces re-imposed before each step) when it is non-NULL. */
int fdtd_reverse(FdtdPlan* plan, const FdtdBuffers* bufs, int32_t t_end, int32_t n_steps, void* stream);

/* Backward loop of the reversible gradient, for t = t_end-1 down to t_end-n_steps
 * (t = -1 is admitted, as the reference's loop runs one step there): reverse step
 * t+1 -> t on bufs (interfaces re-imposed, psi frozen), then the transposed forward
 * step at t.  On entry adj holds the cotangents of the state at t_end, on return
 * those of the state at t_end - n_steps; grad_inv_eps and grad_inv_mu accumulate
 * (fdtdx/fdtd/fdtd.py:324-333 returns both material cotangents).  The first call
 * allocates the plan's adjoint scratch (cotangent twins, detector snapshots);
 * fdtd_plan_device_bytes counts it from then on. */
int fdtd_adjoint(FdtdPlan* plan, const FdtdBuffers* bufs, const FdtdAdjointBuffers* adj, int32_t t_end,
                 int32_t n_steps, void* stream);

/* Backward loop over stored states: the exact gradient of GradientConfig(method="checkpointed"),
 * where the reference differentiates its checkpointed while loop (fdtdx/fdtd/fdtd.py:421-496).
 * states[q], q = 0 .. n_steps, hold the full state (E, H, psi; materials and detector states
 * as in any FdtdBuffers) of step t0 + q, recomputed by the caller from a checkpoint.  For
 * t = t0 + n_steps - 1 down to t0 the transposed forward step at t runs at the stored states
 * of steps t and t + 1 -- no reconstruction, so psi is exact and so is the gradient inside
 * the CPML.  adj as in fdtd_adjoint (cotangents of state t0 + n_steps in, of state t0 out;
 * grad_inv_eps accumulates).  Real fields with 1 or 3 material components; dispersive scenes
 * transpose the ADE step as well (their states carry the polarisation pair, adj its
 * cotangents lam_P_curr / lam_P_prev); grad_inv_mu is not provided (FDTD_EINVAL). */
int fdtd_adjoint_stored(FdtdPlan* plan, const FdtdBuffers* states, int32_t t0, int32_t n_steps,
                        const FdtdAdjointBuffers* adj, void* stream);

/* Tuning of the update kernels: `chunk` x planes per block, `vec` z cells per thread
 * (1, 2 or 4, dividing nz); 0 restores a default.  Invalidates a cached CUDA graph.
 * fdtd_plan_chunk / fdtd_plan_vec return the current values. */
int fdtd_plan_tune(FdtdPlan* plan, int32_t chunk, int32_t vec);
int32_t fdtd_plan_chunk(const FdtdPlan* plan);
int32_t fdtd_plan_vec(const FdtdPlan* plan);
/* The same for the CPML shell boxes of a grid split into a slab-free core and its shell:
 * `chunk` x planes per block (default 4), `vec` z cells per thread (default 1; 2 or 4 need
 * nz % 4 == 0).  Invalidates a cached CUDA graph. */
int fdtd_plan_tune_shell(FdtdPlan* plan, int32_t chunk, int32_t vec);

/* Selects the TMA-pipelined update kernels (enable=1; scenes without periodic axes and
 * with nz % 4 == 0) or the register-queue kernels (enable=0), with a (y, z) tile of
 * ty x tz cells (tz a multiple of 4), `stages` pipeline stages and `chunk` x planes per
 * block; 0 picks a default.  fdtd_plan_uses_tma reports the current choice. */
int fdtd_plan_tune_tma(FdtdPlan* plan, int32_t enable, int32_t tz, int32_t ty, int32_t stages, int32_t chunk);
int32_t fdtd_plan_uses_tma(const FdtdPlan* plan);

/* Where the CPML slab cells of a grid split into a slab-free core and its shell run, when the
 * core runs on the TMA kernels: mode 0, the register-queue shell kernel over the six slab
 * boxes; mode 1, the TMA kernels with in-tile slab terms over the whole x and y extent (the x
 * and y slabs) and the shell kernel over the two z boxes; mode 2, the whole grid in one launch
 * of the TMA kernels with every slab term in the tiles (tile z extent `tz`, 0: picked for nz);
 * mode 3 (split), the plain TMA kernels over the whole grid on the mode-2 tile, then the
 * CPML corrections of the slab cells, one launch per axis (forward and reverse steps); mode 4, the same with the z slabs' terms inside the TMA tiles; mode 5 (the default
 * where the scene admits it), mode 4 for the E half-step and mode 3 for the H half-step.
 * `chunk` x planes per block (0: a default).  fdtd_plan_shell_tma returns the mode in use. */
int fdtd_plan_tune_shell_tma(FdtdPlan* plan, int32_t mode, int32_t tz, int32_t chunk);
int32_t fdtd_plan_shell_tma(const FdtdPlan* plan);

/* Reads and clears the kernels' error word (synchronises the device): FDTD_OK,
 * FDTD_ETIMEOUT when a bounded pipeline wait ran out during an earlier call, or
 * FDTD_ENONFINITE when a finite check (FDTD_FWD_CHECK_FINITE) found a NaN or an infinity. */
int fdtd_plan_status(FdtdPlan* plan);

/* Failure injection for tests of the error paths (no counterpart in the reference, whose
 * errors are Python exceptions at trace time).  No GPU fault is involved in either kind:
 *   FDTD_INJECT_ALLOC        the next `count` device allocations of the library (plan tables,
 *                            adjoint scratch, batch tables) report out-of-memory without
 *                            calling cudaMalloc: the call returns FDTD_ENOMEM;
 *   FDTD_INJECT_WAIT_EXPIRY  the next `count` TMA half-step launches issued outside stream
 *                            capture take their bounded-wait error exit before issuing any
 *                            copy: they update nothing, and the plan's next fdtd_plan_status
 *                            returns FDTD_ETIMEOUT;
 *   FDTD_INJECT_BARRIER_EXPIRY the next `count` fused batch launches (fdtd_batch_set_mode 2)
 *                            run with one block that never arrives at the first grid barrier
 *                            and a short wait limit: the other blocks' waits run out and the
 *                            fdtd_batch_forward call returns FDTD_ETIMEOUT.
 * count = 0 clears a kind.  Process-wide; returns FDTD_EINVAL for an unknown kind. */
#define FDTD_INJECT_ALLOC 1
#define FDTD_INJECT_WAIT_EXPIRY 2
#define FDTD_INJECT_BARRIER_EXPIRY 3
int fdtd_debug_inject(int32_t kind, int32_t count);

/* Number of launches of this library's kernels one forward step issues. */
int32_t fdtd_launches_per_step(const FdtdPlan* plan);

/* Benchmark helper: runs forward steps t0 .. t0+n_steps-1 with CUDA events on `stream`
 * around each launch and writes the mean device time per step, in ms, of:
 * out_ms[0] E core, [1] E CPML shell, [2] E-side sources, [3] H core (with the fused
 * detectors), [4] H CPML shell, [5] H-side sources, [6] detectors, [7] interface
 * recording (a grid that does not split reports its whole update as the shell).
 * Synchronises the stream. */
int fdtd_profile_forward(FdtdPlan* plan, const FdtdBuffers* bufs, int32_t t0, int32_t n_steps, float* out_ms, void* stream);

/* ---- Batched forward path: many simulations stepped together --------------------------
 *
 * No counterpart in the reference (which runs one simulation per call, fdtdx/fdtd/fdtd.py:
 * 421-496); it replaces looping that call over a set of simulations.  A batch holds built
 * plans with their buffers.  One batch step runs every simulation's forward step with
 * one persistent launch per kernel kind (E update, E sources, H update with fused
 * detectors, H sources, interface recording, detectors, reductions, step counters)
 * over a flat list of work units; results equal the per-plan fdtd_forward
 * (same device bodies).  The plans must stay alive and unused elsewhere while the
 * batch exists. */
typedef struct FdtdBatch FdtdBatch;
int fdtd_batch_create(FdtdPlan* const* plans, const FdtdBuffers* bufs, int32_t n, FdtdBatch** out);
void fdtd_batch_destroy(FdtdBatch* batch);
const char* fdtd_batch_last_error(const FdtdBatch* batch);
/* n_steps batch steps.  t0: per-simulation start step (NULL: continue where each
 * stopped).  flags bit 0: CUDA graph of the step loop; bit 1: autotune the tile shapes
 * on the first steps of this call (once per batch; at most n_steps / 4 steps, all of
 * them real simulation steps). */
int fdtd_batch_forward(FdtdBatch* batch, const int32_t* t0, int32_t n_steps, int32_t flags, void* stream);
/* Tile shapes: core x-chunk = each plan's default chunk * num / den, shell x-chunk,
 * resident blocks per SM of the persistent launches.  fdtd_batch_tuning reads them
 * (out4 = {num, den, shell_chunk, blocks_per_sm}). */
int fdtd_batch_tune(FdtdBatch* batch, int32_t chunk_num, int32_t chunk_den, int32_t shell_chunk, int32_t blocks_per_sm);
int fdtd_batch_tuning(const FdtdBatch* batch, int32_t* out4);
/* Execution mode: 0 = persistent launches over the unit lists (default), 1 = each
 * simulation's own per-plan launch chain on its own stream, forked from and joined to the
 * caller's stream (parallel branches of one CUDA graph), 2 = every step of a
 * fdtd_batch_forward call in ONE cooperative launch, the phases of a step separated by a
 * grid-wide barrier whose waits are bounded (an expired wait makes the call return
 * FDTD_ETIMEOUT); in mode 2 fdtd_batch_forward waits for its launch before it returns.
 * The autotuner (fdtd_batch_forward flag bit 1) times the modes and keeps the fastest. */
int fdtd_batch_set_mode(FdtdBatch* batch, int32_t mode);
int32_t fdtd_batch_mode(const FdtdBatch* batch);
/* Launches of this library's kernels one batch step issues (for the whole batch; 1 in
 * mode 2, where one launch runs all the steps of a call). */
int32_t fdtd_batch_launches_per_step(const FdtdBatch* batch);

/* Allocation-free sample of one volume-reducing detector (no counterpart in the
 * reference: there the sample is part of the jitted step, fdtdx/fdtd/update.py:1040-1137).
 *
 * Evaluates the reduced value a FIELD (component mean), FLUX (Poynting flux summed over
 * the region times cell_weight) or ENERGY (energy summed times cell_weight) detector
 * records at one step, from the fields E (after the step), H_prev (H before the step's H
 * update; read, and required, only when det->exact_interpolation and the sample reads H: a
 * FLUX or ENERGY sample, or a FIELD sample of H components) and H, and writes its ncomp floats to
 * the device buffer `out` (ncomp: the recorded components for FIELD, 3 or 1 for FLUX,
 * 1 for ENERGY).  det->slot, det->weights and det->reduce_volume are ignored.
 *
 * It needs no plan and allocates no device memory: the block partial sums live in a
 * static device array of FDTD_NOALLOC_SCRATCH_FLOATS floats, so a region needing more
 * than that many partials (ceil(cells / 256) x ncomp) is rejected with FDTD_EINVAL and a
 * message on stderr.  Nothing in the scratch has to start at zero: every partial is
 * written before it is read, and the step word and slot table it also holds are
 * zero-initialised with the library and never written.  The first call on a device
 * looks up the scratch address (cudaGetSymbolAddress) with that device current; make
 * that first call before any stream capture.  Every later call made outside a capture
 * looks it up again (a device reset may move the array); a call inside a capture uses the
 * address of the last call on that device.  The scratch is shared by all calls on a
 * device: calls that overlap (other streams, other host threads) race on it and must be
 * serialised by the caller.  Same arithmetic as the plan's detector kernels. */
#define FDTD_NOALLOC_SCRATCH_FLOATS 65536
int fdtd_detector_sample_noalloc(const FdtdDetectorDesc* det, int32_t nx, int32_t ny, int32_t nz,
                                 const int32_t periodic[3], const float* E, const float* H_prev, const float* H,
                                 const float* inv_eps, int32_t n_eps, const float* inv_mu, int32_t n_mu,
                                 float inv_mu_scalar, float* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FDTD_GB300_H */
