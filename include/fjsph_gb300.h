/*
 * fjsph_gb300.h -- C ABI of the GB300 WCSPH hot path.
 *
 * This library replaces three subsystems of FJSPH (farg-bristol/FJSPH) with device-resident
 * sm_103a kernels: the neighbour search (src/Neighbours.cpp), the particle residual and its
 * pre-passes (src/Resid.cpp, src/Shifting.cpp, src/Geometry.cpp:14-308, src/Kernel.h,
 * src/Aero.h) and the time integrators with the CFL time-step reduction (src/Runge_Kutta.cpp,
 * src/Newmark_Beta.cpp, src/Integration.cpp).
 *
 * Conventions (all entry points):
 *   - Plain C types only; every pointer is a host pointer unless the name says otherwise.
 *   - Every function returns an int status: FJSPH_OK (0) or a negative FJSPH_E_* code.  The
 *     reference prints and calls exit(-1) on errors; this library never exits.
 *   - A context owns its device memory and one CUDA stream.  Calls on one context must come from
 *     one host thread at a time (the reference functions are not re-entrant either).
 *   - Particle order at the boundary is the reference's index order: boundary blocks first, then
 *     fluid blocks, each block a contiguous index range (LIMITS, src/Var.h:820-883).  Inside the
 *     context particles are kept in cell order; upload and download convert.
 *   - Vectors are stored per particle as `dim` consecutive doubles (x,y[,z]); the 2x2/3x3 L
 *     matrix as dim*dim doubles, row-major.
 */
#ifndef FJSPH_GB300_H
#define FJSPH_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------------------- */
#define FJSPH_OK 0
#define FJSPH_E_ARG (-1)         /* bad argument (null pointer, size, unsupported option)    */
#define FJSPH_E_CUDA (-2)        /* a CUDA runtime call failed                               */
#define FJSPH_E_CAPACITY (-3)    /* particle count above the context capacity                */
#define FJSPH_E_NEIGHBOUR (-4)   /* neighbour list storage could not be grown                */
#define FJSPH_E_NONFINITE (-5)   /* NaN/Inf found in positions or in the residual            */
#define FJSPH_E_UNSUPPORTED (-6) /* variant combination the reference cannot build either    */
#define FJSPH_E_STATE (-7)       /* call order error (e.g. residual before neighbour search) */

/* ---- particle types (src/VarDefs.h:92-102) ------------------------------------------------- */
enum fjsph_part_type {
    FJSPH_BOUND = 0,
    FJSPH_PISTON = 1,
    FJSPH_BUFFER = 2,
    FJSPH_BACK = 3,
    FJSPH_PIPE = 4,
    FJSPH_FREE = 5,
    FJSPH_OUTLET = 6,
    FJSPH_LOST = 7
};

/* ---- compile-time physics variants of the reference, as run-time bits -------------------- */
/* Each bit stands for one -D flag of the reference makefile (README "Building"). */
#define FJSPH_VAR_ALE (1u << 0)      /* -DALE: ALE momentum/continuity + particle shifting  */
#define FJSPH_VAR_LINEAR (1u << 1)   /* -DLINEAR: Marrone pressure form, linear art. visc.  */
#define FJSPH_VAR_NOFROZEN (1u << 2) /* -DNOFROZEN: art. visc. + delta-SPH inside residual   */
#define FJSPH_VAR_NODSPH (1u << 3)   /* -DNODSPH: no delta-SPH continuity term              */
#define FJSPH_VAR_TIC (1u << 4)      /* -DTIC: tensile-instability control                  */
#define FJSPH_VAR_CUBIC (1u << 5)    /* -DCUBIC: cubic spline kernel instead of Wendland C2 */

/* Surface-tension model (-DPAIRWISE default, -DCSF, -DNOST; -DHESF does not build upstream). */
enum fjsph_st_model { FJSPH_ST_PAIRWISE = 0, FJSPH_ST_NOST = 1, FJSPH_ST_CSF = 2 };

/* Enumerations mirrored from src/VarDefs.h:129-166. */
enum fjsph_solver { FJSPH_NEWMARK_BETA = 0, FJSPH_RUNGE_KUTTA = 1 };
enum fjsph_bound_solver { FJSPH_DBC = 0, FJSPH_PRESSURE_G = 1, FJSPH_GHOST = 2 };
enum fjsph_eos { FJSPH_COLE_EOS = 0, FJSPH_ISO_EOS = 1 };
enum fjsph_aero_case { FJSPH_NOAERO = 0, FJSPH_GISSLER = 1, FJSPH_INDUCED_PRESSURE = 2, FJSPH_SKIN_FRIC = 3 };
/* Air velocity source (src/VarDefs.h:168-173): uniform v_inf, the cells of the mesh given to
 * fjsph_mesh_set, the vortex-lattice field of fjsph_vlm_setup (3D). */
enum fjsph_aero_source { FJSPH_CONST_VEL = 0, FJSPH_MESH_INFL = 1, FJSPH_VLM_INFL = 2,
                         /* analytic boundary-layer air field (no reference counterpart):
                          * fjsph_air_power_law */
                         FJSPH_POWER_LAW = 100 };

/* Arithmetic form of the pair kernels. */
enum fjsph_precision {
    FJSPH_PREC_FP64 = 0,  /* plain FP64 everywhere                                            */
    FJSPH_PREC_MIXED = 1  /* FP32 pair arithmetic on cell-relative positions, compensated sums, */
                          /* FP64 membership test / integration / dt / global sums             */
};

/* Aerodynamic closure used inside the residual. */
enum fjsph_aero_closure {
    FJSPH_CLOSURE_PLAIN = 0,  /* Gissler occlusion + drag (src/Aero.h:37-98)         */
    FJSPH_CLOSURE_LEARNED = 1 /* BF16 MLP stand-in for occlusion and drag coefficient */
};

/*
 * Settings: the subset of SIM / FLUID / AERO / INTEG_SETT (src/Var.h:63-394) that the hot path
 * reads, with the values that Set_Values (src/IO.cpp:26-128) derives already filled in.
 * fjsph_settings_defaults() + fjsph_settings_derive() give the reference's defaults and
 * derivations; the Python host layer fills the same struct from a para file.
 */
typedef struct fjsph_settings {
    int32_t dim;            /* SIMDIM: 2 or 3                                           */
    uint32_t variant;       /* FJSPH_VAR_* bits                                         */
    int32_t st_model;       /* fjsph_st_model                                           */
    int32_t precision;      /* fjsph_precision                                          */
    int32_t aero_closure;   /* fjsph_aero_closure                                       */
    int32_t solver_type;    /* fjsph_solver                                             */

    /* FLUID */
    int32_t pressure_rel;   /* fjsph_eos                                                */
    double H, H_sq, sr, H_fac, W_dx, W_correc;
    double rho_rest, rho_pipe, press_pipe, press_back, rho_max, rho_min, rho_var, rho_max_iter;
    double sim_mass, bnd_mass, visc_alpha, speed_sound, mu, nu, sig, gam, B, contangb;
    double dsph_delta, dsph_cont;

    /* SIM */
    double particle_step, dx, scale;
    double grav[3];
    int32_t asource;        /* fjsph_aero_source; FJSPH_VLM_INFL needs fjsph_vlm_setup   */
    int32_t init_hydro_pressure;
    double hydro_height;
    int64_t max_points;

    /* AERO */
    int32_t acase, use_lam, use_TAB_def, use_dx;
    double v_inf[3];
    double L, td, omega, tmax, ycoef, Cf, Ck, Cd, Cb, Cdef, A_sphere, A_plate;
    double v_ref, p_ref, rho_g, mu_g, mass_g, temp_g, R_g, gamma_g, sos, i_sos_sq, M_ref;
    double lam_cutoff, interp_fac, i_interp_fac, n_full, i_n_full, i_n_count;

    /* INTEG_SETT */
    int32_t max_subits, n_stable, n_stable_limit, n_unstable, n_unstable_limit;
    double subits_factor, cfl, cfl_step, cfl_max, cfl_min, current_time, last_frame_time;
    double frame_time_interval, min_residual, delta_t, delta_t_max, delta_t_min;
    double nb_beta, nb_gamma, max_shift_vel;

    /* Extensions of this library (no reference counterpart). */
    int32_t reorder_interval; /* re-sort particle storage every N neighbour searches (0 = never) */
    int32_t learned_judge_interval; /* re-run the plain closure every N steps (learned form) */
} fjsph_settings;

/* One LIMITS entry (src/Var.h:820-881). */
#define FJSPH_MAX_TIMES 16
typedef struct fjsph_block {
    int64_t first, second;      /* index range [first, second)                         */
    int32_t is_fluid;           /* 0 = boundary block, 1 = fluid block                  */
    int32_t bound_solver;       /* fjsph_bound_solver (boundary blocks)                 */
    int32_t no_slip;
    int32_t block_type;         /* shape_type (src/VarDefs.h:116-127); 6 = inletZone    */
    int32_t fixed_vel_or_dynamic;
    int32_t n_times;            /* motion table length; 0 = constant vels[0]           */
    double times[FJSPH_MAX_TIMES];
    double vels[FJSPH_MAX_TIMES][3];
    double delete_norm[3], delconst;
    double insert_norm[3], insconst;
    double aero_norm[3], aeroconst;
} fjsph_block;

/* Inlet bookkeeping of one inletZone block: back[n_back], buffer[n_back][depth] (reference indices). */
typedef struct fjsph_inlet {
    int32_t block;
    int64_t n_back, depth;
    int64_t *back;
    int64_t *buffer;
} fjsph_inlet;

/*
 * Host view of an SPHState (src/Var.h:499-642, only the fields the hot path touches), as
 * structure-of-arrays.  n particles; vector fields hold n*dim doubles, L holds n*dim*dim.
 */
typedef struct fjsph_state_view {
    int64_t n;
    double *xi, *v, *acc, *Af, *aVisc, *cellV, *gradRho, *norm, *vPert; /* n*dim   */
    double *L;                                                            /* n*dim^2 */
    double *Rrho, *rho, *p, *m, *curve, *norm_curve, *woccl, *pDist, *deltaD;
    double *cellP, *cellRho, *colourG, *colour, *lam, *lam_nb, *kernsum;
    int64_t *part_id, *cellID;
    int32_t *b, *surf, *surfzone;
} fjsph_state_view;

/* Opaque device context. */
typedef struct fjsph_ctx fjsph_ctx;

/* Which of the two states a call reads or writes: time n (pn) or the working state (pnp1). */
#define FJSPH_PN 0
#define FJSPH_PNP1 1
#define FJSPH_BOTH 2 /* upload only: the state becomes both pn and pnp1 (one host transfer) */

/* ---- settings helpers (src/Var.h defaults, src/IO.cpp:26-128 Set_Values) -------------------- */
int fjsph_settings_defaults(fjsph_settings *s, int32_t dim);
int fjsph_settings_derive(fjsph_settings *s);

/* ---- context ------------------------------------------------------------------------------ */
/* capacity = maximum particle count (SIM::max_points analogue).  Replaces the setup half of
 * src/FJSPH.cpp:104-149 (state vectors, KD-tree adaptor). */
int fjsph_ctx_create(const fjsph_settings *s, int64_t capacity, fjsph_ctx **out);
int fjsph_ctx_destroy(fjsph_ctx *ctx);
int fjsph_set_settings(fjsph_ctx *ctx, const fjsph_settings *s);
int fjsph_get_settings(fjsph_ctx *ctx, fjsph_settings *s);
/* LIMITS (src/Var.h:883) and the inlet back/buffer tables (src/shapes/inlet.cpp:578-640). */
int fjsph_set_limits(fjsph_ctx *ctx, const fjsph_block *blocks, int32_t nblocks, int64_t n_bound_blocks);
int fjsph_set_inlet(fjsph_ctx *ctx, const fjsph_inlet *inlet);
int fjsph_get_inlet(fjsph_ctx *ctx, fjsph_inlet *inlet); /* current tables, reference indices */
/* The LIMITS table as the particle-set changes of update_data left it (ranges move with
 * insertion and deletion, src/shapes/inlet.cpp:621-626, src/Integration.cpp:190-205). */
int fjsph_get_limits(fjsph_ctx *ctx, fjsph_block *blocks, int32_t max_blocks, int32_t *nblocks);
/* Particles inserted and deleted by update_data since the context was created. */
int fjsph_update_counts(fjsph_ctx *ctx, int64_t *inserted, int64_t *deleted);
/* Replaces the SPHState hand-over between Integrator and its callers (src/Integration.h:15-68).
 * A null array in the view skips that field: an upload leaves the device copy as it is, a
 * download leaves the host array unwritten (at least one array must be given).  Every field a
 * step reads before writing it (FJSPH_STEP_FIELDS below) has to be uploaded before the first
 * step; the others are recomputed inside the step. */
int fjsph_state_upload(fjsph_ctx *ctx, int32_t which, const fjsph_state_view *st);
int fjsph_state_download(fjsph_ctx *ctx, int32_t which, fjsph_state_view *st);
/* The fields a step reads before it writes them: positions, velocities, the previous step's
 * acceleration and density rate (Runge-Kutta and Newmark-Beta weights), density, pressure,
 * mass, the air cell values, the shifting velocity, the frozen dissipation terms and the
 * previous surface detection (the first stage uses them, src/Runge_Kutta.cpp:461-476), the
 * particle type, id and cell.  The rest (Af, gradRho, L, kernsum, colour, colourG, pDist) is
 * recomputed before it is read. */
/* One Integrator::integrate on a host state (src/Integration.h:15-68 with the SPHState in host
 * memory): uploads `in` as pn and pnp1, steps, and downloads pnp1 into `out` (null arrays are
 * skipped both ways; `in` and `out` may share arrays).  The same results as fjsph_state_upload
 * (FJSPH_BOTH), fjsph_integrate and fjsph_state_download, but the copies overlap the step: the
 * inputs travel in groups ordered by their first reader (positions, time-step inputs, packing
 * inputs, the rest) while the search runs, and under Runge-Kutta the fields final after the
 * second search's pre-passes and the last residual travel out during the remaining work.
 * out->n: on entry the particles its arrays can
 * hold (FJSPH_E_CAPACITY after the step if insertion outgrew it), on return the particle count.
 * Not for contexts holding independent simulations (fjsph_set_groups). */
int fjsph_step_host(fjsph_ctx *ctx, const fjsph_state_view *in, fjsph_state_view *out, double *rms_error);
#define FJSPH_STEP_FIELDS \
    "xi v acc Rrho rho p m cellV cellP cellRho vPert aVisc deltaD woccl lam lam_nb curve norm norm_curve " \
    "b part_id cellID surf surfzone"
int fjsph_particle_count(fjsph_ctx *ctx, int64_t *n_total, int64_t *n_bound);

/* ---- neighbour search (src/Neighbours.cpp:7-47) ------------------------------------------- */
/* update_neighbours on pnp1: all pairs with squared distance < sr, self included. */
int fjsph_update_neighbours(fjsph_ctx *ctx, int64_t *n_pairs);
/* Export the lists in reference order: offsets[n+1], idx[n_pairs], d2[n_pairs] (each list sorted
 * by neighbour index).  Any pointer may be NULL to skip it. */
int fjsph_neighbours_export(fjsph_ctx *ctx, int64_t *offsets, int64_t *idx, double *d2);

/* ---- pre-passes ------------------------------------------------------------------------------ */
int fjsph_dsph_prestep(fjsph_ctx *ctx, double *npd);       /* src/Shifting.cpp:12-123      */
int fjsph_get_aero_velocity(fjsph_ctx *ctx);               /* src/Resid.cpp:471-613, constVel */
int fjsph_detect_surface(fjsph_ctx *ctx);                  /* src/Geometry.cpp:14-280      */
int fjsph_dissipation_terms(fjsph_ctx *ctx);               /* src/Shifting.cpp:126-186     */
int fjsph_particle_shift(fjsph_ctx *ctx);                  /* src/Shifting.cpp:189-290     */
int fjsph_check_pipe_outlet(fjsph_ctx *ctx);               /* src/Containment.cpp:822-894 (constVel) */

/* ---- boundary passes and residual on pnp1 -------------------------------------------------- */
int fjsph_get_boundary_pressure(fjsph_ctx *ctx);           /* src/Resid.cpp:21-76          */
int fjsph_boundary_ghost(fjsph_ctx *ctx, int32_t *near_inlet); /* src/Resid.cpp:122-160    */
int fjsph_boundary_dbc(fjsph_ctx *ctx);                    /* src/Resid.cpp:78-117         */
int fjsph_set_no_slip(fjsph_ctx *ctx);                     /* src/Resid.cpp:162-186        */
int fjsph_get_acc_and_rrho(fjsph_ctx *ctx, double npd);    /* src/Resid.cpp:426-469        */

/* ---- integrators and time step --------------------------------------------------------------- */
int fjsph_find_timestep(fjsph_ctx *ctx, double *dt);       /* src/Integration.cpp:370-443  */
/* Get_First_RK (src/Runge_Kutta.cpp:462-476): pnp1 = intermediate(pn, pn, dt/2). */
int fjsph_get_first_rk(fjsph_ctx *ctx, double npd, double *logbase);
/* Runge_Kutta4 (src/Runge_Kutta.cpp:480-515) with st_1 = pnp1 on entry; pnp1 = result. */
int fjsph_runge_kutta4(fjsph_ctx *ctx, double npd, double logbase, double *rms_error);
/* Newmark_Beta::Do_NB_Iter (src/Newmark_Beta.cpp:54-301), one sub-iteration on pnp1. */
int fjsph_nb_iter(fjsph_ctx *ctx, double npd);
/* Newmark_Beta::Newmark_Beta (src/Newmark_Beta.cpp:303-331), full sub-iteration loop. */
int fjsph_newmark_beta(fjsph_ctx *ctx, double npd, double *logbase, int32_t *iteration, double *rms_error);

/* Integrator::integrate_no_update (src/Integration.cpp:27-107). */
int fjsph_integrate_no_update(fjsph_ctx *ctx, double *rms_error);
/* Integrator::integrate (src/Integration.cpp:233-303): one full step incl. update_data. */
int fjsph_integrate(fjsph_ctx *ctx, double *rms_error);
/* Run n_steps of integrate() back to back without host round trips where possible. */
int fjsph_integrate_n(fjsph_ctx *ctx, int32_t n_steps, double *last_error);

/* ---- time-step bound without allocation --------------------------------------------------- */
/* No counterpart in the reference.  The CFL time-step bound of fjsph_find_timestep for callers
 * that may not call cudaMalloc (their device memory belongs to another allocator or pool, or no
 * allocation is allowed on their time-step path).  No context is needed and nothing is
 * allocated: the reduction's scratch is a fixed 256 KB __device__ array held by every GPU that
 * loads this library.
 *   - acc, Af, v, vPert: arrays of `dim` device pointers (x, y[, z] components); Rrho, rho, curve:
 *     device pointers; each holds the n_fluid fluid particles.  vPert is read only with
 *     FJSPH_VAR_ALE (may be NULL otherwise).
 *   - n_fluid <= 16,777,216; larger counts return FJSPH_E_CAPACITY.
 *   - dt (host) receives the time step of src/Integration.cpp:370-443 under the settings' cfl,
 *     dt limits and frame time; maxima7 (host) receives maxf, maxAf, maxdrho, maxRhoi, minST,
 *     maxU, maxShift.  maxShift here is the largest shifting velocity of this call's particles
 *     only; fjsph_find_timestep keeps a running maximum over the context's calls, as the
 *     reference's never-reset member does.
 *   - stream: a cudaStream_t (NULL = default stream); the call synchronises it before returning.
 *   - The first call on a device looks up the scratch array's device address (once per device,
 *     with that device current); make that first call before any stream capture.
 *   - All calls share the scratch array: calls that overlap on the GPU race; serialise them. */
int fjsph_find_timestep_noalloc(const fjsph_settings *s, int64_t n_fluid, const double *const acc[3],
                                const double *const Af[3], const double *Rrho, const double *rho,
                                const double *curve, const double *const v[3], const double *const vPert[3],
                                void *stream, double *dt, double *maxima7);

/* ---- independent simulations in one context ------------------------------------------------- */
/* No reference counterpart.  Many independent simulations of the same settings (the batched
 * droplet workload) share one context: the state holds all of them, each a contiguous range of
 * reference indices first[g] .. first[g + 1] - 1 (first[0] = 0, first[ngroups] = particle count),
 * placed far enough apart that no particle of one is within the support of another.  Each group
 * keeps its own free-stream velocity v_inf[3 g .. 3 g + 2], time step, npd, CFL number, time and
 * Runge-Kutta error, exactly as a context holding it alone would.  Runge-Kutta only; no inlets or
 * deletion planes.  Set after the limits and before (or after) the state upload. */
int fjsph_set_groups(fjsph_ctx *ctx, int32_t ngroups, const int64_t *first, const double *v_inf);
/* n_steps Integrator::integrate steps of every group, enqueued without host round trips.  With
 * use_graph the step is captured once as a CUDA graph (one per pattern of re-ordering searches)
 * and replayed; the neighbour storage is then fixed at 1.5x the lists of the last ordinary step
 * and FJSPH_E_NEIGHBOUR reports lists that outgrew it (run again: the storage grows). */
int fjsph_integrate_groups(fjsph_ctx *ctx, int32_t n_steps, int32_t use_graph);
/* Per-group time, dt of the last step, CFL number, log10 RMS error and steps taken (arrays of
 * ngroups; any pointer may be NULL). */
int fjsph_group_report(fjsph_ctx *ctx, double *time, double *dt, double *cfl, double *err, int64_t *steps);

/* ---- launch-configuration autotuner (split-precision form) --------------------------------- */
/* No reference counterpart.  cfg3 = {block size of the pair sweeps, block size of the residual,
 * pair-list rows prefetched ahead by the residual}; block sizes 32, 64, 96 or 128, rows 1-16. */
int fjsph_set_tuning(fjsph_ctx *ctx, const int32_t *cfg3);
int fjsph_get_tuning(fjsph_ctx *ctx, int32_t *cfg3);
/* Times each candidate (sweep block 64/128; residual block 64/128 x rows ahead 2/4/8) `repeats`
 * times on the current state and neighbour lists, keeps the fastest and returns it in chosen3;
 * times_ms (8 doubles, may be NULL) receives the mean time of every candidate in that order. */
int fjsph_autotune(fjsph_ctx *ctx, int32_t repeats, int32_t *chosen3, double *times_ms);
/* Times the residual in grid order and in the SM-local order (fjsph_set_sweep_order) `repeats`
 * times each with the current tuning, keeps the faster order and returns it in chosen; times_ms
 * (2 doubles, may be NULL) receives the mean time of each, grid order first. */
int fjsph_autotune_order(fjsph_ctx *ctx, int32_t repeats, int32_t *chosen, double *times_ms);

/* ---- learned aerodynamic closure ------------------------------------------------------------ */
/* No counterpart in the reference: a 12 -> 64 -> 64 -> 64 -> 2 GELU network (BF16 weights, FP32
 * accumulation) that stands in for the Gissler occlusion factor and drag coefficient
 * (src/Aero.h:37-98, src/Geometry.cpp:233-255) in the split-precision residual.  Its inputs and
 * outputs per particle are listed in fjsph_gb300/csrc/closure.cuh.  Parameters are one FP32
 * vector of fjsph_mlp_num_params() floats:
 *   W1[64][16] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] W4[8][64] b4[8]
 *   in_shift[16] in_scale[16] out_shift[2] out_scale[2]
 * (row = output; inputs padded to 16 and outputs to 8 with zero weights; the network sees
 * (x - in_shift) * in_scale and returns y * out_scale + out_shift). */
#define FJSPH_MLP_INPUTS 12
#define FJSPH_MLP_OUTPUTS 2
#define FJSPH_CLOSURE_ARM_JUDGE 1 /* next residual: learned closure judged against the plain one */
#define FJSPH_CLOSURE_ARM_LOG 2   /* next residual: plain closure, inputs and targets logged    */

typedef struct fjsph_closure_report {
    int64_t judged;           /* judge evaluations completed                                   */
    int64_t judged_particles; /* particles compared by the last evaluation                     */
    double last_rel_rms;      /* RMS |a_learned - a_plain| / RMS |a_plain|, last evaluation    */
    double max_rel_rms;       /* largest over all evaluations                                  */
    double judge_tol;         /* fallback threshold                                            */
    int64_t logged;           /* samples held in the log                                       */
    int64_t log_capacity;
    int64_t steps;            /* integrate() steps counted by the judge / log schedule         */
    int32_t learned_active;   /* 1 while residuals use the learned closure                     */
    int32_t fallback;         /* 1 once an evaluation exceeded judge_tol (plain closure since) */
} fjsph_closure_report;

int fjsph_mlp_num_params(void);
/* Host arrays: X[n][12] -> Y[n][2] (outputs un-normalised). */
int fjsph_mlp_forward(const float *params, const float *X, int64_t n, float *Y);
/* Mean squared error over the 2 normalised outputs, summed, per sample: loss = (1/n) sum_s
 * sum_o ((y_so - t_so) / out_scale_o)^2 in normalised units, and its gradient with respect to the
 * trainable part of params (the first kNumWeights floats; the normalisation stays fixed). */
int fjsph_mlp_gradient(const float *params, const float *X, const float *T, int64_t n, float *grad, double *loss);
/* Adam on the GPU over (X, T): `epochs` passes in a seeded random order, mini-batches of `batch`
 * samples, learning rate lr with a cosine decay to lr/20.  params is updated in place;
 * final_loss receives the mean loss of the last epoch. */
int fjsph_mlp_train(float *params, const float *X, const float *T, int64_t n, int32_t epochs, int32_t batch, float lr,
                    uint64_t seed, double *final_loss);
/* Weights of the context's learned closure (settings.aero_closure = FJSPH_CLOSURE_LEARNED uses
 * them in the split-precision residual).  Every settings.learned_judge_interval-th step the
 * first residual also runs the plain closure; once the relative RMS aero-force error exceeds
 * judge_tol the context falls back to the plain closure (see fjsph_closure_report). */
int fjsph_closure_set_weights(fjsph_ctx *ctx, const float *params, double judge_tol);
int fjsph_closure_get_weights(fjsph_ctx *ctx, float *params);
/* Sample log on the device: while the plain closure is in use, the first residual of every
 * every_n_steps-th step appends (inputs, targets) of each particle the network would cover.
 * capacity 0 frees the log. */
int fjsph_closure_log(fjsph_ctx *ctx, int64_t capacity, int32_t every_n_steps);
/* Copies up to max_samples logged samples to X[.][12], T[.][2]; *count = samples copied. */
int fjsph_closure_log_read(fjsph_ctx *ctx, float *X, float *T, int64_t max_samples, int64_t *count, int32_t reset);
/* One-shot: make the next residual a judge (FJSPH_CLOSURE_ARM_JUDGE) or log (..._LOG) call. */
int fjsph_closure_arm(fjsph_ctx *ctx, int32_t what);
int fjsph_closure_report_get(fjsph_ctx *ctx, fjsph_closure_report *out);
/* Clears the fallback flag and the judge statistics. */
int fjsph_closure_reset(fjsph_ctx *ctx);

/* ---- vortex-lattice air source (src/VLM.h, src/VLM.cpp) ------------------------------------ */
/* A swept, tapered wing of horseshoe vortices with an optional trailing-edge flap.  Fields keep
 * the reference's para-file meaning ("VLM wing dimensions", "VLM panel counts", ...):
 * span and chord are coords[0] (each side of y = 0) and coords[1]; panels_span and panels_chord
 * the panel counts per side and chordwise; the flap covers span strips
 * [flap_start, flap_start + flap_width) on each side over its last flap_depth chordwise panels,
 * deflected by flap_deg.  aoa_deg is read by the reference but not used in the geometry (the
 * freestream direction carries the incidence).  Velocities are limited to max_vel; max_vel = 2.0
 * (the reference's default) means max_vel_fac x |v_inf|. */
typedef struct fjsph_vlm {
    double span, chord;
    int32_t panels_span, panels_chord;
    double aoa_deg, sweep_deg, taper;
    int32_t flap_start, flap_width, flap_depth, pad;
    double flap_deg;
    double max_vel_fac, max_vel;
} fjsph_vlm;
/* the reference's VLM defaults (src/VLM.h:36-55); span, chord and panel counts are -1 (required) */
int fjsph_vlm_defaults(fjsph_vlm *v);
/* VLM::Init + VLM::GetGamma (src/VLM.cpp:14-118): builds the panels, solves the circulations for
 * the context's v_inf (3D) and keeps them on the device; the air source of a context whose
 * settings name FJSPH_VLM_INFL.  Returns the panel count in *npanels (may be null). */
int fjsph_vlm_setup(fjsph_ctx *ctx, const fjsph_vlm *v, int32_t *npanels);
/* Circulation of every panel (gamma[npanels]) and the panels' vortex ends and control points
 * (A, B, C: 9 doubles per panel, may be null); *npanels receives the count. */
int fjsph_vlm_panels(fjsph_ctx *ctx, double *gamma, double *abc, int32_t *npanels);
/* VLM::getVelocity (src/VLM.cpp:119-140) at n host points pos[3n] into vel[3n], on the device in
 * the context's precision (FP64, or FP32 sums for the split-precision form). */
int fjsph_vlm_velocity(fjsph_ctx *ctx, int64_t n, const double *pos, double *vel);

/* ---- mesh-cell air source (src/Containment.cpp:385-821, src/Resid.cpp:477-519) -------------- */
/* A CFD mesh with a solution per cell (the MESH of src/Var.h:396-451 after the TAU / OpenFOAM
 * readers): vertices, faces as vertex lists (2D: edges of two vertices; 3D: polygons whose first
 * three vertices are the ones the containment test uses, as upstream), each face's right-hand
 * cell (-1 = inner boundary, -2 = outer boundary), each cell's faces, centre, velocity, pressure
 * and density.  Arrays are host pointers, copied by fjsph_mesh_set. */
typedef struct fjsph_mesh {
    int32_t dim;
    int64_t n_verts;
    const double *verts;             /* [dim * n_verts]                                      */
    int64_t n_faces;
    const int64_t *face_offsets;     /* [n_faces + 1] into face_verts                        */
    const int64_t *face_verts;
    const int32_t *face_right;       /* [n_faces]                                            */
    int64_t n_cells;
    const int64_t *cell_face_offsets; /* [n_cells + 1] into cell_faces                       */
    const int64_t *cell_faces;
    const double *cell_centres;      /* [dim * n_cells]                                      */
    const double *cell_vel;          /* [dim * n_cells]                                      */
    const double *cell_p, *cell_rho; /* [n_cells]                                            */
} fjsph_mesh;
/* No reference counterpart: the analytic air field of a context created with asource =
 * FJSPH_POWER_LAW, a boundary layer over a wall normal to axis `axis` (0, 1, 2) at coordinate
 * `wall`: the air velocity at position x is v_inf * min(max((x[axis] - wall) / thickness, 0), 1)^exponent
 * (exponent 1/7: the turbulent 1/7-power law).  It takes the place of the uniform v_inf wherever
 * the reference's constVel source uses it: the aero velocity of get_aero_velocity
 * (src/Resid.cpp:569-611) and the relative air velocity of the Gissler occlusion in
 * Detect_Surface (src/Geometry.cpp:151-164).  params4 = {axis, wall, thickness, exponent};
 * thickness > 0, exponent > 0. */
int fjsph_air_power_law(fjsph_ctx *ctx, const double *params4);
/* Hands the mesh to a context created with asource = FJSPH_MESH_INFL.  FindCell then runs in
 * place of the uniform-source aero velocity pass: free particles below the lambda cutoff take
 * the velocity, pressure and density of the cell they are in (cellID = the cell); a particle
 * that leaves through the outer boundary is deleted at the end of the step. */
int fjsph_mesh_set(fjsph_ctx *ctx, const fjsph_mesh *mesh);

/* ---- restart files (src/H5IO.cpp:395-523, 1027-1060, 1092-1318) ---------------------------- */
/* Write_HDF5 / Read_HDF5 content with the reference's group, dataset and attribute names in a
 * self-describing binary container (no HDF5 library here; the layout is documented in
 * fjsph_gb300/csrc/restart.cpp).  write: pnp1 and the integrator scalars; read: the file's
 * particles become pn and pnp1 (the block layout must be the context's), the current time, CFL
 * and CFL counters are restored, *current_frame receives the frame (may be null). */
int fjsph_restart_write(fjsph_ctx *ctx, const char *path, int64_t current_frame);
int fjsph_restart_read(fjsph_ctx *ctx, const char *path, int64_t *current_frame);

/* ---- initial particles from block files (src/Init.cpp:61-496, src/shapes/) ------------------- */
/* Host-side restatement of Init_Particles: the boundary and fluid block files ("bmap" text,
 * src/shapes/shapes.cpp:400-600) are read, each block checked (check_input) and generated
 * (generate_points: Line/Plane, Square/Cube, Circle/Sphere, Arc/Arch, Cylinder, Inlet,
 * Coordinates), points closer than 0.9 dx to a kept point are culled (Check_Intersection), and
 * the state, the LIMITS entries and the inlet tables are laid out in reference index order,
 * with the hydrostatic start when the settings ask for it.  The settings are the ones after
 * fjsph_settings_derive (dx, masses, EOS constants, grid scale).  Errors that make the reference
 * print and exit(-1) return FJSPH_E_ARG; fjsph_geometry_log holds the reference's messages. */
typedef struct fjsph_geometry fjsph_geometry;
typedef struct fjsph_geometry_block {
    char name[64];
    int32_t is_fluid, shape, sub_shape; /* shape_type (src/VarDefs.h:116-127), -1 = none   */
    int32_t particle_order, write_data;  /* 0 grid / 1 HCP; "Write surface data"             */
    int32_t ni, nj, nk;                  /* counts after check_input                         */
    int64_t estimated;                   /* check_input's point estimate (npts)               */
    int64_t generated;                   /* points made by generate_points                   */
    int64_t kept;                        /* points left by Check_Intersection                */
    double radius;
    double start[3], end[3], right[3], centre[3], normal[3]; /* after check_input            */
} fjsph_geometry_block;
int fjsph_geometry_create(const fjsph_settings *s, fjsph_geometry **out);
int fjsph_geometry_destroy(fjsph_geometry *g);
/* read_shapes_bmap on a file's text / on a file; fluid = 0 for the boundary file, 1 for the
 * fluid file (boundary blocks come first in the state whatever the call order). */
int fjsph_geometry_read(fjsph_geometry *g, const char *text, int32_t fluid);
int fjsph_geometry_read_file(fjsph_geometry *g, const char *path, int32_t fluid);
/* check_input, Generate_Points, Check_Intersection and the Init_Particles layout. */
int fjsph_geometry_build(fjsph_geometry *g);
int fjsph_geometry_sizes(const fjsph_geometry *g, int64_t *n_points, int64_t *n_bound_points,
                         int32_t *n_bound_blocks, int32_t *n_fluid_blocks, int32_t *n_inlets);
/* The SPHPart fields Init_Particles sets (src/Var.h:502-548, src/FJSPH.cpp:116-127: position,
 * velocity, density, pressure, mass, type, id, constant-source cell values, cellID = -3); every
 * other non-null array of the view is zeroed.  out->n is the arrays' capacity. */
int fjsph_geometry_state(const fjsph_geometry *g, fjsph_state_view *out);
int fjsph_geometry_blocks(const fjsph_geometry *g, fjsph_block *blocks, int32_t max_blocks);
int fjsph_geometry_block_info(const fjsph_geometry *g, int32_t k, fjsph_geometry_block *info);
/* Inlet k's tables: with back or buffer null, fills n_back and depth only (a size query). */
int fjsph_geometry_inlet(const fjsph_geometry *g, int32_t k, fjsph_inlet *inlet);
/* The messages check_input and Generate_Points print upstream; *len = full length. */
int fjsph_geometry_log(const fjsph_geometry *g, char *buf, int64_t cap, int64_t *len);

/* ---- diagnostics -------------------------------------------------------------------------- */
/* Step report of src/Integration.cpp:253-265: maxRho_pc, maxf, maxAf, maxShift, iteration. */
int fjsph_step_report(fjsph_ctx *ctx, double *out5);
/* Pair sweeps of the split-precision form (no reference counterpart: a property of this
 * implementation).  FJSPH_PAIRS_LISTS (default): explicit (neighbour, squared distance) lists
 * gathered through the caches.  FJSPH_PAIRS_TILES: the residual stages each tile of cells with
 * its halo in shared memory and walks per-particle member masks (the other sweeps keep the
 * lists).  Both give the same neighbour sets (the reference's FP64 membership test).  A grid too
 * large for the bucket table falls back to lists for that search; tiles_in_use reports what the
 * last search built. */
#define FJSPH_PAIRS_TILES 0
#define FJSPH_PAIRS_LISTS 1
int fjsph_set_pair_mode(fjsph_ctx *ctx, int32_t mode);
int fjsph_get_pair_mode(fjsph_ctx *ctx, int32_t *mode, int32_t *tiles_in_use);
/* Work order of the split-precision residual (no reference counterpart: a property of this
 * implementation; results are identical in both).  FJSPH_ORDER_GRID (default): one thread per
 * particle in launch-grid order.  FJSPH_ORDER_SM: one resident grid whose warps take 32-particle
 * chunks from a contiguous region per SM, so that the warps sharing an SM's L1 work on
 * neighbouring particles. */
#define FJSPH_ORDER_GRID 0
#define FJSPH_ORDER_SM 1
int fjsph_set_sweep_order(fjsph_ctx *ctx, int32_t order);
int fjsph_get_sweep_order(fjsph_ctx *ctx, int32_t *order);
/* Neighbour count (self included) of every particle, in reference order, from the last search
 * (counts: particle-count entries).  No reference counterpart: a diagnostic of the search. */
int fjsph_neighbour_counts(fjsph_ctx *ctx, int32_t *counts);
/* The seven maxima of the last fjsph_find_timestep (Integrator members, src/Integration.h):
 * maxf, maxAf, maxdrho, maxRhoi, minST, maxU, maxShift (the running maximum). */
int fjsph_timestep_maxima(fjsph_ctx *ctx, double *out7);
/* Count and total duration (ms) of kernel launches recorded since the last reset. */
int fjsph_launch_stats(fjsph_ctx *ctx, int64_t *n_launches, int32_t reset);
/* CUDA stream of the context (a cudaStream_t), for callers that time with events. */
int fjsph_ctx_stream(fjsph_ctx *ctx, void **stream);
/* Timing support (no counterpart in the reference, which times whole steps with a wall clock,
 * src/Integration.cpp:239-252).  Events are recorded on the context's stream.
 * fjsph_event_record(ctx, slot) records event `slot` (0..15); fjsph_event_elapsed gives the
 * milliseconds between two recorded slots after synchronising on the later one. */
int fjsph_event_record(fjsph_ctx *ctx, int32_t slot);
int fjsph_event_elapsed(fjsph_ctx *ctx, int32_t slot_a, int32_t slot_b, double *ms);
/* Per-pass device time: when enabled, every pass of the step is bracketed by events.
 * fjsph_profile_read fills ms[FJSPH_NPASS] and launches[FJSPH_NPASS] accumulated since the last
 * read (and clears them); fjsph_profile_pass_name names pass k. */
#define FJSPH_NPASS 13
int fjsph_profile_enable(fjsph_ctx *ctx, int32_t on);
int fjsph_profile_read(fjsph_ctx *ctx, double *ms, int64_t *launches);
const char *fjsph_profile_pass_name(int32_t k);
const char *fjsph_status_string(int status);
/* ABI check for bindings: sizes[0..3] = sizeof(fjsph_settings), sizeof(fjsph_block),
 * sizeof(fjsph_inlet), sizeof(fjsph_state_view).  No counterpart in the reference. */
int fjsph_abi_sizes(int64_t *sizes4);

#ifdef __cplusplus
}
#endif

#endif /* FJSPH_GB300_H */
