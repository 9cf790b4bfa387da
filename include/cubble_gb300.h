/*
 * cubble_gb300 — C ABI of the GB300 (sm_103a) Durian wet-foam time step.
 *
 * The reference (KJLankinen/cubble) exports only `cubble::run(argc, argv)`
 * (src/simulator.cu:1161-1186); its step boundary is internal:
 *   step(Params&, IntegrationParams&)        src/simulator.cu:192-249
 *   integrate(Params&, IntegrationParams&)   src/simulator.cu:251-337
 *   searchNeighbors(Params&)                 src/simulator.cu:60-178
 *   removeBubbles(Params&, int)              src/simulator.cu:180-190
 *   totalEnergy / totalVolume                src/simulator.cu:39-58, 362-379
 * operating on the device SoA owned by `Params` (src/data_definitions.h:302-343).
 * This header is that boundary as a plain C ABI: plain pointers and sizes,
 * `int` status codes (CB_OK == 0) plus cb_last_error(), no exceptions across
 * the boundary, one host thread per context, context-owned device memory and
 * caller-owned host buffers.
 *
 * Each entry point below names the reference function or data it replaces.
 */
#ifndef CUBBLE_GB300_H
#define CUBBLE_GB300_H

#include <stdint.h>

#if defined(__GNUC__)
#define CB_API __attribute__((visibility("default")))
#else
#define CB_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define CB_OK 0
#define CB_ERR_INVALID_ARGUMENT 1 /* bad pointer, size or configuration      */
#define CB_ERR_CUDA 2             /* a CUDA runtime call failed               */
#define CB_ERR_CAPACITY 3         /* bubble, pair or cell capacity exceeded   */
#define CB_ERR_MAX_ATTEMPTS 4     /* reject loop hit cb_config.max_attempts   */
#define CB_ERR_NONFINITE 5        /* NaN/Inf in the predictor-corrector error */
#define CB_ERR_DT_UNDERFLOW 6     /* time step fell below 1e-300              */
#define CB_ERR_NO_DEVICE 7        /* no CUDA device / extension unusable      */
#define CB_ERR_STATE 8            /* call made in the wrong order             */

#define CB_PRECISION_FP64 0  /* plain FP64 form (reference arithmetic)        */
#define CB_PRECISION_MIXED 1 /* FP32 pair geometry on exact 64-bit fixed-point
                                differences, FP64 positions/volume/error     */
#define CB_PRECISION_FP64_FF 2 /* the FP64 form with its pair terms (distance,
                                velocities, gas flux, overlap areas) in
                                float-float (two FP32, ~2^-46 relative) on the
                                FP32 pipe; FP64 state, update and sums       */

/* ------------------------------------------------------------ constants */
/* Mirrors `Constants` (src/data_definitions.h:183-225) plus the host-side
 * knobs of `HostData`/`IntegrationParams` that the step reads
 * (src/data_definitions.h:227-269). All values are the final device values:
 * flow_vel is already multiplied by f0/mu0 and flow_lbb/flow_tfr are absolute
 * coordinates, as after src/simulator.cu:569-570 and :806-811. */
typedef struct cb_config {
    int32_t dimensionality;  /* 2 or 3                                     */
    int32_t wall[3];         /* x, y, z: 1 = wall, 0 = periodic            */
    int32_t use_gas_exchange;/* IntegrationParams.useGasExchange           */
    int32_t use_flow;        /* IntegrationParams.useFlow                  */
    int32_t increment_path;  /* IntegrationParams.incrementPath            */
    int32_t capacity;        /* maximum number of bubbles                  */
    int32_t pair_capacity;   /* maximum number of pairs; 0 = 16 (3D) / 8 (2D) per bubble */
    int32_t max_attempts;    /* reject-loop cap per step; 0 = 64           */
    int32_t precision;       /* CB_PRECISION_*                             */
    int32_t use_graph;       /* 1 = run cb_integrate as one CUDA graph with
                                device-side conditional loops              */
    double lbb[3];           /* lower back bottom corner of the box        */
    double tfr[3];           /* top front right corner of the box          */
    double flow_lbb[3];
    double flow_tfr[3];
    double flow_vel[3];
    double wall_drag;        /* wallDragStrength                           */
    double min_rad;          /* deletion threshold                         */
    double f0_per_mu0;       /* fZeroPerMuZero                             */
    double k_parameter;      /* K                                          */
    double kappa;            /* kappa                                      */
    double skin_radius;      /* Verlet skin                                */
    double bubble_volume_multiplier; /* M of the volume fix                */
    double average_surface_area_in;  /* <A_in>                             */
    double error_tolerance;  /* HostData.errorTolerance                    */
    double time_step;        /* initial dt (HostData.timeStep)             */
    /* Extension, not in the reference: with use_flow and shear_speed != 0
     * the imposed flow is a linear shear instead of addFlowVelocity's box
     * region: every bubble's velocity gains shear_speed * (2 (q - lbb_q) /
     * L_q - 1) along x, q its predicted coordinate on the last axis (z in
     * 3D, y in 2D): -shear_speed at the lower wall, +shear_speed at the
     * upper one. */
    double shear_speed;
} cb_config;

/* Host view of the persistent per-bubble state, keyed by the bubble order of
 * the context (cell order after a search). Mirrors the persistent rows of
 * `Bubbles` (src/data_definitions.h:41-153). Any pointer may be NULL: on
 * load a NULL row is zero-filled (saved_* default to the positions, index to
 * 0..count-1), on get a NULL row is skipped. */
typedef struct cb_state_view {
    int32_t count;
    int32_t pad_;
    double *x, *y, *z, *r;
    double *dxdt, *dydt, *dzdt, *drdt;     /* current velocities   */
    double *dxdto, *dydto, *dzdto, *drdto; /* previous velocities  */
    double *path, *error;
    double *saved_x, *saved_y, *saved_z, *saved_r;
    int32_t *wrap_count_x, *wrap_count_y, *wrap_count_z;
    int32_t *index, *num_neighbors;
} cb_state_view;

/* Host scalars of the step loop (HostData + IntegrationParams results). */
typedef struct cb_report {
    int64_t steps;          /* accepted steps (numIntegrationSteps)        */
    int64_t attempts;       /* step() calls including rejected ones        */
    int64_t searches;       /* neighbour searches (numNeighborsSearched)   */
    int64_t deleted;        /* bubbles removed                             */
    int64_t bubble_steps;   /* sum over accepted steps of the bubble count */
    uint64_t time_integer;  /* HostData.timeInteger                        */
    double time_fraction;   /* HostData.timeFraction                       */
    double time_step;       /* dt of the next attempt                      */
    double max_error;       /* of the last attempt                         */
    double max_radius;      /* HostData.maxBubbleRadius                    */
    double max_expansion;   /* of the last attempt                         */
    int32_t count;          /* bubbles                                     */
    int32_t num_pairs;      /* pairs                                       */
    int32_t status;         /* CB_* status of the device control block     */
    int32_t pad_;
    double dt_min;          /* smallest / largest / summed dt after the    */
    double dt_max;          /* accepted steps since the last               */
    double dt_sum;          /* cb_reset_rows(CB_RESET_DT_STATS)            */
} cb_report;

/* Outputs of one step() attempt (src/simulator.cu:192-249), before the
 * accept/rotate of integrate(). Row pointers may be NULL (skipped). */
typedef struct cb_attempt_view {
    double *xp, *yp, *zp, *rp;             /* corrected values            */
    double *dxdtp, *dydtp, *dzdtp, *drdtp; /* new velocities              */
    double *error;                         /* error row after the attempt */
    double *path_new;                      /* pathNew row                 */
    double *overlap;                       /* per-bubble overlap area     */
    int32_t *delete_flags;                 /* 1 where r <= min_rad        */
    double total_area;                     /* dTotalArea                  */
    double total_area_per_radius;          /* dTotalAreaPerRadius         */
    double total_overlap_area;             /* dTotalOverlapArea           */
    double total_overlap_area_per_radius;  /* dTotalOverlapAreaPerRadius  */
    double total_volume_new;               /* dTotalVolumeNew             */
    double max_error, max_radius, max_expansion;
    int32_t num_to_be_deleted;             /* dNumToBeDeleted             */
    int32_t pad_;
} cb_attempt_view;

typedef struct cb_context cb_context;

/* Last error message of the calling thread ("" if none). */
CB_API const char *cb_last_error(void);

/* Allocates the device state for cfg->capacity bubbles on the current CUDA
 * device. Replaces init()'s allocation and constant upload
 * (src/simulator.cu:608-671). */
CB_API int cb_create(const cb_config *cfg, cb_context **out);
/* Frees everything. Replaces end() (src/simulator.cu:514-525). */
CB_API int cb_destroy(cb_context *ctx);

/* Uploads / downloads the persistent state (host buffers, `count` rows). */
CB_API int cb_load_state(cb_context *ctx, const cb_state_view *state);
CB_API int cb_get_state(cb_context *ctx, cb_state_view *state);

/* Switches the integration options, as stabilize() does
 * (src/simulator.cu:339-360) and simulate() does (:996-1003). */
CB_API int cb_set_options(cb_context *ctx, int32_t use_gas_exchange,
                   int32_t use_flow, int32_t increment_path);
/* Sets dt (HostData.timeStep) and the time accumulator. */
CB_API int cb_set_time(cb_context *ctx, double time_step, uint64_t time_integer,
                double time_fraction);
/* Replaces the device copy of the box and volume-fix constants after the box
 * rescale of init() (src/simulator.cu:793-833). */
CB_API int cb_set_box(cb_context *ctx, const double lbb[3], const double tfr[3],
               double bubble_volume_multiplier, const double flow_lbb[3],
               const double flow_tfr[3]);

/* Euler bootstrap of the Adams-Bashforth history
 * (src/simulator.cu:727-787): dxdto := F(x + dt F(x)), drdto := 0,
 * path := 0. Needs a pair list. */
CB_API int cb_bootstrap(cb_context *ctx);

/* searchNeighbors() (src/simulator.cu:60-178): wrap, cell sort of all rows,
 * saved := positions, pair list, neighbour counts. */
CB_API int cb_search_neighbors(cb_context *ctx);
/* Copies the pair list (Pairs, src/data_definitions.h:157-178). */
CB_API int cb_get_pairs(cb_context *ctx, int32_t *i, int32_t *j, int32_t capacity,
                 int32_t *count);
/* Replaces the pair list (for harnesses that feed a list made elsewhere). */
CB_API int cb_set_pairs(cb_context *ctx, const int32_t *i, const int32_t *j,
                 int32_t count);

/* One step() attempt without accepting it (src/simulator.cu:192-249):
 * predict, pairwise interaction, correct; dt is then updated as step() does.
 * The state stays at the start of the step. */
CB_API int cb_attempt(cb_context *ctx, cb_attempt_view *out);

/* n_steps calls of integrate() (src/simulator.cu:251-337): the reject loop,
 * buffer rotation, time accumulation, removeBubbles() when bubbles fall
 * below min_rad, and searchNeighbors() at half the skin. */
CB_API int cb_integrate(cb_context *ctx, int64_t n_steps, cb_report *report);
/* As cb_integrate, and returns the device time of the call measured with
 * CUDA events on the context's stream. */
CB_API int cb_integrate_timed(cb_context *ctx, int64_t n_steps, cb_report *report,
                       double *device_ms);
CB_API int cb_get_report(cb_context *ctx, cb_report *report);

/* Conditions that end cb_integrate_until after an accepted step: the
 * simulate() loop's stop test (src/simulator.cu:1002-1011: bubbles left
 * <= min_count, or the largest radius >= max_radius, the latter only with
 * gas exchange) and its print / snapshot times (:1017-1029, :1090-1104:
 * time >= time_integer + time_fraction). */
typedef struct cb_stop {
    uint64_t time_integer;
    double time_fraction;
    double max_radius;
    int32_t min_count;
    int32_t pad_;
} cb_stop;

/* Up to max_steps accepted steps (integrate() calls), ending after the
 * first step that meets a condition of *stop; checked on the device, so a
 * graph context runs the whole stretch as one graph launch. The caller
 * reads which condition held from the report (time, count, max_radius). */
CB_API int cb_integrate_until(cb_context *ctx, int64_t max_steps, const cb_stop *stop,
                              cb_report *report);

/* transformPositions (src/kernels.cu:971-990): normalize != 0 maps the
 * positions to [0, 1] of the current box, 0 maps them back from [0, 1]
 * into the box; init()'s box rescale (src/simulator.cu:793-833) is
 * transform(1), cb_set_box(new box), transform(0). */
CB_API int cb_transform_positions(cb_context *ctx, int32_t normalize);

/* Means over the bubbles of r, dxdt, dydt, dzdt, drdt and path
 * (simulate()'s getAvg, src/simulator.cu:1038-1052), in that order. */
CB_API int cb_averages(cb_context *ctx, double means[6]);

/* Resets of simulate() and init(): CB_RESET_ERROR zeroes the error row
 * (resetArrays after each print, src/simulator.cu:1106-1110, and at the end
 * of init, :947-948), CB_RESET_WRAP the wrap counts (:941-945),
 * CB_RESET_DT_STATS the dt statistics of the report. */
#define CB_RESET_ERROR 1
#define CB_RESET_WRAP 2
#define CB_RESET_DT_STATS 4
CB_API int cb_reset_rows(cb_context *ctx, int32_t which);

/* averageSurfaceAreaIn (init() computes it from the initial radii,
 * src/simulator.cu:697-703; the mean-field gas exchange uses it). */
CB_API int cb_set_average_area(cb_context *ctx, double average_surface_area_in);

/* The initial foam of init() (src/simulator.cu:676-711): from the draws of
 * the reference's generator (uniform x, y, z and w, normal r; host rows of
 * `count` doubles, z ignored in 2D) and bubbles_per_dim, places bubble i on
 * its lattice point plus a random offset, fixes its radius
 * (assignDataToBubbles, src/kernels.cu:1026-1071) and loads the result as
 * the state (index = i, rates and path zero). *avg_area receives the mean
 * initial area (averageSurfaceAreaIn), *max_radius the largest radius. The
 * box of the context must be the lattice box: lbb and tfr = lbb +
 * 2 avg_rad bubbles_per_dim. */
CB_API int cb_assign_lattice(cb_context *ctx, const int32_t bubbles_per_dim[3], double avg_rad,
                             const double *ux, const double *uy, const double *uz,
                             const double *uw, const double *nr, int32_t count,
                             double *avg_area, double *max_radius);

/* totalEnergy() (src/simulator.cu:39-58, kernel src/kernels.cu:941-957). */
CB_API int cb_energy(cb_context *ctx, double *energy);
/* Per-bubble energies (saveSnapshot's energy column, src/simulator.cu:389-392). */
CB_API int cb_bubble_energies(cb_context *ctx, double *energy, int32_t capacity);
/* totalVolume() (src/simulator.cu:362-379, kernel src/kernels.cu:1013-1024). */
CB_API int cb_total_volume(cb_context *ctx, double *volume);

/* Measurement: runs `reps` step() attempts without accepting them and
 * returns the mean device time in milliseconds of each of the three attempt
 * kernels (ms[0] predict, ms[1] pairwise interaction, ms[2] correct),
 * measured with CUDA events on the context's stream. */
CB_API int cb_profile_kernels(cb_context *ctx, int32_t reps, double ms[3]);

/* Measurement: `reps` back-to-back searchNeighbors() (src/simulator.cu:60-178)
 * of the current state after one untimed search; *ms = mean device time of
 * one search (CUDA events on the context's stream). The state is left
 * searched; the report's search counter does not count these. */
CB_API int cb_profile_search(cb_context *ctx, int32_t reps, double *ms);

/* ------------------------------------------------------------- tuning
 * Launch and search knobs of a context. None changes the pair set or the
 * arithmetic of a pair; they change how work is cut into threads, blocks and
 * cells (so the bubble order after a search and the order of reductions,
 * which moves FP64 sums by rounding only). No counterpart in the reference,
 * whose launch shape is fixed (5120 x 384, src/data_definitions.h:28-29) and
 * whose cell edge is 2 (maxR + skin) (src/simulator.cu:69-75). */
typedef struct cb_tuning {
    double cell_scale;   /* cell edge of the neighbour search in units of
                            2 maxR + skin, in [1, 4]; 1 = default          */
    int32_t pair_run;    /* mixed form: consecutive pairs per thread of the
                            pair kernel (2, 4 or 8; 32 x that per warp); 0 = 4 */
    int32_t pair_blocks; /* resident blocks per SM of the pair kernel,
                            0..8; 0 = as many as fit                       */
    int32_t step_blocks; /* resident blocks per SM of the predict and correct
                            kernels, 0..8; 0 = as many as fit              */
    int32_t pad_;
} cb_tuning;

/* Sets / reads the knobs of a context (the next integrate rebuilds its
 * graph). */
CB_API int cb_set_tuning(cb_context *ctx, const cb_tuning *tuning);
CB_API int cb_get_tuning(cb_context *ctx, cb_tuning *tuning);

/* Autotuner: on the loaded, searched state, times the pair kernel for every
 * (pair_run, pair_blocks) candidate and the predict + correct kernels for
 * every step_blocks candidate (`reps` attempts each, not accepted: the state
 * does not advance), and one neighbour search per cell_scale candidate (the
 * state is left searched); keeps the fastest of each and returns them in
 * *best. The choice is also kept process-wide for contexts of the same
 * dimensionality, precision and capacity bucket (floor(log2(capacity))):
 * cb_create applies it to every later context of that kind. */
CB_API int cb_autotune(cb_context *ctx, int32_t reps, cb_tuning *best);
/* Forgets every choice cb_autotune kept: later contexts start from the
 * defaults (existing contexts keep their knobs). */
CB_API int cb_forget_tuning(void);

/* Number of kernels this library launched on the context so far (graph
 * kernel nodes are counted per execution). */
CB_API int cb_launch_count(cb_context *ctx, int64_t *count);

/* ------------------------------------------------------------ batches
 * Many independent foams advanced together: the array-job parameter sweep
 * (scripts/triton/array_job.py:54-75 submits one simulate() process per
 * parameter set) as one device job. Every stage of integrate() is one launch
 * over all foams (foam f runs on a virtual grid sized to its capacity), the
 * step loop is one CUDA graph, and each foam keeps its own adaptive dt,
 * accept/reject, search and deletion exactly as a cb_context running
 * integrate() alone. The reference has no batched form.
 *
 * All configs must agree on dimensionality, precision, use_gas_exchange,
 * use_flow and whether any wall is set; capacities and every other
 * parameter may differ. Each foam is a cb_context owned by the batch
 * (cb_batch_context): load its state, search and bootstrap it through the
 * single-foam calls, then advance all foams with cb_batch_integrate. */
typedef struct cb_batch cb_batch;
CB_API int cb_batch_create(const cb_config *configs, int32_t count, cb_batch **out);
CB_API int cb_batch_destroy(cb_batch *batch);
/* The context of foam `index` (owned by the batch; do not cb_destroy it). */
CB_API int cb_batch_context(cb_batch *batch, int32_t index, cb_context **ctx);
/* n_steps accepted steps of every foam whose status is CB_OK; reports[f]
 * (count entries, may be NULL) receives foam f's report. Returns the first
 * foam's error, if any foam's status is not CB_OK at the end. */
CB_API int cb_batch_integrate(cb_batch *batch, int64_t n_steps, cb_report *reports);
/* As cb_batch_integrate; *ms = device time of the whole job (CUDA events). */
CB_API int cb_batch_integrate_timed(cb_batch *batch, int64_t n_steps, cb_report *reports,
                                    double *ms);
/* Bubbles per block of every foam's virtual grid (a multiple of 256,
 * >= 256); the default is 2048. */
CB_API int cb_batch_set_tile(cb_batch *batch, int32_t bubbles_per_block);
/* Autotuner: times `steps_per_trial` steps (these advance the foams) with
 * each candidate tile (512 ... 8192 bubbles per block), then with each
 * cell_scale and, in the mixed form, each pair_run candidate of cb_tuning
 * (applied to every foam), keeps the fastest of each and returns the tile in
 * *tile (the other knobs: cb_get_tuning of any foam's context). */
CB_API int cb_batch_autotune(cb_batch *batch, int32_t steps_per_trial, int32_t *tile);
/* Applies the knobs of cb_tuning to every foam of the batch. */
CB_API int cb_batch_set_tuning(cb_batch *batch, const cb_tuning *tuning);
CB_API int cb_batch_launch_count(cb_batch *batch, int64_t *count);

/* Total potential energy of a foam, as cb_energy computes it, for callers
 * that cannot allocate device memory. No counterpart in the reference.
 *
 * Who needs it: applications whose device memory is owned by their own pool
 * or arena, or code calling from a loop where cudaMalloc would synchronise
 * the device or is not allowed. Such a caller owns the inputs and the
 * output; this call allocates nothing (no cudaMalloc / cudaFree, no library
 * allocator). Its scratch is one static device array inside the library,
 * sized for at most 262,144 bubbles (about 2 MiB), which every GPU that
 * loads the library holds until the process exits.
 *
 * x, y, z (3D only), r: `count` device rows; pair_i, pair_j: `num_pairs`
 * device rows of bubble indices; energy_out: one device double that
 * receives sum_i sum_{pairs of i} (r_i + r_j - |d_ij|)^2 over overlapping
 * pairs. Only dimensionality, wall[] and the box corners of `cfg` are read.
 * `stream` is a cudaStream_t (NULL = the default stream); the work is
 * enqueued there and the call returns without waiting.
 *
 * count > 262,144 is rejected with CB_ERR_CAPACITY before any GPU work.
 * The pair indices are the caller's: a pair with i or j outside [0, count)
 * is skipped without reading or writing anything for it, and the call's
 * result is then NaN (the call stays asynchronous; check the value).
 * Every call looks up the device address of the static array for the
 * current device and context (a host-side lookup once the library's module
 * is loaded, so it stays right after a cudaDeviceReset or a context switch);
 * the first call on a device loads the module, so make that first call
 * before any stream capture. Every call reuses the same array and clears
 * what must start at zero, so calls that overlap on the GPU (different
 * streams, or several host threads) race with each other: serialise them. */
CB_API int cb_energy_noalloc(const cb_config *cfg, const double *x, const double *y,
                             const double *z, const double *r, const int32_t *pair_i,
                             const int32_t *pair_j, int32_t count, int32_t num_pairs,
                             double *energy_out, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* CUBBLE_GB300_H */
