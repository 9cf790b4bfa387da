/*
 * TEST INFRASTRUCTURE — not part of the product.
 *
 * CPU FP64 restatement of the reference's Durian wet-foam step
 * (KJLankinen/cubble src/kernels.cu and src/simulator.cu), used only as the
 * checker by tests/, by __graft_entry__.smoke() and by bench.py's CPU
 * baseline / reference arm. The product path (cubble_gb300) never loads it.
 *
 * The API mirrors include/cubble_gb300.h with a `cbo_` prefix so that a test
 * can drive the oracle and the CUDA library through the same sequence of
 * calls and compare rows keyed by the persistent bubble `index`.
 */
#ifndef CUBBLE_ORACLE_H
#define CUBBLE_ORACLE_H

#include "../include/cubble_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cbo_ctx cbo_ctx;

const char *cbo_last_error(void);
int cbo_create(const cb_config *cfg, cbo_ctx **out);
int cbo_destroy(cbo_ctx *ctx);
/* Threads used by the OpenMP loops. 1 (the default) gives a fully
 * deterministic, sequential evaluation order; >1 is used for timing. */
int cbo_set_threads(cbo_ctx *ctx, int32_t nthreads);
int cbo_load_state(cbo_ctx *ctx, const cb_state_view *state);
int cbo_get_state(cbo_ctx *ctx, cb_state_view *state);
int cbo_set_options(cbo_ctx *ctx, int32_t use_gas_exchange, int32_t use_flow,
                    int32_t increment_path);
int cbo_set_time(cbo_ctx *ctx, double time_step, uint64_t time_integer,
                 double time_fraction);
int cbo_set_box(cbo_ctx *ctx, const double lbb[3], const double tfr[3],
                double bubble_volume_multiplier, const double flow_lbb[3],
                const double flow_tfr[3]);
int cbo_bootstrap(cbo_ctx *ctx);
int cbo_search_neighbors(cbo_ctx *ctx);
int cbo_get_pairs(cbo_ctx *ctx, int32_t *i, int32_t *j, int32_t capacity,
                  int32_t *count);
int cbo_set_pairs(cbo_ctx *ctx, const int32_t *i, const int32_t *j,
                  int32_t count);
int cbo_attempt(cbo_ctx *ctx, cb_attempt_view *out);
int cbo_integrate(cbo_ctx *ctx, int64_t n_steps, cb_report *report);
int cbo_get_report(cbo_ctx *ctx, cb_report *report);
int cbo_energy(cbo_ctx *ctx, double *energy);
int cbo_bubble_energies(cbo_ctx *ctx, double *energy, int32_t capacity);
int cbo_total_volume(cbo_ctx *ctx, double *volume);
/* The cell grid the last search used (for tests of the binning). */
int cbo_cell_dims(cbo_ctx *ctx, int32_t dims[3]);

#ifdef __cplusplus
}
#endif

#endif
