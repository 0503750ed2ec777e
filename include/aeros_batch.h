/*
 * aeros_batch.h — many independent solver domains stepped together.
 *
 * The reference steps one domain at a time (stepLBMCPU, aeros/src/lbm.cpp:907)
 * and has no batching layer; these entry points have no reference counterpart.
 * They sit on top of aeros_lbm.h: a caller creates each domain with
 * aeros_lbm_create (same storage for all members), attaches it to a batch,
 * and steps the batch. Reading fields, forces or statistics of a member goes
 * through the member's own aeros_lbm handle, as for a lone domain.
 *
 * Device side: per lattice step, two persistent launches (the boundary
 * shells of every member, then the interiors) whose warps take work items
 * from a global counter, and a chunk of steps is captured once as a CUDA
 * graph and replayed. Statistics are summed per 32-cell slice and added in
 * exact fixed point, which makes every member's state and statistics
 * independent of the other members, of the schedule and of the tuning: a
 * domain gives the same bits alone as in any mix.
 *
 * Status codes and aeros_consume_error() are those of aeros_lbm.h.
 */
#ifndef AEROS_BATCH_H
#define AEROS_BATCH_H

#include <stdint.h>

#include "aeros_lbm.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct aeros_batch aeros_batch;

/* Launch shape of the batch kernels. A lattice step is two launches: the
 * boundary shells of all members, then their interiors. Work items are runs
 * of 256-cell tiles taken by warps from a global counter. */
typedef struct aeros_batch_tuning {
    int32_t blocks_per_sm;         /* resident blocks per SM of the interior grid (0: occupancy limit) */
    int32_t tiles_per_item;        /* interior tiles per work item: 1, 2, 4 or 8                       */
    int32_t shell_tiles_per_item;  /* shell tiles per work item: 1, 2, 4 or 8                          */
    int32_t chunk_steps;           /* steps per captured graph (even, >= 2)                            */
    int32_t reserved[4];
} aeros_batch_tuning;

/* An empty batch whose members store populations as `storage`
 * (AEROS_STORE_*). The batch owns a CUDA stream. */
int aeros_batch_create(int storage, aeros_batch** out);
/* Detaches every member (the members stay valid) and frees the batch. */
int aeros_batch_destroy(aeros_batch* b);

/* Attaches a domain. Refused (AEROS_ERR_STATE) when it is in another batch,
 * has the thermal lattice on, or stands at an odd AA-pattern parity (it was
 * stepped an odd number of times on its own); AEROS_ERR_INVALID for another
 * storage. A member must be removed before aeros_lbm_destroy. */
int aeros_batch_add(aeros_batch* b, aeros_lbm* domain);
int aeros_batch_remove(aeros_batch* b, aeros_lbm* domain);
int aeros_batch_size(aeros_batch* b, int32_t* n_domains, int64_t* n_cells);

/* Advances every member by nsteps (even, >= 0) lattice steps; waits for the
 * statistics, re-equilibrates members whose divergence guard tripped (as
 * aeros_lbm_step does). */
int aeros_batch_step(aeros_batch* b, int nsteps);

int aeros_batch_set_tuning(aeros_batch* b, const aeros_batch_tuning* t);
int aeros_batch_get_tuning(aeros_batch* b, aeros_batch_tuning* t);

/* Times candidate launch shapes on the live batch (each candidate steps every
 * member trial_steps, even, so the members advance by candidates x
 * trial_steps), keeps the fastest and returns it. The choice changes no
 * result: only the time. */
int aeros_batch_autotune(aeros_batch* b, int trial_steps, aeros_batch_tuning* best);

/* Milliseconds per lattice step of the last aeros_batch_step (CUDA events on
 * the batch stream) and the number of batch-kernel launches it made. */
int aeros_batch_last_step_ms(aeros_batch* b, float* ms);
int aeros_batch_last_launch_count(aeros_batch* b, int64_t* launches);

#ifdef __cplusplus
}
#endif

#endif /* AEROS_BATCH_H */
