/*
 * nwgb_batch.h — batched replicas: many independent worm systems of uneven
 * size (worm count, length, box, activity, bending ...) advanced together,
 * one kernel launch per step for all of them.
 *
 * No reference counterpart: the reference runs one ParticleSystem per
 * process (its parameters live in process-global __constant__ symbols,
 * simulation/particles_kernel_impl.cuh:29-30), so replicas there are
 * separate processes or sequential runs of ParticleSystem::update
 * (simulation/particleSystem.cpp:249-339).  Each replica here follows that
 * same step with its own NwConfig; results equal those of a single-system
 * handle (include/nwgb.h) with the same configuration and strategy up to the
 * order of FP32 sums.
 *
 * Scope: NW_MODEL_WCA_WORMS replicas without SRD solvent.  Every replica
 * has its own cell table and neighbour lists; all replicas share one step
 * counter (each draws its noise from its own seed).
 */
#ifndef NWGB_BATCH_H
#define NWGB_BATCH_H

#include "nwgb.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct nw_batch nw_batch;

/* Launch shape and neighbour search of a batch (what the autotuner picks).
 *  threads_per_block  block size; each block holds whole filaments of one
 *                     replica (128, 256 or 512)
 *  strategy           NW_STRATEGY_VERLET or NW_STRATEGY_CELL_LISTS (the
 *                     sort-free orderings; the sorted scheme is single-system)
 *  neighbor_skin      Verlet skin (sets the list-cell size lj_rcut + skin)
 *  ms_per_step        measured time of one step of the whole batch (output
 *                     of nw_batch_autotune; ignored on input)
 *  cell_capacity      slots per list cell, 8 or 16 (0 on input: 16 if any
 *                     replica's cell_capacity asks for it, else 8; the
 *                     value in use on output) */
typedef struct NwBatchTuning {
    uint32_t threads_per_block;
    int32_t strategy;
    float neighbor_skin;
    float ms_per_step;
    uint32_t cell_capacity;
} NwBatchTuning;

/* Create a batch of n replicas from their configurations (each validated as
 * by nw_config_validate; dt, seed and every force parameter may differ).
 * Initial state is zero, as for nw_create. */
nw_status nw_batch_create(const NwConfig* replicas, int n, nw_batch** out);
nw_status nw_batch_destroy(nw_batch* b);

/* Number of replicas, total beads, and replica r's bead count and offset in
 * the concatenated arrays of nw_batch_device_array. */
nw_status nw_batch_counts(const nw_batch* b, int* n_replicas, uint64_t* total_beads);
nw_status nw_batch_replica(const nw_batch* b, int r, uint32_t* n_beads, uint64_t* bead_offset);

/* State of replica r: NW_POSITION, NW_VELOCITY, NW_TANGENT, NW_FORCE,
 * NW_FORCE_OLD (float4[n_beads of r]).  Synchronous. */
nw_status nw_batch_set_array(nw_batch* b, int r, int array, const void* host, uint32_t start, uint32_t count);
nw_status nw_batch_get_array(nw_batch* b, int r, int array, void* host, uint32_t start, uint32_t count);
/* Device pointer of the concatenated array (all replicas, bead offsets of
 * nw_batch_replica); valid until the next step. */
nw_status nw_batch_device_array(nw_batch* b, int array, void** dptr);

/* Advance every replica by nsteps steps of its own dt.  Asynchronous on the
 * batch's stream; a call of the same nsteps replays one CUDA graph. */
nw_status nw_batch_step(nw_batch* b, int nsteps);
nw_status nw_batch_sync(nw_batch* b);
nw_status nw_batch_set_stream(nw_batch* b, void* stream);
nw_status nw_batch_set_graphs(nw_batch* b, int enabled);
uint64_t nw_batch_get_step(const nw_batch* b);
/* Number of kernels the last nw_batch_step launched. */
nw_status nw_batch_last_launch_count(const nw_batch* b, uint64_t* launches);

/* Current launch shape and neighbour search, and setting them.  Changing
 * them rebuilds the cell tables and lists; the state is kept. */
nw_status nw_batch_get_tuning(const nw_batch* b, NwBatchTuning* t);
nw_status nw_batch_set_tuning(nw_batch* b, const NwBatchTuning* t);

/* Time trial_steps steps of every candidate (block sizes 128, 256, 512;
 * Verlet lists with skins 0.2, 0.3, 0.45 sigma and plain cell lists; 8 or
 * 16 slots per list cell), each from the same saved state, keep the fastest
 * and restore the state.  A candidate whose cells overflow is skipped.  The
 * result is cached for the batch's class: total beads by powers of two and
 * mean packing fraction (beads x pi sigma^2 / 4 over the box area; volume
 * fraction in 3D) by steps of 0.05.  trial_steps = 0 takes the cached tuning
 * of the class without timing when there is one (else times 20 steps).
 * Writes the chosen tuning (with its time) to *chosen if not NULL. */
nw_status nw_batch_autotune(nw_batch* b, int trial_steps, NwBatchTuning* chosen);
/* The (bead-count, packing) class of the batch that keys the tuning cache. */
nw_status nw_batch_tuning_class(const nw_batch* b, int* bead_class, int* packing_class);

#ifdef __cplusplus
}
#endif

#endif /* NWGB_BATCH_H */
