// nw_system.h — the handle behind include/nwgb.h's nw_system (internal:
// shared by the engine and the trajectory writer, not part of the ABI).
#pragma once

#include <vector>

#include "nw_kernels.cuh"

struct GraphEntry {
    int nsteps;
    uint32_t dt_bits;
    uint32_t phase;
    uint64_t version;
    cudaGraphExec_t exec;
    uint64_t launches;
    bool state_ev;  // the graph records nw_system::state_ev
};

struct nw_system {
    NwConfig cfg;
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    nw::StepBuffers B;
    bool lists = false;  // NW_STRATEGY_CELL_LISTS
    uint32_t nb = 0, ns = 0, ntotal = 0, ncells = 0, nchunks = 0, srd_ncells = 0, srd_nchunks = 0;
    uint32_t lncells = 0;  // cells of the per-step bead lists (>= the reference grid's when Verlet cells are finer)
    uint64_t step = 0;
    uint64_t version = 1;
    bool use_graphs = true;
    bool lists_dirty = false;  // list counters must be cleared before the next update
    uint64_t sorted_for = ~0ull;  // step whose sorted order / cell bounds are in the sort buffers
    uint32_t scur = 0;            // solvent buffer holding the current solvent (mirror of *B.scur)
    bool vl = false;              // NW_STRATEGY_VERLET: hash2 holds Verlet-grid hashes
    bool vl_dirty = true;         // Verlet lists must be rebuilt at the next update
    uint64_t hash_for = ~0ull;    // step whose reference hashes are in hash2[cur] (Verlet systems)
    bool tan_stale = false;       // tangents not stored by the step: computed when read
    std::vector<GraphEntry> graphs;
    uint64_t last_launches = 0;
    // early read-back: the step graphs record state_ev once the positions and
    // velocities of their last update are final (before its pair pass), so
    // an asynchronous read of them runs on aux beside the rest of the step;
    // valid while nothing else has been enqueued that writes them
    cudaStream_t aux = nullptr;
    cudaEvent_t state_ev = nullptr, aux_done = nullptr;
    bool state_ev_valid = false;
    bool enqueued_state_ev = false;  // the last enqueue_steps recorded state_ev
    std::vector<void*> allocs;
    // defect search workspace (nw_defects.cu): bounds, counters and marked
    // cells (fixed), the per-cell sums (grown on demand), a pinned host copy
    void* defect_fixed = nullptr;
    void* defect_acc = nullptr;
    size_t defect_acc_bytes = 0;
    uint32_t* defect_host = nullptr;
    // observables workspace (nw_observables.cu): partial sums, the
    // mean-square displacement's reference / last positions and images, the
    // SRD cell sums; grown on demand
    void* obs_ws = nullptr;
    size_t obs_ws_bytes = 0;
    void* obs_msd = nullptr;
    size_t obs_msd_bytes = 0;
    bool obs_msd_on = false;
    void* obs_srd = nullptr;
    size_t obs_srd_bytes = 0;
};
