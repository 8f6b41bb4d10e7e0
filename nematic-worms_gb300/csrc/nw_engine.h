// nw_engine.h — host-side launch helpers shared by the handle API, the
// batched engine and the legacy C-ABI layer.
#pragma once

#include "nw_kernels.cuh"

#include <string>
#include <vector>

namespace nw {

// Optional per-launch timing: an event is recorded on the launch stream
// before every kernel and once after the last, so consecutive event pairs
// bracket exactly one kernel each.
struct Prof {
    std::vector<cudaEvent_t> events;
    std::vector<std::string> names;
    cudaStream_t stream = nullptr;
    void mark(const char* name);  // event, then the kernel `name` follows
    void end();                   // closing event
    void clear();
};

// The neighbour search a configuration runs (NW_STRATEGY_AUTO resolved).
inline int effective_strategy(const NwConfig& c)
{
    if (c.strategy != NW_STRATEGY_AUTO) return c.strategy;
    return c.model == NW_MODEL_WCA_WORMS ? NW_STRATEGY_VERLET : NW_STRATEGY_SORTED;
}

// Kernel parameter block for a configuration and step size.
DevParams make_dev_params(const NwConfig& c, float dt);

// Enqueue one bead step (5 kernels); returns the number of launches.
uint64_t enqueue_bead_step(const DevParams& P, const StepBuffers& B, uint32_t nchunks, uint32_t step_off, float dt,
                           cudaStream_t s, Prof* prof = nullptr);

// Enqueue one SRD collision (7 kernels).  With shift_from_step the grid
// shift is drawn on the device from (seed, step); otherwise `shift` is used.
// buf_sel names the bead buffer holding the current state (0 or 1), or 2 for
// "the buffer of the update being collided" (step & 1).
uint64_t enqueue_srd(const DevParams& P, const StepBuffers& B, uint32_t srd_nchunks, uint32_t step_off, float dt_srd,
                     int shift_from_step, float3 shift, cudaStream_t s, Prof* prof = nullptr, uint32_t buf_sel = 2u);

}  // namespace nw
