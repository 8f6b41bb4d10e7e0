// nw_fused.cuh — launchers of the cell-list step path (nw_fused.cu).
#pragma once

#include "nw_kernels.cuh"

namespace nw {

// Filaments per block of the filament-aligned kernels (about 256 threads).
uint32_t list_filaments_per_block(uint32_t L, uint32_t nf);

// pro(n) with n = *step_base + off: integrate .. hash, insert into list n.
uint64_t launch_bead_pro(const DevParams& P, const StepBuffers& B, uint32_t off, float dt, cudaStream_t s);
// epi(n): pair forces from list n; force = complete F_n.
uint64_t launch_bead_epi(const DevParams& P, const StepBuffers& B, uint32_t off, cudaStream_t s);
// epi(n) followed by pro(n+1) in one kernel.
uint64_t launch_bead_fused(const DevParams& P, const StepBuffers& B, uint32_t off, float dt, cudaStream_t s);

}  // namespace nw
