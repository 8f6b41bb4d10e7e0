// nw_fused.cuh — launchers of the cell-list step path (nw_fused.cu, nw_fused_planar.cu;
// device code in nw_fused_impl.cuh).
#pragma once

#include "nw_kernels.cuh"

namespace nw {

// Options of the pro part of the single-system kernels:
//   kProLazyTangent  tangents are not stored by the step (WCA worms of more
//                    than three beads, whose step never reads them); the
//                    handle API computes them when they are read
constexpr uint32_t kProLazyTangent = 1u;
__host__ __device__ __forceinline__ uint32_t pro_flags(const DevParams& P)
{
    return P.model == NW_MODEL_WCA_WORMS && P.L > 3u ? kProLazyTangent : 0u;
}
// Tangents of the current positions as the pro part computes them.
uint64_t launch_bead_tangents(const DevParams& P, const float4* pos, float4* tan, cudaStream_t s);

// Filaments per block of the filament-aligned kernels (about 256 threads).
uint32_t list_filaments_per_block(uint32_t L, uint32_t nf);

// pro(n) with n = *step_base + off: integrate .. hash, insert into list n.
uint64_t launch_bead_pro(const DevParams& P, const StepBuffers& B, uint32_t off, float dt, cudaStream_t s);
// Verlet systems: the cell list of update n, built only when the pair pass
// of update n rebuilds the neighbour lists (launch after the pro part of n).
uint64_t launch_bead_list(const DevParams& P, const StepBuffers& B, uint32_t off, cudaStream_t s);
// epi(n): pair forces from list n; force = complete F_n.
uint64_t launch_bead_epi(const DevParams& P, const StepBuffers& B, uint32_t off, cudaStream_t s);
// epi(n) followed by pro(n+1) in one kernel.
uint64_t launch_bead_fused(const DevParams& P, const StepBuffers& B, uint32_t off, float dt, cudaStream_t s);

// ---- batched replicas (nw_batch.cu) ------------------------------------------

// One replica of a batch as its blocks see it: its parameter block and where
// its beads, list cells, neighbour lists and blocks start in the batch's
// concatenated buffers.
struct ReplicaSlot {
    DevParams P;
    float dt;
    uint32_t bead_off;  // first bead
    uint32_t cell_off;  // first list cell
    uint32_t blk0;      // first block of the launch
    uint32_t nblk;      // blocks of this replica
    uint32_t fpb;       // filaments per block
    uint32_t pad[2];
    unsigned long long nbr_off;  // first neighbour-list word
};

// kBatchList: a replica's cell list of update n when its pair pass will
// rebuild the Verlet lists (Verlet replicas; launched after each pro part)
enum BatchMode { kBatchPro = 0, kBatchEpi = 1, kBatchFused = 2, kBatchList = 3 };

// One launch over all replicas: block b serves replica block_rep[b].  S holds
// the batch's base pointers; `threads` >= every replica's fpb * L; planar =
// every replica is a planar system.
void launch_batch(int mode, const ReplicaSlot* table, const uint32_t* block_rep, uint32_t blocks, uint32_t threads,
                  size_t smem, uint32_t cap, const StepBuffers& S, uint32_t off, bool planar, cudaStream_t s);

// The two-component launches (nw_fused_planar.cu) behind the launchers above.
uint64_t launch_bead_pro_planar(const DevParams& P, const StepBuffers& B, uint32_t off, float dt, cudaStream_t s);
uint64_t launch_bead_tangents_planar(const DevParams& P, const float4* pos, float4* tan, cudaStream_t s);
uint64_t launch_bead_epi_planar(const DevParams& P, const StepBuffers& B, uint32_t off, cudaStream_t s);
uint64_t launch_bead_fused_planar(const DevParams& P, const StepBuffers& B, uint32_t off, float dt, cudaStream_t s);
void launch_batch_planar(int mode, const ReplicaSlot* table, const uint32_t* block_rep, uint32_t blocks,
                         uint32_t threads, size_t smem, uint32_t cap, const StepBuffers& S, uint32_t off,
                         cudaStream_t s);

}  // namespace nw
