// nw_fused_planar.cu — the cell-list step kernels of planar systems
// (two-dimensional WCA worms), compiled with two vector components
// (device code in nw_fused_impl.cuh).
#include "nw_fused_impl.cuh"

namespace nw {

uint64_t launch_bead_pro_planar(const DevParams& P, const StepBuffers& B, uint32_t off, float dt, cudaStream_t s)
{
    return bead_pro_d<2>(P, B, off, dt, s);
}

uint64_t launch_bead_tangents_planar(const DevParams& P, const float4* pos, float4* tan, cudaStream_t s)
{
    return bead_tangents_d<2>(P, pos, tan, s);
}

uint64_t launch_bead_epi_planar(const DevParams& P, const StepBuffers& B, uint32_t off, cudaStream_t s)
{
    return bead_epi_d<2>(P, B, off, s);
}

uint64_t launch_bead_fused_planar(const DevParams& P, const StepBuffers& B, uint32_t off, float dt, cudaStream_t s)
{
    return bead_fused_d<2>(P, B, off, dt, s);
}

void launch_batch_planar(int mode, const ReplicaSlot* table, const uint32_t* block_rep, uint32_t blocks,
                         uint32_t threads, size_t smem, uint32_t cap, const StepBuffers& S, uint32_t off,
                         cudaStream_t s)
{
    batch_d<2>(mode, table, block_rep, blocks, threads, smem, cap, S, off, s);
}

}  // namespace nw
