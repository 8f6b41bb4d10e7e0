// nw_fused.cu — launchers of the cell-list step path and its three-component
// kernels (device code in nw_fused_impl.cuh); planar systems go to the
// two-component kernels of nw_fused_planar.cu.
#include "nw_fused_impl.cuh"

namespace nw {

uint32_t list_filaments_per_block(uint32_t L, uint32_t nf)
{
    uint32_t fpb = L >= 256 ? 1u : 256u / L;
    if (fpb > nf && nf > 0) fpb = nf;
    return fpb ? fpb : 1u;
}

uint64_t launch_bead_pro(const DevParams& P, const StepBuffers& B, uint32_t off, float dt, cudaStream_t s)
{
    if (P.nb == 0) return 0;
    return planar_system(P) ? launch_bead_pro_planar(P, B, off, dt, s) : bead_pro_d<3>(P, B, off, dt, s);
}

uint64_t launch_bead_tangents(const DevParams& P, const float4* pos, float4* tan, cudaStream_t s)
{
    if (P.nb == 0) return 0;
    return planar_system(P) ? launch_bead_tangents_planar(P, pos, tan, s) : bead_tangents_d<3>(P, pos, tan, s);
}

uint64_t launch_bead_list(const DevParams& P, const StepBuffers& B, uint32_t off, cudaStream_t s)
{
    if (P.nb == 0 || !P.vl_on) return 0;
    const uint32_t blocks = cdiv32(P.nb, 256) < 608u ? cdiv32(P.nb, 256) : 608u;  // 4 blocks per SM
    if (B.cap == 16) launch_pdl(bead_list_kernel<16>, blocks, 256, 0, s, P, B, off);
    else launch_pdl(bead_list_kernel<8>, blocks, 256, 0, s, P, B, off);
    return 1;
}

uint64_t launch_bead_epi(const DevParams& P, const StepBuffers& B, uint32_t off, cudaStream_t s)
{
    if (P.nb == 0) return 0;
    return planar_system(P) ? launch_bead_epi_planar(P, B, off, s) : bead_epi_d<3>(P, B, off, s);
}

uint64_t launch_bead_fused(const DevParams& P, const StepBuffers& B, uint32_t off, float dt, cudaStream_t s)
{
    if (P.nb == 0) return 0;
    return planar_system(P) ? launch_bead_fused_planar(P, B, off, dt, s) : bead_fused_d<3>(P, B, off, dt, s);
}

void launch_batch(int mode, const ReplicaSlot* table, const uint32_t* block_rep, uint32_t blocks, uint32_t threads,
                  size_t smem, uint32_t cap, const StepBuffers& S, uint32_t off, bool planar, cudaStream_t s)
{
    if (blocks == 0) return;
    if (planar) launch_batch_planar(mode, table, block_rep, blocks, threads, smem, cap, S, off, s);
    else batch_d<3>(mode, table, block_rep, blocks, threads, smem, cap, S, off, s);
}

}  // namespace nw
