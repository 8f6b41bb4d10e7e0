// nw_sort.cu — kernels of the general stable radix sort declared in nw_sort.cuh.
#include "nw_sort.cuh"

namespace nw {

// Digit histogram of one tile: ghist[d * nblocks + b].
__global__ void __launch_bounds__(256) radix_hist_kernel(const uint32_t* __restrict__ keys, uint32_t n, int shift,
                                                         uint32_t* __restrict__ ghist, uint32_t nblocks)
{
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * kRadixTile;
#pragma unroll
    for (uint32_t r = 0; r < kRadixItems; ++r) {
        const uint32_t e = base + r * kRadixThreads + threadIdx.x;
        if (e < n) atomicAdd(&h[(keys[e] >> shift) & 255u], 1u);
    }
    __syncthreads();
    ghist[threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter of one tile: rounds of 256 consecutive keys; inside a round
// the rank of a key among equal digits is (earlier warps' counts) + (earlier
// lanes of its warp), so input order is kept.
__global__ void __launch_bounds__(256) radix_scatter_kernel(const uint32_t* __restrict__ kin,
                                                            const uint32_t* __restrict__ vin,
                                                            uint32_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                                            uint32_t n, int shift,
                                                            const uint32_t* __restrict__ goffset, uint32_t nblocks)
{
    __shared__ uint32_t s_base[256];
    __shared__ uint32_t s_run[256];
    __shared__ uint32_t s_cnt[8][257];
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    s_base[tid] = goffset[tid * nblocks + blockIdx.x];
    s_run[tid] = 0;
    const uint32_t lt = (1u << lane) - 1u;
    const uint32_t base = blockIdx.x * kRadixTile;
    for (uint32_t r = 0; r < kRadixItems; ++r) {
#pragma unroll
        for (int w = 0; w < 8; ++w) s_cnt[w][tid] = 0;
        if (tid == 0)
            for (int w = 0; w < 8; ++w) s_cnt[w][256] = 0;
        __syncthreads();
        const uint32_t e = base + r * kRadixThreads + tid;
        const bool valid = e < n;
        const uint32_t key = valid ? kin[e] : 0u;
        const uint32_t d = valid ? ((key >> shift) & 255u) : 256u;
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const uint32_t rank = __popc(peers & lt);
        if (rank == 0) s_cnt[warp][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            uint32_t before = 0;
            for (uint32_t w = 0; w < warp; ++w) before += s_cnt[w][d];
            const uint32_t pos = s_base[d] + s_run[d] + before + rank;
            kout[pos] = key;
            vout[pos] = vin[e];
        }
        __syncthreads();
        uint32_t add = 0;
#pragma unroll
        for (int w = 0; w < 8; ++w) add += s_cnt[w][tid];
        s_run[tid] += add;
        __syncthreads();
    }
}

}  // namespace nw
