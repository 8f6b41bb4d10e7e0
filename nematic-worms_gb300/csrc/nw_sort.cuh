// nw_sort.cuh — general stable key/value sort (LSD radix, 8-bit digits) for
// arbitrary 32-bit keys.  The step itself uses the cell counting sort of
// nw_kernels.cuh; this sort backs the legacy sortParticles symbol
// (simulation/particleSystem_cuda.cu:277-282, thrust::sort_by_key), whose
// keys are not known to be cell indices.
#pragma once

#include "nw_kernels.cuh"

namespace nw {

constexpr uint32_t kRadixThreads = 256;
constexpr uint32_t kRadixItems = 8;
constexpr uint32_t kRadixTile = kRadixThreads * kRadixItems;  // 2048 keys per block

// Digit histogram of one tile: ghist[d * nblocks + b].
__global__ void __launch_bounds__(256) radix_hist_kernel(const uint32_t* __restrict__ keys, uint32_t n, int shift,
                                                         uint32_t* __restrict__ ghist, uint32_t nblocks);

// Stable scatter of one tile (rounds of 256 consecutive keys; the rank of a
// key among equal digits is earlier warps' counts + earlier lanes of its warp).
__global__ void __launch_bounds__(256) radix_scatter_kernel(const uint32_t* __restrict__ kin,
                                                            const uint32_t* __restrict__ vin,
                                                            uint32_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                                            uint32_t n, int shift,
                                                            const uint32_t* __restrict__ goffset, uint32_t nblocks);

// Scratch of one radix sort of up to `capacity` keys.
struct RadixScratch {
    uint32_t* keys_alt = nullptr;
    uint32_t* vals_alt = nullptr;
    uint32_t* ghist = nullptr;
    uint32_t* goffset = nullptr;
    uint32_t* chunk = nullptr;
    uint32_t capacity = 0;
};

// Carve the scratch of a sort of up to n keys out of one buffer of 32-bit
// words.  Every sub-array starts on a 256-byte boundary (the scan reads and
// writes 16-byte vectors).  Returns the words needed; with base == nullptr
// only the size is computed.
inline size_t radix_scratch_layout(uint32_t n, uint32_t* base, RadixScratch* out)
{
    auto up = [](size_t w) { return (w + 63) & ~size_t(63); };
    const size_t nblocks = (n + kRadixTile - 1) / kRadixTile;
    const size_t m = 256 * (nblocks ? nblocks : 1);
    const size_t hist = up(m + 8);
    const size_t chunk = up((m + kChunk - 1) / kChunk + 1);
    const size_t keys = up(n ? n : 1);
    if (base && out) {
        out->keys_alt = base;
        out->vals_alt = base + keys;
        out->ghist = base + 2 * keys;
        out->goffset = out->ghist + hist;
        out->chunk = out->goffset + hist;
        out->capacity = n;
    }
    return 2 * keys + 2 * hist + chunk;
}

// Sort (keys, vals) in place, stable, 4 passes; scratch must hold n keys.
inline void radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t n, const RadixScratch& S, cudaStream_t s)
{
    if (n < 2) return;
    const uint32_t nblocks = (n + kRadixTile - 1) / kRadixTile;
    const uint32_t m = 256u * nblocks;
    const uint32_t nchunks = (m + kChunk - 1) / kChunk;
    uint32_t *ki = keys, *vi = vals, *ko = S.keys_alt, *vo = S.vals_alt;
    for (int shift = 0; shift < 32; shift += 8) {
        radix_hist_kernel<<<nblocks, 256, 0, s>>>(ki, n, shift, S.ghist, nblocks);
        chunk_sum_kernel<<<nchunks, 512, 0, s>>>(S.ghist, m, S.chunk, nullptr, nullptr);
        scan_cells_kernel<false><<<nchunks, 512, 0, s>>>(S.ghist, S.chunk, m, S.goffset, nullptr, nullptr, nullptr,
                                                          nullptr, nullptr);
        radix_scatter_kernel<<<nblocks, 256, 0, s>>>(ki, vi, ko, vo, n, shift, S.goffset, nblocks);
        uint32_t* t = ki;
        ki = ko;
        ko = t;
        t = vi;
        vi = vo;
        vo = t;
    }
}

}  // namespace nw
