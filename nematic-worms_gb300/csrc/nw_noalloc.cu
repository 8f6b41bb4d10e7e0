// nw_noalloc.cu — a stable key/value sort that allocates no device memory.
//
// sortParticles (nw_legacy.cu) takes its scratch from cudaMalloc on first
// use.  Some callers cannot allow that: their device memory is owned in full
// by another allocator (a framework's caching allocator, or a fixed budget
// taken at start-up), or they run a tight loop in which cudaMalloc's implicit
// device-wide synchronisation is not acceptable.  nw_sort_particles_noalloc
// gives them the same sort with its scratch in a fixed array compiled into
// this library.
#include <cstdio>
#include <mutex>

#include "../../include/nw_legacy.h"
#include "nw_sort.cuh"

namespace nw {
namespace {

// Largest key count the fixed scratch holds.
constexpr uint32_t kNoAllocMaxKeys = 1u << 18;  // 262,144

// Words of scratch for kNoAllocMaxKeys keys, by the layout of
// radix_scratch_layout: two 64-word-rounded key/value copies, two digit
// histograms of 256 entries per 2048-key tile (+8), the chunk totals.
constexpr size_t round64(size_t w) { return (w + 63) & ~size_t(63); }
constexpr size_t kTiles = (kNoAllocMaxKeys + kRadixTile - 1) / kRadixTile;
constexpr size_t kHistWords = round64(256 * kTiles + 8);
constexpr size_t kChunkWords = round64((256 * kTiles + kChunk - 1) / kChunk + 1);
constexpr size_t kNoAllocWords = 2 * round64(kNoAllocMaxKeys) + 2 * kHistWords + kChunkWords;

// The scratch itself: about 2.4 MB held by every GPU that loads the library,
// until the process exits.  Every call shares it.
__device__ __align__(256) uint32_t g_noalloc_sort_scratch[kNoAllocWords];

constexpr int kMaxDevices = 64;
uint32_t* g_scratch_addr[kMaxDevices] = {};
std::mutex g_setup_mu;

// Device address of the scratch on the current device (the symbol's
// host-side name is not a device address).  Looked up again on every call
// made outside stream capture, so that a context re-created after
// cudaDeviceReset (which can place the symbol elsewhere) is picked up; calls
// made while the legacy stream captures use the address of the last call
// made outside capture on this device.
nw_status scratch_address(uint32_t** out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return NW_ERR_CUDA;
    }
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(0, &cap) != cudaSuccess) {
        cudaGetLastError();
        return NW_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_addr[dev] || cap == cudaStreamCaptureStatusNone) {
        if (cap != cudaStreamCaptureStatusNone) {
            std::fprintf(stderr, "[nwgb] nw_sort_particles_noalloc: first call on a device made inside stream "
                                 "capture; make it once outside capture first\n");
            return NW_ERR_INVALID;
        }
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_sort_scratch);
        if (e != cudaSuccess || !p) {
            std::fprintf(stderr, "[nwgb] nw_sort_particles_noalloc: cudaGetSymbolAddress failed: %s\n",
                         cudaGetErrorString(e));
            cudaGetLastError();
            return NW_ERR_CUDA;
        }
        g_scratch_addr[dev] = static_cast<uint32_t*>(p);
    }
    *out = g_scratch_addr[dev];
    return NW_OK;
}

}  // namespace
}  // namespace nw

extern "C" int nw_sort_particles_noalloc(uint* dGridParticleHash, uint* dGridParticleIndex, uint numParticles)
{
    using namespace nw;
    if (numParticles > kNoAllocMaxKeys) {
        std::fprintf(stderr,
                     "[nwgb] nw_sort_particles_noalloc: %u keys exceed the fixed scratch (at most %u keys); "
                     "use sortParticles\n",
                     numParticles, kNoAllocMaxKeys);
        return NW_ERR_INVALID;
    }
    if (numParticles < 2) return NW_OK;
    if (!dGridParticleHash || !dGridParticleIndex) return NW_ERR_INVALID;
    // an error left by earlier, unrelated work is reported here and left in
    // place for its owner, so that the check after the launches below only
    // sees this call's own launches
    if (cudaPeekAtLastError() != cudaSuccess) {
        std::fprintf(stderr, "[nwgb] nw_sort_particles_noalloc: a CUDA error is pending from earlier work: %s\n",
                     cudaGetErrorString(cudaPeekAtLastError()));
        return NW_ERR_CUDA;
    }
    if (radix_scratch_layout(kNoAllocMaxKeys, nullptr, nullptr) > kNoAllocWords) return NW_ERR_INVALID;
    uint32_t* base = nullptr;
    const nw_status st = scratch_address(&base);
    if (st != NW_OK) return st;
    // Carved for the maximum key count, so every call uses the same sub-arrays.
    // No word needs clearing: each pass writes its histograms, offsets and
    // key/value copies in full before reading them.
    RadixScratch S;
    radix_scratch_layout(kNoAllocMaxKeys, base, &S);
    radix_sort_pairs(dGridParticleHash, dGridParticleIndex, numParticles, S, 0);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        std::fprintf(stderr, "[nwgb] nw_sort_particles_noalloc: %s\n", cudaGetErrorString(e));
        return NW_ERR_CUDA;
    }
    return NW_OK;
}
