// nw_batch.cu — batched replicas (include/nwgb_batch.h): many WCA worm
// systems of uneven size stepped by one kernel launch per step.
//
// Layout in HBM: every per-bead array is the concatenation of the replicas'
// arrays (replica r at bead offset boff[r]); the per-step cell lists and the
// Verlet lists are concatenations of per-replica tables (offsets in each
// replica's ReplicaSlot).  A launch's block b serves replica block_rep[b],
// whose parameter block it copies into shared memory before running the same
// pro / epi / fused step bodies as a single system (nw_fused_impl.cuh).
#include <cmath>
#include <cstring>
#include <mutex>
#include <utility>
#include <vector>

#include "../../include/nwgb_batch.h"
#include "nw_engine.h"
#include "nw_fused.cuh"

using namespace nw;

namespace {

struct BatchGraph {
    int nsteps;
    uint64_t version;
    cudaGraphExec_t exec;
    uint64_t launches;
};

uint32_t cdivu(uint64_t a, uint32_t b) { return (uint32_t)((a + b - 1) / b); }

}  // namespace

struct nw_batch {
    std::vector<NwConfig> cfg;
    int R = 0;
    cudaStream_t own_stream = nullptr, stream = nullptr;
    NwBatchTuning tune{};
    std::vector<uint32_t> nb;
    std::vector<uint64_t> boff;
    uint64_t total = 0;
    // launch layout of the current tuning
    std::vector<ReplicaSlot> slots;
    ReplicaSlot* d_slots = nullptr;
    uint32_t* d_block_rep = nullptr;
    uint32_t blocks = 0, threads = 0, cap = 8;
    size_t smem = 0;
    StepBuffers B{};
    std::vector<void*> state_allocs, list_allocs;
    uint64_t step = 0, version = 1, last_launches = 0;
    bool use_graphs = true, vl = false, vl_dirty = true, lists_dirty = true;
    bool tan_stale = false;  // tangents of lazy replicas (pro_flags) computed when read
    bool planar = false;     // every replica is two-dimensional (the planar kernels)
    std::vector<BatchGraph> graphs;
};

namespace {

// ---- tuning cache: one tuning per (bead-count, packing) class of batches ----
struct TuneKey {
    int beads;    // floor(log2(total beads))
    int packing;  // floor(mean packing fraction / 0.05)
};

TuneKey tune_key(const nw_batch* b)
{
    TuneKey k{0, 0};
    uint64_t n = b->total;
    while (n > 1) {
        n >>= 1;
        ++k.beads;
    }
    constexpr double kPi = 3.14159265358979323846;
    double phi = 0.0;
    for (const auto& c : b->cfg) {
        const double s = c.lj_sigma, nb = (double)c.num_filaments * c.filament_size;
        if (c.dim >= 3)
            phi += nb * (kPi / 6.0) * s * s * s / ((double)c.box[0] * c.box[1] * c.box[2]);
        else
            phi += nb * (kPi / 4.0) * s * s / ((double)c.box[0] * c.box[1]);
    }
    if (!b->cfg.empty()) phi /= (double)b->cfg.size();
    k.packing = (int)std::floor(phi / 0.05);
    return k;
}

std::mutex g_tune_mutex;
std::vector<std::pair<TuneKey, NwBatchTuning>> g_tune_cache;

bool tune_cache_find(const TuneKey& k, NwBatchTuning* t)
{
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    for (const auto& e : g_tune_cache)
        if (e.first.beads == k.beads && e.first.packing == k.packing) {
            *t = e.second;
            return true;
        }
    return false;
}

void tune_cache_store(const TuneKey& k, const NwBatchTuning& t)
{
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    for (auto& e : g_tune_cache)
        if (e.first.beads == k.beads && e.first.packing == k.packing) {
            e.second = t;
            return;
        }
    g_tune_cache.push_back({k, t});
}

nw_status cuda_st(cudaError_t e)
{
    if (e == cudaSuccess) return NW_OK;
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? NW_ERR_NOMEM : NW_ERR_CUDA;
}

template <class T>
nw_status balloc(std::vector<void*>& list, T** p, size_t n)
{
    *p = nullptr;
    void* q = nullptr;
    if (cudaMalloc(&q, (n ? n : 1) * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        return NW_ERR_NOMEM;
    }
    list.push_back(q);
    *p = reinterpret_cast<T*>(q);
    return NW_OK;
}

void free_list(std::vector<void*>& list)
{
    for (void* p : list) cudaFree(p);
    list.clear();
}

void drop_graphs(nw_batch* b)
{
    for (auto& g : b->graphs) cudaGraphExecDestroy(g.exec);
    b->graphs.clear();
}

uint32_t cur_buffer(const nw_batch* b) { return (uint32_t)((b->step + 1ull) & 1ull); }

// (Re)build the launch layout, list tables and neighbour lists for tuning t.
nw_status configure(nw_batch* b, const NwBatchTuning& t)
{
    if (t.threads_per_block != 128 && t.threads_per_block != 256 && t.threads_per_block != 512) return NW_ERR_INVALID;
    if (t.strategy != NW_STRATEGY_VERLET && t.strategy != NW_STRATEGY_CELL_LISTS) return NW_ERR_INVALID;
    if (!(t.neighbor_skin >= 0.0f) || !std::isfinite(t.neighbor_skin)) return NW_ERR_INVALID;
    if (t.cell_capacity != 0 && t.cell_capacity != 8 && t.cell_capacity != 16) return NW_ERR_INVALID;
    cudaStreamSynchronize(b->stream);
    drop_graphs(b);
    free_list(b->list_allocs);
    uint32_t maxL = 1;
    bool reverse = false;
    b->cap = 8;
    for (const auto& c : b->cfg) {
        maxL = c.filament_size > maxL ? c.filament_size : maxL;
        reverse |= c.reverse_probability > 0.0f;
        if (c.cell_capacity == 16) b->cap = 16;
    }
    if (t.cell_capacity) b->cap = t.cell_capacity;
    uint32_t threads = t.threads_per_block;
    const uint32_t need = (maxL + 31u) & ~31u;
    if (need > threads) threads = need;
    if (threads > 512) return NW_ERR_UNSUPPORTED;
    b->threads = threads;
    b->smem = (size_t)threads * sizeof(float4) * (reverse ? 3u : 1u) + (size_t)threads * 3u * sizeof(float4);
    b->slots.assign(b->R, ReplicaSlot{});
    std::vector<uint32_t> block_rep;
    uint64_t cells = 0, nbr_words = 0;
    b->vl = false;
    for (int r = 0; r < b->R; ++r) {
        NwConfig c = b->cfg[r];
        c.strategy = t.strategy;
        c.neighbor_skin = t.neighbor_skin;
        ReplicaSlot& e = b->slots[r];
        std::memset(&e, 0, sizeof(e));
        e.P = make_dev_params(c, c.dt);
        e.dt = c.dt;
        e.bead_off = (uint32_t)b->boff[r];
        e.cell_off = (uint32_t)cells;
        e.nbr_off = nbr_words;
        uint32_t fpb = threads / c.filament_size;
        if (fpb < 1) fpb = 1;
        if (fpb > c.num_filaments && c.num_filaments > 0) fpb = c.num_filaments;
        e.fpb = fpb;
        e.blk0 = (uint32_t)block_rep.size();
        e.nblk = c.num_filaments ? cdivu(c.num_filaments, fpb) : 0u;
        for (uint32_t k = 0; k < e.nblk; ++k) block_rep.push_back((uint32_t)r);
        cells += e.P.lncells;
        if (e.P.vl_on) {
            b->vl = true;
            nbr_words += (uint64_t)e.P.vl_cap * b->nb[r];
        }
    }
    if (cells >= (1ull << 32) || nbr_words >= (1ull << 40)) return NW_ERR_INVALID;
    b->blocks = (uint32_t)block_rep.size();
    nw_status st = NW_OK;
    auto A = [&](nw_status x) {
        if (st == NW_OK) st = x;
    };
    StepBuffers& B = b->B;
    for (int k = 0; k < 3; ++k) A(balloc(b->list_allocs, &B.lcount[k], cells + 8));
    for (int k = 0; k < 2; ++k) A(balloc(b->list_allocs, &B.lslot[k], cells * b->cap + 8));
    B.cap = b->cap;
    B.nbr = B.nnb = B.vstate = nullptr;
    if (b->vl) {
        A(balloc(b->list_allocs, &B.nbr, nbr_words + 8));
        A(balloc(b->list_allocs, &B.nnb, b->total + 8));
        A(balloc(b->list_allocs, &B.vstate, 8ull * b->R));
    }
    A(balloc(b->list_allocs, &b->d_slots, b->slots.size()));
    A(balloc(b->list_allocs, &b->d_block_rep, block_rep.size() + 1));
    if (st != NW_OK) return st;
    cudaError_t e = cudaMemcpy(b->d_slots, b->slots.data(), b->slots.size() * sizeof(ReplicaSlot),
                               cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !block_rep.empty())
        e = cudaMemcpy(b->d_block_rep, block_rep.data(), block_rep.size() * 4, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_st(e);
    b->tune = t;
    b->tune.cell_capacity = b->cap;
    b->version++;
    b->lists_dirty = true;
    b->vl_dirty = true;
    return NW_OK;
}

// Zero the list counters and force a list build where the state changed.
cudaError_t clean(nw_batch* b)
{
    cudaError_t e = cudaSuccess;
    if (b->lists_dirty) {
        uint64_t cells = 0;
        for (const auto& s : b->slots) cells += s.P.lncells;
        for (int k = 0; k < 3 && e == cudaSuccess; ++k)
            e = cudaMemsetAsync(b->B.lcount[k], 0, (cells + 8) * 4, b->stream);
        if (e != cudaSuccess) return e;
        b->lists_dirty = false;
    }
    if (b->vl && b->vl_dirty) {
        std::vector<uint32_t> init(8ull * b->R, 0u);
        for (int r = 0; r < b->R; ++r) {
            init[8ull * r] = init[8ull * r + 1] = 0x7f000000u;  // a list build at the first pair pass
            init[8ull * r + 6] = 7u;                            // every count buffer counts as filled
        }
        // pageable source: the copy is staged before the call returns
        e = cudaMemcpyAsync(b->B.vstate, init.data(), init.size() * 4, cudaMemcpyHostToDevice, b->stream);
        if (e != cudaSuccess) return e;
        b->vl_dirty = false;
    }
    return e;
}

uint64_t enqueue(nw_batch* b, int nsteps)
{
    if (b->blocks == 0) return 0;
    uint64_t launches = 0;
    auto L = [&](int mode, uint32_t off) {
        launch_batch(mode, b->d_slots, b->d_block_rep, b->blocks, b->threads, b->smem, b->cap, b->B, off, b->planar,
                     b->stream);
        ++launches;
    };
    L(kBatchPro, 0u);
    if (b->vl) L(kBatchList, 0u);
    for (int j = 0; j < nsteps; ++j) {
        if (j == nsteps - 1) {
            L(kBatchEpi, (uint32_t)j);
        } else {
            L(kBatchFused, (uint32_t)j);
            if (b->vl) L(kBatchList, (uint32_t)(j + 1));
        }
    }
    advance_step_kernel<<<1, 1, 0, b->stream>>>(b->B.step_base, (unsigned long long)nsteps);
    return launches + 1ull;
}

nw_status state_ptr(nw_batch* b, int array, float4** p)
{
    const uint32_t cur = cur_buffer(b);
    switch (array) {
    case NW_POSITION: *p = b->B.pos2[cur]; return NW_OK;
    case NW_VELOCITY: *p = b->B.vel2[cur]; return NW_OK;
    case NW_TANGENT: *p = b->B.tan2[cur]; return NW_OK;
    case NW_FORCE: *p = b->B.force; return NW_OK;
    case NW_FORCE_OLD: *p = b->B.force_old; return NW_OK;
    default: return NW_ERR_INVALID;
    }
}

// Tangents of the replicas whose step does not store them, from the current
// positions (as the single-system engine does when they are read).
cudaError_t materialize_tangents(nw_batch* b)
{
    if (!b->tan_stale) return cudaSuccess;
    const uint32_t cur = cur_buffer(b);
    for (int r = 0; r < b->R; ++r) {
        const DevParams& P = b->slots[r].P;
        if (pro_flags(P) & kProLazyTangent)
            launch_bead_tangents(P, b->B.pos2[cur] + b->boff[r], b->B.tan2[cur] + b->boff[r], b->stream);
    }
    const cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) b->tan_stale = false;
    return e;
}

nw_status set_step(nw_batch* b, uint64_t step)
{
    const uint32_t from = cur_buffer(b);
    const uint64_t old = b->step;
    b->step = step;
    const uint32_t to = cur_buffer(b);
    cudaError_t e = cudaSuccess;
    if (from != to) {
        const size_t n = b->total * 16;
        e = cudaMemcpyAsync(b->B.pos2[to], b->B.pos2[from], n, cudaMemcpyDeviceToDevice, b->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(b->B.vel2[to], b->B.vel2[from], n, cudaMemcpyDeviceToDevice, b->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(b->B.tan2[to], b->B.tan2[from], n, cudaMemcpyDeviceToDevice, b->stream);
    }
    unsigned long long v = step;
    if (e == cudaSuccess) e = cudaMemcpyAsync(b->B.step_base, &v, 8, cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) {
        b->step = old;
        return cuda_st(e);
    }
    b->lists_dirty = true;
    b->vl_dirty = true;
    return NW_OK;
}

}  // namespace

extern "C" {

nw_status nw_batch_create(const NwConfig* replicas, int n, nw_batch** out)
{
    if (!out) return NW_ERR_INVALID;
    *out = nullptr;
    if (!replicas || n <= 0) return NW_ERR_INVALID;
    for (int r = 0; r < n; ++r) {
        const nw_status st = nw_config_validate(&replicas[r]);
        if (st != NW_OK) return st;
        if (replicas[r].model != NW_MODEL_WCA_WORMS || replicas[r].srd_enabled) return NW_ERR_UNSUPPORTED;
        if (replicas[r].filament_size > 512) return NW_ERR_UNSUPPORTED;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return NW_ERR_NO_DEVICE;
    }
    nw_batch* b = new nw_batch();
    b->cfg.assign(replicas, replicas + n);
    b->R = n;
    b->planar = true;
    for (int r = 0; r < n; ++r) b->planar = b->planar && replicas[r].dim == 2;  // all are WCA worms
    if (cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete b;
        return NW_ERR_CUDA;
    }
    b->stream = b->own_stream;
    for (int r = 0; r < n; ++r) {
        b->nb.push_back(replicas[r].num_filaments * replicas[r].filament_size);
        b->boff.push_back(b->total);
        b->total += b->nb.back();
    }
    nw_status st = b->total >= (1ull << 31) ? NW_ERR_INVALID : NW_OK;
    auto A = [&](nw_status x) {
        if (st == NW_OK) st = x;
    };
    StepBuffers& B = b->B;
    std::memset(&B, 0, sizeof(B));
    const size_t nbt = b->total + 8;
    for (int k = 0; k < 2; ++k) {
        A(balloc(b->state_allocs, &B.pos2[k], nbt));
        A(balloc(b->state_allocs, &B.vel2[k], nbt));
        A(balloc(b->state_allocs, &B.tan2[k], nbt));
        A(balloc(b->state_allocs, &B.hash2[k], nbt));
    }
    A(balloc(b->state_allocs, &B.force, nbt));
    A(balloc(b->state_allocs, &B.force_old, nbt));
    A(balloc(b->state_allocs, &B.err, 4));
    A(balloc(b->state_allocs, &B.step_base, 1));
    cudaError_t e = cudaSuccess;
    if (st == NW_OK) {
        for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
            e = cudaMemset(B.pos2[k], 0, nbt * 16);
            if (e == cudaSuccess) e = cudaMemset(B.vel2[k], 0, nbt * 16);
            if (e == cudaSuccess) e = cudaMemset(B.tan2[k], 0, nbt * 16);
            if (e == cudaSuccess) e = cudaMemset(B.hash2[k], 0, nbt * 4);
        }
        if (e == cudaSuccess) e = cudaMemset(B.force, 0, nbt * 16);
        if (e == cudaSuccess) e = cudaMemset(B.force_old, 0, nbt * 16);
        if (e == cudaSuccess) e = cudaMemset(B.err, 0, 16);
        if (e == cudaSuccess) e = cudaMemset(B.step_base, 0, 8);
        if (e != cudaSuccess) st = cuda_st(e);
    }
    if (st == NW_OK) {
        NwBatchTuning t{256u, NW_STRATEGY_VERLET, 0.3f, 0.0f};
        st = configure(b, t);
    }
    if (st != NW_OK) {
        nw_batch_destroy(b);
        return st;
    }
    *out = b;
    return NW_OK;
}

nw_status nw_batch_destroy(nw_batch* b)
{
    if (!b) return NW_ERR_INVALID;
    cudaStreamSynchronize(b->stream);
    drop_graphs(b);
    free_list(b->list_allocs);
    free_list(b->state_allocs);
    if (b->own_stream) cudaStreamDestroy(b->own_stream);
    delete b;
    return NW_OK;
}

nw_status nw_batch_counts(const nw_batch* b, int* n_replicas, uint64_t* total_beads)
{
    if (!b) return NW_ERR_INVALID;
    if (n_replicas) *n_replicas = b->R;
    if (total_beads) *total_beads = b->total;
    return NW_OK;
}

nw_status nw_batch_replica(const nw_batch* b, int r, uint32_t* n_beads, uint64_t* bead_offset)
{
    if (!b || r < 0 || r >= b->R) return NW_ERR_INVALID;
    if (n_beads) *n_beads = b->nb[r];
    if (bead_offset) *bead_offset = b->boff[r];
    return NW_OK;
}

static nw_status batch_transfer(nw_batch* b, int r, int array, void* host, uint32_t start, uint32_t count, bool to_dev)
{
    if (!b || r < 0 || r >= b->R || !host) return NW_ERR_INVALID;
    if ((uint64_t)start + count > b->nb[r]) return NW_ERR_INVALID;
    float4* base = nullptr;
    const nw_status st = state_ptr(b, array, &base);
    if (st != NW_OK) return st;
    if (!count) return NW_OK;
    if (array == NW_TANGENT) {
        const cudaError_t m = materialize_tangents(b);  // also before a partial write
        if (m != cudaSuccess) return cuda_st(m);
    }
    float4* d = base + b->boff[r] + start;
    cudaError_t e = to_dev ? cudaMemcpyAsync(d, host, (size_t)count * 16, cudaMemcpyHostToDevice, b->stream)
                           : cudaMemcpyAsync(host, d, (size_t)count * 16, cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (to_dev && array == NW_POSITION) b->vl_dirty = true;
    return cuda_st(e);
}

nw_status nw_batch_set_array(nw_batch* b, int r, int array, const void* host, uint32_t start, uint32_t count)
{
    return batch_transfer(b, r, array, const_cast<void*>(host), start, count, true);
}

nw_status nw_batch_get_array(nw_batch* b, int r, int array, void* host, uint32_t start, uint32_t count)
{
    return batch_transfer(b, r, array, host, start, count, false);
}

nw_status nw_batch_device_array(nw_batch* b, int array, void** dptr)
{
    if (!b || !dptr) return NW_ERR_INVALID;
    float4* p = nullptr;
    const nw_status st = state_ptr(b, array, &p);
    if (st != NW_OK) return st;
    if (array == NW_POSITION) b->vl_dirty = true;  // the caller may move beads through it
    if (array == NW_TANGENT) {
        cudaError_t e = materialize_tangents(b);
        if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
        if (e != cudaSuccess) return cuda_st(e);
    }
    *dptr = p;
    return NW_OK;
}

nw_status nw_batch_step(nw_batch* b, int nsteps)
{
    if (!b || nsteps < 0) return NW_ERR_INVALID;
    if (nsteps == 0) return NW_OK;
    cudaError_t e = clean(b);
    if (e != cudaSuccess) return cuda_st(e);
    if (b->use_graphs && nsteps > 1) {
        BatchGraph* hit = nullptr;
        for (auto& g : b->graphs)
            if (g.nsteps == nsteps && g.version == b->version) hit = &g;
        if (!hit) {
            if (b->graphs.size() >= 8) drop_graphs(b);
            cudaGraph_t graph = nullptr;
            e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
            if (e != cudaSuccess) return cuda_st(e);
            const uint64_t launches = enqueue(b, nsteps);
            e = cudaStreamEndCapture(b->stream, &graph);
            if (e != cudaSuccess) return cuda_st(e);
            cudaGraphExec_t exec = nullptr;
            e = cudaGraphInstantiate(&exec, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) return cuda_st(e);
            b->graphs.push_back({nsteps, b->version, exec, launches});
            hit = &b->graphs.back();
        }
        e = cudaGraphLaunch(hit->exec, b->stream);
        b->last_launches = hit->launches;
    } else {
        b->last_launches = enqueue(b, nsteps);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return cuda_st(e);
    b->step += (uint64_t)nsteps;
    b->tan_stale = true;
    return NW_OK;
}

nw_status nw_batch_sync(nw_batch* b)
{
    if (!b) return NW_ERR_INVALID;
    cudaError_t e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return cuda_st(e);
    uint32_t f = 0;
    e = cudaMemcpy(&f, b->B.err, 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && f) e = cudaMemset(b->B.err, 0, 4);
    if (e != cudaSuccess) return cuda_st(e);
    if (f & NW_EFLAG_NONFINITE) return NW_ERR_NONFINITE;
    if (f & (NW_EFLAG_CELL_OVERFLOW | NW_EFLAG_NEIGHBOR_OVERFLOW)) return NW_ERR_CELL_OVERFLOW;
    if (f & NW_EFLAG_TIMEOUT) return NW_ERR_TIMEOUT;
    if (f & NW_EFLAG_BAD_INDEX) return NW_ERR_INVALID;
    return NW_OK;
}

nw_status nw_batch_set_stream(nw_batch* b, void* stream)
{
    if (!b) return NW_ERR_INVALID;
    cudaStreamSynchronize(b->stream);
    b->stream = stream ? (cudaStream_t)stream : b->own_stream;
    drop_graphs(b);
    return NW_OK;
}

nw_status nw_batch_set_graphs(nw_batch* b, int enabled)
{
    if (!b) return NW_ERR_INVALID;
    b->use_graphs = enabled != 0;
    return NW_OK;
}

uint64_t nw_batch_get_step(const nw_batch* b) { return b ? b->step : 0ull; }

nw_status nw_batch_last_launch_count(const nw_batch* b, uint64_t* launches)
{
    if (!b || !launches) return NW_ERR_INVALID;
    *launches = b->last_launches;
    return NW_OK;
}

nw_status nw_batch_get_tuning(const nw_batch* b, NwBatchTuning* t)
{
    if (!b || !t) return NW_ERR_INVALID;
    *t = b->tune;
    return NW_OK;
}

nw_status nw_batch_set_tuning(nw_batch* b, const NwBatchTuning* t)
{
    if (!b || !t) return NW_ERR_INVALID;
    const NwBatchTuning old = b->tune;
    nw_status st = configure(b, *t);
    if (st != NW_OK) configure(b, old);
    return st;
}

nw_status nw_batch_tuning_class(const nw_batch* b, int* bead_class, int* packing_class)
{
    if (!b) return NW_ERR_INVALID;
    const TuneKey k = tune_key(b);
    if (bead_class) *bead_class = k.beads;
    if (packing_class) *packing_class = k.packing;
    return NW_OK;
}

nw_status nw_batch_autotune(nw_batch* b, int trial_steps, NwBatchTuning* chosen)
{
    if (!b || trial_steps < 0 || trial_steps == 1) return NW_ERR_INVALID;
    const TuneKey key = tune_key(b);
    if (trial_steps == 0) {
        NwBatchTuning cached;
        if (tune_cache_find(key, &cached)) {
            nw_status st = configure(b, cached);
            if (st != NW_OK) return st;
            b->tune.ms_per_step = cached.ms_per_step;
            if (chosen) *chosen = b->tune;
            return NW_OK;
        }
        trial_steps = 20;
    }
    cudaError_t e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return cuda_st(e);
    // saved state: the current buffers of position, velocity, tangent, force, old force
    const uint64_t step0 = b->step;
    const size_t bytes = b->total * 16 + 16;
    std::vector<void*> scratch;
    float4* save[5] = {};
    for (int k = 0; k < 5; ++k)
        if (balloc(scratch, &save[k], b->total + 1) != NW_OK) {
            free_list(scratch);
            return NW_ERR_NOMEM;
        }
    const int arrays[5] = {NW_POSITION, NW_VELOCITY, NW_TANGENT, NW_FORCE, NW_FORCE_OLD};
    auto copy_state = [&](bool out) -> nw_status {
        for (int k = 0; k < 5; ++k) {
            float4* p = nullptr;
            state_ptr(b, arrays[k], &p);
            cudaError_t x = out ? cudaMemcpyAsync(save[k], p, bytes, cudaMemcpyDeviceToDevice, b->stream)
                                : cudaMemcpyAsync(p, save[k], bytes, cudaMemcpyDeviceToDevice, b->stream);
            if (x != cudaSuccess) return cuda_st(x);
        }
        return cuda_st(cudaStreamSynchronize(b->stream));
    };
    auto restore = [&]() -> nw_status {
        nw_status s = set_step(b, step0);
        if (s == NW_OK) s = copy_state(false);
        return s;
    };
    nw_status st = copy_state(true);
    const NwBatchTuning start = b->tune;
    NwBatchTuning best = start;
    best.ms_per_step = INFINITY;
    const uint32_t threads[3] = {128u, 256u, 512u};
    const uint32_t caps[2] = {8u, 16u};
    const NwBatchTuning searches[4] = {{0, NW_STRATEGY_VERLET, 0.2f, 0, 0}, {0, NW_STRATEGY_VERLET, 0.3f, 0, 0},
                                       {0, NW_STRATEGY_VERLET, 0.45f, 0, 0}, {0, NW_STRATEGY_CELL_LISTS, 0.3f, 0, 0}};
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEventCreate(&ev0);
    cudaEventCreate(&ev1);
    for (int a = 0; a < 3 && st == NW_OK; ++a)
        for (int s = 0; s < 4 && st == NW_OK; ++s)
            for (int c = 0; c < 2 && st == NW_OK; ++c) {
                NwBatchTuning t = searches[s];
                t.threads_per_block = threads[a];
                t.cell_capacity = caps[c];
                // a candidate the replicas cannot run (e.g. lists too large) is skipped
                if (configure(b, t) != NW_OK) continue;
                st = restore();
                if (st == NW_OK) st = nw_batch_step(b, trial_steps);  // capture + warm
                if (st == NW_OK) st = nw_batch_sync(b);
                if (st == NW_ERR_CELL_OVERFLOW) {  // cells too small for this state: skipped
                    st = NW_OK;
                    continue;
                }
                if (st == NW_OK) st = restore();
                if (st != NW_OK) break;
                cudaEventRecord(ev0, b->stream);
                st = nw_batch_step(b, trial_steps);
                cudaEventRecord(ev1, b->stream);
                if (st == NW_OK) st = nw_batch_sync(b);
                if (st == NW_ERR_CELL_OVERFLOW) {
                    st = NW_OK;
                    continue;
                }
                float ms = 0.f;
                cudaEventElapsedTime(&ms, ev0, ev1);
                t.ms_per_step = ms / (float)trial_steps;
                if (st == NW_OK && t.ms_per_step < best.ms_per_step) best = t;
            }
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    if (st == NW_OK) st = configure(b, best.ms_per_step < INFINITY ? best : start);
    if (st == NW_OK) st = restore();
    b->tune.ms_per_step = best.ms_per_step < INFINITY ? best.ms_per_step : 0.0f;
    free_list(scratch);
    if (st == NW_OK && best.ms_per_step < INFINITY) tune_cache_store(key, b->tune);
    if (st == NW_OK && chosen) *chosen = b->tune;
    return st;
}

}  // extern "C"
