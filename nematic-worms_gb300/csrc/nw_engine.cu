// nw_engine.cu — the handle API of include/nwgb.h: system lifetime, state
// transfer, the step launcher with CUDA-graph replay, SRD, checkpoints.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "nw_engine.h"
#include "nw_fused.cuh"
#include "nw_system.h"

namespace nw {

DevParams make_dev_params(const NwConfig& c, float dt)
{
    DevParams P;
    std::memset(&P, 0, sizeof(P));
    P.model = c.model;
    P.dim = c.dim;
    P.hash_mode = c.hash_mode;
    P.nf = c.num_filaments;
    P.L = c.filament_size;
    P.nb = c.num_filaments * c.filament_size;
    P.ns = c.srd_enabled ? c.num_solvent : 0u;
    P.ntotal = P.nb + P.ns;
    P.ncells = 1;
    for (int a = 0; a < 3; ++a) {
        P.grid[a] = c.grid[a];
        P.ncells *= c.grid[a];
        P.cell[a] = c.cell_size[a];
        P.origin[a] = c.origin[a];
        P.box[a] = c.box[a];
        P.bnd[a] = c.boundary[a];
        P.srd_grid[a] = c.srd_grid[a] ? c.srd_grid[a] : 1u;
        P.srd_cell[a] = c.srd_cell_size[a];
        P.inv_cell[a] = 1.0f / c.cell_size[a];
        P.srd_inv_cell[a] = c.srd_cell_size[a] > 0.0f ? 1.0f / c.srd_cell_size[a] : 0.0f;
        P.ibox[a] = c.boundary[a] == NW_PERIODIC && c.box[a] > 0.0f ? 1.0f / c.box[a] : 0.0f;
    }
    P.srd_ncells = P.srd_grid[0] * P.srd_grid[1] * P.srd_grid[2];
    P.radius = c.radius;
    P.mass = c.mass;
    P.bond_k = c.bond_k;
    P.bond_r0 = c.bond_r0;
    P.bend_k = c.bend_k;
    const float s6 = powf(c.lj_sigma, 6.0f);
    P.lj_amp = 24.0f * c.lj_epsilon * s6;
    P.lj_two_s6 = 2.0f * s6;
    P.lj_rc2 = c.lj_rcut * c.lj_rcut;
    P.lj_exclude = c.lj_exclude;
    P.spring = c.spring;
    P.damping = c.damping;
    P.shear = c.shear;
    P.bdamp = c.boundary_damping;
    P.activity = c.activity;
    P.reverse_p = c.reverse_probability;
    P.reverse_on = c.reverse_probability > 0.0f;
    P.gamma = c.gamma;
    float s2 = 2.0f * c.gamma * c.kT;
    if (c.noise_dt_scaling) s2 = s2 / dt;
    P.noise_sigma = sqrtf(s2);
    P.langevin_on = (!c.srd_enabled || c.langevin_with_srd) ? 1 : 0;
    P.srd_on = c.srd_enabled;
    P.srd_alpha = c.srd_alpha;
    P.srd_sin_a = (float)std::sin((double)c.srd_alpha);
    P.srd_cos_a = (float)std::cos((double)c.srd_alpha);
    P.srd_kT = c.srd_kT;
    P.srd_shift_lo = c.srd_shift_lo;
    P.srd_rotate_beads = c.srd_rotate_beads;
    P.srd_thermo = c.srd_thermostat;
    P.seed_lo = (uint32_t)c.seed;
    P.seed_hi = (uint32_t)(c.seed >> 32);
    fast_div_params(P.grid[0] ? P.grid[0] : 1u, P.div_gx_m, P.div_gx_k);
    fast_div_params(P.grid[0] * P.grid[1] ? P.grid[0] * P.grid[1] : 1u, P.div_gxy_m, P.div_gxy_k);
    // per-step bead lists: the reference grid, or the Verlet list grid
    P.vl_on = effective_strategy(c) == NW_STRATEGY_VERLET && c.model == NW_MODEL_WCA_WORMS;
    const float skin = c.neighbor_skin > 0.0f ? c.neighbor_skin : 0.3f * c.lj_sigma;
    const float rl = c.lj_rcut + skin;
    P.vl_r2 = rl * rl;
    P.vl_half_skin = 0.5f * skin;
    P.vl_cap = c.neighbor_capacity ? c.neighbor_capacity : 32u;
    P.lncells = 1;
    for (int a = 0; a < 3; ++a) {
        if (P.vl_on) {
            // cells a little wider than the list radius, tiling the box exactly
            uint32_t G = 1;
            if (c.grid[a] > 1u) {
                const float g = std::floor(c.box[a] / (rl * 1.0001f));
                G = g >= 1.0f ? (uint32_t)g : 1u;
            }
            P.lgrid[a] = G;
            P.linv[a] = (float)G / c.box[a];
        } else {
            P.lgrid[a] = P.grid[a];
            P.linv[a] = P.inv_cell[a];
        }
        P.lncells *= P.lgrid[a];
    }
    fast_div_params(P.lgrid[0], P.ldiv_x_m, P.ldiv_x_k);
    fast_div_params(P.lgrid[0] * P.lgrid[1], P.ldiv_xy_m, P.ldiv_xy_k);
    return P;
}

static uint32_t cdiv(uint64_t a, uint32_t b) { return (uint32_t)((a + b - 1) / b); }

void Prof::mark(const char* name)
{
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, stream);
    events.push_back(e);
    names.emplace_back(name);
}

void Prof::end()
{
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, stream);
    events.push_back(e);
    names.emplace_back("");
}

void Prof::clear()
{
    for (auto e : events) cudaEventDestroy(e);
    events.clear();
    names.clear();
}

#define NW_MARK(name) \
    if (prof) prof->mark(name)

uint64_t enqueue_bead_step(const DevParams& P, const StepBuffers& B, uint32_t nchunks, uint32_t step_off, float dt,
                           cudaStream_t s, Prof* prof)
{
    if (P.nb == 0) return 0;
    const uint32_t fpb = list_filaments_per_block(P.L, P.nf);
    const uint32_t beads = fpb * P.L;
    const uint32_t threads = (beads + 31u) & ~31u;
    const size_t smem = (size_t)beads * sizeof(float4) * (P.reverse_on ? 3u : 1u);
    NW_MARK("filament_pass");
    filament_pass_kernel<<<cdiv(P.nf, fpb), threads, smem, s>>>(P, B, step_off, dt, fpb);
    NW_MARK("chunk_sum");
    chunk_sum_kernel<<<nchunks, 512, 0, s>>>(B.cell_count, P.ncells, B.chunk_count, nullptr, nullptr);
    NW_MARK("scan_cells");
    scan_cells_kernel<true><<<nchunks, 512, 0, s>>>(B.cell_count, B.chunk_count, P.ncells, B.cell_offset, B.cell_start,
                                                    B.cell_end, nullptr, nullptr, nullptr);
    NW_MARK("scatter");
    scatter_kernel<<<cdiv(P.nb, 256), 256, 0, s>>>(B.hash, B.slot, B.cell_offset, B.tmp_index, P.nb);
    if (P.model == NW_MODEL_REF_DEM) {
        NW_MARK("stable_gather");
        stable_gather_kernel<true><<<cdiv(P.nb, 256), 256, 0, s>>>(P, B);
        NW_MARK("pair_ref");
        if (P.grid[2] == 1u) {
            const uint32_t tiles = cdiv(P.grid[0], kRefTX) * cdiv(P.grid[1], kRefTY);
            pair_ref_tiled_kernel<<<tiles, kRefThreads, kRefSmem, s>>>(P, B);
        } else {
            pair_ref_kernel<<<cdiv(P.nb, 256), 256, 0, s>>>(P, B);
        }
    } else {
        NW_MARK("stable_gather");
        stable_gather_kernel<false><<<cdiv(P.nb, 256), 256, 0, s>>>(P, B);
        NW_MARK("pair_wca");
        pair_wca_kernel<<<cdiv(P.nb, 256), 256, 0, s>>>(P, B);
    }
    return 6;
}

uint64_t enqueue_srd(const DevParams& P, const StepBuffers& B, uint32_t srd_nchunks, uint32_t step_off, float dt_srd,
                     int shift_from_step, float3 shift, cudaStream_t s, Prof* prof, uint32_t buf_sel)
{
    if (P.ntotal == 0) return 0;
    NW_MARK("srd_hash");
    srd_hash_kernel<<<cdiv(P.ntotal, 256), 256, 0, s>>>(P, B, step_off, shift_from_step, shift, buf_sel);
    NW_MARK("srd_chunk_sum");
    // bead and solvent counts side by side (grid rows 0 and 1)
    chunk_sum_kernel<<<dim3(srd_nchunks, 2), 512, 0, s>>>(B.srd_bcount, P.srd_ncells, B.srd_bchunk, B.srd_scount,
                                                          B.srd_schunk);
    NW_MARK("srd_scan_cells");
    scan_cells_kernel<false><<<dim3(srd_nchunks, 2), 512, 0, s>>>(B.srd_bcount, B.srd_bchunk, P.srd_ncells,
                                                                  B.srd_boff, nullptr, nullptr, B.srd_scount,
                                                                  B.srd_schunk, B.srd_soff);
    NW_MARK("srd_scatter");
    srd_scatter_kernel<<<cdiv(P.ntotal, 256), 256, 0, s>>>(P, B);
    NW_MARK("srd_collide");
    srd_collide_kernel<<<cdiv(P.srd_ncells, 128), 128, 0, s>>>(P, B, step_off, dt_srd, buf_sel);
    NW_MARK("srd_collide_big");
    srd_collide_big_kernel<<<kSrdBigBlocks, kBigWarps * 32, 0, s>>>(P, B, step_off, dt_srd, buf_sel);
    srd_flip_kernel<<<1, 1, 0, s>>>(B.scur);
    return 7;
}

// Histogram of bead hashes (the counting sort's first pass, for the sorted
// order and cell bounds read from a cell-list system).
__global__ void __launch_bounds__(256) count_hash_kernel(const uint32_t* __restrict__ hash, uint32_t n,
                                                         uint32_t* __restrict__ count, uint32_t* __restrict__ slot)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) slot[i] = count_into_cell(count, hash[i]);
}

// Reference-grid cell hash of every bead (systems whose per-step lists live
// on the Verlet grid compute it only when it is read).
__global__ void __launch_bounds__(256) ref_hash_kernel(const DevParams P, const float4* __restrict__ pos,
                                                       uint32_t* __restrict__ hash)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < P.nb) hash[i] = bead_hash(P, f3(pos[i]));
}

// Positions set between updates of a Verlet system: staged in the free
// position buffer, moved into the current one while the largest squared
// displacement is taken (non-negative floats order as their bits); the
// displacement is then added to the lists' bound, so unchanged or slightly
// moved beads keep their lists and larger moves rebuild them.
__global__ void __launch_bounds__(256) set_positions_kernel(const float4* __restrict__ src, float4* __restrict__ dst,
                                                            uint32_t n, uint32_t* __restrict__ dmax)
{
    uint32_t m = 0u;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 a = src[i], b = dst[i];
        const float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
        const float d2 = dx * dx + dy * dy + dz * dz;
        const uint32_t bits = d2 == d2 ? __float_as_uint(d2) : 0x7f800000u;  // NaN counts as unbounded
        m = bits > m ? bits : m;
        dst[i] = a;
    }
    __shared__ uint32_t s_m[8];
    m = __reduce_max_sync(0xffffffffu, m);
    if ((threadIdx.x & 31u) == 0u) s_m[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {  // one atomic per block on the shared word
        for (uint32_t q = 1; q < (blockDim.x >> 5); ++q) m = s_m[q] > m ? s_m[q] : m;
        if (m) atomicMax(dmax, m);
    }
}

__global__ void vl_add_displacement_kernel(uint32_t* __restrict__ vstate, uint32_t slot)
{
    const float d = sqrtf(__uint_as_float(vstate[5]));
    vstate[slot] = __float_as_uint(__uint_as_float(vstate[slot]) + d);
    vstate[5] = 0u;
}

}  // namespace nw

using namespace nw;

namespace {

nw_status alloc(nw_system* s, void** p, size_t bytes)
{
    *p = nullptr;
    if (bytes == 0) bytes = 16;
    if (cudaMalloc(p, bytes) != cudaSuccess) {
        cudaGetLastError();
        return NW_ERR_NOMEM;
    }
    s->allocs.push_back(*p);
    return NW_OK;
}

template <class T>
nw_status alloc_n(nw_system* s, T** p, size_t n)
{
    return alloc(s, reinterpret_cast<void**>(p), n * sizeof(T));
}

void free_all(nw_system* s)
{
    for (auto& g : s->graphs) cudaGraphExecDestroy(g.exec);
    s->graphs.clear();
    for (void* p : s->allocs) cudaFree(p);
    s->allocs.clear();
    cudaFree(s->defect_fixed);
    cudaFree(s->defect_acc);
    cudaFreeHost(s->defect_host);
    s->defect_fixed = s->defect_acc = nullptr;
    s->defect_host = nullptr;
    s->defect_acc_bytes = 0;
    cudaFree(s->obs_ws);
    cudaFree(s->obs_msd);
    cudaFree(s->obs_srd);
    s->obs_ws = s->obs_msd = s->obs_srd = nullptr;
    s->obs_ws_bytes = s->obs_msd_bytes = s->obs_srd_bytes = 0;
    s->obs_msd_on = false;
    if (s->aux) cudaStreamDestroy(s->aux);
    if (s->state_ev) cudaEventDestroy(s->state_ev);
    if (s->aux_done) cudaEventDestroy(s->aux_done);
    s->aux = nullptr;
    s->state_ev = s->aux_done = nullptr;
    s->state_ev_valid = false;
    if (s->own_stream) cudaStreamDestroy(s->own_stream);
    s->own_stream = nullptr;
}

void drop_graphs(nw_system* s)
{
    for (auto& g : s->graphs) cudaGraphExecDestroy(g.exec);
    s->graphs.clear();
    s->version++;
}

nw_status cuda_status(cudaError_t e)
{
    if (e == cudaSuccess) return NW_OK;
    if (e == cudaErrorMemoryAllocation) return NW_ERR_NOMEM;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return NW_ERR_NO_DEVICE;
    std::fprintf(stderr, "[nwgb] CUDA error: %s\n", cudaGetErrorString(e));
    return NW_ERR_CUDA;
}

// Bead buffer holding the state after the last update.
uint32_t cur_buffer(const nw_system* s) { return s->lists ? (uint32_t)((s->step + 1ull) & 1ull) : 0u; }

// Parity of the number of SRD collisions in updates [first, first + nsteps):
// each collision moves the solvent to the other buffer.
uint32_t collision_parity(const nw_system* s, uint64_t first, int nsteps)
{
    if (!s->cfg.srd_enabled || nsteps <= 0) return 0u;
    const uint64_t gap = s->cfg.srd_gap ? s->cfg.srd_gap : 1u;
    const uint64_t last = first + (uint64_t)nsteps - 1ull;
    const uint64_t upto_last = last / gap + 1ull;            // multiples of gap in [0, last]
    const uint64_t before = first ? (first - 1ull) / gap + 1ull : 0ull;  // in [0, first)
    return (uint32_t)((upto_last - before) & 1ull);
}

// Clear the list counters when the step counter changed under them.
cudaError_t clean_lists(nw_system* s)
{
    if (s->vl && s->vl_dirty) {
        // an unbounded displacement forces a list build at the next pair pass;
        // every cell-list count buffer counts as filled (word 6)
        const uint32_t init[8] = {0x7f000000u, 0x7f000000u, 0u, 0u, 0u, 0u, 7u, 0u};
        cudaError_t e = cudaMemcpyAsync(s->B.vstate, init, sizeof(init), cudaMemcpyHostToDevice, s->stream);
        if (e != cudaSuccess) return e;
        s->vl_dirty = false;
    }
    if (!s->lists || !s->lists_dirty) return cudaSuccess;
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 3 && e == cudaSuccess; ++k)
        e = cudaMemsetAsync(s->B.lcount[k], 0, ((size_t)s->lncells + 8) * 4, s->stream);
    if (e == cudaSuccess) s->lists_dirty = false;
    return e;
}

// Enqueue `nsteps` updates starting at device step base + 0 and advance the base.
uint64_t enqueue_steps(nw_system* s, int nsteps, float dt, uint64_t first_step, Prof* prof = nullptr)
{
    const DevParams P = make_dev_params(s->cfg, dt);
    const bool srd = s->cfg.srd_enabled != 0;
    const uint32_t gap = s->cfg.srd_gap ? s->cfg.srd_gap : 1u;
    const float dt_srd = dt * (float)gap;
    uint64_t launches = 0;
    // positions and velocities of the last update are final here (an event
    // node of the graph under capture); single updates only, the round trip of
    // a caller that feeds and reads the state every update (longer calls keep
    // their graphs free of the extra node)
    bool state_marked = nsteps != 1 || prof;
    s->enqueued_state_ev = false;
    auto mark_state = [&]() {
        cudaStreamCaptureStatus cst = cudaStreamCaptureStatusNone;
        const bool ok =
            cudaStreamIsCapturing(s->stream, &cst) == cudaSuccess &&
            cudaEventRecordWithFlags(s->state_ev, s->stream, cst == cudaStreamCaptureStatusActive
                                                                 ? cudaEventRecordExternal
                                                                 : cudaEventRecordDefault) == cudaSuccess;
        if (!ok) cudaGetLastError();  // no early read-back after this call
        s->enqueued_state_ev = ok;
        state_marked = true;
    };
    if (!s->lists) {
        for (int j = 0; j < nsteps; ++j) {
            launches += enqueue_bead_step(P, s->B, s->nchunks, (uint32_t)j, dt, s->stream, prof);
            if (srd && ((first_step + (uint64_t)j) % gap) == 0)
                launches += enqueue_srd(P, s->B, s->srd_nchunks, (uint32_t)j, dt_srd, 1, make_float3(0.f, 0.f, 0.f),
                                        s->stream, prof, 2u);
        }
    } else {
        // WCA pair forces depend on positions only, so a collision (which
        // changes bead velocities) can run between the pro part of update j
        // and its pair pass, keeping the pair/integrate chain fused; REF_DEM
        // pair forces read velocities, so its collision follows the pair pass.
        const bool wca = P.model == NW_MODEL_WCA_WORMS;
        auto list = [&](uint32_t j) {
            if (!P.vl_on) return;
            NW_MARK("bead_list");
            launches += launch_bead_list(P, s->B, j, s->stream);
        };
        auto collide = [&](uint32_t j) {
            launches += enqueue_srd(P, s->B, s->srd_nchunks, j, dt_srd, 1, make_float3(0.f, 0.f, 0.f), s->stream,
                                    prof, 2u);
        };
        NW_MARK("bead_pro");
        launches += launch_bead_pro(P, s->B, 0u, dt, s->stream);
        list(0u);
        for (int j = 0; j < nsteps; ++j) {
            const bool srd_now = srd && ((first_step + (uint64_t)j) % gap) == 0;
            if (srd_now && wca) collide((uint32_t)j);
            if (j == nsteps - 1 || (srd_now && !wca)) {
                // WCA: the last update's pair pass changes forces only
                if (j == nsteps - 1 && wca && !state_marked) mark_state();
                NW_MARK("bead_epi");
                launches += launch_bead_epi(P, s->B, (uint32_t)j, s->stream);
                if (srd_now && !wca) collide((uint32_t)j);
                if (j < nsteps - 1) {
                    NW_MARK("bead_pro");
                    launches += launch_bead_pro(P, s->B, (uint32_t)(j + 1), dt, s->stream);
                    list((uint32_t)(j + 1));
                }
            } else {
                NW_MARK("bead_fused");
                launches += launch_bead_fused(P, s->B, (uint32_t)j, dt, s->stream);
                list((uint32_t)(j + 1));
            }
        }
    }
    if (!state_marked) mark_state();
    if (prof) prof->mark("advance_step");
    advance_step_kernel<<<1, 1, 0, s->stream>>>(s->B.step_base, (unsigned long long)nsteps);
    if (prof) prof->end();
    return launches + 1;
}

// Sorted order and cell bounds of the current bead hashes (cell-list systems
// keep no sorted order between updates; this runs the counting sort once).
// Systems whose step does not store tangents (pro_flags) compute them from
// the current positions when they are read.
bool lazy_tangents(const nw_system* s)
{
    return s->lists && (pro_flags(make_dev_params(s->cfg, s->cfg.dt)) & kProLazyTangent) != 0u;
}

cudaError_t materialize_tangents(nw_system* s)
{
    if (!s->tan_stale) return cudaSuccess;
    const DevParams P = make_dev_params(s->cfg, s->cfg.dt);
    const uint32_t cur = cur_buffer(s);
    launch_bead_tangents(P, s->B.pos2[cur], s->B.tan2[cur], s->stream);
    const cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) s->tan_stale = false;
    return e;
}

cudaError_t ensure_hash(nw_system* s)
{
    if (!s->vl || s->hash_for == s->step || s->nb == 0) return cudaSuccess;
    const DevParams P = make_dev_params(s->cfg, s->cfg.dt);
    const uint32_t cur = cur_buffer(s);
    ref_hash_kernel<<<cdiv(s->nb, 256), 256, 0, s->stream>>>(P, s->B.pos2[cur], s->B.hash2[cur]);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) s->hash_for = s->step;
    return e;
}

cudaError_t ensure_sorted(nw_system* s)
{
    if (!s->lists || s->sorted_for == s->step || s->nb == 0) return cudaSuccess;
    cudaError_t eh = ensure_hash(s);
    if (eh != cudaSuccess) return eh;
    const DevParams P = make_dev_params(s->cfg, s->cfg.dt);
    StepBuffers B = s->B;
    const uint32_t cur = cur_buffer(s);
    B.hash = B.hash2[cur];
    B.pos = B.pos2[cur];
    count_hash_kernel<<<cdiv(s->nb, 256), 256, 0, s->stream>>>(B.hash, s->nb, B.cell_count, B.slot);
    chunk_sum_kernel<<<s->nchunks, 512, 0, s->stream>>>(B.cell_count, P.ncells, B.chunk_count, nullptr, nullptr);
    scan_cells_kernel<true><<<s->nchunks, 512, 0, s->stream>>>(B.cell_count, B.chunk_count, P.ncells, B.cell_offset,
                                                               B.cell_start, B.cell_end, nullptr, nullptr, nullptr);
    scatter_kernel<<<cdiv(s->nb, 256), 256, 0, s->stream>>>(B.hash, B.slot, B.cell_offset, B.tmp_index, s->nb);
    stable_gather_kernel<false><<<cdiv(s->nb, 256), 256, 0, s->stream>>>(P, B);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) s->sorted_for = s->step;
    return e;
}

enum class Dir { ToDevice, ToHost };

// Copy `count` elements of an API array between host and device.  Position /
// velocity arrays are beads [0, nb) then solvent [nb, nb + ns) in two stores.
nw_status transfer(nw_system* s, int array, void* host, uint32_t start, uint32_t count, Dir dir, bool wait = true)
{
    // an asynchronous read of positions or velocities right after a step
    // starts on aux once they are final (state_ev), beside the step's pair
    // pass; the engine's stream then waits for it
    const bool early = dir == Dir::ToHost && !wait && s->state_ev_valid &&
                       (array == NW_POSITION || array == NW_VELOCITY);
    if (dir == Dir::ToDevice) s->state_ev_valid = false;
    cudaStream_t cs = s->stream;
    if (early) {
        if (cudaStreamWaitEvent(s->aux, s->state_ev, 0) != cudaSuccess) return cuda_status(cudaGetLastError());
        cs = s->aux;
    }
    const uint32_t cur = cur_buffer(s);
    const StepBuffers& B = s->B;
    void* bead_ptr = nullptr;
    void* solv_ptr = nullptr;
    size_t elem = 16;
    size_t nbead = s->nb, ntot = s->nb;
    switch (array) {
    case NW_POSITION: bead_ptr = B.pos2[cur]; solv_ptr = B.spos2[s->scur]; ntot = s->ntotal; break;
    case NW_VELOCITY: bead_ptr = B.vel2[cur]; solv_ptr = B.svel2[s->scur]; ntot = s->ntotal; break;
    case NW_TANGENT: {
        cudaError_t e = materialize_tangents(s);  // also before a partial write
        if (e != cudaSuccess) return cuda_status(e);
        bead_ptr = B.tan2[cur];
        break;
    }
    case NW_FORCE: bead_ptr = B.force; break;
    case NW_FORCE_OLD: bead_ptr = B.force_old; break;
    case NW_HASH: {
        if (dir == Dir::ToHost) {
            cudaError_t e = ensure_hash(s);
            if (e != cudaSuccess) return cuda_status(e);
        }
        bead_ptr = B.hash2[cur];
        elem = 4;
        break;
    }
    case NW_SORTED_INDEX:
    case NW_CELL_START:
    case NW_CELL_END: {
        if (dir == Dir::ToDevice) return NW_ERR_INVALID;
        cudaError_t e = ensure_sorted(s);
        if (e != cudaSuccess) return cuda_status(e);
        elem = 4;
        if (array == NW_SORTED_INDEX) bead_ptr = B.sorted_index;
        else {
            bead_ptr = array == NW_CELL_START ? B.cell_start : B.cell_end;
            nbead = ntot = s->ncells;
        }
        break;
    }
    case NW_SRD_SORTED_INDEX: bead_ptr = B.srd_sorted_index; elem = 4; nbead = ntot = s->cfg.srd_enabled ? s->ntotal : 0; break;
    case NW_SRD_CELL_START: bead_ptr = B.srd_start; elem = 4; nbead = ntot = s->cfg.srd_enabled ? s->srd_ncells : 0; break;
    case NW_SRD_CELL_END: bead_ptr = B.srd_end; elem = 4; nbead = ntot = s->cfg.srd_enabled ? s->srd_ncells : 0; break;
    case NW_SRD_CELL_MEAN: bead_ptr = B.srd_mean; nbead = ntot = s->cfg.srd_enabled ? s->srd_ncells : 0; break;
    default: return NW_ERR_INVALID;
    }
    if ((uint64_t)start + count > ntot) return NW_ERR_INVALID;
    if (!count) return NW_OK;
    if (dir == Dir::ToDevice && (array == NW_HASH || array >= NW_SRD_SORTED_INDEX)) return NW_ERR_INVALID;
    cudaError_t e = cudaSuccess;
    char* h = static_cast<char*>(host);
    const uint64_t end = (uint64_t)start + count;
    // bead part; positions of a Verlet system with valid lists go through the
    // free buffer so that the lists' displacement bound takes the move
    bool moved_through_stage = false;
    if (start < nbead && dir == Dir::ToDevice && array == NW_POSITION && s->vl && !s->vl_dirty &&
        B.pos2[0] != B.pos2[1]) {
        const uint64_t a = start, b = end < nbead ? end : nbead;
        float4* stage = B.pos2[cur ^ 1u] + a;
        e = cudaMemcpyAsync(stage, h, (b - a) * elem, cudaMemcpyHostToDevice, s->stream);
        if (e == cudaSuccess) {
            const uint32_t n = (uint32_t)(b - a);
            const uint32_t blocks = std::min<uint32_t>((n + 255u) / 256u, 4u * 152u);
            set_positions_kernel<<<blocks, 256, 0, s->stream>>>(stage, B.pos2[cur] + a, n, B.vstate + 5);
            vl_add_displacement_kernel<<<1, 1, 0, s->stream>>>(B.vstate, (uint32_t)((s->step + 1ull) & 1ull));
            e = cudaGetLastError();
        }
        h += (b - a) * elem;
        moved_through_stage = true;
    } else if (start < nbead) {
        const uint64_t a = start, b = end < nbead ? end : nbead;
        char* d = static_cast<char*>(bead_ptr) + a * elem;
        e = dir == Dir::ToDevice ? cudaMemcpyAsync(d, h, (b - a) * elem, cudaMemcpyHostToDevice, s->stream)
                                 : cudaMemcpyAsync(h, d, (b - a) * elem, cudaMemcpyDeviceToHost, cs);
        h += (b - a) * elem;
    }
    // solvent part
    if (e == cudaSuccess && end > nbead) {
        const uint64_t a = start > nbead ? start : nbead, b = end;
        char* d = static_cast<char*>(solv_ptr) + (a - nbead) * elem;
        e = dir == Dir::ToDevice ? cudaMemcpyAsync(d, h, (b - a) * elem, cudaMemcpyHostToDevice, s->stream)
                                 : cudaMemcpyAsync(h, d, (b - a) * elem, cudaMemcpyDeviceToHost, cs);
    }
    if (e == cudaSuccess && early) {
        e = cudaEventRecord(s->aux_done, s->aux);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s->stream, s->aux_done, 0);
    }
    if (e == cudaSuccess && wait) e = cudaStreamSynchronize(s->stream);
    if (dir == Dir::ToDevice) {
        s->sorted_for = ~0ull;
        s->hash_for = ~0ull;
        if (array == NW_POSITION && !moved_through_stage) s->vl_dirty = true;
    }
    return cuda_status(e);
}

}  // namespace

extern "C" {

nw_status nw_create(const NwConfig* cfg, nw_system** out)
{
    if (!out) return NW_ERR_INVALID;
    *out = nullptr;
    nw_status st = nw_config_validate(cfg);
    if (st != NW_OK) return st;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return NW_ERR_NO_DEVICE;
    }
    nw_system* s = new nw_system();
    s->cfg = *cfg;
    cudaGetDevice(&s->device);
    if (cudaStreamCreateWithFlags(&s->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete s;
        return NW_ERR_CUDA;
    }
    s->stream = s->own_stream;
    // the cell-tiled REF_DEM pair pass stages more than the default 48 KB
    if (cudaFuncSetAttribute(pair_ref_tiled_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRefSmem) !=
        cudaSuccess) {
        cudaGetLastError();
        cudaStreamDestroy(s->own_stream);
        delete s;
        return NW_ERR_CUDA;
    }
    s->lists = effective_strategy(*cfg) != NW_STRATEGY_SORTED;
    const DevParams P0 = make_dev_params(*cfg, cfg->dt);
    s->vl = P0.vl_on != 0;
    if (P0.lncells >= (1u << 30)) {
        cudaStreamDestroy(s->own_stream);
        delete s;
        return NW_ERR_INVALID;
    }
    s->nb = cfg->num_filaments * cfg->filament_size;
    s->ns = cfg->srd_enabled ? cfg->num_solvent : 0u;
    s->ntotal = s->nb + s->ns;
    s->ncells = cfg->grid[0] * cfg->grid[1] * cfg->grid[2];
    s->lncells = P0.lncells > s->ncells ? P0.lncells : s->ncells;
    s->nchunks = (s->ncells + kChunk - 1) / kChunk;
    s->srd_ncells = cfg->srd_enabled ? cfg->srd_grid[0] * cfg->srd_grid[1] * cfg->srd_grid[2] : 0u;
    s->srd_nchunks = (s->srd_ncells + kChunk - 1) / kChunk;
    if (cudaStreamCreateWithFlags(&s->aux, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->state_ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->aux_done, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        if (s->aux) cudaStreamDestroy(s->aux);
        if (s->state_ev) cudaEventDestroy(s->state_ev);
        cudaStreamDestroy(s->own_stream);
        delete s;
        return NW_ERR_CUDA;
    }
    StepBuffers& B = s->B;
    std::memset(&B, 0, sizeof(B));
    const size_t nb = s->nb, ns = s->ns, C = s->ncells;
    const bool ref = cfg->model == NW_MODEL_REF_DEM;
    B.cap = cfg->cell_capacity ? cfg->cell_capacity : (ref ? 16u : 8u);
    st = NW_OK;
    auto A = [&](nw_status x) {
        if (st == NW_OK) st = x;
    };
    const int nbuf = s->lists ? 2 : 1;
    for (int k = 0; k < nbuf; ++k) {
        A(alloc_n(s, &B.pos2[k], nb));
        A(alloc_n(s, &B.vel2[k], nb));
        A(alloc_n(s, &B.tan2[k], nb));
        A(alloc_n(s, &B.hash2[k], nb));
    }
    if (!s->lists) {
        B.pos2[1] = B.pos2[0];
        B.vel2[1] = B.vel2[0];
        B.tan2[1] = B.tan2[0];
        B.hash2[1] = B.hash2[0];
    }
    B.pos = B.pos2[0];
    B.vel = B.vel2[0];
    B.tangent = B.tan2[0];
    B.hash = B.hash2[0];
    A(alloc_n(s, &B.force, nb));
    A(alloc_n(s, &B.force_old, nb));
    for (int k = 0; k < 2; ++k) {
        A(alloc_n(s, &B.spos2[k], ns));
        A(alloc_n(s, &B.svel2[k], ns));
    }
    A(alloc_n(s, &B.scur, 4));
    A(alloc_n(s, &B.slot, nb));
    A(alloc_n(s, &B.tmp_index, nb));
    A(alloc_n(s, &B.sorted_index, nb));
    A(alloc_n(s, &B.sorted_hash, nb));
    A(alloc_n(s, &B.cell_count, C + 8));
    A(alloc_n(s, &B.cell_offset, C + 8));
    A(alloc_n(s, &B.cell_start, C + 8));
    A(alloc_n(s, &B.cell_end, C + 8));
    A(alloc_n(s, &B.chunk_count, (size_t)s->nchunks + 1));
    A(alloc_n(s, &B.sorted_pos, nb));
    if (ref && !s->lists) {
        A(alloc_n(s, &B.sorted_vel, nb));
        A(alloc_n(s, &B.sorted_tan, nb));
    }
    if (s->lists) {
        const size_t LC = P0.lncells > C ? P0.lncells : C;
        for (int k = 0; k < 3; ++k) A(alloc_n(s, &B.lcount[k], LC + 8));
        for (int k = 0; k < 2; ++k) A(alloc_n(s, &B.lslot[k], LC * B.cap + 8));
    }
    if (s->vl) {
        A(alloc_n(s, &B.nbr, (size_t)P0.vl_cap * nb + 8));
        A(alloc_n(s, &B.nnb, nb + 8));
        A(alloc_n(s, &B.vstate, 8));
    }
    if (cfg->srd_enabled) {
        const size_t Cs = s->srd_ncells, nt = s->ntotal;
        A(alloc_n(s, &B.srd_hash, nt));
        A(alloc_n(s, &B.srd_slot, nt));
        A(alloc_n(s, &B.srd_btmp, nb));
        A(alloc_n(s, &B.srd_stmp, ns));
        A(alloc_n(s, &B.srd_sorted_index, nt));
        A(alloc_n(s, &B.srd_bcount, Cs + 8));
        A(alloc_n(s, &B.srd_scount, Cs + 8));
        A(alloc_n(s, &B.srd_boff, Cs + 8));
        A(alloc_n(s, &B.srd_soff, Cs + 8));
        A(alloc_n(s, &B.srd_start, Cs + 8));
        A(alloc_n(s, &B.srd_end, Cs + 8));
        A(alloc_n(s, &B.srd_bchunk, (size_t)s->srd_nchunks + 1));
        A(alloc_n(s, &B.srd_schunk, (size_t)s->srd_nchunks + 1));
        A(alloc_n(s, &B.srd_mean, Cs));
        A(alloc_n(s, &B.srd_big, Cs + 8));
        A(alloc_n(s, &B.srd_nbig, 4));
    }
    A(alloc_n(s, &B.err, 4));
    A(alloc_n(s, &B.step_base, 1));
    if (st != NW_OK) {
        free_all(s);
        delete s;
        return st;
    }
    // counters must start at zero; state starts empty
    cudaError_t e = cudaSuccess;
    auto Z = [&](void* p, size_t bytes, int v = 0) {
        if (p && e == cudaSuccess) e = cudaMemsetAsync(p, v, bytes, s->stream);
    };
    for (int k = 0; k < nbuf; ++k) {
        Z(B.pos2[k], nb * 16);
        Z(B.vel2[k], nb * 16);
        Z(B.tan2[k], nb * 16);
        Z(B.hash2[k], nb * 4);
    }
    Z(B.force, nb * 16);
    Z(B.force_old, nb * 16);
    for (int k = 0; k < 2; ++k) {
        Z(B.spos2[k], ns * 16);
        Z(B.svel2[k], ns * 16);
    }
    Z(B.scur, 4);
    Z(B.cell_count, (C + 8) * 4);
    Z(B.chunk_count, ((size_t)s->nchunks + 1) * 4);
    Z(B.cell_start, (C + 8) * 4, 0xff);
    Z(B.cell_end, (C + 8) * 4, 0xff);
    if (s->lists)
        for (int k = 0; k < 3; ++k) Z(B.lcount[k], ((size_t)s->lncells + 8) * 4);
    if (cfg->srd_enabled) {
        Z(B.srd_bcount, ((size_t)s->srd_ncells + 8) * 4);
        Z(B.srd_scount, ((size_t)s->srd_ncells + 8) * 4);
        Z(B.srd_mean, (size_t)s->srd_ncells * 16);
    }
    Z(B.err, 16);
    Z(B.step_base, 8);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) {
        st = cuda_status(e);
        free_all(s);
        delete s;
        return st;
    }
    *out = s;
    return NW_OK;
}

nw_status nw_destroy(nw_system* s)
{
    if (!s) return NW_ERR_INVALID;
    if (s->stream) cudaStreamSynchronize(s->stream);
    free_all(s);
    delete s;
    return NW_OK;
}

nw_status nw_set_config(nw_system* s, const NwConfig* cfg)
{
    if (!s || !cfg) return NW_ERR_INVALID;
    nw_status st = nw_config_validate(cfg);
    if (st != NW_OK) return st;
    const NwConfig& o = s->cfg;
    if (cfg->model != o.model || cfg->num_filaments != o.num_filaments || cfg->filament_size != o.filament_size ||
        cfg->srd_enabled != o.srd_enabled || (cfg->srd_enabled && cfg->num_solvent != o.num_solvent) ||
        cfg->strategy != o.strategy || cfg->cell_capacity != o.cell_capacity)
        return NW_ERR_INVALID;
    for (int a = 0; a < 3; ++a)
        if (cfg->grid[a] != o.grid[a] || (cfg->srd_enabled && cfg->srd_grid[a] != o.srd_grid[a]))
            return NW_ERR_INVALID;
    // the list buffers were sized for the old list grid and list capacity
    const DevParams Pn = make_dev_params(*cfg, cfg->dt), Po = make_dev_params(o, o.dt);
    if (Pn.vl_on != Po.vl_on || Pn.lncells != Po.lncells || (Pn.vl_on && Pn.vl_cap != Po.vl_cap))
        return NW_ERR_INVALID;
    for (int a = 0; a < 3; ++a)
        if (Pn.lgrid[a] != Po.lgrid[a]) return NW_ERR_INVALID;
    s->cfg = *cfg;
    s->state_ev_valid = false;
    s->vl_dirty = true;  // radii or the box may have changed
    s->hash_for = ~0ull;
    s->sorted_for = ~0ull;
    drop_graphs(s);
    return NW_OK;
}

nw_status nw_get_config(const nw_system* s, NwConfig* cfg)
{
    if (!s || !cfg) return NW_ERR_INVALID;
    *cfg = s->cfg;
    return NW_OK;
}

nw_status nw_get_counts(const nw_system* s, uint32_t* nb, uint32_t* ns, uint32_t* nc, uint32_t* nsc)
{
    if (!s) return NW_ERR_INVALID;
    if (nb) *nb = s->nb;
    if (ns) *ns = s->ns;
    if (nc) *nc = s->ncells;
    if (nsc) *nsc = s->srd_ncells;
    return NW_OK;
}

nw_status nw_set_array(nw_system* s, int array, const void* host, uint32_t start, uint32_t count)
{
    if (!s || (!host && count)) return NW_ERR_INVALID;
    return transfer(s, array, const_cast<void*>(host), start, count, Dir::ToDevice);
}

nw_status nw_get_array(nw_system* s, int array, void* host, uint32_t start, uint32_t count)
{
    if (!s || (!host && count)) return NW_ERR_INVALID;
    return transfer(s, array, host, start, count, Dir::ToHost);
}

nw_status nw_set_array_async(nw_system* s, int array, const void* host, uint32_t start, uint32_t count)
{
    if (!s || (!host && count)) return NW_ERR_INVALID;
    return transfer(s, array, const_cast<void*>(host), start, count, Dir::ToDevice, false);
}

nw_status nw_get_array_async(nw_system* s, int array, void* host, uint32_t start, uint32_t count)
{
    if (!s || (!host && count)) return NW_ERR_INVALID;
    return transfer(s, array, host, start, count, Dir::ToHost, false);
}

nw_status nw_device_array(nw_system* s, int array, void** dptr)
{
    if (!s || !dptr) return NW_ERR_INVALID;
    s->state_ev_valid = false;  // the caller may write through the pointer
    const uint32_t cur = cur_buffer(s);
    const StepBuffers& B = s->B;
    void* p = nullptr;
    switch (array) {
    case NW_POSITION:
        p = B.pos2[cur];
        s->vl_dirty = true;  // the caller may move beads through the pointer
        s->hash_for = ~0ull;
        s->sorted_for = ~0ull;
        break;
    case NW_VELOCITY: p = B.vel2[cur]; break;
    case NW_TANGENT: {
        cudaError_t e = materialize_tangents(s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess) return cuda_status(e);
        p = B.tan2[cur];
        break;
    }
    case NW_FORCE: p = B.force; break;
    case NW_FORCE_OLD: p = B.force_old; break;
    case NW_HASH: {
        cudaError_t e = ensure_hash(s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess) return cuda_status(e);
        p = B.hash2[cur];
        break;
    }
    case NW_SORTED_INDEX:
    case NW_CELL_START:
    case NW_CELL_END: {
        cudaError_t e = ensure_sorted(s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess) return cuda_status(e);
        p = array == NW_SORTED_INDEX ? (void*)B.sorted_index : array == NW_CELL_START ? (void*)B.cell_start
                                                                                      : (void*)B.cell_end;
        break;
    }
    case NW_SRD_SORTED_INDEX: p = B.srd_sorted_index; break;
    case NW_SRD_CELL_START: p = B.srd_start; break;
    case NW_SRD_CELL_END: p = B.srd_end; break;
    case NW_SRD_CELL_MEAN: p = B.srd_mean; break;
    default: return NW_ERR_INVALID;
    }
    if (!p) return NW_ERR_INVALID;
    *dptr = p;
    return NW_OK;
}

nw_status nw_zero_forces(nw_system* s)
{
    if (!s) return NW_ERR_INVALID;
    cudaError_t e = cudaMemsetAsync(s->B.force, 0, (size_t)s->nb * 16, s->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->B.force_old, 0, (size_t)s->nb * 16, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    return cuda_status(e);
}

// The cached graph of nsteps updates from an update index of the given SRD
// phase, captured on first use.  A graph depends on the host state only
// through the phase (which updates collide); buffers are picked on the device
// from the step counter.
static cudaError_t find_graph(nw_system* s, int nsteps, float dt, uint64_t first_step, GraphEntry** out)
{
    const uint32_t phase = s->cfg.srd_enabled ? (uint32_t)(first_step % s->cfg.srd_gap) : 0u;
    uint32_t bits;
    std::memcpy(&bits, &dt, 4);
    for (auto& g : s->graphs)
        if (g.nsteps == nsteps && g.dt_bits == bits && g.phase == phase && g.version == s->version) {
            *out = &g;
            return cudaSuccess;
        }
    if (s->graphs.size() >= 24) drop_graphs(s);  // single steps take one graph per collision phase
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    uint64_t launches = enqueue_steps(s, nsteps, dt, first_step);
    e = cudaStreamEndCapture(s->stream, &graph);
    if (e != cudaSuccess) return e;
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return e;
    s->graphs.push_back({nsteps, bits, phase, s->version, exec, launches, s->enqueued_state_ev});
    *out = &s->graphs.back();
    return cudaSuccess;
}

nw_status nw_step_prepare(nw_system* s, int nsteps, float dt, uint64_t first_step)
{
    if (!s || nsteps < 0) return NW_ERR_INVALID;
    if (nsteps == 0 || !s->use_graphs) return NW_OK;
    if (!(dt > 0.0f)) dt = s->cfg.dt;
    if (!std::isfinite(dt)) return NW_ERR_INVALID;
    GraphEntry* g = nullptr;
    return cuda_status(find_graph(s, nsteps, dt, first_step, &g));
}

nw_status nw_step(nw_system* s, int nsteps, float dt)
{
    if (!s || nsteps < 0) return NW_ERR_INVALID;
    if (nsteps == 0) return NW_OK;
    if (!(dt > 0.0f)) dt = s->cfg.dt;
    if (!std::isfinite(dt)) return NW_ERR_INVALID;
    cudaError_t e = clean_lists(s);
    if (e != cudaSuccess) return cuda_status(e);
    if (s->use_graphs) {
        GraphEntry* hit = nullptr;
        e = find_graph(s, nsteps, dt, s->step, &hit);
        if (e != cudaSuccess) return cuda_status(e);
        e = cudaGraphLaunch(hit->exec, s->stream);
        s->last_launches = hit->launches;
        s->state_ev_valid = hit->state_ev;
    } else {
        s->last_launches = enqueue_steps(s, nsteps, dt, s->step);
        s->state_ev_valid = s->enqueued_state_ev;
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        s->state_ev_valid = false;
        return cuda_status(e);
    }
    s->scur ^= collision_parity(s, s->step, nsteps);
    s->step += (uint64_t)nsteps;
    if (lazy_tangents(s)) s->tan_stale = true;
    return NW_OK;
}

nw_status nw_error_word(nw_system* s, uint32_t* flags)
{
    if (!s) return NW_ERR_INVALID;
    uint32_t f = 0;
    cudaError_t e = cudaMemcpyAsync(&f, s->B.err, 4, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->B.err, 0, 4, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (flags) *flags = f;
    return cuda_status(e);
}

nw_status nw_sync(nw_system* s)
{
    if (!s) return NW_ERR_INVALID;
    uint32_t f = 0;
    nw_status st = nw_error_word(s, &f);
    if (st != NW_OK) return st;
    if (f & NW_EFLAG_NONFINITE) return NW_ERR_NONFINITE;
    if (f & (NW_EFLAG_CELL_OVERFLOW | NW_EFLAG_NEIGHBOR_OVERFLOW)) return NW_ERR_CELL_OVERFLOW;
    if (f & NW_EFLAG_TIMEOUT) return NW_ERR_TIMEOUT;
    if (f & NW_EFLAG_BAD_INDEX) return NW_ERR_INVALID;
    return NW_OK;
}

nw_status nw_get_step(const nw_system* s, uint64_t* step)
{
    if (!s || !step) return NW_ERR_INVALID;
    *step = s->step;
    return NW_OK;
}

nw_status nw_set_step(nw_system* s, uint64_t step)
{
    if (!s) return NW_ERR_INVALID;
    if (s->lists && ((step ^ s->step) & 1ull)) {
        // keep the state in the buffer the new step count names as current
        const uint32_t from = cur_buffer(s), to = from ^ 1u;
        const size_t nb = s->nb;
        cudaError_t e = cudaMemcpyAsync(s->B.pos2[to], s->B.pos2[from], nb * 16, cudaMemcpyDeviceToDevice, s->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(s->B.vel2[to], s->B.vel2[from], nb * 16, cudaMemcpyDeviceToDevice, s->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(s->B.tan2[to], s->B.tan2[from], nb * 16, cudaMemcpyDeviceToDevice, s->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(s->B.hash2[to], s->B.hash2[from], nb * 4, cudaMemcpyDeviceToDevice, s->stream);
        if (e != cudaSuccess) return cuda_status(e);
    }
    unsigned long long v = step;
    cudaError_t e = cudaMemcpyAsync(s->B.step_base, &v, 8, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess) {
        s->step = step;
        s->state_ev_valid = false;
        s->lists_dirty = true;
        s->vl_dirty = true;
        s->sorted_for = ~0ull;
        s->hash_for = ~0ull;
    }
    return cuda_status(e);
}

nw_status nw_set_stream(nw_system* s, void* stream)
{
    if (!s) return NW_ERR_INVALID;
    cudaStreamSynchronize(s->stream);
    s->stream = stream ? (cudaStream_t)stream : s->own_stream;
    drop_graphs(s);
    return NW_OK;
}

nw_status nw_set_graphs(nw_system* s, int enabled)
{
    if (!s) return NW_ERR_INVALID;
    s->use_graphs = enabled != 0;
    return NW_OK;
}

nw_status nw_srd_collide(nw_system* s, float dt_srd, const float shift[3])
{
    if (!s || !shift) return NW_ERR_INVALID;
    if (!s->cfg.srd_enabled) return NW_ERR_UNSUPPORTED;
    const DevParams P = make_dev_params(s->cfg, s->cfg.dt);
    s->last_launches = enqueue_srd(P, s->B, s->srd_nchunks, 0u, dt_srd, 0, make_float3(shift[0], shift[1], shift[2]),
                                   s->stream, nullptr, cur_buffer(s));
    s->scur ^= 1u;
    s->state_ev_valid = false;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    return cuda_status(e);
}

// ---- checkpoints ---------------------------------------------------------------

struct CkptHeader {
    char magic[8];
    uint32_t version, cfg_bytes, nb, ntotal;
    uint64_t step;
};

nw_status nw_checkpoint_size(const nw_system* s, size_t* bytes)
{
    if (!s || !bytes) return NW_ERR_INVALID;
    *bytes = sizeof(CkptHeader) + sizeof(NwConfig) + (size_t)s->ntotal * 32 + (size_t)s->nb * 48;
    return NW_OK;
}

nw_status nw_checkpoint_save(nw_system* s, void* buf, size_t bytes)
{
    size_t need = 0;
    if (nw_checkpoint_size(s, &need) != NW_OK || !buf || bytes < need) return NW_ERR_INVALID;
    char* p = (char*)buf;
    CkptHeader h;
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, "NWGBCKP", 8);
    h.version = 2;
    h.cfg_bytes = sizeof(NwConfig);
    h.nb = s->nb;
    h.ntotal = s->ntotal;
    h.step = s->step;
    std::memcpy(p, &h, sizeof(h));
    p += sizeof(h);
    std::memcpy(p, &s->cfg, sizeof(NwConfig));
    p += sizeof(NwConfig);
    const int arrays[] = {NW_POSITION, NW_VELOCITY, NW_FORCE, NW_FORCE_OLD, NW_TANGENT};
    for (int a : arrays) {
        const uint32_t n = (a == NW_POSITION || a == NW_VELOCITY) ? s->ntotal : s->nb;
        nw_status st = transfer(s, a, p, 0, n, Dir::ToHost);
        if (st != NW_OK) return st;
        p += (size_t)n * 16;
    }
    return NW_OK;
}

nw_status nw_checkpoint_load(nw_system* s, const void* buf, size_t bytes)
{
    size_t need = 0;
    if (nw_checkpoint_size(s, &need) != NW_OK || !buf || bytes < need) return NW_ERR_INVALID;
    const char* p = (const char*)buf;
    CkptHeader h;
    std::memcpy(&h, p, sizeof(h));
    if (std::memcmp(h.magic, "NWGBCKP", 8) != 0 || h.version != 2 || h.cfg_bytes != sizeof(NwConfig) ||
        h.nb != s->nb || h.ntotal != s->ntotal)
        return NW_ERR_INVALID;
    p += sizeof(h);
    NwConfig cfg;
    std::memcpy(&cfg, p, sizeof(cfg));
    p += sizeof(NwConfig);
    nw_status st = nw_set_config(s, &cfg);
    if (st != NW_OK) return st;
    st = nw_set_step(s, h.step);
    if (st != NW_OK) return st;
    const int arrays[] = {NW_POSITION, NW_VELOCITY, NW_FORCE, NW_FORCE_OLD, NW_TANGENT};
    for (int a : arrays) {
        const uint32_t n = (a == NW_POSITION || a == NW_VELOCITY) ? s->ntotal : s->nb;
        st = transfer(s, a, const_cast<char*>(p), 0, n, Dir::ToDevice);
        if (st != NW_OK) return st;
        p += (size_t)n * 16;
    }
    return NW_OK;
}

nw_status nw_last_launch_count(const nw_system* s, uint64_t* launches)
{
    if (!s || !launches) return NW_ERR_INVALID;
    *launches = s->last_launches;
    return NW_OK;
}

nw_status nw_profile_steps(nw_system* s, int nsteps, float dt, NwKernelTime* out, int max_entries, int* n_entries)
{
    if (!s || nsteps < 1 || !out || max_entries < 1 || !n_entries) return NW_ERR_INVALID;
    if (!(dt > 0.0f)) dt = s->cfg.dt;
    cudaError_t e = clean_lists(s);
    if (e != cudaSuccess) return cuda_status(e);
    Prof prof;
    prof.stream = s->stream;
    s->state_ev_valid = false;  // the profiled launches record no state event
    s->last_launches = enqueue_steps(s, nsteps, dt, s->step, &prof);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) {
        prof.clear();
        return cuda_status(e);
    }
    s->scur ^= collision_parity(s, s->step, nsteps);
    s->step += (uint64_t)nsteps;
    if (lazy_tangents(s)) s->tan_stale = true;
    int n = 0;
    for (size_t k = 0; k + 1 < prof.events.size(); ++k) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, prof.events[k], prof.events[k + 1]);
        int slot = -1;
        for (int q = 0; q < n; ++q)
            if (std::strncmp(out[q].name, prof.names[k].c_str(), sizeof(out[q].name)) == 0) slot = q;
        if (slot < 0) {
            if (n >= max_entries) continue;
            slot = n++;
            std::memset(&out[slot], 0, sizeof(out[slot]));
            std::strncpy(out[slot].name, prof.names[k].c_str(), sizeof(out[slot].name) - 1);
        }
        out[slot].total_ms += ms;
        out[slot].launches += 1;
    }
    *n_entries = n;
    prof.clear();
    return NW_OK;
}

}  // extern "C"
