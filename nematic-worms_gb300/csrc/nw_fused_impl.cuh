// nw_fused_impl.cuh — device code and launch templates of the cell-list step
// path: capped per-cell bead lists instead of a full sort, and the pair pass
// of update n fused with the integrate / bonded / hash pass of update n + 1
// in one kernel.  Compiled once per vector dimension: nw_fused.cu holds the
// three-component kernels and the launchers, nw_fused_planar.cu the
// two-component kernels of planar systems.
//
// Update n (ParticleSystem::update, simulation/particleSystem.cpp:249-339) is
//   pro(n): integrate -> [reverse] -> Langevin -> bending, tangents [bonds,
//           drive] -> cell hash -> insert into list n      (reads buffers n-1)
//   epi(n): pair forces from list n, force[i] = F_n complete (reads buffers n)
// and a call of M updates launches pro(s), then fused(n -> n+1) = epi(n) +
// pro(n+1) for every n not followed by an SRD collision, and epi(last).
// Bead state is double-buffered ([n & 1] written by update n), so a block
// integrating update n+1 never overwrites positions another block still reads
// for the pair forces of update n.  Members of a cell are visited in
// ascending bead index (a sorting network over the cell's slots), which is
// the order of the reference's stable sort: forces accumulate in the same
// order as with the sorted arrays, and runs are bit-identical.
#pragma once

#include <utility>

#include "nw_fused.cuh"

namespace nw {
namespace {

// Buffer k of a double / triple buffer by selects rather than an indexed
// load: a StepBuffers copy in registers (the batch kernel's) stays there.
template <class T>
__device__ __forceinline__ T* pick2(T* const (&a)[2], uint32_t k)
{
    return k ? a[1] : a[0];
}
__device__ __forceinline__ uint32_t* pick3(uint32_t* const (&a)[3], uint32_t k)
{
    return k == 0u ? a[0] : (k == 1u ? a[1] : a[2]);
}

// Programmatic dependent launch: the step kernels are launched with the
// stream-serialisation attribute relaxed, so that a kernel's blocks may be
// scheduled while the previous kernel's last blocks still run.  Each step
// kernel first waits (griddepcontrol.wait) until the previous kernel has
// completed and its writes are visible, exactly the stream order, and then
// lets the next launch begin.  Launched without the attribute both
// instructions return at once.  NW_PDL=0 builds plain launches.
#ifndef NW_PDL
#define NW_PDL 1
#endif
__device__ __forceinline__ void pdl_enter()
{
#if NW_PDL
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#endif
}

template <class... KArgs, class... Args>
inline void launch_pdl(void (*kernel)(KArgs...), uint32_t grid, uint32_t block, size_t smem, cudaStream_t s,
                       Args&&... args)
{
#if NW_PDL
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
#else
    kernel<<<grid, block, smem, s>>>(std::forward<Args>(args)...);
#endif
}

// Ascending bitonic sort of N (power of two) registers, fully unrolled.
template <int N>
__device__ __forceinline__ void bitonic_sort(uint32_t (&a)[N])
{
#pragma unroll
    for (int size = 2; size <= N; size <<= 1)
#pragma unroll
        for (int stride = size / 2; stride > 0; stride >>= 1)
#pragma unroll
            for (int i = 0; i < N; ++i) {
                const int j = i ^ stride;
                if (j > i) {
                    const bool up = (i & size) == 0;
                    const uint32_t x = a[i], y = a[j];
                    if ((x > y) == up) {
                        a[i] = y;
                        a[j] = x;
                    }
                }
            }
}

// Members of cell c in ascending index; returns their number (<= CAP).
template <int CAP>
__device__ __forceinline__ int cell_members(const uint32_t* __restrict__ cnt, const uint32_t* __restrict__ slots,
                                            uint32_t c, uint32_t (&ids)[CAP])
{
    uint32_t k = __ldg(cnt + c);
    if (k == 0) return 0;
    if (k > (uint32_t)CAP) k = CAP;  // the overflow was flagged when the list was filled
    const uint4* src = reinterpret_cast<const uint4*>(slots + (size_t)c * CAP);
#pragma unroll
    for (int q = 0; q < CAP / 4; ++q) {
        uint4 v = make_uint4(kEmpty, kEmpty, kEmpty, kEmpty);
        if ((uint32_t)(4 * q) < k) v = __ldg(src + q);
        ids[4 * q] = v.x;
        ids[4 * q + 1] = v.y;
        ids[4 * q + 2] = v.z;
        ids[4 * q + 3] = v.w;
    }
#pragma unroll
    for (int m = 0; m < CAP; ++m)
        if ((uint32_t)m >= k) ids[m] = kEmpty;
    if (k == 2) {
        if (ids[0] > ids[1]) {
            const uint32_t t = ids[0];
            ids[0] = ids[1];
            ids[1] = t;
        }
    } else if (k > 2) {
        bitonic_sort<CAP>(ids);
    }
    return (int)k;
}

// WCA_WORMS pair force on bead i from the lists (distinct neighbour cells in
// z, y, x order; same law, exclusion and order as pair_wca_kernel).
template <int CAP, int D>
__device__ __forceinline__ float3 wca_list_force(const DevParams& P, const float4* __restrict__ pos,
                                                 const uint32_t* __restrict__ cnt,
                                                 const uint32_t* __restrict__ slots, uint32_t i, float3 r,
                                                 uint32_t own)
{
    const uint32_t fbase = (i / P.L) * P.L;
    float3 f = zero3();
    for_neighbour_cells<true>(P, r, own, [&](uint32_t h) {
        uint32_t ids[CAP];
        const int k = cell_members<CAP>(cnt, slots, h, ids);
#pragma unroll
        for (int m = 0; m < CAP; ++m) {
            if (m >= k) break;
            const uint32_t j = ids[m];
            if (j == i || lj_excluded(P, i, j, fbase)) continue;
            float3 dr = subv<D>(f3(__ldg(pos + j)), r);
            min_image_near<D>(P, dr);
            const float rr = dotv<D>(dr, dr);
            if (rr > P.lj_rc2) continue;
            sub_scaled<D>(f, wca_lj(P, rr), dr);
        }
    });
    return f;
}

// collideCell over one list cell (particles_kernel_impl.cuh:492-556).
template <int CAP>
__device__ __forceinline__ float3 ref_list_cell(const DevParams& P, const float4* __restrict__ pos,
                                                const float4* __restrict__ vel, const float4* __restrict__ tan,
                                                const uint32_t* __restrict__ cnt, const uint32_t* __restrict__ slots,
                                                uint32_t h, uint32_t i, float3 r, float3 v, float3 t, uint32_t fI,
                                                uint32_t cI)
{
    float3 sum = zero3();
    uint32_t ids[CAP];
    const int k = cell_members<CAP>(cnt, slots, h, ids);
    const float cd = P.radius + P.radius;
#pragma unroll
    for (int m = 0; m < CAP; ++m) {
        if (m >= k) break;
        const uint32_t j = ids[m];
        if (j == i) continue;
        const float3 r2 = f3(__ldg(pos + j));
        const uint32_t fJ = j / P.L, cJ = j - fJ * P.L;
        const bool same = fI == fJ;
        if (same && ((cI + 1u == cJ) || (cI - 1u == cJ))) {
            float3 rel = r2 - r;
            const float d = min_image_len(P, rel);
            const float3 nrm = rel / d;
            sum += (-P.bond_k * (P.bond_r0 - d)) * nrm;
        } else {
            float3 rel = r2 - r;
            const float d = min_image_len(P, rel);
            if (d < cd) {
                const float3 nrm = rel / d;
                const float3 rv = f3(__ldg(vel + j)) - v;
                const float3 tv = rv - dot3(rv, nrm) * nrm;
                float3 F = (-P.spring * (cd - d)) * nrm;
                F += P.damping * rv;
                F += P.shear * tv;
                sum += F;
            }
        }
        if (!same) {
            float3 rel = r2 - r;
            const float d = min_image_len(P, rel);
            const float3 t2 = f3(__ldg(tan + j));
            if (dot3(t, t2) < -0.5f) sum += ((-P.activity) * (t - t2)) / (2.0f * d);
        }
    }
    return sum;
}

// REF_DEM pair force on bead i: the reference's 27 offsets in z, y, x order;
// with one z layer each (x, y) cell sum is reused for the three z offsets.
template <int CAP>
__device__ __forceinline__ float3 ref_list_force(const DevParams& P, const float4* __restrict__ pos,
                                                 const float4* __restrict__ vel, const float4* __restrict__ tan,
                                                 const uint32_t* __restrict__ cnt,
                                                 const uint32_t* __restrict__ slots, uint32_t i, float3 r)
{
    const float3 v = f3(__ldg(vel + i));
    const float3 t = f3(__ldg(tan + i));
    const int3 g = grid_pos(P, r);
    const uint32_t fI = i / P.L, cI = i - fI * P.L;
    float3 total = zero3();
    if (P.grid[2] == 1u) {
        float3 cs[9];
#pragma unroll
        for (int y = -1; y <= 1; ++y)
#pragma unroll
            for (int x = -1; x <= 1; ++x) {
                const uint32_t h =
                    cell_hash(P, cell_coord(P, 0, g.x + x), cell_coord(P, 1, g.y + y), cell_coord(P, 2, g.z));
                cs[(y + 1) * 3 + (x + 1)] = ref_list_cell<CAP>(P, pos, vel, tan, cnt, slots, h, i, r, v, t, fI, cI);
            }
#pragma unroll
        for (int z = 0; z < 3; ++z)
#pragma unroll
            for (int k = 0; k < 9; ++k) total += cs[k];
    } else {
        for (int z = -1; z <= 1; ++z)
            for (int y = -1; y <= 1; ++y)
                for (int x = -1; x <= 1; ++x) {
                    const uint32_t h =
                        cell_hash(P, cell_coord(P, 0, g.x + x), cell_coord(P, 1, g.y + y), cell_coord(P, 2, g.z + z));
                    total += ref_list_cell<CAP>(P, pos, vel, tan, cnt, slots, h, i, r, v, t, fI, cI);
                }
    }
    return total;
}

// Displacement bound of the state after update n: the bound after update
// n - 1 (zero if the lists were built then) plus update n's largest bead
// displacement.  Every block reads the same words, so all agree.
__device__ __forceinline__ float vl_bound(const StepBuffers& S, unsigned long long n)
{
    return __uint_as_float(S.vstate[(uint32_t)((n + 1ull) & 1ull)]) +
           __uint_as_float(S.vstate[2u + (uint32_t)(n % 3ull)]);
}

// Verlet pair force: the bead's list from the last build, each pair still
// tested against lj_rcut.  Pairs are summed in list order, which is the
// cell-scan order of the build.  Neighbours are fetched in batches so that
// the batch's index loads, then its position gathers, are in flight together:
// four at a time, or six in the planar loop (verlet_force_planar), which
// gathers only x and y (8 bytes each, so the batch fits the register budget).
// A batch's pairs are evaluated without branches, a pair beyond the cut-off
// (or past the end of the list, fetched as bead i itself) adding 0 * dr.
template <int D>
__device__ __forceinline__ float3 verlet_force(const DevParams& P, const StepBuffers& S,
                                               const float4* __restrict__ pos, uint32_t i, float3 r)
{
    uint32_t k = __ldg(S.nnb + i);
    if (k > P.vl_cap) k = P.vl_cap;
    float3 f = zero3();
    const uint32_t* __restrict__ col = S.nbr + i;
    for (uint32_t m = 0; m < k; m += 4) {
        uint32_t j[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) j[q] = m + q < k ? __ldg(col + (size_t)(m + q) * P.nb) : i;
        float4 pj[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) pj[q] = __ldg(pos + j[q]);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            float3 dr = subv<D>(f3(pj[q]), r);
            min_image_near<D>(P, dr);
            const float rr = dotv<D>(dr, dr);
            const bool in = m + q < k && rr <= P.lj_rc2;
            sub_scaled<D>(f, in ? wca_lj(P, rr) : 0.0f, dr);
        }
    }
    return f;
}

// The planar loop's list length and first batch of six entries, loaded
// before the rebuild decision so that they travel with the bound's words;
// entries past the list are masked by its length, and rows beyond the list
// capacity (at least 4) are read as row 0.
constexpr int kPlanarBatch = 6;
struct PlanarHead {
    uint32_t k;
    uint32_t j[kPlanarBatch];
};

__device__ __forceinline__ PlanarHead planar_head(const DevParams& P, const StepBuffers& S, uint32_t i)
{
    PlanarHead h;
    h.k = __ldg(S.nnb + i);
#pragma unroll
    for (int q = 0; q < kPlanarBatch; ++q) h.j[q] = __ldg(S.nbr + i + (size_t)((uint32_t)q < P.vl_cap ? q : 0) * P.nb);
    return h;
}

// verlet_force of planar systems: x and y of six neighbours gathered per
// batch (8 bytes each), the first batch from the head.
__device__ __forceinline__ float3 verlet_force_planar(const DevParams& P, const StepBuffers& S,
                                                      const float4* __restrict__ pos, uint32_t i, float3 r,
                                                      const PlanarHead& h)
{
    constexpr int D = 2;
    const uint32_t k = h.k > P.vl_cap ? P.vl_cap : h.k;
    float3 f = zero3();
    const uint32_t* __restrict__ col = S.nbr + i;
    for (uint32_t m = 0; m < k; m += kPlanarBatch) {
        uint32_t j[kPlanarBatch];
        if (m == 0) {
#pragma unroll
            for (int q = 0; q < kPlanarBatch; ++q) j[q] = (uint32_t)q < k ? h.j[q] : i;
        } else {
#pragma unroll
            for (int q = 0; q < kPlanarBatch; ++q) j[q] = m + q < k ? __ldg(col + (size_t)(m + q) * P.nb) : i;
        }
        float2 pj[kPlanarBatch];
#pragma unroll
        for (int q = 0; q < kPlanarBatch; ++q) pj[q] = __ldg(reinterpret_cast<const float2*>(pos + j[q]));
#pragma unroll
        for (int q = 0; q < kPlanarBatch; ++q) {
            float3 dr = make_float3(pj[q].x - r.x, pj[q].y - r.y, 0.f);
            min_image_near<D>(P, dr);
            const float rr = dotv<D>(dr, dr);
            const bool in = m + q < k && rr <= P.lj_rc2;
            sub_scaled<D>(f, in ? wca_lj(P, rr) : 0.0f, dr);
        }
    }
    return f;
}

// List build: the cell scan of wca_list_force on the Verlet grid, recording
// every non-excluded bead within lj_rcut + skin and summing the LJ force of
// those within lj_rcut.
template <int CAP, int D>
__device__ __forceinline__ float3 verlet_build_force(const DevParams& P, const StepBuffers& S,
                                                     const float4* __restrict__ pos,
                                                     const uint32_t* __restrict__ cnt,
                                                     const uint32_t* __restrict__ slots, uint32_t i, float3 r,
                                                     uint32_t own)
{
    const uint32_t fbase = (i / P.L) * P.L;
    uint32_t k = 0;
    uint32_t* col = S.nbr + i;
    float3 f = zero3();
    for_neighbour_cells<true>(P, r, own, [&](uint32_t h) {
        uint32_t ids[CAP];
        const int kc = cell_members<CAP>(cnt, slots, h, ids);
#pragma unroll
        for (int m = 0; m < CAP; ++m) {
            if (m >= kc) break;
            const uint32_t j = ids[m];
            if (j == i || lj_excluded(P, i, j, fbase)) continue;
            float3 dr = subv<D>(f3(__ldg(pos + j)), r);
            min_image_near<D>(P, dr);
            const float rr = dotv<D>(dr, dr);
            if (rr > P.vl_r2) continue;
            if (k < P.vl_cap) col[(size_t)k * P.nb] = j;
            ++k;
            if (rr > P.lj_rc2) continue;
            sub_scaled<D>(f, wca_lj(P, rr), dr);
        }
    });
    S.nnb[i] = k < P.vl_cap ? k : P.vl_cap;
    if (k > P.vl_cap) atomicOr(S.err, (uint32_t)NW_EFLAG_NEIGHBOR_OVERFLOW);
    return f;
}

// Bookkeeping of the Verlet lists by the kernel that runs the pair pass of
// update n (one thread): the bound after update n, a cleared maximum for
// update n + 2, and which cell-list count buffers hold entries (bit b of
// vstate[kVlFilled] for lcount[b]): buffer n % 3 when update n rebuilt (its
// cell list was filled), not buffer (n + 1) % 3, which pro(n) emptied in an
// earlier kernel.  pro(n + 1), running beside this, reads only bit
// (n + 2) % 3, which this write leaves as it was.
constexpr uint32_t kVlFilled = 6;
__device__ __forceinline__ void vl_commit(const StepBuffers& S, unsigned long long n, bool rebuilt, float bound)
{
    S.vstate[(uint32_t)(n & 1ull)] = __float_as_uint(rebuilt ? 0.0f : bound);
    S.vstate[2u + (uint32_t)((n + 2ull) % 3ull)] = 0u;
    uint32_t filled = S.vstate[kVlFilled] & ~(1u << (uint32_t)((n + 1ull) % 3ull));
    if (rebuilt) filled |= 1u << (uint32_t)(n % 3ull);
    S.vstate[kVlFilled] = filled;
}

// Pair force of bead i for update n (reads the update-n buffers and list).
// blk = the block's index among the blocks of its system.  D = 2: planar
// WCA systems (REF_DEM systems are always D = 3); their loop's first batch
// is loaded before the rebuild decision (planar_head).  kWide = false (the
// batch kernel, whose parameter block is read from shared memory and whose
// registers are tighter) keeps the four-wide loop: the batch measured 1 %
// faster with it, the single system 1.5 % slower.
template <int CAP, bool kRef, int D, bool kWide = true>
__device__ __forceinline__ float3 list_pair_force(const DevParams& P, const StepBuffers& S, unsigned long long n,
                                                  uint32_t i, uint32_t blk)
{
    const uint32_t cur = (uint32_t)(n & 1ull);
    const uint32_t* cnt = pick3(S.lcount, (uint32_t)(n % 3ull));
    const uint32_t* slots = pick2(S.lslot, cur);
    const float3 r = f3(pick2(S.pos2, cur)[i]);
    if (kRef) return ref_list_force<CAP>(P, pick2(S.pos2, cur), pick2(S.vel2, cur), pick2(S.tan2, cur), cnt, slots, i, r);
    if (P.vl_on) {
        PlanarHead head{};
        if constexpr (D == 2 && kWide) head = planar_head(P, S, i);
        const float bound = vl_bound(S, n);
        const bool rebuild = !(bound <= P.vl_half_skin);  // a NaN bound rebuilds too
        if (blk == 0 && threadIdx.x == 0) vl_commit(S, n, rebuild, bound);
        if (!rebuild) {
            if constexpr (D == 2 && kWide) return verlet_force_planar(P, S, pick2(S.pos2, cur), i, r, head);
            else return verlet_force<D>(P, S, pick2(S.pos2, cur), i, r);
        }
        return verlet_build_force<CAP, D>(P, S, pick2(S.pos2, cur), cnt, slots, i, r, pick2(S.hash2, cur)[i]);
    }
    return wca_list_force<CAP, D>(P, pick2(S.pos2, cur), cnt, slots, i, r, pick2(S.hash2, cur)[i]);
}

// Resident blocks of 256 threads per SM that the WCA fused kernel is
// compiled for (the register budget: 65536 / (256 * 6) -> 40 registers).
#ifndef NW_FUSED_MIN_BLOCKS
#define NW_FUSED_MIN_BLOCKS 6
#endif

// Shared-memory bytes of the pro part for a block of `beads` beads.
__host__ __device__ __forceinline__ size_t pro_smem(uint32_t beads, bool reverse)
{
    return (size_t)beads * sizeof(float4) * (reverse ? 3u : 1u) + (size_t)beads * 3u * sizeof(float4);
}

// pro(n) for the block's filaments: every thread of the block must call it.
// fprev = F_{n-1} of this thread's bead (complete force of the previous update);
// blk / nblk = the block's index among, and the number of, its system's blocks.
// D = 2: a planar WCA system (z carried, forces in the plane).
template <int CAP, int D>
__device__ __forceinline__ void pro_part(const DevParams& P, const StepBuffers& S, unsigned long long n, float dt,
                                         uint32_t fpb, bool active, uint32_t i, float3 fprev, uint32_t blk,
                                         uint32_t nblk, bool insert = true, uint32_t pflags = 0u)
{
    extern __shared__ float4 sm[];
    const uint32_t L = P.L;
    const uint32_t beads = fpb * L;
    const uint32_t t = threadIdx.x;
    const uint32_t w0 = blk * fpb;
    const uint32_t in = (uint32_t)((n + 1ull) & 1ull), out = (uint32_t)(n & 1ull);
    float4* smp = sm;                                       // positions [beads]
    float4* smx = sm + (P.reverse_on ? 3u : 1u) * beads;    // triple forces [3][beads]

    // lists of update n+1 must start empty: clear them while nobody reads them
    // (Verlet systems fill them only for a rebuild: clear a buffer only when
    // a build filled it since it was last cleared)
    {
        const uint32_t b = (uint32_t)((n + 1ull) % 3ull);
        if (!P.vl_on || ((S.vstate[kVlFilled] >> b) & 1u)) {
            uint32_t* nxt = pick3(S.lcount, b);
            const uint32_t stride = nblk * blockDim.x;
            for (uint32_t c = blk * blockDim.x + t; c < P.lncells; c += stride) nxt[c] = 0u;
        }
    }

    float4 nP = make_float4(0.f, 0.f, 0.f, 0.f), nV = nP, nFo = nP;
    float disp2 = 0.f;  // squared displacement of this update (Verlet list bound)
    if (active) {
        const float4 P4 = pick2(S.pos2, in)[i], V4 = pick2(S.vel2, in)[i], Fo4 = S.force_old[i];
        float3 p = f3(P4), v = f3(V4);
        const float3 f = fprev, fo = f3(Fo4);
        // velocity Verlet (particles_kernel_impl.cuh:93-97), per axis:
        // v += (f + f_old) / 2 dt, dr = v dt + (f / 2) dt dt, r += dr
        auto verlet = [dt](float fa, float foa, float& va, float& pa) {
            va += (0.5f * (fa + foa)) * dt;
            const float d = va * dt + ((0.5f * fa) * dt) * dt;
            pa += d;
            return d;
        };
        float3 dr;
        dr.x = verlet(f.x, fo.x, v.x, p.x);
        dr.y = verlet(f.y, fo.y, v.y, p.y);
        dr.z = D == 3 ? verlet(f.z, fo.z, v.z, p.z) : 0.f;
        disp2 = dotv<D>(dr, dr);
        apply_boundaries<D>(P, p, v, dr, P.radius);
        nP = make_float4(p.x, p.y, p.z, P4.w);
        nV = make_float4(v.x, v.y, v.z, V4.w);
        nFo = make_float4(f.x, f.y, D == 3 ? f.z : 0.f, Fo4.w);
    }
    if (P.reverse_on) {
        // reverseFilamentsKernel (particles_kernel_impl.cuh:820-857)
        if (active) {
            smp[t] = nP;
            smp[beads + t] = nV;
            smp[2 * beads + t] = nFo;
        }
        __syncthreads();
        if (active) {
            const uint32_t wl = t / L, c = t - wl * L;
            const float u = u01(rng_draw(P, w0 + wl, n, kRngReverse).x);
            if (u <= P.reverse_p) {
                const uint32_t src = wl * L + (L - 1u - c);
                disp2 = 3.0e38f;  // bead indices moved: the lists must be rebuilt
                nP = smp[src];
                nV = smp[beads + src];
                nFo = smp[2 * beads + src];
            }
        }
        __syncthreads();
    }
    // largest displacement of update n (float bits order like the values): a
    // warp maximum, then one atomic per block (one per warp on a single word
    // serialises in L2 and cost 1.4 us of a 26 us step kernel)
    __shared__ uint32_t s_dmax[32];
    if (P.vl_on) {
        const uint32_t m = __reduce_max_sync(0xffffffffu, __float_as_uint(disp2));
        if ((t & 31u) == 0u) s_dmax[t >> 5] = m;
    }
    if (active) smp[t] = nP;
    __syncthreads();
    if (P.vl_on && t == 0) {
        uint32_t m = 0u;
        for (uint32_t q = 0; q < (blockDim.x + 31u) >> 5; ++q) m = s_dmax[q] > m ? s_dmax[q] : m;
        if (m) atomicMax(&S.vstate[2u + (uint32_t)(n % 3ull)], __float_as_uint(sqrtf(__uint_as_float(m))));
    }
    const uint32_t wl = active ? t / L : 0u, c = active ? t - wl * L : 0u;
    const float4* R = smp + wl * L;
    // each bending triple once, by the thread of its first bead
    if (active && L >= 3 && c + 2 < L) {
        const Triple tr = bend_triple<D>(P, f3(R[c]), f3(R[c + 1]), f3(R[c + 2]));
        smx[t] = make_float4(tr.fi.x, tr.fi.y, tr.fi.z, 0.f);
        smx[beads + t] = make_float4(tr.fj.x, tr.fj.y, tr.fj.z, 0.f);
        smx[2 * beads + t] = make_float4(tr.fk.x, tr.fk.y, tr.fk.z, 0.f);
    }
    __syncthreads();
    if (!active) return;

    float3 fs = zero3();
    if (P.langevin_on) {
        // langevinKernel (particles_kernel_impl.cuh:859-874), Philox noise in registers
        const uint4 x = rng_draw(P, i, n, kRngLangevin);
        if constexpr (D == 2) {
            const float2 z = normal2(x);
            fs = make_float3((0.f - P.gamma * nV.x) + P.noise_sigma * z.x,
                             (0.f - P.gamma * nV.y) + P.noise_sigma * z.y, 0.f);
        } else {
            const float3 g = noise3(P, x);
            float3 fl = zero3() - P.gamma * f3(nV);
            fl += g;
            fs = fl;
        }
    }
    // bending contributions in the reference's triple order p = c-2, c-1, c
    if (L >= 3) {
        if (c >= 2) fs = addv<D>(fs, f3(smx[2 * beads + t - 2]));
        if (c >= 1 && c + 1 < L) fs = addv<D>(fs, f3(smx[beads + t - 1]));
        if (c + 2 < L) fs = addv<D>(fs, f3(smx[t]));
    }
    bool wt = false;
    float3 tg = zero3();
    const bool eager_tan = !(pflags & kProLazyTangent);
    if (eager_tan && L >= 3) {
        if (c == 0) {
            tg = tangent_of<D>(P, f3(R[0]), f3(R[1]));
            wt = true;
        } else if (c == L - 1) {
            if (L > 3) {
                tg = tangent_of<D>(P, f3(R[L - 2]), f3(R[L - 1]));
                wt = true;
            }
        } else {
            tg = tangent_of<D>(P, f3(R[c - 1]), f3(R[c + 1]));
            wt = true;
        }
    }
    if (P.model == NW_MODEL_WCA_WORMS) {
        const float3 me = f3(R[c]);
        if (c > 0) wca_bond<D>(P, me, f3(R[c - 1]), fs);
        if (c + 1 < L) wca_bond_drive<D>(P, me, f3(R[c + 1]), fs);
    }
    pick2(S.pos2, out)[i] = nP;
    pick2(S.vel2, out)[i] = nV;
    S.force_old[i] = nFo;
    S.force[i] = make_float4(fs.x, fs.y, fs.z, 0.f);
    if (eager_tan) pick2(S.tan2, out)[i] = wt ? make_float4(tg.x, tg.y, tg.z, 0.f) : pick2(S.tan2, in)[i];
    if (!finitev<D>(f3(nP)) || !finitev<D>(fs)) atomicOr(S.err, (uint32_t)NW_EFLAG_NONFINITE);

    if (!insert) return;  // Verlet systems: bead_list_kernel fills list n when a rebuild needs it
    const uint32_t h = P.vl_on ? list_hash(P, f3(nP)) : bead_hash(P, f3(nP));
    pick2(S.hash2, out)[i] = h;
    const uint32_t slot = atomicAdd(&pick3(S.lcount, (uint32_t)(n % 3ull))[h], 1u);
    if (slot < (uint32_t)CAP) pick2(S.lslot, out)[(size_t)h * CAP + slot] = i;
    else atomicOr(S.err, (uint32_t)NW_EFLAG_CELL_OVERFLOW);
}

// The cell list of update n for a Verlet system, built only when the pair
// pass of update n will rebuild the neighbour lists: the same predicate on
// the same words (the displacement bound after update n), so the two always
// agree.  Otherwise every block leaves after reading the bound.
template <int CAP>
__global__ void __launch_bounds__(256) bead_list_kernel(const DevParams P, const StepBuffers S, uint32_t off)
{
    pdl_enter();
    const unsigned long long n = *S.step_base + off;
    if (vl_bound(S, n) <= P.vl_half_skin) return;
    const uint32_t out = (uint32_t)(n & 1ull);
    const float4* __restrict__ pos = pick2(S.pos2, out);
    uint32_t* hash = pick2(S.hash2, out);
    uint32_t* cnt = pick3(S.lcount, (uint32_t)(n % 3ull));
    uint32_t* slots = pick2(S.lslot, out);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < P.nb; i += gridDim.x * blockDim.x) {
        const uint32_t h = list_hash(P, f3(pos[i]));
        hash[i] = h;
        const uint32_t slot = atomicAdd(cnt + h, 1u);
        if (slot < (uint32_t)CAP) slots[(size_t)h * CAP + slot] = i;
        else atomicOr(S.err, (uint32_t)NW_EFLAG_CELL_OVERFLOW);
    }
}

template <int CAP, int MAXT, int D>
__global__ void __launch_bounds__(MAXT) bead_pro_kernel(const DevParams P, const StepBuffers S, uint32_t off, float dt,
                                                        uint32_t fpb, uint32_t pflags)
{
    pdl_enter();
    const unsigned long long n = *S.step_base + off;
    const uint32_t i = blockIdx.x * fpb * P.L + threadIdx.x;
    const bool active = threadIdx.x < fpb * P.L && i < P.nb;
    const float3 fprev = active ? f3(S.force[i]) : zero3();
    pro_part<CAP, D>(P, S, n, dt, fpb, active, i, fprev, blockIdx.x, gridDim.x, !P.vl_on, pflags);
}

template <int CAP, bool kRef, int D>
__global__ void __launch_bounds__(256) bead_epi_kernel(const DevParams P, const StepBuffers S, uint32_t off)
{
    pdl_enter();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.nb) return;
    const unsigned long long n = *S.step_base + off;
    const float3 pair = list_pair_force<CAP, kRef, D>(P, S, n, i, blockIdx.x);
    float4 F = S.force[i];
    F.x += pair.x;
    F.y += pair.y;
    if constexpr (D == 3) F.z += pair.z;
    S.force[i] = F;
    if (!finitev<D>(f3(F))) atomicOr(S.err, (uint32_t)NW_EFLAG_NONFINITE);
}

// epi(n) then pro(n+1): the complete force of update n stays in a register.
template <int CAP, bool kRef, int MAXT, int D>
__global__ void __launch_bounds__(MAXT, (MAXT == 256 && !kRef) ? NW_FUSED_MIN_BLOCKS : 1)
    bead_fused_kernel(const DevParams P, const StepBuffers S, uint32_t off, float dt, uint32_t fpb, uint32_t pflags)
{
    pdl_enter();
    const unsigned long long n = *S.step_base + off;
    const uint32_t i = blockIdx.x * fpb * P.L + threadIdx.x;
    const bool active = threadIdx.x < fpb * P.L && i < P.nb;
    float3 Fn = zero3();
    if (active) {
        const float3 pair = list_pair_force<CAP, kRef, D>(P, S, n, i, blockIdx.x);
        const float4 F = S.force[i];
        Fn = make_float3(F.x + pair.x, F.y + pair.y, D == 3 ? F.z + pair.z : 0.f);
        if (!finitev<D>(Fn)) atomicOr(S.err, (uint32_t)NW_EFLAG_NONFINITE);
    }
    pro_part<CAP, D>(P, S, n + 1ull, dt, fpb, active, i, Fn, blockIdx.x, gridDim.x, !P.vl_on, pflags);
}

// A batch block: copy its replica's parameter block into shared memory and
// run pro, epi or fused for that replica's slice of the batch buffers.
template <int CAP, int MODE, int MAXT, int D>
__global__ void __launch_bounds__(MAXT, MAXT == 256 ? 6 : 1) batch_kernel(const ReplicaSlot* __restrict__ table,
                                                     const uint32_t* __restrict__ block_rep, const StepBuffers S0,
                                                     uint32_t off)
{
    __shared__ DevParams sP;
    const uint32_t r = __ldg(block_rep + blockIdx.x);
    const ReplicaSlot* e = table + r;
    if (MODE == kBatchList) {
        // leave before staging the parameter block unless this replica rebuilds
        // (two round trips: the step counter beside the replica index, then the
        // replica's bound beside its skin)
        if (!S0.vstate) return;
        const unsigned long long n0 = *S0.step_base + off;
        const uint32_t* vs = S0.vstate + 8u * r;
        const float bound = __uint_as_float(vs[(uint32_t)((n0 + 1ull) & 1ull)]) +
                            __uint_as_float(vs[2u + (uint32_t)(n0 % 3ull)]);
        if (!e->P.vl_on || bound <= e->P.vl_half_skin) return;
    }
    {
        const uint32_t* src = reinterpret_cast<const uint32_t*>(&e->P);
        uint32_t* dst = reinterpret_cast<uint32_t*>(&sP);
        for (uint32_t w = threadIdx.x; w < (uint32_t)(sizeof(DevParams) / 4); w += blockDim.x) dst[w] = __ldg(src + w);
    }
    __syncthreads();
    const DevParams& P = sP;
    const uint32_t bo = e->bead_off, co = e->cell_off, blk = blockIdx.x - e->blk0, nblk = e->nblk, fpb = e->fpb;
    const float dt = e->dt;
    StepBuffers S = S0;
    for (int k = 0; k < 2; ++k) {
        S.pos2[k] += bo;
        S.vel2[k] += bo;
        S.tan2[k] += bo;
        S.hash2[k] += bo;
        S.lslot[k] += (size_t)co * CAP;
    }
    for (int k = 0; k < 3; ++k) S.lcount[k] += co;
    S.force += bo;
    S.force_old += bo;
    if (S.nbr) S.nbr += e->nbr_off;
    if (S.nnb) S.nnb += bo;
    if (S.vstate) S.vstate += 8u * r;
    const unsigned long long n = *S.step_base + off;
    const uint32_t i = blk * fpb * P.L + threadIdx.x;
    const bool active = threadIdx.x < fpb * P.L && i < P.nb;
    if (MODE == kBatchList) {
        // this replica's cell list of update n, only when its pair pass rebuilds
        if (!P.vl_on || vl_bound(S, n) <= P.vl_half_skin || !active) return;
        const uint32_t out = (uint32_t)(n & 1ull);
        const uint32_t h = list_hash(P, f3(pick2(S.pos2, out)[i]));
        pick2(S.hash2, out)[i] = h;
        const uint32_t slot = atomicAdd(&pick3(S.lcount, (uint32_t)(n % 3ull))[h], 1u);
        if (slot < (uint32_t)CAP) pick2(S.lslot, out)[(size_t)h * CAP + slot] = i;
        else atomicOr(S.err, (uint32_t)NW_EFLAG_CELL_OVERFLOW);
        return;
    }
    if (MODE == kBatchPro) {
        const float3 fprev = active ? f3(S.force[i]) : zero3();
        pro_part<CAP, D>(P, S, n, dt, fpb, active, i, fprev, blk, nblk, !P.vl_on, pro_flags(P));
        return;
    }
    float3 Fn = zero3();
    if (active) {
        const float3 pair = list_pair_force<CAP, false, D, false>(P, S, n, i, blk);
        const float4 F = S.force[i];
        Fn = make_float3(F.x + pair.x, F.y + pair.y, D == 3 ? F.z + pair.z : F.z);
        if (!finitev<D>(Fn)) atomicOr(S.err, (uint32_t)NW_EFLAG_NONFINITE);
        if (MODE == kBatchEpi) S.force[i] = make_float4(Fn.x, Fn.y, Fn.z, F.w);
    }
    if (MODE == kBatchFused) pro_part<CAP, D>(P, S, n + 1ull, dt, fpb, active, i, Fn, blk, nblk, !P.vl_on, pro_flags(P));
}

// Bead tangents of the current positions, as the pro part writes them
// (systems whose step leaves them to be computed when read).
template <int D>
__global__ void __launch_bounds__(256) bead_tangent_kernel(const DevParams P, const float4* __restrict__ pos,
                                                           float4* __restrict__ tan)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.nb) return;
    const uint32_t L = P.L, c = i % L, b = i - c;
    float3 tg;
    if (c == 0) tg = tangent_of<D>(P, f3(pos[b]), f3(pos[b + 1]));
    else if (c == L - 1) tg = tangent_of<D>(P, f3(pos[b + L - 2]), f3(pos[b + L - 1]));
    else tg = tangent_of<D>(P, f3(pos[i - 1]), f3(pos[i + 1]));
    tan[i] = make_float4(tg.x, tg.y, tg.z, 0.f);
}

inline uint32_t cdiv32(uint64_t a, uint32_t b) { return (uint32_t)((a + b - 1) / b); }

inline void pro_shape(const DevParams& P, uint32_t& fpb, uint32_t& threads, size_t& smem)
{
    fpb = list_filaments_per_block(P.L, P.nf);
    const uint32_t beads = fpb * P.L;
    threads = (beads + 31u) & ~31u;
    smem = pro_smem(beads, P.reverse_on != 0);
}

// ---- launchers of one dimension (D = 3, or 2 for planar systems) ------------

template <int D>
uint64_t bead_pro_d(const DevParams& P, const StepBuffers& B, uint32_t off, float dt, cudaStream_t s)
{
    uint32_t fpb, threads;
    size_t smem;
    pro_shape(P, fpb, threads, smem);
    const uint32_t blocks = cdiv32(P.nf, fpb);
    const bool big = threads > 256;  // filaments longer than 256 beads: one per block, up to 1024 threads
    const uint32_t pf = pro_flags(P);
    if (B.cap == 16) {
        if (big) launch_pdl(bead_pro_kernel<16, 1024, D>, blocks, threads, smem, s, P, B, off, dt, fpb, pf);
        else launch_pdl(bead_pro_kernel<16, 256, D>, blocks, threads, smem, s, P, B, off, dt, fpb, pf);
    } else {
        if (big) launch_pdl(bead_pro_kernel<8, 1024, D>, blocks, threads, smem, s, P, B, off, dt, fpb, pf);
        else launch_pdl(bead_pro_kernel<8, 256, D>, blocks, threads, smem, s, P, B, off, dt, fpb, pf);
    }
    return 1;
}

template <int D>
uint64_t bead_tangents_d(const DevParams& P, const float4* pos, float4* tan, cudaStream_t s)
{
    bead_tangent_kernel<D><<<cdiv32(P.nb, 256), 256, 0, s>>>(P, pos, tan);
    return 1;
}

// REF_DEM systems are never planar: their pair kernels exist for D = 3 only.
template <int D>
uint64_t bead_epi_d(const DevParams& P, const StepBuffers& B, uint32_t off, cudaStream_t s)
{
    const uint32_t blocks = cdiv32(P.nb, 256);
    const bool ref = P.model == NW_MODEL_REF_DEM;
    if constexpr (D == 3) {
        if (ref) {
            if (B.cap == 16) launch_pdl(bead_epi_kernel<16, true, 3>, blocks, 256, 0, s, P, B, off);
            else launch_pdl(bead_epi_kernel<8, true, 3>, blocks, 256, 0, s, P, B, off);
            return 1;
        }
    }
    if (B.cap == 16) launch_pdl(bead_epi_kernel<16, false, D>, blocks, 256, 0, s, P, B, off);
    else launch_pdl(bead_epi_kernel<8, false, D>, blocks, 256, 0, s, P, B, off);
    return 1;
}

template <int D>
uint64_t bead_fused_d(const DevParams& P, const StepBuffers& B, uint32_t off, float dt, cudaStream_t s)
{
    uint32_t fpb, threads;
    size_t smem;
    pro_shape(P, fpb, threads, smem);
    const uint32_t blocks = cdiv32(P.nf, fpb);
    const bool ref = P.model == NW_MODEL_REF_DEM;
    const bool big = threads > 256;
    const uint32_t pf = pro_flags(P);
#define NW_FUSED(CAPV, REFV)                                                                                   \
    do {                                                                                                       \
        if (big) launch_pdl(bead_fused_kernel<CAPV, REFV, 1024, D>, blocks, threads, smem, s, P, B, off, dt, fpb, pf); \
        else launch_pdl(bead_fused_kernel<CAPV, REFV, 256, D>, blocks, threads, smem, s, P, B, off, dt, fpb, pf);      \
    } while (0)
    if constexpr (D == 3) {
        if (ref) {
            if (B.cap == 16) NW_FUSED(16, true);
            else NW_FUSED(8, true);
            return 1;
        }
    }
    if (B.cap == 16) NW_FUSED(16, false);
    else NW_FUSED(8, false);
#undef NW_FUSED
    return 1;
}

template <int D>
void batch_d(int mode, const ReplicaSlot* table, const uint32_t* block_rep, uint32_t blocks, uint32_t threads,
             size_t smem, uint32_t cap, const StepBuffers& S, uint32_t off, cudaStream_t s)
{
    const bool big = threads > 256;
#define NW_BATCH(CAPV, MODEV)                                                                                    \
    do {                                                                                                         \
        if (big) batch_kernel<CAPV, MODEV, 512, D><<<blocks, threads, smem, s>>>(table, block_rep, S, off);     \
        else batch_kernel<CAPV, MODEV, 256, D><<<blocks, threads, smem, s>>>(table, block_rep, S, off);         \
    } while (0)
#define NW_BATCH_MODE(CAPV)                                      \
    do {                                                         \
        if (mode == kBatchPro) NW_BATCH(CAPV, kBatchPro);        \
        else if (mode == kBatchEpi) NW_BATCH(CAPV, kBatchEpi);   \
        else if (mode == kBatchList) NW_BATCH(CAPV, kBatchList); \
        else NW_BATCH(CAPV, kBatchFused);                        \
    } while (0)
    if (cap == 16) NW_BATCH_MODE(16);
    else NW_BATCH_MODE(8);
#undef NW_BATCH_MODE
#undef NW_BATCH
}

}  // namespace
}  // namespace nw
