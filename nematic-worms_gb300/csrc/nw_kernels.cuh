// nw_kernels.cuh — the step kernels of the GB300 worm engine.
//
// Sorted strategy (the reference's scheme), six launches per step:
//   filament_pass   integrate + [reverse] + Langevin + bending/tangents
//                   [+ bonds + drive] + cell hash + counting-sort slot
//   chunk_sum       totals of 4096-cell chunks of the cell counts
//   scan_cells      cell offsets / starts / ends from the cell counts
//   scatter         bucket the bead indices by cell
//   stable_gather   order every bucket by index (the stable sort) and
//                   gather positions (+ velocities and tangents) in cell order
//   pair_*          pair forces over the 3x3(x3) neighbour cells
// The cell-list and Verlet strategies (nw_fused_impl.cuh) run one fused kernel
// per step instead.  Every srd_gap steps an SRD collision adds seven:
//   srd_hash, chunk_sum and scan_cells (bead and solvent buckets side by
//   side), srd_scatter, srd_collide, srd_collide_big, srd_flip.
//
// No float atomics are used anywhere: every output element has exactly one
// writer, so repeated runs are bit-identical.
#pragma once

#include "nw_device.cuh"

namespace nw {

// Beyond these occupancies a cell is reported (NW_EFLAG_CELL_OVERFLOW) and
// processed with bounded work; physical states never get close.
constexpr uint32_t kStableCap = 128;  // members ordered exactly up to this count
constexpr uint32_t kPairCap = 1024;   // members scanned per neighbour cell

struct StepBuffers {
    // Bead state.  pos2/vel2/tan2/hash2 are double buffers: the cell-list path
    // writes update n into [n & 1] while other blocks still read [(n-1) & 1];
    // the sorted path updates in place, with both entries naming one array.
    float4 *pos2[2], *vel2[2], *tan2[2];
    uint32_t* hash2[2];
    // in-place views of the sorted path (= pos2[0], ...)
    float4 *pos, *vel, *force, *force_old, *tangent;
    uint32_t *hash, *slot, *tmp_index, *sorted_index, *sorted_hash;
    // solvent state (particle nb + k is solvent k), kept in the cell order of
    // the last collision: each collision reads [*scur] and writes [*scur ^ 1]
    float4 *spos2[2], *svel2[2];
    uint32_t* scur;
    // capped per-cell bead lists of the cell-list path: counts of update n in
    // lcount[n % 3], members in lslot[n & 1][cell * cap + slot]
    uint32_t *lcount[3], *lslot[2];
    uint32_t cap;
    // Verlet lists (vl_on): neighbours of bead i in nbr[k * nb + i], k < nnb[i];
    // vstate[0..1] displacement bound of the state after update n in [n & 1],
    // vstate[2..4] maximum bead displacement of update n in [2 + n % 3]
    // (float bits; the bound counts from the last list build), vstate[5] the
    // largest move of positions set from the host, vstate[6] bit b set while
    // lcount[b] holds entries of a list build
    uint32_t *nbr, *nnb, *vstate;
    uint32_t *cell_count, *cell_offset, *cell_start, *cell_end, *chunk_count;
    float4 *sorted_pos, *sorted_vel, *sorted_tan;
    // SRD collision: per-particle cell hash and slot (beads [0, nb), solvent
    // [nb, ntotal)); beads and solvent are bucketed separately (a cell's
    // members in the stable order are its beads, then its solvent)
    uint32_t *srd_hash, *srd_slot, *srd_btmp, *srd_stmp, *srd_sorted_index;
    uint32_t *srd_bcount, *srd_scount, *srd_boff, *srd_soff, *srd_bchunk, *srd_schunk;
    uint32_t *srd_start, *srd_end;
    float4* srd_mean;
    // SRD cells of more than kLaneCap members, handed to
    // srd_collide_big_kernel: srd_big[0 .. *srd_nbig)
    uint32_t *srd_big, *srd_nbig;
    uint32_t* err;
    unsigned long long* step_base;
};

__device__ __forceinline__ uint32_t warp_sum(uint32_t x)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t x)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    return x;
}

// Count one element into its cell; the returned slot orders the cell's
// members arbitrarily (the stable order is restored when the bucket is read).
__device__ __forceinline__ uint32_t count_into_cell(uint32_t* cell_count, uint32_t h)
{
    return atomicAdd(&cell_count[h], 1u);
}

// ---- bonded helpers ----------------------------------------------------------

struct Triple {
    float3 fi, fj, fk;
};
// The bonded and pair laws below avoid IEEE division and square-root
// sequences (with their slow-path calls): they start from the hardware
// approximations (__fdividef, rsqrtf; <= 2 ulp) and, where the reference's
// result involves cancellation (r - r0 of a bond, the bending projections,
// the two LJ terms), refine them by one Newton-Raphson step whose residual
// is formed exactly with an FMA (P. Markstein, "Computation of elementary
// functions on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34,
// 1990).  Inputs are finite, positive and normal (squared separations of
// distinct beads).  nw_math_probe exposes the three for tests.

// 1/x to about 1 ulp: y' = y + y (1 - x y).
__device__ __forceinline__ float rcp_nr(float x)
{
    const float y = __fdividef(1.0f, x);
    return fmaf(y, fmaf(-x, y, 1.0f), y);
}

// sqrt(q) to about 1 ulp from y ~ 1/sqrt(q): r = q y, r' = r + (y / 2) (q - r^2).
__device__ __forceinline__ float sqrt_nr(float q, float y)
{
    const float r = q * y;
    return fmaf(0.5f * y, fmaf(-r, r, q), r);
}

// a / b to about 1 ulp: t = a (1/b), t' = t + (1/b) (a - b t).
__device__ __forceinline__ float div_nr(float a, float b)
{
    const float y = rcp_nr(b);
    const float t = a * y;
    return fmaf(fmaf(-b, t, a), y, t);
}

// One bending triple (filamentKernel, particles_kernel_impl.cuh:777-800):
// A = k_b / (d_ij d_jk), F_i = -A (r_jk - r_ij (r_ij . r_jk) / d_ij^2),
// F_k = -A (r_jk (r_ij . r_jk) / d_jk^2 - r_ij), F_j = -F_i - F_k.
// D = 2: in the xy plane (planar arithmetic, nw_device.cuh).
template <int D = 3>
__device__ __forceinline__ Triple bend_triple(const DevParams& P, float3 ri, float3 rj, float3 rk)
{
    float3 rij = subv<D>(rj, ri), rjk = subv<D>(rk, rj);
    min_image_near<D>(P, rij);
    min_image_near<D>(P, rjk);
    const float qij = dotv<D>(rij, rij), qjk = dotv<D>(rjk, rjk);
    const float dd = dotv<D>(rij, rjk);
    const float A = P.bend_k * (rsqrtf(qij) * rsqrtf(qjk));
    const float3 B = scalev<D>(div_nr(dd, qij), rij);
    const float3 C = scalev<D>(div_nr(dd, qjk), rjk);
    Triple t;
    t.fi = scalev<D>(-A, subv<D>(rjk, B));
    t.fk = scalev<D>(-A, subv<D>(C, rij));
    t.fj = subv<D>(make_float3(-t.fi.x, -t.fi.y, -t.fi.z), t.fk);
    return t;
}

// getTangent (particles_kernel_impl.cuh:303-309): the unit vector a -> b.
template <int D = 3>
__device__ __forceinline__ float3 tangent_of(const DevParams& P, float3 a, float3 b)
{
    float3 rel = subv<D>(b, a);
    min_image_near<D>(P, rel);
    return scalev<D>(rsqrtf(dotv<D>(rel, rel)), rel);
}

// Archived harmonic bond (NWWormsKernel_InternalForce.h:37-59):
// F_i = k (|r| - r0) r / |r| with r = r_j - r_i.
template <int D = 3>
__device__ __forceinline__ void wca_bond(const DevParams& P, float3 ri, float3 rj, float3& f)
{
    float3 dr = subv<D>(rj, ri);
    min_image_near<D>(P, dr);
    const float q = dotv<D>(dr, dr);
    const float ir = rsqrtf(q);
    const float fm = -(P.bond_k * (sqrt_nr(q, ir) - P.bond_r0)) * ir;
    sub_scaled<D>(f, fm, dr);
}

// Archived tangent drive (NWWormsKernel_DriveForce.h:21-34): F_act along
// the unit vector to the next bead.
template <int D = 3>
__device__ __forceinline__ void wca_drive(const DevParams& P, float3 ri, float3 rn, float3& f)
{
    float3 dr = subv<D>(rn, ri);
    min_image_near<D>(P, dr);
    const float s = P.activity * rsqrtf(dotv<D>(dr, dr));
    f.x += s * dr.x;
    f.y += s * dr.y;
    if constexpr (D == 3) f.z += s * dr.z;
}

// The bond to the next bead and the drive along it share one separation
// and one reciprocal square root.
template <int D = 3>
__device__ __forceinline__ void wca_bond_drive(const DevParams& P, float3 ri, float3 rn, float3& f)
{
    float3 dr = subv<D>(rn, ri);
    min_image_near<D>(P, dr);
    const float q = dotv<D>(dr, dr);
    const float ir = rsqrtf(q);
    const float fm = -(P.bond_k * (sqrt_nr(q, ir) - P.bond_r0)) * ir;
    const float s = P.activity * ir;
    f.x += s * dr.x - fm * dr.x;
    f.y += s * dr.y - fm * dr.y;
    if constexpr (D == 3) f.z += s * dr.z - fm * dr.z;
}

// Repulsive LJ magnitude of NWWormsKernel_LennardJones.h:38-50,
// 24 eps s^6 (2 s^6 / r^14 - 1 / r^8), from one reciprocal of r^2.
__device__ __forceinline__ float wca_lj(const DevParams& P, float rr)
{
    const float ir = rcp_nr(rr);
    const float ir2 = ir * ir;
    const float ir4 = ir2 * ir2;
    return P.lj_amp * (P.lj_two_s6 * (ir4 * ir2 * ir) - ir4);
}

// Same-filament pairs closer than lj_exclude along the chain take no LJ
// force; fbase = first bead of bead i's filament.
__device__ __forceinline__ bool lj_excluded(const DevParams& P, uint32_t i, uint32_t j, uint32_t fbase)
{
    const int d = (int)j - (int)i;
    return d <= P.lj_exclude && d >= -P.lj_exclude && j - fbase < P.L;
}

// ---- K1: filament pass ---------------------------------------------------------
// A block owns `fpb` whole filaments (beads [w0*L, (w0+fpb)*L) in storage
// order), so reversal and every bonded term stay inside the block's shared
// memory.  Follows ParticleSystem::update steps integrate -> reverse ->
// Langevin -> filamentForces -> calcHash (simulation/particleSystem.cpp:257-299).
__global__ void __launch_bounds__(1024) filament_pass_kernel(const DevParams P, const StepBuffers S, uint32_t step_off,
                                                             float dt, uint32_t fpb);

// ---- K2: cell scan ---------------------------------------------------------------
// Block b scans cells [b*4096, (b+1)*4096); the totals of all earlier chunks
// come from chunk_sum_kernel, so no block waits on another.
// offset[c] = exclusive prefix, offset[ncells] = total; start/end in the
// reference's format (0xffffffff for empty cells); counts are reset to zero.
// A grid two blocks high scans a second array (count2, chunk_count2 ->
// offset2; no bounds) in its second row.
template <bool kBounds>
__global__ void __launch_bounds__(512) scan_cells_kernel(uint32_t* __restrict__ count,
                                                         const uint32_t* __restrict__ chunk_count, uint32_t ncells,
                                                         uint32_t* __restrict__ offset, uint32_t* __restrict__ start,
                                                         uint32_t* __restrict__ end, uint32_t* __restrict__ count2,
                                                         const uint32_t* __restrict__ chunk_count2,
                                                         uint32_t* __restrict__ offset2)
{
    if (blockIdx.y) {
        count = count2;
        chunk_count = chunk_count2;
        offset = offset2;
    }
    const bool bounds = kBounds && blockIdx.y == 0;
    __shared__ uint32_t s_w[16];
    __shared__ uint32_t s_base;
    const uint32_t b = blockIdx.x, tid = threadIdx.x, lane = tid & 31u, wid = tid >> 5;
    uint32_t part = 0;
    for (uint32_t k = tid; k < b; k += 512u) part += chunk_count[k];
    part = warp_sum(part);
    if (lane == 0) s_w[wid] = part;
    __syncthreads();
    if (wid == 0) {
        uint32_t x = lane < 16u ? s_w[lane] : 0u;
        x = warp_sum(x);
        if (lane == 0) s_base = x;
    }
    __syncthreads();
    const uint32_t base = s_base;
    __syncthreads();

    const uint32_t c0 = b * kChunk + tid * 8u;
    uint32_t cnt[8];
    uint32_t tot = 0;
    if (c0 + 8u <= ncells) {
        const uint4 a = *reinterpret_cast<const uint4*>(count + c0);
        const uint4 d = *reinterpret_cast<const uint4*>(count + c0 + 4);
        cnt[0] = a.x; cnt[1] = a.y; cnt[2] = a.z; cnt[3] = a.w;
        cnt[4] = d.x; cnt[5] = d.y; cnt[6] = d.z; cnt[7] = d.w;
    } else {
#pragma unroll
        for (int k = 0; k < 8; ++k) cnt[k] = (c0 + k < ncells) ? count[c0 + k] : 0u;
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) tot += cnt[k];
    const uint32_t incl = warp_incl_scan(tot);
    if (lane == 31u) s_w[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        const uint32_t x = lane < 16u ? s_w[lane] : 0u;
        const uint32_t xi = warp_incl_scan(x);
        if (lane < 16u) s_w[lane] = xi - x;
    }
    __syncthreads();
    uint32_t run = base + s_w[wid] + incl - tot;
    if (c0 + 8u <= ncells) {
        uint32_t o[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            o[k] = run;
            run += cnt[k];
        }
        *reinterpret_cast<uint4*>(offset + c0) = make_uint4(o[0], o[1], o[2], o[3]);
        *reinterpret_cast<uint4*>(offset + c0 + 4) = make_uint4(o[4], o[5], o[6], o[7]);
        if (bounds) {
            uint32_t s[8], e[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                s[k] = cnt[k] ? o[k] : kEmpty;
                e[k] = cnt[k] ? o[k] + cnt[k] : kEmpty;
            }
            *reinterpret_cast<uint4*>(start + c0) = make_uint4(s[0], s[1], s[2], s[3]);
            *reinterpret_cast<uint4*>(start + c0 + 4) = make_uint4(s[4], s[5], s[6], s[7]);
            *reinterpret_cast<uint4*>(end + c0) = make_uint4(e[0], e[1], e[2], e[3]);
            *reinterpret_cast<uint4*>(end + c0 + 4) = make_uint4(e[4], e[5], e[6], e[7]);
        }
        *reinterpret_cast<uint4*>(count + c0) = make_uint4(0u, 0u, 0u, 0u);
        *reinterpret_cast<uint4*>(count + c0 + 4) = make_uint4(0u, 0u, 0u, 0u);
    } else {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const uint32_t c = c0 + k;
            if (c < ncells) {
                offset[c] = run;
                if (bounds) {
                    start[c] = cnt[k] ? run : kEmpty;
                    end[c] = cnt[k] ? run + cnt[k] : kEmpty;
                }
                count[c] = 0u;
            }
            run += cnt[k];
        }
    }
    if (c0 < ncells && c0 + 8u >= ncells) offset[ncells] = run;
}

// Sum of each 4096-entry chunk of the cell counts (feeds scan_cells_kernel,
// whose blocks then need no communication with one another).  A grid two
// blocks high does a second array (a2 -> chunk2) in its second row.
__global__ void __launch_bounds__(512) chunk_sum_kernel(const uint32_t* __restrict__ a, uint32_t m,
                                                        uint32_t* __restrict__ chunk, const uint32_t* __restrict__ a2,
                                                        uint32_t* __restrict__ chunk2);

// ---- K3: scatter into cell buckets (arbitrary order inside a bucket) -------------
__global__ void __launch_bounds__(256) scatter_kernel(const uint32_t* __restrict__ hash,
                                                      const uint32_t* __restrict__ slot,
                                                      const uint32_t* __restrict__ offset, uint32_t* __restrict__ tmp,
                                                      uint32_t n);

// Rank of element `i` among the members of its bucket (= stable position).
__device__ __forceinline__ uint32_t bucket_rank(const uint32_t* __restrict__ tmp, uint32_t lo, uint32_t hi, uint32_t i,
                                                uint32_t q, uint32_t* err)
{
    if (hi - lo > kStableCap) {
        if (q == lo) atomicOr(err, (uint32_t)NW_EFLAG_CELL_OVERFLOW);
        return q - lo;
    }
    uint32_t r = 0;
    for (uint32_t k = lo; k < hi; ++k) r += tmp[k] < i;
    return r;
}

// ---- K4: stable order + gather ---------------------------------------------------
// Completes the stable sort (thrust::sort_by_key order: by hash, ties by
// index) and performs reorderDataAndFindCellStartD's gather
// (particles_kernel_impl.cuh:406-420).
template <bool kRef>
__global__ void __launch_bounds__(256) stable_gather_kernel(const DevParams P, const StepBuffers S)
{
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= P.nb) return;
    const uint32_t i = S.tmp_index[q];
    const uint32_t h = S.hash[i];
    const uint32_t lo = S.cell_offset[h], hi = S.cell_offset[h + 1];
    const uint32_t d = lo + bucket_rank(S.tmp_index, lo, hi, i, q, S.err);
    S.sorted_index[d] = i;
    S.sorted_hash[d] = h;
    S.sorted_pos[d] = S.pos[i];
    if (kRef) {
        S.sorted_vel[d] = S.vel[i];
        S.sorted_tan[d] = S.tangent[i];
    }
}

// ---- K5: pair forces ---------------------------------------------------------------

// Member range [s0, s1) of cell h, checked against the particle count (cell
// bounds handed in through the legacy C ABI are caller data); false if empty.
__device__ __forceinline__ bool cell_range(const DevParams& P, const StepBuffers& S, uint32_t h, uint32_t& s0,
                                           uint32_t& s1)
{
    s0 = __ldg(&S.cell_start[h]);
    if (s0 == kEmpty) return false;
    s1 = __ldg(&S.cell_end[h]);
    if (s0 >= P.nb || s1 > P.nb || s1 < s0) {
        atomicOr(S.err, (uint32_t)NW_EFLAG_BAD_INDEX);
        return false;
    }
    if (s1 - s0 > kPairCap) {
        atomicOr(S.err, (uint32_t)NW_EFLAG_CELL_OVERFLOW);
        s1 = s0 + kPairCap;
    }
    return true;
}

// collideCell for one neighbour cell (particles_kernel_impl.cuh:492-556).
__device__ __forceinline__ float3 ref_cell_sum(const DevParams& P, const StepBuffers& S, uint32_t h, uint32_t p,
                                               float3 r, float3 v, float3 t, uint32_t fI, uint32_t cI)
{
    float3 sum = zero3();
    uint32_t s0, s1;
    if (!cell_range(P, S, h, s0, s1)) return sum;
    const float cd = P.radius + P.radius;
    for (uint32_t j = s0; j < s1; ++j) {
        if (j == p) continue;
        const float3 r2 = f3(__ldg(&S.sorted_pos[j]));
        const float3 v2 = f3(__ldg(&S.sorted_vel[j]));
        const float3 t2 = f3(__ldg(&S.sorted_tan[j]));
        const uint32_t o = __ldg(&S.sorted_index[j]);
        const uint32_t fJ = o / P.L, cJ = o - fJ * P.L;
        const bool same = fI == fJ;
        if (same && ((cI + 1u == cJ) || (cI - 1u == cJ))) {
            // bondHookean (:466-473)
            float3 rel = r2 - r;
            const float d = min_image_len(P, rel);
            const float3 n = rel / d;
            sum += (-P.bond_k * (P.bond_r0 - d)) * n;
        } else {
            // collideParticles (:427-462)
            float3 rel = r2 - r;
            const float d = min_image_len(P, rel);
            if (d < cd) {
                const float3 n = rel / d;
                const float3 rv = v2 - v;
                const float3 tv = rv - dot3(rv, n) * n;
                float3 F = (-P.spring * (cd - d)) * n;
                F += P.damping * rv;
                F += P.shear * tv;
                sum += F;
            }
        }
        if (!same) {
            // extensileForce (:477-487)
            float3 rel = r2 - r;
            const float d = min_image_len(P, rel);
            if (dot3(t, t2) < -0.5f) sum += ((-P.activity) * (t - t2)) / (2.0f * d);
        }
    }
    return sum;
}

// REF_DEM: collideFilamentsKernel (particles_kernel_impl.cuh:694-744).  With a
// single z layer every (x, y) neighbour cell is reached by all three z
// offsets; its sum is computed once and added three times in the reference's
// z, y, x order, which reproduces the reference's accumulation exactly.
__global__ void __launch_bounds__(256) pair_ref_kernel(const DevParams P, const StepBuffers S);

// REF_DEM pair pass over tiles of kRefTX x kRefTY cells of a single z layer
// (layout in nw_kernels.cu).  Grid: ceil(gx / kRefTX) * ceil(gy / kRefTY)
// blocks of kRefThreads with kRefSmem bytes of dynamic shared memory (above
// the default 48 KB: the kernel's attribute is raised when a system is made).
constexpr uint32_t kRefTX = 32, kRefTY = 4, kRefG = 4, kRefThreads = 256;
constexpr uint32_t kRefHX = kRefTX + 2, kRefHalo = kRefHX * (kRefTY + 2);
constexpr uint32_t kRefStage = 1024;
constexpr size_t kRefSmem = (size_t)kRefStage * (3 * 16 + 2 * 4) + (size_t)(2 * kRefHalo + 1) * 4;
static_assert(kRefHalo <= kRefThreads, "one thread per halo cell");
static_assert(32 % kRefG == 0, "lane groups within a warp");
__global__ void __launch_bounds__(kRefThreads) pair_ref_tiled_kernel(const DevParams P, const StepBuffers S);

// Neighbour cell c + o (o in -1..1) of an axis of G cells as the
// distinct-cell visit takes it: wrapped on periodic axes, absent beyond a
// wall, and absent when an earlier offset already gave the same cell
// (possible only with fewer than three cells on the axis).
__device__ __forceinline__ bool nb_cell(int G, bool per, uint32_t c, int o, uint32_t& out)
{
    auto at = [&](int oo, int& x) -> bool {
        x = (int)c + oo;
        if (per) {
            if (x < 0) x += G;
            else if (x >= G) x -= G;
            return true;
        }
        return x >= 0 && x < G;
    };
    int x;
    if (!at(o, x)) return false;
    if (G < 3) {
        for (int q = -1; q < o; ++q) {
            int y;
            if (at(q, y) && y == x) return false;
        }
    }
    out = (uint32_t)x;
    return true;
}

// visit(h) for every distinct neighbour cell h of a bead at r whose own
// cell hash is `own`, in the reference's z, y, x order.  kList selects the
// per-step list grid (the Verlet grid when vl_on) instead of the reference
// grid.
template <bool kList, class Visit>
__device__ __forceinline__ void for_neighbour_cells(const DevParams& P, float3 r, uint32_t own, Visit visit)
{
    const bool coarse = kList && P.vl_on;
    const uint32_t G0 = coarse ? P.lgrid[0] : P.grid[0];
    const uint32_t G1 = coarse ? P.lgrid[1] : P.grid[1];
    const uint32_t G2 = coarse ? P.lgrid[2] : P.grid[2];
    uint32_t c0, c1, c2 = 0;
    if (!coarse && P.hash_mode == NW_HASH_MASK) {
        const int3 g = grid_pos(P, r);
        c0 = cell_coord(P, 0, g.x);
        c1 = cell_coord(P, 1, g.y);
        c2 = cell_coord(P, 2, g.z);
    } else {
        // modulo/clamp hash h = (c2 * G1 + c1) * G0 + c0, divided by multiply-shift
        uint32_t rest = own;
        if (G2 > 1u) {
            c2 = fast_div(own, coarse ? P.ldiv_xy_m : P.div_gxy_m, coarse ? P.ldiv_xy_k : P.div_gxy_k);
            rest = own - c2 * (G0 * G1);
        }
        c1 = fast_div(rest, coarse ? P.ldiv_x_m : P.div_gx_m, coarse ? P.ldiv_x_k : P.div_gx_k);
        c0 = rest - c1 * G0;
    }
#pragma unroll 1
    for (int dz = -1; dz <= 1; ++dz) {
        uint32_t z;
        if (!nb_cell((int)G2, P.bnd[2] == NW_PERIODIC, c2, dz, z)) continue;
#pragma unroll 1
        for (int dy = -1; dy <= 1; ++dy) {
            uint32_t y;
            if (!nb_cell((int)G1, P.bnd[1] == NW_PERIODIC, c1, dy, y)) continue;
            const uint32_t row = (z * G1 + y) * G0;
#pragma unroll 1
            for (int dx = -1; dx <= 1; ++dx) {
                uint32_t x;
                if (!nb_cell((int)G0, P.bnd[0] == NW_PERIODIC, c0, dx, x)) continue;
                visit(row + x);
            }
        }
    }
}

// WCA_WORMS pair pass: repulsive LJ to every bead within lj_rcut in the
// distinct neighbour cells, except same-filament pairs |i - j| <= lj_exclude
// (NWWormsKernel_LennardJones.h:38-50, NWWormsKernel_InternalForce.h:196-208,
// NWDeviceFunctions.h:73-76).
__global__ void __launch_bounds__(256) pair_wca_kernel(const DevParams P, const StepBuffers S);

// ---- SRD -------------------------------------------------------------------------

// Random grid shift of the collision at `step`: (lo + U) * cell per axis,
// no z shift in 2D (the reference draws frand() * cell for x and y,
// simulation/particleSystem.cpp:345-346).
__device__ __forceinline__ float3 srd_shift_of(const DevParams& P, unsigned long long step)
{
    const uint4 x = rng_draw(P, 0u, step, kRngSrdShift);
    return make_float3((P.srd_shift_lo + u01(x.x)) * P.srd_cell[0], (P.srd_shift_lo + u01(x.y)) * P.srd_cell[1],
                       P.dim >= 3 ? (P.srd_shift_lo + u01(x.z)) * P.srd_cell[2] : 0.0f);
}

// calcHashD(srd = true) over beads and solvent + counting-sort slot.
__global__ void __launch_bounds__(256) srd_hash_kernel(const DevParams P, const StepBuffers S, uint32_t step_off,
                                                       int shift_from_step, float3 shift, uint32_t buf_sel);

// SRD collision, a warp per 32 consecutive cells staged in shared memory,
// one cell per thread: members in stable (index) order, then the reference's
// isokinetic thermostat (particles_kernel_impl.cuh:605-637) or none, the
// mass-weighted cell mean (:560-594), the +/- alpha rotation of (v - u)
// (:640-691), the relative-velocity thermostat when selected, and the
// solvent's ballistic streaming by dt_srd (solvent_integrator, :145-205).
__global__ void __launch_bounds__(128, 8) srd_collide_kernel(const DevParams P, const StepBuffers S, uint32_t step_off,
                                                             float dt_srd, uint32_t buf_sel);

__global__ void __launch_bounds__(256) srd_scatter_kernel(const DevParams P, const StepBuffers S);
// One warp per SRD cell of the srd_big list (grid-stride over the list).
__global__ void __launch_bounds__(128) srd_collide_big_kernel(const DevParams P, const StepBuffers S,
                                                              uint32_t step_off, float dt_srd, uint32_t buf_sel);
// Tuning of the collision's two paths (overridable at compile time):
// blocks of srd_collide_big_kernel, and the largest cell one lane of
// srd_collide_kernel collides (larger cells go to the warp-per-cell kernel).
#ifndef NW_SRD_BIG_BLOCKS
#define NW_SRD_BIG_BLOCKS 912  // 6 blocks per SM (its shared memory allows 6, its registers 7)
#endif
#ifndef NW_SRD_LANE_CAP
#define NW_SRD_LANE_CAP 16
#endif
constexpr uint32_t kSrdBigBlocks = NW_SRD_BIG_BLOCKS;
constexpr uint32_t kLaneCap = NW_SRD_LANE_CAP;  // members of a cell collided by one lane of srd_collide_kernel
constexpr uint32_t kBigWarps = 4;        // warps (cells at a time) per block of srd_collide_big_kernel
constexpr uint32_t kBigCap = 384;        // members of a cell ordered exactly by srd_collide_big_kernel
__global__ void srd_flip_kernel(uint32_t* scur);

__global__ void advance_step_kernel(unsigned long long* step_base, unsigned long long k);

}  // namespace nw
