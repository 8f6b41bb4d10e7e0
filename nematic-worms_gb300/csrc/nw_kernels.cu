// nw_kernels.cu — definitions of the non-template step kernels declared in
// nw_kernels.cuh (one translation unit owns each kernel).
#include "nw_kernels.cuh"

namespace nw {

namespace {

// The filament pass with D vector components (D = 2: planar systems).
template <int D>
__device__ __forceinline__ void filament_pass(const DevParams& P, const StepBuffers& S, uint32_t step_off, float dt,
                                              uint32_t fpb)
{
    extern __shared__ float4 sm[];
    const uint32_t L = P.L;
    const uint32_t beads = fpb * L;
    const uint32_t t = threadIdx.x;
    const uint32_t w0 = blockIdx.x * fpb;
    const uint32_t i = w0 * L + t;
    const bool active = t < beads && i < P.nb;
    const unsigned long long step = *S.step_base + step_off;

    float4 nP = make_float4(0.f, 0.f, 0.f, 0.f), nV = nP, nFo = nP;
    if (active) {
        const float4 P4 = S.pos[i], V4 = S.vel[i], F4 = S.force[i], Fo4 = S.force_old[i];
        float3 p = f3(P4), v = f3(V4);
        const float3 f = f3(F4), fo = f3(Fo4);
        // velocity Verlet (particles_kernel_impl.cuh:93-97), per axis
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
        apply_boundaries<D>(P, p, v, dr, P.radius);
        nP = make_float4(p.x, p.y, p.z, P4.w);
        nV = make_float4(v.x, v.y, v.z, V4.w);
        nFo = make_float4(f.x, f.y, D == 3 ? f.z : 0.f, Fo4.w);
    }
    if (P.reverse_on) {
        // reverseFilamentsKernel (particles_kernel_impl.cuh:820-857)
        if (active) {
            sm[t] = nP;
            sm[beads + t] = nV;
            sm[2 * beads + t] = nFo;
        }
        __syncthreads();
        if (active) {
            const uint32_t wl = t / L, c = t - wl * L;
            const float u = u01(rng_draw(P, w0 + wl, step, kRngReverse).x);
            if (u <= P.reverse_p) {
                const uint32_t src = wl * L + (L - 1u - c);
                nP = sm[src];
                nV = sm[beads + src];
                nFo = sm[2 * beads + src];
            }
        }
        __syncthreads();
    }
    if (active) sm[t] = nP;
    __syncthreads();
    if (!active) return;

    const uint32_t wl = t / L, c = t - wl * L;
    const float4* R = sm + wl * L;
    float3 fs = zero3();
    if (P.langevin_on) {
        // langevinKernel (particles_kernel_impl.cuh:859-874), Philox noise in registers
        const float3 g = noise3(P, rng_draw(P, i, step, kRngLangevin));
        float3 fl = zero3() - P.gamma * f3(nV);
        fl += g;
        fs = D == 3 ? fl : make_float3(fl.x, fl.y, 0.f);
    }
    // bending contributions in the reference's triple order p = c-2, c-1, c
    if (L >= 3) {
        if (c >= 2) fs = addv<D>(fs, bend_triple<D>(P, f3(R[c - 2]), f3(R[c - 1]), f3(R[c])).fk);
        if (c >= 1 && c + 1 < L) fs = addv<D>(fs, bend_triple<D>(P, f3(R[c - 1]), f3(R[c]), f3(R[c + 1])).fj);
        if (c + 2 < L) fs = addv<D>(fs, bend_triple<D>(P, f3(R[c]), f3(R[c + 1]), f3(R[c + 2])).fi);
    }
    bool wt = false;
    float3 tg = zero3();
    if (L >= 3) {
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
    S.pos[i] = nP;
    S.vel[i] = nV;
    S.force_old[i] = nFo;
    S.force[i] = make_float4(fs.x, fs.y, fs.z, 0.f);
    if (wt) S.tangent[i] = make_float4(tg.x, tg.y, tg.z, 0.f);
    if (!finitev<D>(f3(nP)) || !finitev<D>(fs)) atomicOr(S.err, (uint32_t)NW_EFLAG_NONFINITE);

    const uint32_t h = bead_hash(P, f3(nP));
    S.hash[i] = h;
    S.slot[i] = count_into_cell(S.cell_count, h);
}

}  // namespace

__global__ void __launch_bounds__(1024) filament_pass_kernel(const DevParams P, const StepBuffers S, uint32_t step_off,
                                                             float dt, uint32_t fpb)
{
    if (planar_system(P)) filament_pass<2>(P, S, step_off, dt, fpb);
    else filament_pass<3>(P, S, step_off, dt, fpb);
}

__global__ void __launch_bounds__(512) chunk_sum_kernel(const uint32_t* __restrict__ a, uint32_t m,
                                                        uint32_t* __restrict__ chunk, const uint32_t* __restrict__ a2,
                                                        uint32_t* __restrict__ chunk2)
{
    if (blockIdx.y) {
        a = a2;
        chunk = chunk2;
    }
    __shared__ uint32_t s_w[16];
    const uint32_t c0 = blockIdx.x * kChunk;
    uint32_t x = 0;
    if (c0 + kChunk <= m) {
        const uint4* v = reinterpret_cast<const uint4*>(a + c0);
        for (uint32_t k = threadIdx.x; k < kChunk / 4u; k += 512u) {
            const uint4 q = v[k];
            x += q.x + q.y + q.z + q.w;
        }
    } else {
        for (uint32_t k = threadIdx.x; k < kChunk; k += 512u)
            if (c0 + k < m) x += a[c0 + k];
    }
    x = warp_sum(x);
    if ((threadIdx.x & 31u) == 0) s_w[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x < 32) {
        uint32_t y = threadIdx.x < 16 ? s_w[threadIdx.x] : 0u;
        y = warp_sum(y);
        if (threadIdx.x == 0) chunk[blockIdx.x] = y;
    }
}

__global__ void __launch_bounds__(256) scatter_kernel(const uint32_t* __restrict__ hash,
                                                      const uint32_t* __restrict__ slot,
                                                      const uint32_t* __restrict__ offset, uint32_t* __restrict__ tmp,
                                                      uint32_t n)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) tmp[offset[hash[i]] + slot[i]] = i;
}

// collideFilamentsKernel's force on the bead at sorted position p, from the
// sorted arrays in global memory (added to force[original index]).
__device__ __forceinline__ void ref_pair_bead(const DevParams& P, const StepBuffers& S, uint32_t p)
{
    const float3 r = f3(S.sorted_pos[p]);
    const float3 v = f3(S.sorted_vel[p]);
    const float3 t = f3(S.sorted_tan[p]);
    const int3 g = grid_pos(P, r);
    const uint32_t me = S.sorted_index[p];
    if (me >= P.nb) {
        atomicOr(S.err, (uint32_t)NW_EFLAG_BAD_INDEX);
        return;
    }
    const uint32_t fI = me / P.L, cI = me - fI * P.L;
    float3 total = zero3();
    if (P.grid[2] == 1u) {
        float3 cs[9];
#pragma unroll
        for (int y = -1; y <= 1; ++y)
#pragma unroll
            for (int x = -1; x <= 1; ++x) {
                const uint32_t h = cell_hash(P, cell_coord(P, 0, g.x + x), cell_coord(P, 1, g.y + y), cell_coord(P, 2, g.z));
                cs[(y + 1) * 3 + (x + 1)] = ref_cell_sum(P, S, h, p, r, v, t, fI, cI);
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
                    total += ref_cell_sum(P, S, h, p, r, v, t, fI, cI);
                }
    }
    float4 F = S.force[me];
    F.x += total.x;
    F.y += total.y;
    F.z += total.z;
    S.force[me] = F;
    if (!finite3(f3(F))) atomicOr(S.err, (uint32_t)NW_EFLAG_NONFINITE);
}

__global__ void __launch_bounds__(256) pair_ref_kernel(const DevParams P, const StepBuffers S)
{
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < P.nb) ref_pair_bead(P, S, p);
}

// ---- REF_DEM pair pass, cell-tiled (single z layer) ---------------------------
//
// The thread-per-bead form above (the reference's own layout) spends most of
// its issue slots on divergence: each lane walks 27 cells of 0-2 members and
// branches per member (8 of 32 lanes active in the reference's kernel on the
// 400k-bead lattice).  Here a block takes a tile of kRefTX x kRefTY cells of
// the sorted order, stages the members of the tile and its one-cell halo
// (pos, vel, tangent, original index and filament) in shared memory with
// coalesced loads, and gives each central bead a group of kRefG lanes that
// stride over its candidates: the members of the 3 x 3 halo cells around its
// own, which lie in three contiguous runs of the staged arrays (one per halo
// row, cells x-1 .. x+1).  The group's partial sums are combined by shuffles
// in a fixed order, so results do not depend on scheduling.  With one z layer
// every (x, y) neighbour cell is reached by the reference's three z offsets,
// so the bead's sum is added three times; a cell reached by two x or y offsets
// (grids narrower than 3 cells) appears twice in the halo and is summed twice,
// as in the reference.  A tile whose halo holds more than kRefStage members
// takes the thread-per-bead form.  Same pair laws as collideCell
// (particles_kernel_impl.cuh:427-556), with the divisions by the separation
// taken from a Newton-refined reciprocal.

__device__ __forceinline__ float3 ref_pair_law(const DevParams& P, float3 r, float3 v, float3 t, float3 r2, float3 v2,
                                               float3 t2, bool same, bool bonded)
{
    float3 rel = r2 - r;
    min_image(P, rel);
    const float q = dot3(rel, rel);
    const float d = sqrt_nr(q, rsqrtf(q));
    const float id = rcp_nr(d);
    const float3 n = rel * id;
    float3 F = zero3();
    const float cd = P.radius + P.radius;
    if (bonded) {
        // bondHookean (:466-473)
        F = (-P.bond_k * (P.bond_r0 - d)) * n;
    } else if (d < cd) {
        // collideParticles (:427-462)
        const float3 rv = v2 - v;
        const float3 tv = rv - dot3(rv, n) * n;
        F = (-P.spring * (cd - d)) * n;
        F += P.damping * rv;
        F += P.shear * tv;
    }
    // extensileForce (:477-487): other filaments, anti-aligned tangents
    if (!same && dot3(t, t2) < -0.5f) F += ((-P.activity) * (t - t2)) * (0.5f * id);
    return F;
}

__global__ void __launch_bounds__(kRefThreads) pair_ref_tiled_kernel(const DevParams P, const StepBuffers S)
{
    extern __shared__ float4 smr[];
    float4* spos = smr;
    float4* svel = spos + kRefStage;
    float4* stan = svel + kRefStage;
    uint32_t* sidx = reinterpret_cast<uint32_t*>(stan + kRefStage);  // original index
    uint32_t* sfil = sidx + kRefStage;                               // its filament
    uint32_t* soff = sfil + kRefStage;                               // kRefHalo + 1 staged offsets
    uint32_t* sbeg = soff + kRefHalo + 1;                            // sorted start of each halo cell
    __shared__ uint32_t s_total, s_bad;
    __shared__ uint32_t wsum[kRefThreads / 32];

    const uint32_t tid = threadIdx.x;
    const uint32_t tiles_x = (P.grid[0] + kRefTX - 1) / kRefTX;
    const int x0 = (int)((blockIdx.x % tiles_x) * kRefTX);
    const int y0 = (int)((blockIdx.x / tiles_x) * kRefTY);

    // 1. member counts of the halo cells (halo row-major), exclusive scan
    uint32_t cnt = 0, beg = 0;
    if (tid < kRefHalo) {
        const int hx = (int)(tid % kRefHX), hy = (int)(tid / kRefHX);
        const uint32_t h = cell_hash(P, cell_coord(P, 0, x0 + hx - 1), cell_coord(P, 1, y0 + hy - 1), 0u);
        uint32_t s1;
        if (cell_range(P, S, h, beg, s1)) cnt = s1 - beg;
    }
    const uint32_t lane = tid & 31u, warp = tid >> 5;
    const uint32_t inc = warp_incl_scan(cnt);
    if (lane == 31u) wsum[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < kRefThreads / 32 ? wsum[lane] : 0u;
        w = warp_incl_scan(w);
        if (lane < kRefThreads / 32) wsum[lane] = w;
    }
    __syncthreads();
    const uint32_t excl = inc - cnt + (warp ? wsum[warp - 1] : 0u);
    if (tid < kRefHalo) {
        soff[tid] = excl;
        sbeg[tid] = beg;
    }
    if (tid == kRefThreads - 1) {
        s_total = excl + cnt;
        soff[kRefHalo] = excl + cnt;
        s_bad = 0u;
    }
    __syncthreads();
    const uint32_t total = s_total;
    if (total > kRefStage) {
        // crowded tile: the thread-per-bead form for its central cells
        for (uint32_t hy = 1; hy <= kRefTY; ++hy) {
            if (y0 + (int)hy - 1 >= (int)P.grid[1]) break;
            for (uint32_t hx = 1 + warp; hx <= kRefTX; hx += kRefThreads / 32) {
                if (x0 + (int)hx - 1 >= (int)P.grid[0]) break;
                const uint32_t c = hy * kRefHX + hx;
                const uint32_t n = soff[c + 1] - soff[c], b = sbeg[c];
                for (uint32_t k = lane; k < n; k += 32u) ref_pair_bead(P, S, b + k);
            }
        }
        return;
    }
    // 2. stage the members: element e of halo cell c is sorted position sbeg[c] + e - soff[c]
    for (uint32_t e = tid; e < total; e += kRefThreads) {
        uint32_t lo = 0, hi = kRefHalo;  // the last c with soff[c] <= e
        while (hi - lo > 1u) {
            const uint32_t mid = (lo + hi) >> 1;
            if (soff[mid] <= e) lo = mid;
            else hi = mid;
        }
        const uint32_t j = sbeg[lo] + (e - soff[lo]);
        spos[e] = __ldg(&S.sorted_pos[j]);
        svel[e] = __ldg(&S.sorted_vel[j]);
        stan[e] = __ldg(&S.sorted_tan[j]);
        const uint32_t o = __ldg(&S.sorted_index[j]);
        if (o >= P.nb) s_bad = 1u;
        sidx[e] = o;
        sfil[e] = o / P.L;
    }
    __syncthreads();
    if (s_bad) {
        if (tid == 0) atomicOr(S.err, (uint32_t)NW_EFLAG_BAD_INDEX);
        return;
    }
    // 3. central beads (cells of the tile inside the grid), kRefG lanes each
    uint32_t row_lo[kRefTY], row_n[kRefTY], nc = 0;
    const uint32_t nx = (uint32_t)max(0, min((int)kRefTX, (int)P.grid[0] - x0));
#pragma unroll
    for (uint32_t r = 0; r < kRefTY; ++r) {
        const uint32_t hy = r + 1;
        const uint32_t w = y0 + (int)hy - 1 < (int)P.grid[1] ? nx : 0u;
        row_lo[r] = soff[hy * kRefHX + 1];
        row_n[r] = soff[hy * kRefHX + 1 + w] - row_lo[r];
        nc += row_n[r];
    }
    constexpr uint32_t kBeadsPerPass = kRefThreads / kRefG;
    const uint32_t g = tid % kRefG;
    const uint32_t passes = (nc + kBeadsPerPass - 1) / kBeadsPerPass;
    for (uint32_t pass = 0; pass < passes; ++pass) {
        const uint32_t c0 = pass * kBeadsPerPass + tid / kRefG;
        const bool live = c0 < nc;
        float3 sum = zero3();
        uint32_t q = 0;
        if (live) {
            uint32_t hy = 1, c = c0;
#pragma unroll
            for (uint32_t r = 0; r < kRefTY; ++r) {
                if (c < row_n[r]) {
                    q = row_lo[r] + c;
                    hy = r + 1;
                    break;
                }
                c -= row_n[r];
            }
            // the bead's halo cell: the last cell of its row with soff <= q
            uint32_t lo = hy * kRefHX + 1, hi = hy * kRefHX + kRefTX + 1;
            while (hi - lo > 1u) {
                const uint32_t mid = (lo + hi) >> 1;
                if (soff[mid] <= q) lo = mid;
                else hi = mid;
            }
            const uint32_t hx = lo - hy * kRefHX;
            const float3 r = f3(spos[q]), v = f3(svel[q]), t = f3(stan[q]);
            const uint32_t me = sidx[q], fI = sfil[q], cI = me - fI * P.L;
            const uint32_t a0 = soff[(hy - 1) * kRefHX + hx - 1], n0 = soff[(hy - 1) * kRefHX + hx + 2] - a0;
            const uint32_t a1 = soff[hy * kRefHX + hx - 1], n1 = soff[hy * kRefHX + hx + 2] - a1;
            const uint32_t a2 = soff[(hy + 1) * kRefHX + hx - 1], n2 = soff[(hy + 1) * kRefHX + hx + 2] - a2;
            const uint32_t m = n0 + n1 + n2;
            for (uint32_t k = g; k < m; k += kRefG) {
                const uint32_t j = k < n0 ? a0 + k : (k < n0 + n1 ? a1 + (k - n0) : a2 + (k - n0 - n1));
                const uint32_t o = sidx[j];
                if (o == me) continue;
                const uint32_t fJ = sfil[j], cJ = o - fJ * P.L;
                const bool same = fI == fJ;
                const bool bonded = same && ((cI + 1u == cJ) || (cI - 1u == cJ));
                sum += ref_pair_law(P, r, v, t, f3(spos[j]), f3(svel[j]), f3(stan[j]), same, bonded);
            }
        }
        // fixed-order combination of the group's partial sums
#pragma unroll
        for (uint32_t o = 1; o < kRefG; o <<= 1) {
            sum.x += __shfl_xor_sync(0xffffffffu, sum.x, o, kRefG);
            sum.y += __shfl_xor_sync(0xffffffffu, sum.y, o, kRefG);
            sum.z += __shfl_xor_sync(0xffffffffu, sum.z, o, kRefG);
        }
        if (live && g == 0) {
            const uint32_t me = sidx[q];
            const float3 tot = (sum + sum) + sum;  // the three z offsets of one layer
            float4 F = S.force[me];
            F.x += tot.x;
            F.y += tot.y;
            F.z += tot.z;
            S.force[me] = F;
            if (!finite3(f3(F))) atomicOr(S.err, (uint32_t)NW_EFLAG_NONFINITE);
        }
    }
}

namespace {

// WCA pair forces from the sorted arrays with D vector components.
template <int D>
__device__ __forceinline__ void pair_wca(const DevParams& P, const StepBuffers& S)
{
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.nb) return;
    const float3 r = f3(S.sorted_pos[p]);
    const uint32_t me = S.sorted_index[p];
    if (me >= P.nb) {
        atomicOr(S.err, (uint32_t)NW_EFLAG_BAD_INDEX);
        return;
    }
    const uint32_t fbase = (me / P.L) * P.L;
    float3 f = zero3();
    for_neighbour_cells<false>(P, r, S.sorted_hash[p], [&](uint32_t h) {
        uint32_t s0, s1;
        if (!cell_range(P, S, h, s0, s1)) return;
        for (uint32_t j = s0; j < s1; ++j) {
            if (j == p) continue;
            const uint32_t o = __ldg(&S.sorted_index[j]);
            if (lj_excluded(P, me, o, fbase)) continue;
            float3 dr = subv<D>(f3(__ldg(&S.sorted_pos[j])), r);
            min_image_near<D>(P, dr);
            const float rr = dotv<D>(dr, dr);
            if (rr > P.lj_rc2) continue;
            sub_scaled<D>(f, wca_lj(P, rr), dr);
        }
    });
    float4 F = S.force[me];
    F.x += f.x;
    F.y += f.y;
    if constexpr (D == 3) F.z += f.z;
    S.force[me] = F;
    if (!finitev<D>(f3(F))) atomicOr(S.err, (uint32_t)NW_EFLAG_NONFINITE);
}

}  // namespace

__global__ void __launch_bounds__(256) pair_wca_kernel(const DevParams P, const StepBuffers S)
{
    if (planar_system(P)) pair_wca<2>(P, S);
    else pair_wca<3>(P, S);
}

// SRD cell hash of every particle (beads from the current bead buffer,
// solvent from the current solvent buffer) and its slot in its cell's bead
// or solvent bucket.  The solvent is stored in cell order, so equal keys come
// in runs along the warp: the first lane of each run takes the run's slots
// with one atomic.  The grid shift of a scheduled collision is drawn once per
// block.
__global__ void __launch_bounds__(256) srd_hash_kernel(const DevParams P, const StepBuffers S, uint32_t step_off,
                                                       int shift_from_step, float3 shift, uint32_t buf_sel)
{
    __shared__ float s_shift[3];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < P.ntotal;
    const bool bead = i < P.nb;
    // the step counter and the solvent buffer index side by side, then the
    // particle's position, all before the shift's barrier
    const unsigned long long step = *S.step_base + step_off;
    const uint32_t sc = *S.scur;
    const uint32_t cur = buf_sel < 2u ? buf_sel : (uint32_t)(step & 1ull);
    float4 p4 = make_float4(0.f, 0.f, 0.f, 0.f);
    if (valid) p4 = bead ? S.pos2[cur][i] : S.spos2[sc][i - P.nb];
    if (shift_from_step) {
        if (threadIdx.x == 0) {
            const float3 d = srd_shift_of(P, step);
            s_shift[0] = d.x;
            s_shift[1] = d.y;
            s_shift[2] = d.z;
        }
        __syncthreads();
        shift = make_float3(s_shift[0], s_shift[1], s_shift[2]);
    }
    uint32_t h = 0, key = 0xffffffffu;  // no cell hash reaches 2^31 - 1 with the bead bit set
    if (valid) {
        h = srd_hash(P, f3(p4), shift);
        S.srd_hash[i] = h;
        key = h | (bead ? 0x80000000u : 0u);
    }
    // every lane of the warp takes part (blockDim is a multiple of 32)
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t prev = __shfl_up_sync(0xffffffffu, key, 1);
    const uint32_t heads = __ballot_sync(0xffffffffu, lane == 0u || prev != key);
    const uint32_t upto = (2u << lane) - 1u;  // lanes 0..lane (all 32 bits for lane 31)
    const uint32_t start = 31u - (uint32_t)__clz(heads & upto);
    const uint32_t after = heads & ~upto;
    const uint32_t end = after ? (uint32_t)(__ffs(after) - 1) : 32u;
    uint32_t base = 0;
    if (valid && lane == start) base = atomicAdd(bead ? &S.srd_bcount[h] : &S.srd_scount[h], end - start);
    base = __shfl_sync(0xffffffffu, base, (int)start);
    if (valid) S.srd_slot[i] = base + (lane - start);
}

// Bucket every particle: beads by bead index, solvent by solvent index.
__global__ void __launch_bounds__(256) srd_scatter_kernel(const DevParams P, const StepBuffers S)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.ntotal) return;
    if (i == 0) *S.srd_nbig = 0;  // the list is filled by the collision that follows
    const uint32_t h = S.srd_hash[i], slot = S.srd_slot[i];
    if (i < P.nb) S.srd_btmp[S.srd_boff[h] + slot] = i;
    else S.srd_stmp[S.srd_soff[h] + slot] = i - P.nb;
}

// SRD collision.  A warp owns 32 consecutive cells; their members are one
// contiguous range of the stable (cell, index) order and their solvent one
// contiguous range of the new solvent storage.  So the warp gathers the
// members' velocities and positions lane-strided into shared memory (the
// previous collision's cell order keeps them in a compact region), each
// thread takes its own cell's sums from shared memory, every lane then
// updates the members of its slots, and the warp writes the stable order and
// the streamed solvent back coalesced.
//
// Per cell, in the member order (the cell's beads, then its solvent, each by
// index): the reference's isokinetic scaling (particles_kernel_impl.cuh:605-637)
// or none, the mass-weighted cell mean (:560-594), the +/- alpha rotation of
// (v - u) (:640-691), the relative-velocity thermostat when selected, and the
// solvent's ballistic streaming by dt_srd (solvent_integrator, :145-205).
// Beads are written in place, the solvent to the other solvent buffer.
// A warp holding more than kWarpCap members takes its cells in rounds that
// fit.  A cell of more than kLaneCap members goes to srd_collide_big_kernel
// (a warp per cell), so that no lane's serial loops run far longer than its
// neighbours'.
constexpr int kCollideWarps = 4;
// 192 members per warp (32 cells at up to 6 members on average) keeps
// 8 blocks of 4 warps resident per SM (27 KB of shared memory, 64 registers).
constexpr uint32_t kWarpCap = 192;
static_assert(kLaneCap <= kWarpCap, "a cell of the warp path fits the staging alone");
static_assert(5 * ((kWarpCap + 31) / 32) <= 32, "a lane's slot-to-cell fields fit one register");

__global__ void __launch_bounds__(kCollideWarps * 32, 8) srd_collide_kernel(const DevParams P, const StepBuffers S,
                                                                         uint32_t step_off, float dt_srd,
                                                                         uint32_t buf_sel)
{
    __shared__ uint32_t s_id[kCollideWarps][kWarpCap];
    __shared__ float4 s_v[kCollideWarps][kWarpCap];
    __shared__ float4 s_p[kCollideWarps][kWarpCap];
    const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = c < P.srd_ncells;
    const unsigned long long step = *S.step_base + step_off;
    const uint32_t cur = buf_sel < 2u ? buf_sel : (uint32_t)(step & 1ull);
    const uint32_t a = *S.scur;
    const float4* __restrict__ sv_old = S.svel2[a];
    const float4* __restrict__ sp_old = S.spos2[a];
    float4* __restrict__ sv_new = S.svel2[a ^ 1u];
    float4* __restrict__ sp_new = S.spos2[a ^ 1u];
    float4* __restrict__ bvel = S.vel2[cur];
    uint32_t b0 = 0, nbc = 0, s0 = 0, nsc = 0;
    if (valid) {
        b0 = S.srd_boff[c];
        nbc = S.srd_boff[c + 1] - b0;
        s0 = S.srd_soff[c];
        nsc = S.srd_soff[c + 1] - s0;
    }
    const uint32_t nall = nbc + nsc;
    const uint32_t start = b0 + s0;  // particles before this cell in the stable order
    if (valid) {
        S.srd_start[c] = nall ? start : kEmpty;
        S.srd_end[c] = nall ? start + nall : kEmpty;
    }
    // a cell of more than kLaneCap members is collided by a whole warp in
    // srd_collide_big_kernel; here it counts as empty
    const bool big = nall > kLaneCap;
    if (valid && big) S.srd_big[atomicAdd(S.srd_nbig, 1u)] = c;
    const uint32_t n = big ? 0u : nall;
    const uint32_t incl = warp_incl_scan(n);
    const uint32_t loc = incl - n;  // this cell's members in the warp's staging
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    if (total == 0u) {  // uniform over the warp
        if (valid && !big) S.srd_mean[c] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    const uint32_t gdelta = start - loc;  // stable-order position of staged slot j of this cell: gdelta + j
    // Rounds of consecutive cells whose members fit the staging buffers
    // (one round unless the warp holds more than kWarpCap members).
    uint32_t first = 0;
    while (first < 32u) {
        const uint32_t base = __shfl_sync(0xffffffffu, loc, (int)first);
        const uint32_t fm = __ballot_sync(0xffffffffu, lane >= first && loc + n - base <= kWarpCap);
        const uint32_t last = 31u - (uint32_t)__clz(fm);
        const uint32_t rtotal = __shfl_sync(0xffffffffu, loc + n, (int)last) - base;
        const bool mine = lane >= first && lane <= last;
        // members of the round's cells in stable order: ids < nb are beads, nb + k
        // is solvent k.  The bucket entries are loaded lane-strided (consecutive
        // cells' entries are consecutive in the buckets), each into its cell's
        // segment; then every lane orders its own cell's segment in shared memory.
        // A lane visits the same slots (j0 + lane) in the three loops below, so
        // the cell of each of its (at most kWarpCap / 32 = 6) slots is found once
        // and kept in 5-bit fields of one register.
        uint32_t qpack = 0;
#pragma unroll 2
        for (uint32_t j0 = 0; j0 < rtotal; j0 += 32u) {
            const uint32_t j = j0 + lane, slot = base + (j < rtotal ? j : 0u);
            uint32_t q = 0;  // the last cell whose segment starts at or before slot
#pragma unroll
            for (uint32_t st = 16; st; st >>= 1) {
                const uint32_t lq = __shfl_sync(0xffffffffu, loc, (int)(q + st));
                if (lq <= slot) q += st;
            }
            qpack |= q << (5u * (j0 >> 5));
            const uint32_t lq = __shfl_sync(0xffffffffu, loc, (int)q), nq = __shfl_sync(0xffffffffu, nbc, (int)q);
            const uint32_t bq = __shfl_sync(0xffffffffu, b0, (int)q), sq = __shfl_sync(0xffffffffu, s0, (int)q);
            if (j < rtotal) {
                const uint32_t k = slot - lq;
                s_id[w][j] = k < nq ? S.srd_btmp[bq + k] : P.nb + S.srd_stmp[sq + (k - nq)];
            }
        }
        __syncwarp();
        if (mine) {
            uint32_t* ids = &s_id[w][loc - base];
            for (uint32_t k = 1; k < n; ++k) {  // insertion sort of the cell's segment
                const uint32_t x = ids[k];
                uint32_t m = k;
                while (m > 0 && ids[m - 1] > x) {
                    ids[m] = ids[m - 1];
                    --m;
                }
                ids[m] = x;
            }
        }
        __syncwarp();
        for (uint32_t j0 = 0; j0 < rtotal; j0 += 32u) {
            const uint32_t j = j0 + lane, slot = base + (j < rtotal ? j : 0u);
            const uint32_t q = (qpack >> (5u * (j0 >> 5))) & 31u;  // the cell of slot
            const uint32_t gq = __shfl_sync(0xffffffffu, gdelta, (int)q);
            if (j < rtotal) {
                const uint32_t id = s_id[w][j];
                S.srd_sorted_index[gq + slot] = id;
                if (id < P.nb) {
                    s_v[w][j] = bvel[id];
                } else {
                    s_v[w][j] = sv_old[id - P.nb];
                    s_p[w][j] = sp_old[id - P.nb];
                }
            }
        }
        __syncwarp();
        // per cell, by its lane: [lab isokinetic factor], mean velocity, rotation
        // sign, [relative-velocity thermostat factor]
        const bool lab = P.srd_thermo == NW_SRD_THERMO_REF_LAB;
        const float ca = P.srd_cos_a;
        float3 u = zero3();
        float lam1 = 1.0f, sa = 0.0f, lam2 = 1.0f;
        bool scale2 = false;
        if (mine && n > 0) {
            const uint32_t* ids = &s_id[w][loc - base];
            const float4* V_ = &s_v[w][loc - base];
            float E = 0.f;
            if (lab)
                for (uint32_t k = 0; k < n; ++k) {
                    const float4 V = V_[k];
                    const float3 v = f3(V);
                    E += (0.5f * V.w) * dot3(v, v);
                }
            // reference isokinetic rule: lambda scales every member before the mean
            lam1 = lab ? sqrtf(P.srd_kT / E) : 1.0f;
            float M = 0.f;
            for (uint32_t k = 0; k < n; ++k) {
                const float4 V = V_[k];
                u += V.w * (lab ? make_float3(lam1 * V.x, lam1 * V.y, lam1 * V.z) : f3(V));
                M += V.w;
            }
            if (M > 0.f) {
                const float inv = 1.0f / M;
                u = u * inv;
            }
            // rotation by +alpha or -alpha with equal probability
            const bool plus = u01(rng_draw(P, c, step, kRngSrdRot).x) > 0.5f;
            sa = plus ? P.srd_sin_a : -P.srd_sin_a;
            if (P.srd_thermo == NW_SRD_THERMO_CELL_REL) {
                uint32_t nrot = 0;
                float ke = 0.f;
                for (uint32_t k = 0; k < n; ++k) {
                    if (ids[k] < P.nb && !P.srd_rotate_beads) continue;
                    const float4 V = V_[k];
                    const float3 d = (lab ? make_float3(lam1 * V.x, lam1 * V.y, lam1 * V.z) : f3(V)) - u;
                    const float rx = d.x * ca - d.y * sa;
                    const float ry = d.x * sa + d.y * ca;
                    ke += (0.5f * V.w) * (rx * rx + ry * ry);
                    ++nrot;
                }
                if (nrot >= 2u && ke > 0.f) {
                    lam2 = sqrtf(((float)(nrot - 1u) * P.srd_kT) / ke);
                    scale2 = true;
                }
            }
        }
        // every member updated by the lane of its slot (the cell's factors from
        // the cell's lane): rotation, thermostat, solvent streaming, and the
        // member's destination in the new solvent storage (beads: none)
        __syncwarp();
        for (uint32_t j0 = 0; j0 < rtotal; j0 += 32u) {
            const uint32_t j = j0 + lane, slot = base + (j < rtotal ? j : 0u);
            const uint32_t q = (qpack >> (5u * (j0 >> 5))) & 31u;  // the cell of slot
            const float3 uq = make_float3(__shfl_sync(0xffffffffu, u.x, (int)q), __shfl_sync(0xffffffffu, u.y, (int)q),
                                          __shfl_sync(0xffffffffu, u.z, (int)q));
            const float l1 = __shfl_sync(0xffffffffu, lam1, (int)q), saq = __shfl_sync(0xffffffffu, sa, (int)q);
            const float l2 = __shfl_sync(0xffffffffu, lam2, (int)q);
            const bool sc2 = __shfl_sync(0xffffffffu, (int)scale2, (int)q) != 0;
            const uint32_t lq = __shfl_sync(0xffffffffu, loc, (int)q), nq = __shfl_sync(0xffffffffu, nbc, (int)q);
            const uint32_t sq = __shfl_sync(0xffffffffu, s0, (int)q);
            if (j < rtotal) {
                const uint32_t id = s_id[w][j], k = slot - lq;
                const bool is_bead = id < P.nb;
                const float4 V = s_v[w][j];
                float3 v = lab ? make_float3(l1 * V.x, l1 * V.y, l1 * V.z) : f3(V);
                if (!is_bead || P.srd_rotate_beads) {
                    const float3 d = v - uq;
                    const float rx = d.x * ca - d.y * saq;
                    const float ry = d.x * saq + d.y * ca;
                    v = make_float3(uq.x + rx, uq.y + ry, uq.z + d.z);
                    if (sc2) v = make_float3(uq.x + l2 * (v.x - uq.x), uq.y + l2 * (v.y - uq.y), v.z);
                }
                if (is_bead) {
                    if (lab || P.srd_rotate_beads) bvel[id] = make_float4(v.x, v.y, v.z, V.w);
                    s_id[w][j] = kEmpty;
                } else {
                    const float4 P4 = s_p[w][j];
                    float3 p = f3(P4);
                    const float3 dr = dt_srd * v;
                    p += dr;
                    apply_boundaries(P, p, v, dr, 0.0f);
                    s_p[w][j] = make_float4(p.x, p.y, p.z, P4.w);
                    s_v[w][j] = make_float4(v.x, v.y, v.z, V.w);
                    s_id[w][j] = sq + (k - nq);
                }
            }
        }
        if (mine && valid && !big) S.srd_mean[c] = make_float4(u.x, u.y, u.z, 0.f);
        __syncwarp();
        for (uint32_t k = lane; k < rtotal; k += 32) {
            const uint32_t d = s_id[w][k];
            if (d != kEmpty) {
                sp_new[d] = s_p[w][k];
                sv_new[d] = s_v[w][k];
            }
        }
        __syncwarp();
        first = last + 1u;
    }
}

__device__ __forceinline__ float warp_allsum(float x)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}

// The collision of srd_collide_kernel for one cell of more than kLaneCap
// members, by one warp: members ranked by index in shared memory (the stable
// order; beyond kBigCap members the bucket order, and the overflow is
// reported), velocities gathered once into shared memory, sums as
// lane-strided partials combined by a fixed butterfly (the same result on
// every run), then the per-member update by all lanes.
__global__ void __launch_bounds__(kBigWarps * 32) srd_collide_big_kernel(const DevParams P, const StepBuffers S,
                                                                         uint32_t step_off, float dt_srd,
                                                                         uint32_t buf_sel)
{
    __shared__ uint32_t s_in[kBigWarps][kBigCap];
    __shared__ uint32_t s_id[kBigWarps][kBigCap];
    __shared__ float4 s_v[kBigWarps][kBigCap];
    const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    const uint32_t nbig = *S.srd_nbig;
    const unsigned long long step = *S.step_base + step_off;
    const uint32_t cur = buf_sel < 2u ? buf_sel : (uint32_t)(step & 1ull);
    const uint32_t a = *S.scur;
    const float4* __restrict__ sv_old = S.svel2[a];
    const float4* __restrict__ sp_old = S.spos2[a];
    float4* __restrict__ sv_new = S.svel2[a ^ 1u];
    float4* __restrict__ sp_new = S.spos2[a ^ 1u];
    float4* __restrict__ bvel = S.vel2[cur];
    const bool lab = P.srd_thermo == NW_SRD_THERMO_REF_LAB;
    const bool rel = P.srd_thermo == NW_SRD_THERMO_CELL_REL;
    for (uint32_t q = blockIdx.x * kBigWarps + w; q < nbig; q += gridDim.x * kBigWarps) {
        const uint32_t c = S.srd_big[q];
        const uint32_t b0 = S.srd_boff[c], b1 = S.srd_boff[c + 1];
        const uint32_t s0 = S.srd_soff[c], s1 = S.srd_soff[c + 1];
        const uint32_t nbc = b1 - b0, n = nbc + (s1 - s0);
        const uint32_t start = b0 + s0;
        // beyond kBigCap members: bucket order, reported, bounded work
        const bool fits = n <= kBigCap;
        if (!fits && lane == 0) atomicOr(S.err, (uint32_t)NW_EFLAG_CELL_OVERFLOW);
        auto raw = [&](uint32_t k) -> uint32_t {
            return k < nbc ? S.srd_btmp[b0 + k] : P.nb + S.srd_stmp[s0 + (k - nbc)];
        };
        if (fits) {
            for (uint32_t k = lane; k < n; k += 32) s_in[w][k] = raw(k);
            __syncwarp();
            for (uint32_t k = lane; k < n; k += 32) {
                const uint32_t x = s_in[w][k];
                uint32_t r = 0;
                for (uint32_t j = 0; j < n; ++j) r += s_in[w][j] < x;
                s_id[w][r] = x;
            }
            __syncwarp();
        }
        auto member = [&](uint32_t k) -> uint32_t { return fits ? s_id[w][k] : raw(k); };
        auto vel_of = [&](uint32_t k, uint32_t id) -> float4 {
            return fits ? s_v[w][k] : (id < P.nb ? bvel[id] : sv_old[id - P.nb]);
        };
        float E = 0.f;
        for (uint32_t k = lane; k < n; k += 32) {
            const uint32_t id = member(k);
            S.srd_sorted_index[start + k] = id;
            const float4 V = id < P.nb ? bvel[id] : sv_old[id - P.nb];
            if (fits) s_v[w][k] = V;
            E += (0.5f * V.w) * (V.x * V.x + V.y * V.y + V.z * V.z);
        }
        __syncwarp();
        E = warp_allsum(E);
        const float lam1 = lab ? sqrtf(P.srd_kT / E) : 1.0f;
        float ux = 0.f, uy = 0.f, uz = 0.f, M = 0.f;
        for (uint32_t k = lane; k < n; k += 32) {
            const float4 V = vel_of(k, member(k));
            const float sx = lab ? lam1 * V.x : V.x, sy = lab ? lam1 * V.y : V.y, sz = lab ? lam1 * V.z : V.z;
            ux += V.w * sx;
            uy += V.w * sy;
            uz += V.w * sz;
            M += V.w;
        }
        ux = warp_allsum(ux);
        uy = warp_allsum(uy);
        uz = warp_allsum(uz);
        M = warp_allsum(M);
        if (M > 0.f) {
            const float inv = 1.0f / M;
            ux *= inv;
            uy *= inv;
            uz *= inv;
        }
        const bool plus = u01(rng_draw(P, c, step, kRngSrdRot).x) > 0.5f;
        const float sa = plus ? P.srd_sin_a : -P.srd_sin_a, ca = P.srd_cos_a;
        float lam2 = 1.0f;
        bool scale2 = false;
        if (rel) {
            float ke = 0.f, nrot = 0.f;
            for (uint32_t k = lane; k < n; k += 32) {
                if (member(k) < P.nb && !P.srd_rotate_beads) continue;
                const float4 V = vel_of(k, member(k));
                const float dx = (lab ? lam1 * V.x : V.x) - ux, dy = (lab ? lam1 * V.y : V.y) - uy;
                const float rx = dx * ca - dy * sa, ry = dx * sa + dy * ca;
                ke += (0.5f * V.w) * (rx * rx + ry * ry);
                nrot += 1.f;
            }
            ke = warp_allsum(ke);
            nrot = warp_allsum(nrot);
            if (nrot >= 2.f && ke > 0.f) {
                lam2 = sqrtf(((nrot - 1.f) * P.srd_kT) / ke);
                scale2 = true;
            }
        }
        for (uint32_t k = lane; k < n; k += 32) {
            const uint32_t id = member(k);
            const bool is_bead = id < P.nb;
            const float4 V = vel_of(k, id);
            float3 v = lab ? make_float3(lam1 * V.x, lam1 * V.y, lam1 * V.z) : f3(V);
            if (!is_bead || P.srd_rotate_beads) {
                const float dx = v.x - ux, dy = v.y - uy, dz = v.z - uz;
                const float rx = dx * ca - dy * sa, ry = dx * sa + dy * ca;
                v = make_float3(ux + rx, uy + ry, uz + dz);
                if (scale2) v = make_float3(ux + lam2 * (v.x - ux), uy + lam2 * (v.y - uy), v.z);
            }
            if (is_bead) {
                if (lab || P.srd_rotate_beads) bvel[id] = make_float4(v.x, v.y, v.z, V.w);
            } else {
                const float4 P4 = sp_old[id - P.nb];
                float3 p = f3(P4);
                const float3 dr = dt_srd * v;
                p += dr;
                apply_boundaries(P, p, v, dr, 0.0f);
                const uint32_t dst = s0 + (k - nbc);
                sp_new[dst] = make_float4(p.x, p.y, p.z, P4.w);
                sv_new[dst] = make_float4(v.x, v.y, v.z, V.w);
            }
        }
        if (lane == 0) S.srd_mean[c] = make_float4(ux, uy, uz, 0.f);
        __syncwarp();
    }
}

// The collision just written the solvent to the other buffer.
__global__ void srd_flip_kernel(uint32_t* scur) { *scur ^= 1u; }

__global__ void advance_step_kernel(unsigned long long* step_base, unsigned long long k) { *step_base += k; }

}  // namespace nw

namespace {

__global__ void math_probe_kernel(const float* a, const float* b, uint32_t n, float4* out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float x = a[i], y = b[i];
    const float r = rsqrtf(x);
    out[i] = make_float4(nw::rcp_nr(x), nw::sqrt_nr(x, r), nw::div_nr(x, y), r);
}

}  // namespace

extern "C" nw_status nw_math_probe(const float* a, const float* b, uint32_t n, float* out)
{
    if (!a || !b || !out) return NW_ERR_INVALID;
    if (n == 0) return NW_OK;
    float *da = nullptr, *db = nullptr, *dout = nullptr;
    cudaError_t e = cudaMalloc(&da, (size_t)n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&db, (size_t)n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dout, (size_t)n * 16);
    if (e == cudaSuccess) e = cudaMemcpy(da, a, (size_t)n * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(db, b, (size_t)n * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        math_probe_kernel<<<(n + 255) / 256, 256>>>(da, db, n, reinterpret_cast<float4*>(dout));
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, dout, (size_t)n * 16, cudaMemcpyDeviceToHost);
    cudaFree(da);
    cudaFree(db);
    cudaFree(dout);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return NW_ERR_CUDA;
    }
    return NW_OK;
}
