// nw_device.cuh — device-side building blocks of the GB300 worm engine:
// the kernel parameter block, float3 arithmetic, Philox4x32-10, cell hashing,
// minimum image and the boundary rules.  Arithmetic follows the reference's
// FP32 operation order so that cell hashes are bit-identical and forces agree
// to rounding (simulation/particles_kernel_impl.cuh).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/nwgb.h"

namespace nw {

constexpr uint32_t kEmpty = 0xffffffffu;
constexpr int kChunkLog2 = 12;  // cells per scan chunk = 4096
constexpr uint32_t kChunk = 1u << kChunkLog2;

enum : uint32_t { kRngLangevin = 1, kRngReverse = 2, kRngSrdShift = 3, kRngSrdRot = 4, kRngInit = 5 };

// Everything a kernel needs, derived once on the host from NwConfig and
// passed by value (kernel parameter space), so many systems can coexist.
struct DevParams {
    int32_t model, dim, hash_mode;
    uint32_t nf, L, nb, ns, ntotal;
    uint32_t grid[3];
    uint32_t ncells;
    float cell[3], origin[3], box[3];
    int32_t bnd[3];
    float radius, mass;
    float bond_k, bond_r0, bend_k;
    float lj_amp, lj_two_s6, lj_rc2;
    int32_t lj_exclude;
    float spring, damping, shear, bdamp;
    float activity, reverse_p;
    float gamma, noise_sigma;
    int32_t langevin_on, reverse_on;
    int32_t srd_on;
    uint32_t srd_grid[3];
    uint32_t srd_ncells;
    float srd_cell[3];
    float srd_alpha, srd_kT, srd_shift_lo;
    float srd_sin_a, srd_cos_a;  // sin and cos of the rotation angle alpha
    int32_t srd_rotate_beads, srd_thermo;
    uint32_t seed_lo, seed_hi;
    // multiply-shift divisors by grid[0] and grid[0] * grid[1] (see fast_div)
    uint32_t div_gx_m, div_gx_k, div_gxy_m, div_gxy_k;
    // float reciprocals of the bead and SRD cell sizes (see floor_div)
    float inv_cell[3], srd_inv_cell[3];
    // cell grid of the per-step bead lists: the reference grid, or with
    // Verlet lists (vl_on) cells of at least lj_rcut + skin on the same box
    int32_t vl_on;
    uint32_t lgrid[3], lncells;
    float linv[3];  // lgrid / box
    uint32_t ldiv_x_m, ldiv_x_k, ldiv_xy_m, ldiv_xy_k;
    float vl_r2;         // (lj_rcut + skin)^2
    float vl_half_skin;  // lists stay valid while the displacement bound is below this
    uint32_t vl_cap;     // neighbours per bead list
    float ibox[3];       // 1 / box on periodic axes, 0 on the others (min_image_near)
};

// Planar systems (two-dimensional WCA worms) compute with two vector
// components, as the archived two-dimensional worm kernels do; their step
// kernels are compiled for D = 2 (planar arithmetic below).
__host__ __device__ __forceinline__ bool planar_system(const DevParams& P)
{
    return P.model == NW_MODEL_WCA_WORMS && P.dim == 2;
}

// floor(n / d) for n < 2^30 and 1 <= d < 2^30 with m = floor(2^k / d) + 1,
// k = 30 + ceil(log2 d): n * m / 2^k = n / d + e with 0 < e < 1 / d
// (Granlund and Montgomery, "Division by invariant integers using
// multiplication", PLDI 1994).
__host__ __device__ __forceinline__ uint32_t fast_div(uint32_t n, uint32_t m, uint32_t k)
{
    return (uint32_t)(((unsigned long long)n * m) >> k);
}

inline void fast_div_params(uint32_t d, uint32_t& m, uint32_t& k)
{
    uint32_t l = 0;
    while ((1ull << l) < (unsigned long long)d) ++l;
    k = 30u + l;
    m = (uint32_t)((1ull << k) / d + 1ull);
}

// ---- float3 helpers --------------------------------------------------------
__device__ __forceinline__ float3 f3(float4 a) { return make_float3(a.x, a.y, a.z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return make_float3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator/(float3 a, float s) { return make_float3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float3 operator-(float3 a) { return make_float3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ void operator+=(float3& a, float3 b) { a.x += b.x; a.y += b.y; a.z += b.z; }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 zero3() { return make_float3(0.f, 0.f, 0.f); }
__device__ __forceinline__ bool finite3(float3 a) { return isfinite(a.x) && isfinite(a.y) && isfinite(a.z); }

// ---- planar arithmetic -------------------------------------------------------
// Two-dimensional WCA worm systems compute in the xy plane, as the archived
// worm kernels do with two components per vector (NWWormsKernel_*.h, built
// with _D_ = 2).  With D = 2 the helpers below drop every z operation: a
// bead's z coordinate and velocity are carried unchanged and its forces have
// z = 0.  D = 3 is the three-component arithmetic of the other systems.
template <int D>
__device__ __forceinline__ float dotv(float3 a, float3 b)
{
    if constexpr (D == 2) return a.x * b.x + a.y * b.y;
    else return a.x * b.x + a.y * b.y + a.z * b.z;
}
// a - b (z = 0 for D = 2)
template <int D>
__device__ __forceinline__ float3 subv(float3 a, float3 b)
{
    if constexpr (D == 2) return make_float3(a.x - b.x, a.y - b.y, 0.f);
    else return make_float3(a.x - b.x, a.y - b.y, a.z - b.z);
}
// s a (z = 0 for D = 2)
template <int D>
__device__ __forceinline__ float3 scalev(float s, float3 a)
{
    if constexpr (D == 2) return make_float3(s * a.x, s * a.y, 0.f);
    else return make_float3(s * a.x, s * a.y, s * a.z);
}
// a + b (a's z for D = 2)
template <int D>
__device__ __forceinline__ float3 addv(float3 a, float3 b)
{
    if constexpr (D == 2) return make_float3(a.x + b.x, a.y + b.y, a.z);
    else return make_float3(a.x + b.x, a.y + b.y, a.z + b.z);
}
// f -= s a, component by component (f's z untouched for D = 2)
template <int D>
__device__ __forceinline__ void sub_scaled(float3& f, float s, float3 a)
{
    f.x -= s * a.x;
    f.y -= s * a.y;
    if constexpr (D == 3) f.z -= s * a.z;
}
template <int D>
__device__ __forceinline__ bool finitev(float3 a)
{
    if constexpr (D == 2) return isfinite(a.x) && isfinite(a.y);
    else return isfinite(a.x) && isfinite(a.y) && isfinite(a.z);
}

// ---- Philox4x32-10 (Salmon et al., SC'11) ----------------------------------
__host__ __device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
#ifdef __CUDA_ARCH__
        const uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
#else
        const uint64_t p0 = (uint64_t)0xD2511F53u * c.x, p1 = (uint64_t)0xCD9E8D57u * c.z;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
#endif
        c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
    }
    return c;
}

__host__ __device__ __forceinline__ uint4 rng_draw(const DevParams& P, uint32_t index, uint64_t step, uint32_t stream)
{
    return philox4x32_10(make_uint4(index, (uint32_t)step, (uint32_t)(step >> 32), stream), P.seed_lo, P.seed_hi);
}

// Uniform in (0, 1) from the top 23 bits; exact in FP32.
__host__ __device__ __forceinline__ float u01(uint32_t x) { return ((float)(x >> 9) + 0.5f) * 1.1920928955078125e-07f; }

// Two Box-Muller pairs: four standard normals.
// The first Box-Muller pair of normal4 only (2D systems use two components).
__device__ __forceinline__ float2 normal2(uint4 x)
{
    float s0, c0;
    const float r0 = sqrtf(-2.0f * logf(u01(x.x)));
    sincospif(2.0f * u01(x.y), &s0, &c0);
    return make_float2(r0 * c0, r0 * s0);
}

__device__ __forceinline__ float4 normal4(uint4 x)
{
    float s0, c0, s1, c1;
    const float r0 = sqrtf(-2.0f * logf(u01(x.x)));
    const float r1 = sqrtf(-2.0f * logf(u01(x.z)));
    sincospif(2.0f * u01(x.y), &s0, &c0);
    sincospif(2.0f * u01(x.w), &s1, &c1);
    return make_float4(r0 * c0, r0 * s0, r1 * c1, r1 * s1);
}

// Langevin noise sigma * (z0, z1[, z2]) of one Philox draw; 2D systems need
// only the first Box-Muller pair.
__device__ __forceinline__ float3 noise3(const DevParams& P, uint4 x)
{
    if (P.dim >= 3) {
        const float4 z = normal4(x);
        return make_float3(P.noise_sigma * z.x, P.noise_sigma * z.y, P.noise_sigma * z.z);
    }
    const float2 z = normal2(x);
    return make_float3(P.noise_sigma * z.x, P.noise_sigma * z.y, 0.f);
}

// ---- geometry ----------------------------------------------------------------

// lengthPeriodic (particles_kernel_impl.cuh:279-301): single-shift minimum
// image on periodic axes, in place.
__device__ __forceinline__ float min_image_len(const DevParams& P, float3& d)
{
    if (P.bnd[0] == NW_PERIODIC) {
        const float h = P.box[0] / 2.0f;
        if (d.x > h) d.x -= P.box[0];
        else if (d.x < -h) d.x += P.box[0];
    }
    if (P.bnd[1] == NW_PERIODIC) {
        const float h = P.box[1] / 2.0f;
        if (d.y > h) d.y -= P.box[1];
        else if (d.y < -h) d.y += P.box[1];
    }
    if (P.bnd[2] == NW_PERIODIC) {
        const float h = P.box[2] / 2.0f;
        if (d.z > h) d.z -= P.box[2];
        else if (d.z < -h) d.z += P.box[2];
    }
    return sqrtf(dot3(d, d));
}

__device__ __forceinline__ void min_image(const DevParams& P, float3& d)
{
    if (P.bnd[0] == NW_PERIODIC) {
        const float h = P.box[0] / 2.0f;
        if (d.x > h) d.x -= P.box[0];
        else if (d.x < -h) d.x += P.box[0];
    }
    if (P.bnd[1] == NW_PERIODIC) {
        const float h = P.box[1] / 2.0f;
        if (d.y > h) d.y -= P.box[1];
        else if (d.y < -h) d.y += P.box[1];
    }
    if (P.bnd[2] == NW_PERIODIC) {
        const float h = P.box[2] / 2.0f;
        if (d.z > h) d.z -= P.box[2];
        else if (d.z < -h) d.z += P.box[2];
    }
}

// Minimum image of a separation known to be far below half the box on every
// periodic axis (bonded neighbours, Verlet and cell-list candidates within
// the list radius): d -= box * rint(d / box), with the rounding done by
// adding and subtracting 1.5 * 2^23 (exact for |d / box| < 2^22), so three
// FMA-pipe instructions per axis and no branch.  For |d| < box / 2 the shift
// is 0 and d is unchanged; for box / 2 < |d| < box it is one box, subtracted
// with one rounding exactly as min_image does.  The two can differ only
// where d / box lies within rounding of +-1/2, i.e. for pairs half a box
// apart, which no force or list of these paths reaches.  Non-periodic axes
// have ibox = 0 and keep d.
template <int D = 3>
__device__ __forceinline__ void min_image_near(const DevParams& P, float3& d)
{
    constexpr float kRound = 12582912.0f;  // 1.5 * 2^23
    d.x = fmaf(-P.box[0], fmaf(d.x, P.ibox[0], kRound) - kRound, d.x);
    d.y = fmaf(-P.box[1], fmaf(d.y, P.ibox[1], kRound) - kRound, d.y);
    if constexpr (D == 3) d.z = fmaf(-P.box[2], fmaf(d.z, P.ibox[2], kRound) - kRound, d.z);
}

// floor(x / c) as the reference computes it (IEEE quotient, floor,
// saturating float -> int), for c > 0 with ic = 1/c rounded to float.
// x * ic and the IEEE quotient both lie within 1.2e-7 |q| of the exact x / c,
// so their floors agree unless an integer lies within that distance; only
// then is the division itself evaluated.
__device__ __forceinline__ int floor_div(float x, float c, float ic)
{
    const float q = x * ic;
    const float n = rintf(q);
    if (fabsf(q - n) <= fabsf(q) * 5.0e-7f) return (int)floorf(x / c);
    return (int)floorf(q);
}

// calcGridPos (particles_kernel_impl.cuh:231-238).
__device__ __forceinline__ int3 grid_pos(const DevParams& P, float3 p)
{
    int3 g;
    g.x = floor_div(p.x - P.origin[0], P.cell[0], P.inv_cell[0]);
    g.y = floor_div(p.y - P.origin[1], P.cell[1], P.inv_cell[1]);
    // a single layer maps every z to cell 0 in all hash modes
    g.z = P.grid[2] == 1u ? 0 : floor_div(p.z - P.origin[2], P.cell[2], P.inv_cell[2]);
    return g;
}

// g mod G in [0, G): one compare for the cells inside the box and one add or
// subtract for a single wrap; the integer remainder only beyond that.
__device__ __forceinline__ uint32_t wrap_mod(int g, uint32_t G)
{
    const int n = (int)G;
    if (g >= 0) {
        if (g < n) return (uint32_t)g;
        if (g - n < n) return (uint32_t)(g - n);
    } else if (g >= -n) {
        return (uint32_t)(g + n);
    }
    const int m = g % n;
    return (uint32_t)(m < 0 ? m + n : m);
}

__device__ __forceinline__ uint32_t clamp_cell(int g, uint32_t G)
{
    return g < 0 ? 0u : ((uint32_t)g >= G ? G - 1u : (uint32_t)g);
}

// Cell coordinate of one axis (power-of-two mask, or modulo / clamp).
__device__ __forceinline__ uint32_t cell_coord(const DevParams& P, int a, int g)
{
    if (P.hash_mode == NW_HASH_MASK) return (uint32_t)g & (P.grid[a] - 1u);
    return P.bnd[a] == NW_PERIODIC ? wrap_mod(g, P.grid[a]) : clamp_cell(g, P.grid[a]);
}

// calcGridHash (particles_kernel_impl.cuh:252-258), mask form uses 24-bit multiplies.
__device__ __forceinline__ uint32_t cell_hash(const DevParams& P, uint32_t cx, uint32_t cy, uint32_t cz)
{
    if (P.hash_mode == NW_HASH_MASK)
        return __umul24(__umul24(cz, P.grid[1]), P.grid[0]) + __umul24(cy, P.grid[0]) + cx;
    return (cz * P.grid[1] + cy) * P.grid[0] + cx;
}

__device__ __forceinline__ uint32_t bead_hash(const DevParams& P, float3 p)
{
    const int3 g = grid_pos(P, p);
    return cell_hash(P, cell_coord(P, 0, g.x), cell_coord(P, 1, g.y), cell_coord(P, 2, g.z));
}

// Cell of a bead on the Verlet list grid (modulo hash, no exactness
// requirement: insertion and lookup use this one function).
__device__ __forceinline__ uint32_t list_hash(const DevParams& P, float3 p)
{
    const float x[3] = {p.x, p.y, p.z};
    uint32_t c[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const uint32_t G = P.lgrid[a];
        const int g = G == 1u ? 0 : (int)floorf((x[a] - P.origin[a]) * P.linv[a]);
        c[a] = P.bnd[a] == NW_PERIODIC ? wrap_mod(g, G) : clamp_cell(g, G);
    }
    return (c[2] * P.lgrid[1] + c[1]) * P.lgrid[0] + c[0];
}

// positionRelativeToBox + calcGridPosSRD + calcGridHashSRD
// (particles_kernel_impl.cuh:208-228, 241-249, 261-276); wall axes clamped.
__device__ __forceinline__ uint32_t srd_hash(const DevParams& P, float3 p, float3 shift)
{
    const float t[3] = {p.x + shift.x, p.y + shift.y, p.z + shift.z};
    uint32_t c[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const uint32_t G = P.srd_grid[a];
        if (G == 1u) {  // a single layer (the z axis of 2D systems): cell 0 in every mode
            c[a] = 0u;
            continue;
        }
        float rel = t[a] - P.origin[a];
        if (P.bnd[a] == NW_PERIODIC) {
            if (rel >= P.box[a]) rel -= P.box[a];
            else if (rel < 0.0f) rel += P.box[a];
        }
        const int g = floor_div(rel, P.srd_cell[a], P.srd_inv_cell[a]);
        if (P.bnd[a] == NW_PERIODIC)
            c[a] = P.hash_mode == NW_HASH_MASK ? ((uint32_t)g & (G - 1u)) : wrap_mod(g, G);
        else
            c[a] = clamp_cell(g, G);
    }
    if (P.hash_mode == NW_HASH_MASK)
        return __umul24(__umul24(c[2], P.srd_grid[1]), P.srd_grid[0]) + __umul24(c[1], P.srd_grid[0]) + c[0];
    return (c[2] * P.srd_grid[1] + c[1]) * P.srd_grid[0] + c[0];
}

// periodicBoundary / dampedWallBoundary / noslipWallBoundary in
// filament_integrator's axis order (particles_kernel_impl.cuh:34-68, 99-134);
// planar systems (D = 2) leave the z axis alone.
template <int D = 3>
__device__ __forceinline__ void apply_boundaries(const DevParams& P, float3& p, float3& v, float3 dr, float rad)
{
    float* pp = &p.x;
    float* vv = &v.x;
#pragma unroll
    for (int a = 0; a < D; ++a) {
        const float L0 = P.origin[a], L = P.box[a];
        const int b = P.bnd[a];
        if (b == NW_PERIODIC) {
            if (pp[a] < L0) pp[a] += L;
            else if (pp[a] > L + L0) pp[a] -= L;
        } else if (b == NW_WALL) {
            if (pp[a] < L0 + rad) {
                pp[a] = L0 + rad;
                vv[a] *= P.bdamp;
            } else if (pp[a] > (L + L0) - rad) {
                pp[a] = (L + L0) - rad;
                vv[a] *= P.bdamp;
            }
        } else if (b == NW_WALL_NO_SLIP && a < 2) {
            bool hit = false;
            float target = 0.f;
            if (pp[a] < L0 + rad) {
                hit = true;
                target = L0 + rad;
            } else if (pp[a] > (L + L0) - rad) {
                hit = true;
                target = (L + L0) - rad;
            }
            if (hit) {
                p = p - dr;
                pp[a] = target;
                const float nx = a == 0 ? 1.f : 0.f, ny = a == 1 ? 1.f : 0.f;
                v = make_float3(-v.x * nx, -v.y * ny, D == 3 ? -v.z * 0.f : v.z);
            }
        }
    }
}

// Filament of a bead index (beads are stored filament by filament).
__device__ __forceinline__ uint32_t div_L(uint32_t i, uint32_t L) { return i / L; }

}  // namespace nw
