/*
 * nw_oracle.c — CPU oracle of the nematic-worm step.  TEST INFRASTRUCTURE ONLY:
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it as
 * the checker; the product (libnwgb.so) never links or calls it.
 *
 * Shared, precision-independent parts live here (RNG, cell hashing in FP32,
 * the stable sort, cell bounds); the FP32/FP64 physics is nw_oracle_impl.h,
 * included twice below.
 */
#include "nw_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Per-bead force scale: when set, every force term added to bead i adds to
 * nwo_fscale[i] (in double) the magnitude of its parts before they cancel
 * (for a WCA pair both LJ powers, for a bond k (r + r0), for the bending
 * projections each part, for Langevin friction and noise each).  A rounding
 * error of relative size u in any part moves the bead's net force by at most
 * about u times this scale, however much the parts cancel, so parity tests
 * normalise per-bead force differences by it. */
double* nwo_fscale = NULL;

void nwo_set_force_scale(double* buf)
{
    nwo_fscale = buf;
}

int nwo_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void nwo_set_num_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ---- Philox4x32-10 -------------------------------------------------------
 * Round function and constants as published by Salmon et al. (SC'11):
 * multipliers 0xD2511F53 / 0xCD9E8D57, Weyl key increments 0x9E3779B9 /
 * 0xBB67AE85, ten rounds, key bumped before every round but the first. */
void nwo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        uint64_t p0 = (uint64_t)0xD2511F53u * (uint64_t)c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * (uint64_t)c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

float nwo_u01(uint32_t x)
{
    return ((float)(x >> 9) + 0.5f) * 1.1920928955078125e-07f; /* 2^-23 */
}

static void philox_draw(uint64_t seed, uint32_t index, uint64_t step, uint32_t stream, uint32_t out[4])
{
    uint32_t ctr[4] = {index, (uint32_t)step, (uint32_t)(step >> 32), stream};
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    nwo_philox4x32_10(ctr, key, out);
}

void nwo_uniform4(uint64_t seed, uint32_t index, uint64_t step, uint32_t stream, float out[4])
{
    uint32_t x[4];
    philox_draw(seed, index, step, stream, x);
    for (int k = 0; k < 4; ++k) out[k] = nwo_u01(x[k]);
}

/* Box-Muller: z0 = sqrt(-2 ln u1) cos(2 pi u2), z1 = sqrt(-2 ln u1) sin(2 pi u2). */
void nwo_normal4(uint64_t seed, uint32_t index, uint64_t step, uint32_t stream, double out[4])
{
    float u[4];
    nwo_uniform4(seed, index, step, stream, u);
    const double two_pi = 6.283185307179586476925286766559;
    for (int k = 0; k < 2; ++k) {
        double r = sqrt(-2.0 * log((double)u[2 * k]));
        double th = two_pi * (double)u[2 * k + 1];
        out[2 * k] = r * cos(th);
        out[2 * k + 1] = r * sin(th);
    }
}

/* ---- cell hashing (FP32, bit-exact to the device) -------------------------- */

/* float -> int conversion with the device's saturating round-toward-zero
 * semantics (NaN -> 0). */
static int f2i_sat(float x)
{
    if (x != x) return 0;
    if (x >= 2147483648.0f) return 2147483647;
    if (x < -2147483648.0f) return (-2147483647 - 1);
    return (int)x;
}

/* __umul24: product of the low 24 bits of each operand, low 32 bits kept. */
static uint32_t umul24(uint32_t a, uint32_t b)
{
    return (uint32_t)((uint64_t)(a & 0xffffffu) * (uint64_t)(b & 0xffffffu));
}

static uint32_t wrap_mod(int g, uint32_t G)
{
    long long m = (long long)g % (long long)G;
    if (m < 0) m += G;
    return (uint32_t)m;
}

static uint32_t clamp_cell(int g, uint32_t G)
{
    if (g < 0) return 0;
    if ((uint32_t)g >= G) return G - 1;
    return (uint32_t)g;
}

uint32_t nwo_num_cells(const NwConfig* cfg)
{
    return cfg->grid[0] * cfg->grid[1] * cfg->grid[2];
}

uint32_t nwo_num_srd_cells(const NwConfig* cfg)
{
    return cfg->srd_grid[0] * cfg->srd_grid[1] * cfg->srd_grid[2];
}

/* calcGridPos + calcGridHash (simulation/particles_kernel_impl.cuh:231-238, 252-258). */
static uint32_t bead_hash(const NwConfig* cfg, const float* p)
{
    int g[3];
    for (int a = 0; a < 3; ++a) {
        float d = p[a] - cfg->origin[a];
        float q = d / cfg->cell_size[a];
        g[a] = f2i_sat(floorf(q));
    }
    if (cfg->hash_mode == NW_HASH_MASK) {
        uint32_t gx = (uint32_t)g[0] & (cfg->grid[0] - 1u);
        uint32_t gy = (uint32_t)g[1] & (cfg->grid[1] - 1u);
        uint32_t gz = (uint32_t)g[2] & (cfg->grid[2] - 1u);
        return umul24(umul24(gz, cfg->grid[1]), cfg->grid[0]) + umul24(gy, cfg->grid[0]) + gx;
    }
    uint32_t c[3];
    for (int a = 0; a < 3; ++a)
        c[a] = cfg->boundary[a] == NW_PERIODIC ? wrap_mod(g[a], cfg->grid[a]) : clamp_cell(g[a], cfg->grid[a]);
    return (c[2] * cfg->grid[1] + c[1]) * cfg->grid[0] + c[0];
}

/* positionRelativeToBox + calcGridPosSRD + calcGridHashSRD
 * (simulation/particles_kernel_impl.cuh:208-228, 241-249, 261-276).  Wall
 * axes are clamped into the grid (the reference leaves them unwrapped). */
static uint32_t srd_hash(const NwConfig* cfg, const float* p, const float shift[3])
{
    int g[3];
    for (int a = 0; a < 3; ++a) {
        float t = p[a] + shift[a];
        float rel = t - cfg->origin[a];
        if (cfg->boundary[a] == NW_PERIODIC) {
            if (rel >= cfg->box[a]) rel -= cfg->box[a];
            else if (rel < 0.0f) rel += cfg->box[a];
        }
        float q = rel / cfg->srd_cell_size[a];
        g[a] = f2i_sat(floorf(q));
    }
    uint32_t c[3];
    for (int a = 0; a < 3; ++a) {
        uint32_t G = cfg->srd_grid[a];
        if (cfg->boundary[a] == NW_PERIODIC)
            c[a] = cfg->hash_mode == NW_HASH_MASK ? ((uint32_t)g[a] & (G - 1u)) : wrap_mod(g[a], G);
        else
            c[a] = clamp_cell(g[a], G);
    }
    if (cfg->hash_mode == NW_HASH_MASK)
        return umul24(umul24(c[2], cfg->srd_grid[1]), cfg->srd_grid[0]) + umul24(c[1], cfg->srd_grid[0]) + c[0];
    return (c[2] * cfg->srd_grid[1] + c[1]) * cfg->srd_grid[0] + c[0];
}

void nwo_calc_hash(const NwConfig* cfg, const float* pos, uint32_t n, uint32_t* hash, uint32_t* index)
{
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)n; ++i) {
        hash[i] = bead_hash(cfg, pos + 4 * i);
        index[i] = (uint32_t)i;
    }
}

void nwo_calc_hash_srd(const NwConfig* cfg, const float* pos, uint32_t n, const float shift[3],
                       uint32_t* hash, uint32_t* index)
{
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)n; ++i) {
        hash[i] = srd_hash(cfg, pos + 4 * i, shift);
        index[i] = (uint32_t)i;
    }
}

/* Stable LSD radix sort on 8-bit digits (ties keep their input order, as in
 * thrust::sort_by_key). */
void nwo_sort_by_key(uint32_t* keys, uint32_t* values, uint32_t n)
{
    if (n < 2) return;
    uint32_t* k2 = (uint32_t*)malloc(sizeof(uint32_t) * n);
    uint32_t* v2 = (uint32_t*)malloc(sizeof(uint32_t) * n);
    uint32_t *ks = keys, *vs = values, *kd = k2, *vd = v2;
    for (int shift = 0; shift < 32; shift += 8) {
        size_t count[257];
        memset(count, 0, sizeof(count));
        for (uint32_t i = 0; i < n; ++i) count[((ks[i] >> shift) & 0xffu) + 1]++;
        if (count[((ks[0] >> shift) & 0xffu) + 1] == n) continue; /* digit constant: pass is identity */
        for (int d = 0; d < 256; ++d) count[d + 1] += count[d];
        for (uint32_t i = 0; i < n; ++i) {
            size_t dst = count[(ks[i] >> shift) & 0xffu]++;
            kd[dst] = ks[i];
            vd[dst] = vs[i];
        }
        uint32_t* t = ks; ks = kd; kd = t;
        t = vs; vs = vd; vd = t;
    }
    if (ks != keys) {
        memcpy(keys, ks, sizeof(uint32_t) * n);
        memcpy(values, vs, sizeof(uint32_t) * n);
    }
    free(k2);
    free(v2);
}

void nwo_cell_bounds(const uint32_t* sorted_hash, uint32_t n, uint32_t num_cells,
                     uint32_t* cell_start, uint32_t* cell_end)
{
    for (uint32_t c = 0; c < num_cells; ++c) cell_start[c] = NWO_EMPTY;
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t h = sorted_hash[i];
        if (i == 0 || h != sorted_hash[i - 1]) {
            if (h < num_cells) cell_start[h] = i;
            if (i > 0 && sorted_hash[i - 1] < num_cells) cell_end[sorted_hash[i - 1]] = i;
        }
        if (i == n - 1 && h < num_cells) cell_end[h] = i + 1;
    }
}

/* ---- precision-dependent physics ------------------------------------------ */

#define R float
#define S f32
#define RS(name) name##_f32
#include "nw_oracle_impl.h"
#undef R
#undef S
#undef RS

#define R double
#define S f64
#define RS(name) name##_f64
#include "nw_oracle_impl.h"
#undef R
#undef S
#undef RS
