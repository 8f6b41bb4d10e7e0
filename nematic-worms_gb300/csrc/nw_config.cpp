// nw_config.cpp — configuration defaults, derivation and validation of the
// C ABI (include/nwgb.h).  Host code only.
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "../../include/nwgb.h"

namespace {

bool is_pow2(uint32_t x) { return x && !(x & (x - 1)); }
bool finite_pos(float x) { return std::isfinite(x) && x > 0.0f; }

}  // namespace

extern "C" {

uint32_t nw_abi_version(void) { return NW_ABI_VERSION; }

size_t nw_config_size(void) { return sizeof(NwConfig); }

nw_status nw_config_finalize(NwConfig* c)
{
    if (!c) return NW_ERR_INVALID;
    for (int a = 0; a < 3; ++a) {
        c->box[a] = (float)c->grid[a] * c->cell_size[a];
        c->origin[a] = -c->box[a] / 2.0f;
    }
    return NW_OK;
}

nw_status nw_reference_reset(const NwConfig* c, float* pos, float* vel, float* tan)
{
    if (!c || !pos || !vel || !tan) return NW_ERR_INVALID;
    const uint32_t L = c->filament_size, M = c->num_filaments;
    const uint64_t nb = (uint64_t)M * L;
    const uint64_t ns = c->srd_enabled ? c->num_solvent : 0;
    const float R = c->radius, bl = c->bond_r0;
    const float flen = (float)L * bl + 2.0f * R;
    const long xdim = (long)std::floor(c->box[0] / flen);
    const long ydim = (long)std::floor(c->box[1] / (2.0f * R));
    if (nb && (xdim <= 0 || ydim <= 0)) return NW_ERR_INVALID;
    const long plane = xdim * ydim;
    srand(1);
    auto frand = []() { return (float)rand() / (float)RAND_MAX; };
    for (uint64_t i = 0; i < nb; ++i) {
        const long w = (long)(i / L);
        const float x = ((float)(w % xdim) * flen + R) + (float)(i % L) * bl;
        const float y = 2.0f * R * (float)((w / xdim) % ydim + 1);
        const float z = 2.0f * R * (float)(w / plane + 1);
        float* p = pos + 4 * i;
        p[0] = x + c->origin[0];
        p[1] = y + c->origin[1];
        p[2] = z + c->origin[2];
        p[3] = R;
        float* v = vel + 4 * i;
        for (int a = 0; a < 3; ++a) v[a] = 0.1f * (frand() * 2.0f - 1.0f);
        v[3] = c->mass;
        float* t = tan + 4 * i;
        t[0] = 1.0f;
        t[1] = t[2] = t[3] = 0.0f;
    }
    for (uint32_t w = 0; w < M; ++w) {
        if (frand() < 0.5f) continue;
        for (uint32_t p = 0; p < L / 2; ++p) {
            const uint64_t i = (uint64_t)w * L + p, j = (uint64_t)(w + 1) * L - 1 - p;
            for (int a = 0; a < 4; ++a) {
                float tmp = pos[4 * i + a];
                pos[4 * i + a] = pos[4 * j + a];
                pos[4 * j + a] = tmp;
            }
            for (int a = 0; a < 4; ++a) {
                tan[4 * i + a] = -tan[4 * i + a];
                tan[4 * j + a] = -tan[4 * j + a];
            }
        }
    }
    for (uint64_t s = 0; s < ns; ++s) {
        float* p = pos + 4 * (nb + s);
        for (int a = 0; a < 3; ++a) p[a] = c->box[a] * frand() + c->origin[a];
        p[3] = 0.0f;
        float* v = vel + 4 * (nb + s);
        for (int a = 0; a < 3; ++a) v[a] = 5.0f * (frand() * 2.0f - 1.0f);
        v[3] = c->solvent_mass;
    }
    return NW_OK;
}

nw_status nw_config_default(NwConfig* c, int model, uint32_t nf, uint32_t L, uint32_t gx, uint32_t gy, uint32_t gz,
                            int srd)
{
    if (!c) return NW_ERR_INVALID;
    std::memset(c, 0, sizeof(*c));
    c->abi_version = NW_ABI_VERSION;
    c->model = model;
    c->num_filaments = nf;
    c->filament_size = L;
    c->grid[0] = gx;
    c->grid[1] = gy;
    c->grid[2] = gz;
    c->boundary[0] = c->boundary[1] = c->boundary[2] = NW_PERIODIC;
    c->radius = 0.5f;
    c->mass = 1.0f;
    c->lj_epsilon = 1.0f;
    c->lj_sigma = 1.0f;
    c->lj_rcut = 1.12246205f;  // 2^(1/6) sigma, the archived engine's _216 constant
    c->lj_exclude = 2;
    c->srd_enabled = srd ? 1 : 0;
    c->solvent_mass = 1.0f;
    c->srd_alpha = 2.26893f;  // 130 degrees
    if (model == NW_MODEL_REF_DEM) {
        // ParticleSystem constructor defaults (simulation/particleSystem.cpp:64-105)
        c->dim = 3;
        c->hash_mode = NW_HASH_MASK;
        const float cell = c->radius * 2.0f;
        c->cell_size[0] = c->cell_size[1] = c->cell_size[2] = cell;
        c->bond_k = 57.0f;
        c->bond_r0 = c->radius * 0.8f;
        c->bend_k = 0.001f;
        c->spring = 0.5f;
        c->damping = 0.02f;
        c->shear = 0.1f;
        c->attraction = 0.0f;
        c->boundary_damping = -0.5f;
        c->activity = 0.1f;
        c->reverse_probability = 0.0f;
        c->kT = 1.0f;
        c->gamma = 0.01f;
        c->noise_dt_scaling = 0;
        c->dt = 0.002f;  // main.cpp's default time step (simulation/main.cpp:25)
        // _initSolventParams (simulation/particleSystem.cpp:124-148)
        c->srd_grid[0] = gx / 2u ? gx / 2u : 1u;
        c->srd_grid[1] = gy / 2u ? gy / 2u : 1u;
        c->srd_grid[2] = gz / 2u ? gz / 2u : 1u;
        for (int a = 0; a < 3; ++a) c->srd_cell_size[a] = cell * 2.0f;
        c->srd_gap = 5;
        c->srd_kT = c->kT;
        c->srd_shift_lo = 0.0f;
        c->srd_rotate_beads = 0;
        c->srd_thermostat = NW_SRD_THERMO_REF_LAB;
        c->num_solvent = srd ? (uint32_t)(10.0f * (float)(c->srd_grid[0] * c->srd_grid[1] * c->srd_grid[2])) : 0u;
    } else {
        // 2D WCA worms: eps = sigma = 1, bond k = 57, r0 = 0.8, bend k = 10,
        // F_act = 0.5, gamma = 2, kT = 0.1, dt = 0.005; cell edge = cut-off.
        c->dim = gz > 1 ? 3 : 2;
        c->hash_mode = NW_HASH_MODULO;
        c->cell_size[0] = c->cell_size[1] = c->cell_size[2] = c->lj_rcut;
        c->bond_k = 57.0f;
        c->bond_r0 = 0.8f;
        c->bend_k = 10.0f;
        c->activity = 0.5f;
        c->kT = 0.1f;
        c->gamma = 2.0f;
        c->noise_dt_scaling = 1;
        c->boundary_damping = -0.5f;
        c->dt = 0.005f;
        // SRD: unit cells, density 4, collision every 10 steps, shift in [-a/2, a/2)
        c->srd_cell_size[0] = c->srd_cell_size[1] = 1.0f;
        c->srd_gap = 10;
        c->srd_kT = c->kT;
        c->srd_shift_lo = -0.5f;
        c->srd_rotate_beads = 1;
        c->srd_thermostat = NW_SRD_THERMO_CELL_REL;
    }
    nw_config_finalize(c);
    if (model != NW_MODEL_REF_DEM) {
        for (int a = 0; a < 3; ++a) {
            if (a == 2 && c->dim < 3) {
                c->srd_grid[2] = 1;
                c->srd_cell_size[2] = c->box[2] > 0.f ? c->box[2] : 1.0f;
                continue;
            }
            float g = std::floor(c->box[a] / c->srd_cell_size[a]);
            c->srd_grid[a] = g >= 1.0f ? (uint32_t)g : 1u;
            c->srd_cell_size[a] = c->box[a] / (float)c->srd_grid[a];
        }
        c->num_solvent = srd ? 4u * c->srd_grid[0] * c->srd_grid[1] * c->srd_grid[2] : 0u;
    }
    return NW_OK;
}

nw_status nw_config_validate(const NwConfig* c)
{
    if (!c) return NW_ERR_INVALID;
    if (c->abi_version != NW_ABI_VERSION) return NW_ERR_INVALID;
    if (c->model != NW_MODEL_WCA_WORMS && c->model != NW_MODEL_REF_DEM) return NW_ERR_INVALID;
    if (c->dim != 2 && c->dim != 3) return NW_ERR_INVALID;
    if (c->filament_size < 1 || c->filament_size > 1024) return NW_ERR_INVALID;
    const uint64_t nb = (uint64_t)c->num_filaments * c->filament_size;
    if (nb >= (1ull << 31)) return NW_ERR_INVALID;
    uint64_t ncells = 1;
    for (int a = 0; a < 3; ++a) {
        if (c->grid[a] < 1) return NW_ERR_INVALID;
        if (!finite_pos(c->cell_size[a])) return NW_ERR_INVALID;
        if (c->boundary[a] < NW_PERIODIC || c->boundary[a] > NW_WALL_NO_SLIP) return NW_ERR_INVALID;
        if (c->hash_mode == NW_HASH_MASK && !is_pow2(c->grid[a])) return NW_ERR_INVALID;
        if (std::fabs(c->box[a] - (float)c->grid[a] * c->cell_size[a]) > 1e-4f * c->box[a] + 1e-6f)
            return NW_ERR_INVALID;
        ncells *= c->grid[a];
    }
    if (ncells >= (1ull << 30)) return NW_ERR_INVALID;
    if (c->hash_mode != NW_HASH_MODULO && c->hash_mode != NW_HASH_MASK) return NW_ERR_INVALID;
    if (c->model == NW_MODEL_WCA_WORMS) {
        if (!finite_pos(c->lj_rcut) || !finite_pos(c->lj_sigma)) return NW_ERR_INVALID;
        // the 3x3(x3) stencil must cover the cut-off sphere
        for (int a = 0; a < 3; ++a)
            if (c->grid[a] > 1 && c->cell_size[a] < c->lj_rcut * (1.0f - 1e-6f)) return NW_ERR_INVALID;
    }
    if (!std::isfinite(c->dt)) return NW_ERR_INVALID;
    if (c->strategy < NW_STRATEGY_AUTO || c->strategy > NW_STRATEGY_VERLET) return NW_ERR_INVALID;
    if (c->strategy == NW_STRATEGY_VERLET && c->model != NW_MODEL_WCA_WORMS) return NW_ERR_INVALID;
    if (c->cell_capacity != 0 && c->cell_capacity != 8 && c->cell_capacity != 16) return NW_ERR_INVALID;
    if (!std::isfinite(c->neighbor_skin) || c->neighbor_skin < 0.0f) return NW_ERR_INVALID;
    if (c->neighbor_capacity != 0 && (c->neighbor_capacity < 4 || c->neighbor_capacity > 256)) return NW_ERR_INVALID;
    if (c->srd_enabled) {
        uint64_t nsc = 1;
        for (int a = 0; a < 3; ++a) {
            if (c->srd_grid[a] < 1 || !finite_pos(c->srd_cell_size[a])) return NW_ERR_INVALID;
            if (c->hash_mode == NW_HASH_MASK && !is_pow2(c->srd_grid[a])) return NW_ERR_INVALID;
            nsc *= c->srd_grid[a];
        }
        if (nsc >= (1ull << 30)) return NW_ERR_INVALID;
        if (c->srd_gap < 1) return NW_ERR_INVALID;
        if (nb + (uint64_t)c->num_solvent >= (1ull << 31)) return NW_ERR_INVALID;
        if (c->srd_thermostat < NW_SRD_THERMO_NONE || c->srd_thermostat > NW_SRD_THERMO_CELL_REL)
            return NW_ERR_INVALID;
    }
    return NW_OK;
}

const char* nw_status_string(nw_status s)
{
    switch (s) {
    case NW_OK: return "ok";
    case NW_ERR_CUDA: return "CUDA runtime error";
    case NW_ERR_INVALID: return "invalid argument or configuration";
    case NW_ERR_CELL_OVERFLOW: return "cell occupancy above kernel capacity";
    case NW_ERR_NONFINITE: return "non-finite position or force";
    case NW_ERR_TIMEOUT: return "bounded device wait timed out";
    case NW_ERR_NOMEM: return "out of memory";
    case NW_ERR_UNSUPPORTED: return "unsupported configuration";
    case NW_ERR_NO_DEVICE: return "no CUDA device";
    case NW_ERR_IO: return "file could not be opened or written";
    default: return "unknown status";
    }
}

}  // extern "C"
