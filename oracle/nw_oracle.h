/*
 * nw_oracle.h — CPU oracle of the nematic-worm step.  TEST INFRASTRUCTURE ONLY.
 *
 * This is a plain-C restatement of the reference's step, used by tests/,
 * __graft_entry__.smoke() and the CPU-baseline leg of bench.py as the checker.
 * No product code path may call it.
 *
 * Every routine exists in an FP32 flavour (suffix _f32, float arithmetic in
 * the reference's operation order) and an FP64 flavour (suffix _f64).  Cell
 * hashing always uses FP32 arithmetic so that cell assignment is bit-identical
 * to the GPU's.  Arrays are float4-style AoS: REAL[4*n] with x, y, z, w.
 *
 * Parity pinning: tests compare these routines with the reference's own
 * kernel source compiled for the CPU (oracle/ref_emu, output in oracle/_ref)
 * and with golden vectors generated from it (tests/golden).
 */
#ifndef NW_ORACLE_H
#define NW_ORACLE_H

#include <stdint.h>
#include "../include/nwgb.h"

#ifdef __cplusplus
extern "C" {
#endif

#define NWO_EMPTY 0xffffffffu

/* RNG streams: counter = {index, step_lo, step_hi, stream}, key = seed. */
enum { NWO_RNG_LANGEVIN = 1, NWO_RNG_REVERSE = 2, NWO_RNG_SRD_SHIFT = 3, NWO_RNG_SRD_ROT = 4, NWO_RNG_INIT = 5 };

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
 * easy as 1, 2, 3", SC'11). */
void nwo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* Uniform in (0, 1) from the top 23 bits: ((x >> 9) + 0.5) * 2^-23 (exact in float). */
float nwo_u01(uint32_t x);
/* Four standard normals (two Box-Muller pairs) for (index, step, stream). */
void nwo_normal4(uint64_t seed, uint32_t index, uint64_t step, uint32_t stream, double out[4]);
/* Four uniforms in (0,1) for (index, step, stream). */
void nwo_uniform4(uint64_t seed, uint32_t index, uint64_t step, uint32_t stream, float out[4]);

/* a1: bead cell hash, calcHashD with srd=false (simulation/particles_kernel_impl.cuh:231-238,
 * 252-258, 312-342).  pos is float4[n].  index[i] = i. */
void nwo_calc_hash(const NwConfig* cfg, const float* pos, uint32_t n, uint32_t* hash, uint32_t* index);
/* a9: SRD cell hash, calcHashD with srd=true (:208-228, 241-249, 261-276). */
void nwo_calc_hash_srd(const NwConfig* cfg, const float* pos, uint32_t n, const float shift[3],
                       uint32_t* hash, uint32_t* index);
/* a2: stable key/value sort (thrust::sort_by_key, simulation/particleSystem_cuda.cu:277-282). */
void nwo_sort_by_key(uint32_t* keys, uint32_t* values, uint32_t n);
/* a3: cell start/end of the sorted hash (reorderDataAndFindCellStartD,
 * simulation/particles_kernel_impl.cuh:346-424).  cell_start is filled with
 * 0xffffffff first (particleSystem_cuda.cu:188); cell_end is written only for
 * non-empty cells. */
void nwo_cell_bounds(const uint32_t* sorted_hash, uint32_t n, uint32_t num_cells,
                     uint32_t* cell_start, uint32_t* cell_end);
uint32_t nwo_num_cells(const NwConfig* cfg);
uint32_t nwo_num_srd_cells(const NwConfig* cfg);

#define NWO_DECLARE(R, S)                                                                          \
    /* a7: filament_integrator (simulation/particles_kernel_impl.cuh:34-142). */                  \
    void nwo_integrate_##S(const NwConfig* cfg, R* pos, R* vel, R* force, R* force_old,           \
                           uint32_t n, R dt);                                                     \
    /* a9: solvent_integrator (:145-205), applied to [start, start+count). */                     \
    void nwo_integrate_solvent_##S(const NwConfig* cfg, R* pos, R* vel, uint32_t start,           \
                                   uint32_t count, R dt);                                         \
    /* a8: reverseFilamentsKernel (:820-857). uniform[num_filaments]. */                          \
    void nwo_reverse_##S(const NwConfig* cfg, R* force, R* force_old, R* vel, R* pos,             \
                         const float* uniform, uint32_t num_filaments);                           \
    /* a6: langevinKernel (:859-874): f += -gamma v + noise.xyz, noise float4[n]. */              \
    void nwo_langevin_##S(const NwConfig* cfg, R* force, const R* vel, const R* noise,            \
                          uint32_t n);                                                            \
    /* a5: filamentKernel (:751-818) bending + tangents; WCA_WORMS adds the archived              \
     * harmonic bonds (NWWormsKernel_InternalForce.h:37-59) and tangent drive                     \
     * (NWWormsKernel_DriveForce.h:21-34). */                                                     \
    void nwo_filament_##S(const NwConfig* cfg, R* force, R* tangent, const R* pos,                \
                          uint32_t num_filaments);                                                \
    /* a4/a4': pair forces through the cell list.  sorted_index/cell_start/cell_end               \
     * from the bead sort; pos/vel/tangent in ORIGINAL order (gathered inside). */                \
    void nwo_pair_##S(const NwConfig* cfg, R* force, const R* pos, const R* vel,                  \
                      const R* tangent, const uint32_t* sorted_index,                             \
                      const uint32_t* cell_start, const uint32_t* cell_end, uint32_t n);          \
    /* WCA_WORMS pair forces by brute force O(n^2) (independent cross-check). */                  \
    void nwo_pair_wca_bruteforce_##S(const NwConfig* cfg, R* force, const R* pos, uint32_t n);    \
    /* a9: the SRD sub-step (_solventUpdate, simulation/particleSystem.cpp:341-413):              \
     * hash with shift, stable sort, cell thermostat, cell mean, rotation, solvent                \
     * streaming by dt_srd.  rot_uniform[n_srd_cells] or NULL (Philox by step).                   \
     * Optional outputs: sorted_index[n_total], cell_start/end[n_srd_cells],                      \
     * cell_mean float4-style R[4*n_srd_cells]. */                                                \
    void nwo_srd_##S(const NwConfig* cfg, R* pos, R* vel, uint32_t n_beads, uint32_t n_solvent,   \
                     const float shift[3], const float* rot_uniform, uint64_t step, R dt_srd,     \
                     uint32_t* sorted_index, uint32_t* cell_start, uint32_t* cell_end,            \
                     R* cell_mean);                                                               \
    /* The full step (ParticleSystem::update, simulation/particleSystem.cpp:249-339) with          \
     * Philox noise keyed by (seed, step).  Optional outputs of the bead sort. */                 \
    void nwo_step_##S(const NwConfig* cfg, R* pos, R* vel, R* force, R* force_old, R* tangent,    \
                      uint64_t step, R dt, uint32_t* hash_out, uint32_t* sorted_index_out,        \
                      uint32_t* cell_start_out, uint32_t* cell_end_out);                          \
    /* SRD grid shift of a collision at `step` (world units). */                                  \
    void nwo_srd_shift_##S(const NwConfig* cfg, uint64_t step, float shift[3]);                   \
    /* Relabel the solvent in the collision's stable cell order (the engine's storage order). */  \
    void nwo_reorder_solvent_##S(R* pos, R* vel, uint32_t n_beads, uint32_t n_solvent,            \
                                 const uint32_t* sorted_index);

NWO_DECLARE(float, f32)
NWO_DECLARE(double, f64)

/* Number of host threads the oracle uses (OpenMP); 1 when built without it. */
/* Per-bead force scale buffer (n_beads doubles, caller-zeroed) that every
 * following force computation adds its term magnitudes to; NULL switches it off. */
void nwo_set_force_scale(double* buf);
int nwo_num_threads(void);
void nwo_set_num_threads(int n);

#ifdef __cplusplus
}
#endif

#endif
