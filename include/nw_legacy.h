/*
 * nw_legacy.h — the reference's C-ABI launch layer, implemented on the GB300
 * kernels of libnwgb.so.
 *
 * Replaces: simulation/particleSystem.cuh:12-112 (declarations) and
 * simulation/particleSystem_cuda.cu:36-371 (definitions).  Every symbol has
 * the reference's name and signature, so the reference's
 * particleSystem.cpp links against libnwgb.so unchanged.  Semantics follow
 * the reference, including its quirks (power-of-two mask hashing, the 2D
 * triple visit of neighbour cells, Langevin noise without 1/sqrt(dt), the
 * lab-frame SRD thermostat that also scales beads, beads excluded from the
 * SRD rotation).
 *
 * Differences from the reference, by design:
 *  - no function calls exit(); failures are printed and recorded, and
 *    nw_legacy_last_status() returns the last one;
 *  - random numbers come from a counter-based Philox4x32-10 stream instead
 *    of cuRAND's XORWOW generator (simulation/particleSystem_cuda.cu:53);
 *  - all work is issued on the legacy default stream, as in the reference.
 */
#ifndef NW_LEGACY_H
#define NW_LEGACY_H

#include <stdint.h>
#ifndef __cplusplus
#include <stdbool.h>
#endif

#include "../nematic-worms_gb300/compat/particles_kernel.cuh"

#ifdef __cplusplus
#define NW_DEFAULT_FALSE = false
#else
#define NW_DEFAULT_FALSE
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* particleSystem_cuda.cu:40-54 — pick the device (-device=N), start the RNG. */
void cudaInit(int argc, char** argv);
/* particleSystem_cuda.cu:56-59 — n uniforms in (0, 1). */
void randomizeUniform(float* device, uint n);
/* particleSystem_cuda.cu:61-64 — n normals N(mean, stddev). */
void randomizeGaussian(float* device, uint n, float mean, float stddev);
/* particleSystem_cuda.cu:66-69 (declared with int size in particleSystem.cuh:19). */
void allocateArray(void** devPtr, int size);
/* particleSystem_cuda.cu:71-74 */
void freeArray(void* devPtr);
/* particleSystem_cuda.cu:76-79 */
void threadSync(void);
/* particleSystem_cuda.cu:86-90; the graphics-resource argument is ignored. */
void copyArrayFromDevice(void* host, const void* device, struct cudaGraphicsResource** cuda_vbo_resource, int size);
/* particleSystem_cuda.cu:81-84 */
void copyArrayToDevice(void* device, const void* host, int offset, int size);
/* particleSystem_cuda.cu:92-96 */
void setParameters(struct SimParams* hostParams);
/* particleSystem_cuda.cu:98-102 */
void setSolventParameters(struct SolventParams* solventParams);
/* particleSystem_cuda.cu:117-133 — velocity Verlet + boundaries; f := 0, f_old := f. */
void integrateFilaments(float* pos, float* vel, float* f, float* f_old, float deltaTime, uint numParticles);
/* particleSystem_cuda.cu:136-149 — ballistic solvent streaming. */
void integrateSolvent(float* pos, float* vel, float deltaTime, uint startIndex, uint numSolvent);
/* particleSystem_cuda.cu:151-169 — bead (srd = false) or shifted SRD (srd = true) cell hash. */
void calcHash(uint* gridParticleHash, uint* gridParticleIndex, float* pos, int numParticles, bool srd NW_DEFAULT_FALSE);
/* particleSystem_cuda.cu:171-205 — cell start/end + gather into sorted order. */
void reorderDataAndFindCellStart(uint* cellStart, uint* cellEnd, float* sortedPos, float* sortedVel,
                                 float* sortedTangent, uint* gridParticleHash, uint* gridParticleIndex, float* pos,
                                 float* vel, float* tangent, uint numParticles, uint numCells);
/* particleSystem_cuda.cu:207-235 — DEM contact, cell-list bond, extensile drive. */
void collideFilaments(float* force, float* sortedPos, float* sortedVel, float* sortedTangent, uint* gridParticleIndex,
                      uint* cellStart, uint* cellEnd, uint numParticles, uint numCells);
/* particleSystem_cuda.cu:237-256 — SRD rotation of the solvent about the cell mean. */
void collideSolvent(float* pos, float* vel, float* solventCellCOM, float* random, uint numSolventCells,
                    uint numParticles);
/* particleSystem_cuda.cu:258-274 — bending forces and tangents (count passed as float, as in the reference). */
void filamentForces(float* force, float* tangent, float* pos, float numFilaments);
/* particleSystem_cuda.cu:277-282 — stable sort of (hash, index) pairs by hash. */
void sortParticles(uint* dGridParticleHash, uint* dGridParticleIndex, uint numParticles);
/* No counterpart in the reference.  The same stable sort as sortParticles,
 * for callers that cannot allocate device memory: those whose device memory
 * is owned in full by another allocator (a framework's caching allocator, a
 * budget fixed at start-up) and those whose timing-critical loop cannot take
 * cudaMalloc's implicit device-wide synchronisation.  Its scratch is one
 * fixed array compiled into the library (about 2.4 MB, held by every GPU that
 * loads the library until the process exits); it calls no allocator.
 * At most 262,144 keys: larger counts return NW_ERR_INVALID (2) and leave
 * the arrays untouched.  Returns an nw_status (0 = OK).  The first call on a
 * device looks up the array's device address, so make that first call before
 * any stream capture (a first call inside capture returns NW_ERR_INVALID);
 * calls outside capture look it up again, so after a cudaDeviceReset make one
 * call outside capture before capturing again.  A CUDA error already pending
 * from earlier work is returned as NW_ERR_CUDA before anything is launched
 * and left pending.  All calls share the one array; calls that overlap on
 * the GPU race.  Runs on the legacy default stream, like sortParticles. */
int nw_sort_particles_noalloc(uint* dGridParticleHash, uint* dGridParticleIndex, uint numParticles);
/* particleSystem_cuda.cu:284-306 — random filament reversal. */
void reverseFilaments(float* force, float* forceOld, float* vel, float* pos, float* uniform, uint numFilaments);
/* particleSystem_cuda.cu:308-328 — f += -gamma v + N(0, sqrt(2 gamma kT)). */
void langevinThermostat(float* force, float* vel, float* random, float gamma, float kbT, uint numParticles);
/* particleSystem_cuda.cu:331-349 */
void solventCellCentorOfMomentum(float* solventCellCOM, float* sortedVel, uint* cellStart, uint* cellEnd,
                                 uint* gridParticleIndex, uint numCells);
/* particleSystem_cuda.cu:351-369 */
void solventIsokineticThermostat(float* vel, float* sortedVel, uint* cellStart, uint* cellEnd, uint* gridParticleIndex,
                                 uint numCells);

/* ---- extensions (no counterpart symbol in the reference) ------------------ */

/* Status of the last failing legacy call (0 = none), cleared by reading. */
int nw_legacy_last_status(void);
/* Seed of the legacy RNG stream (the reference never seeds cuRAND). */
void nw_legacy_seed(uint64_t seed);
/* The kernel parts of langevinThermostat, reverseFilaments and collideSolvent
 * with a caller-supplied random buffer (for injecting the same numbers into
 * the reference and this implementation). */
void nw_legacy_langevin_apply(float* force, float* vel, const float* gaussian, uint numParticles);
void nw_legacy_reverse_apply(float* force, float* forceOld, float* vel, float* pos, const float* uniform,
                             uint numFilaments);
void nw_legacy_collide_solvent_apply(float* pos, float* vel, const float* solventCellCOM, const float* uniform,
                                     uint numParticles);

#ifdef __cplusplus
}
#endif

#endif
