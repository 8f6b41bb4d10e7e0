/*
 * ref_emu_modern.cpp — runs the reference's own modern kernel source
 * (simulation/particles_kernel_impl.cuh, included unmodified from the
 * reference tree at build time) on the CPU.  TEST INFRASTRUCTURE ONLY: it
 * pins the oracle and generates golden vectors; nothing in the product
 * links it.
 *
 * Emulation model: a launch <<<blocks, threads>>> runs every thread to
 * completion, block by block, in increasing threadIdx order.  The kernels
 * used here either have no intra-block communication or (reorder) only read
 * shared values written by lower-numbered threads, so this order gives the
 * device result.  Each wrapper mirrors the launch in the reference's C-ABI
 * layer (simulation/particleSystem_cuda.cu), with the same 256-thread blocks.
 */
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>
#include <tuple>

static uint3 nwemu_threadIdx, nwemu_blockIdx;
static dim3 nwemu_blockDim;
#define threadIdx nwemu_threadIdx
#define blockIdx nwemu_blockIdx
#define blockDim nwemu_blockDim

static inline unsigned int __umul24(unsigned int a, unsigned int b)
{
    return (unsigned int)((unsigned long long)(a & 0xffffffu) * (unsigned long long)(b & 0xffffffu));
}
static inline int __mul24(int a, int b)
{
    /* signed 24-bit multiply: sign-extend the low 24 bits of each operand */
    long long x = (long long)((int)((unsigned)a << 8) >> 8);
    long long y = (long long)((int)((unsigned)b << 8) >> 8);
    return (int)(unsigned int)(unsigned long long)(x * y);
}

/* thrust::get on the std::tuple of references the functor wrappers pass */
namespace thrust {
template <int I, class T>
auto& get(T& t) { return std::get<I>(t); }
}

/* Every header the kernel file pulls in is parsed first; `volatile` (a
 * register-spill hint in the device code, meaningless for a sequential CPU
 * run) is then erased only while the kernel file itself is parsed, so that
 * its volatile float4 temporaries can be passed to helper_math.h by value. */
#include <stdio.h>
#include "vector_functions.h"
#include "helper_math.h"
#include "math_constants.h"
#include <cooperative_groups.h>
#define volatile
#include "particles_kernel_impl.cuh"
#undef volatile

/* dynamic shared memory of reorderDataAndFindCellStartD */
unsigned int sharedHash[257];

#include "../../include/nwgb.h"

template <class Fn>
static void launch(uint32_t n, Fn fn)
{
    if (n == 0) return;
    uint32_t threads = n < 256u ? n : 256u;
    uint32_t blocks = (n + threads - 1) / threads;
    nwemu_blockDim = dim3(threads, 1, 1);
    for (uint32_t b = 0; b < blocks; ++b) {
        nwemu_blockIdx = make_uint3(b, 0, 0);
        for (uint32_t t = 0; t < threads; ++t) {
            nwemu_threadIdx = make_uint3(t, 0, 0);
            fn();
        }
    }
}

static void load_params(const NwConfig* c, const float* shift)
{
    SimParams p;
    memset(&p, 0, sizeof(p));
    p.gravity = make_float3(c->gravity[0], c->gravity[1], c->gravity[2]);
    p.particleRadius = c->radius;
    p.particleMass = c->mass;
    p.gridSize = make_uint3(c->grid[0], c->grid[1], c->grid[2]);
    p.numCells = c->grid[0] * c->grid[1] * c->grid[2];
    p.origin = make_float3(c->origin[0], c->origin[1], c->origin[2]);
    p.boxSize = make_float3(c->box[0], c->box[1], c->box[2]);
    p.cellSize = make_float3(c->cell_size[0], c->cell_size[1], c->cell_size[2]);
    p.boundaryX = (BoundaryType)c->boundary[0];
    p.boundaryY = (BoundaryType)c->boundary[1];
    p.boundaryZ = (BoundaryType)c->boundary[2];
    p.numFilaments = c->num_filaments;
    p.filamentSize = c->filament_size;
    p.numParticles = c->num_filaments * c->filament_size;
    p.bondSpringK = c->bond_k;
    p.bondSpringL = c->bond_r0;
    p.bondBendingK = c->bend_k;
    p.activity = c->activity;
    p.reverseProbability = c->reverse_probability;
    p.kbT = c->kT;
    p.gamma = c->gamma;
    p.spring = c->spring;
    p.damping = c->damping;
    p.shear = c->shear;
    p.attraction = c->attraction;
    p.boundaryDamping = c->boundary_damping;
    params = p;

    SolventParams s;
    memset(&s, 0, sizeof(s));
    s.enabled = c->srd_enabled != 0;
    s.gridSize = make_uint3(c->srd_grid[0], c->srd_grid[1], c->srd_grid[2]);
    s.numCells = c->srd_grid[0] * c->srd_grid[1] * c->srd_grid[2];
    s.randOffset = shift ? make_float3(shift[0], shift[1], shift[2]) : make_float3(0.f, 0.f, 0.f);
    s.cellSize = make_float3(c->srd_cell_size[0], c->srd_cell_size[1], c->srd_cell_size[2]);
    s.numParticles = c->num_solvent;
    s.alpha = c->srd_alpha;
    s.kbT = c->srd_kT;
    s.particleMass = c->solvent_mass;
    srd = s;
}

extern "C" {

/* calcHash (simulation/particleSystem_cuda.cu:151-169) */
void ref_calc_hash(const NwConfig* c, const float* shift, uint32_t* hash, uint32_t* index, float* pos,
                   uint32_t n, int use_srd)
{
    load_params(c, shift);
    launch(n, [&] { calcHashD(hash, index, (float4*)pos, n, use_srd != 0); });
}

/* reorderDataAndFindCellStart (simulation/particleSystem_cuda.cu:171-205) */
void ref_reorder(const NwConfig* c, uint32_t* cellStart, uint32_t* cellEnd, float* sortedPos, float* sortedVel,
                 float* sortedTangent, uint32_t* hash, uint32_t* index, float* pos, float* vel, float* tangent,
                 uint32_t n, uint32_t numCells)
{
    load_params(c, nullptr);
    memset(cellStart, 0xff, sizeof(uint32_t) * numCells);
    launch(n, [&] {
        reorderDataAndFindCellStartD(cellStart, cellEnd, (float4*)sortedPos, (float4*)sortedVel,
                                     (float4*)sortedTangent, hash, index, (float4*)pos, (float4*)vel,
                                     (float4*)tangent, n);
    });
}

/* collideFilaments (simulation/particleSystem_cuda.cu:207-235) */
void ref_collide_filaments(const NwConfig* c, float* force, float* sortedPos, float* sortedVel, float* sortedTangent,
                           uint32_t* index, uint32_t* cellStart, uint32_t* cellEnd, uint32_t n)
{
    load_params(c, nullptr);
    launch(n, [&] {
        collideFilamentsKernel((float4*)force, (float4*)sortedPos, (float4*)sortedVel, (float4*)sortedTangent, index,
                               cellStart, cellEnd, n);
    });
}

/* filamentForces (simulation/particleSystem_cuda.cu:258-274) */
void ref_filament_forces(const NwConfig* c, float* force, float* tangent, float* pos, uint32_t numFilaments)
{
    load_params(c, nullptr);
    launch(numFilaments, [&] { filamentKernel((float4*)force, (float4*)tangent, (float4*)pos, numFilaments); });
}

/* langevinThermostat kernel part (simulation/particleSystem_cuda.cu:308-328) with
 * an injected noise buffer in place of curandGenerateNormal */
void ref_langevin(const NwConfig* c, float* force, float* vel, float* gaussian, uint32_t n)
{
    load_params(c, nullptr);
    launch(n, [&] { langevinKernel((float4*)force, (float4*)vel, (float4*)gaussian, n); });
}

/* integrateFilaments (simulation/particleSystem_cuda.cu:117-133): the thrust
 * functor applied to every particle */
void ref_integrate(const NwConfig* c, float* pos, float* vel, float* f, float* fo, float dt, uint32_t n)
{
    load_params(c, nullptr);
    filament_integrator op(dt);
    float4 *P = (float4*)pos, *V = (float4*)vel, *F = (float4*)f, *Fo = (float4*)fo;
    for (uint32_t i = 0; i < n; ++i) op(std::tuple<float4&, float4&, float4&, float4&>(P[i], V[i], F[i], Fo[i]));
}

/* integrateSolvent (simulation/particleSystem_cuda.cu:136-149) */
void ref_integrate_solvent(const NwConfig* c, float* pos, float* vel, float dt, uint32_t start, uint32_t count)
{
    load_params(c, nullptr);
    solvent_integrator op(dt);
    float4 *P = (float4*)pos, *V = (float4*)vel;
    for (uint32_t i = start; i < start + count; ++i) op(std::tuple<float4&, float4&>(P[i], V[i]));
}

/* reverseFilaments kernel part (simulation/particleSystem_cuda.cu:284-306) */
void ref_reverse(const NwConfig* c, float* force, float* forceOld, float* vel, float* pos, float* uniform,
                 uint32_t numFilaments)
{
    load_params(c, nullptr);
    launch(numFilaments, [&] {
        reverseFilamentsKernel((float4*)force, (float4*)forceOld, (float4*)vel, (float4*)pos, uniform, numFilaments);
    });
}

/* solventIsokineticThermostat (simulation/particleSystem_cuda.cu:351-369) */
void ref_srd_thermostat(const NwConfig* c, float* vel, float* sortedVel, uint32_t* cellStart, uint32_t* cellEnd,
                        uint32_t* index, uint32_t numCells)
{
    load_params(c, nullptr);
    launch(numCells, [&] {
        isokineticThermostatSRD((float4*)vel, (float4*)sortedVel, cellStart, cellEnd, index, numCells);
    });
}

/* solventCellCentorOfMomentum (simulation/particleSystem_cuda.cu:331-349) */
void ref_srd_com(const NwConfig* c, float* com, float* sortedVel, uint32_t* cellStart, uint32_t* cellEnd,
                 uint32_t* index, uint32_t numCells)
{
    load_params(c, nullptr);
    launch(numCells, [&] {
        cellCenterOfMomentumSRD((float4*)com, (float4*)sortedVel, cellStart, cellEnd, index, numCells);
    });
}

/* collideSolvent kernel part (simulation/particleSystem_cuda.cu:237-256) with an
 * injected per-cell uniform buffer */
void ref_collide_solvent(const NwConfig* c, const float* shift, float* pos, float* vel, float* com, float* uniform,
                         uint32_t nTotal)
{
    load_params(c, shift);
    launch(nTotal, [&] { collideSolventKernel((float4*)pos, (float4*)vel, (float4*)com, uniform, nTotal); });
}

size_t ref_sizeof_simparams(void) { return sizeof(SimParams); }

} /* extern "C" */
