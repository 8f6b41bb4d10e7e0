/*
 * nwref_host.cu — host side of the reference CUDA build on the GPU.
 *
 * TEST INFRASTRUCTURE ONLY: the checker and the speed denominator for the
 * engine; nothing in the product links or loads it.
 *
 * The reference's device code (simulation/particles_kernel_impl.cuh, built
 * unmodified for sm_103a into oracle/_ref/nwref_kernels.fatbin by
 * oracle/ref_cuda/Makefile) is loaded with the driver API.  This file issues
 * the reference's launches the way its C-ABI layer does
 * (simulation/particleSystem_cuda.cu:36-371): the same kernels, 256-thread
 * blocks from computeGridSize, the same dynamic shared memory, the same
 * cudaMemset of the cell starts, thrust::sort_by_key for the sort, cuRAND's
 * default generator (never seeded) for the random buffers, parameters copied
 * to the module's __constant__ symbols before every update, all on the
 * legacy default stream.  The two thrust::for_each integrators run as one
 * thread per element (nwref_kernels.cu).  The host orchestration restates
 * ParticleSystem::update / _solventUpdate (simulation/particleSystem.cpp:
 * 249-413) and the buffer set of _initialize (:172-223); unlike the
 * reference, force and old force start at zero (:202-203 leaves them
 * uninitialised).
 *
 * The reference's x86 host objects cannot run on the Arm GPU host and its
 * source tree is not there, so this harness (built on either host by the
 * package build) stands in for particleSystem_cuda.cu's host half; the
 * fatbin travels.
 */
#include <cuda.h>
#include <math.h>
#include <cuda_runtime.h>
#include <curand.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <thrust/device_ptr.h>
#include <thrust/sort.h>

#include "../../nematic-worms_gb300/compat/particles_kernel.cuh"

namespace {

char g_err[512];
bool g_ready = false;
CUmodule g_mod;
CUdeviceptr g_params, g_srd;
curandGenerator_t g_rng;

enum {
    K_HASH, K_REORDER, K_COM, K_ISO, K_COLLIDE_SOLVENT, K_COLLIDE_FIL, K_FILAMENT, K_REVERSE, K_LANGEVIN,
    K_INT_FIL, K_INT_SOLVENT, K_COUNT
};
/* Itanium-mangled names of the reference's kernels (their signatures in
 * simulation/particles_kernel_impl.cuh:312-874) and the two functor entry
 * points of nwref_kernels.cu. */
const char* const k_names[K_COUNT] = {
    "_Z9calcHashDPjS_P6float4jb",
    "_Z28reorderDataAndFindCellStartDPjS_P6float4S1_S1_S_S_S1_S1_S1_j",
    "_Z23cellCenterOfMomentumSRDP6float4S0_PjS1_S1_j",
    "_Z23isokineticThermostatSRDP6float4S0_PjS1_S1_j",
    "_Z20collideSolventKernelP6float4S0_S0_Pfj",
    "_Z22collideFilamentsKernelP6float4S0_S0_S0_PjS1_S1_j",
    "_Z14filamentKernelP6float4S0_S0_j",
    "_Z22reverseFilamentsKernelP6float4S0_S0_S0_Pfj",
    "_Z14langevinKernelP6float4S0_S0_j",
    "nwref_filament_integrator",
    "nwref_solvent_integrator",
};
CUfunction g_fn[K_COUNT];

int fail(const char* what, int code)
{
    snprintf(g_err, sizeof g_err, "%s (code %d)", what, code);
    fprintf(stderr, "nwref: %s\n", g_err);
    return code ? code : -1;
}

/* particleSystem_cuda.cu:105-115 */
void grid_size(uint n, uint block, uint& blocks, uint& threads)
{
    threads = n < block ? n : block;
    blocks = (n + threads - 1) / threads;
}

int launch(int k, uint n, void** args, uint smem = 0)
{
    if (!g_ready) return fail("nwref_init has not succeeded", -2);
    if (n == 0) return 0;
    uint blocks, threads;
    grid_size(n, 256, blocks, threads);
    CUresult r = cuLaunchKernel(g_fn[k], blocks, 1, 1, threads, 1, 1, smem, nullptr, args, nullptr);
    if (r != CUDA_SUCCESS) return fail(k_names[k], (int)r);
    return 0;
}

}  // namespace

extern "C" {

const char* nwref_error(void) { return g_err; }

/* Load the fatbin into the current device's primary context, resolve the
 * kernels and the two __constant__ parameter blocks (checking their sizes
 * against this layout), create cuRAND's default generator
 * (particleSystem_cuda.cu:40-54). */
int nwref_init(const char* fatbin_path)
{
    if (g_ready) return 0;
    cudaError_t ce = cudaFree(nullptr);
    if (ce != cudaSuccess) return fail("CUDA runtime initialisation", (int)ce);
    CUresult r = cuModuleLoad(&g_mod, fatbin_path);
    if (r != CUDA_SUCCESS) return fail("cuModuleLoad of the reference fatbin", (int)r);
    for (int k = 0; k < K_COUNT; ++k) {
        r = cuModuleGetFunction(&g_fn[k], g_mod, k_names[k]);
        if (r != CUDA_SUCCESS) return fail(k_names[k], (int)r);
    }
    size_t bytes = 0;
    r = cuModuleGetGlobal(&g_params, &bytes, g_mod, "params");
    if (r != CUDA_SUCCESS) return fail("params symbol", (int)r);
    if (bytes != sizeof(SimParams)) return fail("SimParams size differs from the reference's", (int)bytes);
    r = cuModuleGetGlobal(&g_srd, &bytes, g_mod, "srd");
    if (r != CUDA_SUCCESS) return fail("srd symbol", (int)r);
    if (bytes != sizeof(SolventParams)) return fail("SolventParams size differs from the reference's", (int)bytes);
    curandStatus_t cs = curandCreateGenerator(&g_rng, CURAND_RNG_PSEUDO_DEFAULT);
    if (cs != CURAND_STATUS_SUCCESS) return fail("curandCreateGenerator", (int)cs);
    g_ready = true;
    return 0;
}

/* ---- the reference's C-ABI layer, symbol by symbol ------------------------ */

int nwref_randomizeUniform(float* device, uint n)
{
    curandStatus_t s = curandGenerateUniform(g_rng, device, n);
    return s == CURAND_STATUS_SUCCESS ? 0 : fail("curandGenerateUniform", (int)s);
}

int nwref_randomizeGaussian(float* device, uint n, float mean, float stddev)
{
    curandStatus_t s = curandGenerateNormal(g_rng, device, n, mean, stddev);
    return s == CURAND_STATUS_SUCCESS ? 0 : fail("curandGenerateNormal", (int)s);
}

int nwref_setParameters(const SimParams* p)
{
    CUresult r = cuMemcpyHtoD(g_params, p, sizeof(SimParams));
    return r == CUDA_SUCCESS ? 0 : fail("setParameters", (int)r);
}

int nwref_setSolventParameters(const SolventParams* p)
{
    CUresult r = cuMemcpyHtoD(g_srd, p, sizeof(SolventParams));
    return r == CUDA_SUCCESS ? 0 : fail("setSolventParameters", (int)r);
}

int nwref_integrateFilaments(float* pos, float* vel, float* f, float* f_old, float dt, uint n)
{
    void* a[] = {&pos, &vel, &f, &f_old, &dt, &n};
    return launch(K_INT_FIL, n, a);
}

int nwref_integrateSolvent(float* pos, float* vel, float dt, uint start, uint n)
{
    void* a[] = {&pos, &vel, &dt, &start, &n};
    return launch(K_INT_SOLVENT, n, a);
}

int nwref_calcHash(uint* hash, uint* index, float* pos, int n, bool srd)
{
    uint un = (uint)n;
    void* a[] = {&hash, &index, &pos, &un, &srd};
    return launch(K_HASH, un, a);
}

int nwref_reorderDataAndFindCellStart(uint* cellStart, uint* cellEnd, float* sortedPos, float* sortedVel,
                                      float* sortedTangent, uint* hash, uint* index, float* pos, float* vel,
                                      float* tangent, uint n, uint numCells)
{
    cudaError_t e = cudaMemset(cellStart, 0xff, numCells * sizeof(uint));
    if (e != cudaSuccess) return fail("cudaMemset(cellStart)", (int)e);
    if (n == 0) return 0;
    uint blocks, threads;
    grid_size(n, 256, blocks, threads);
    void* a[] = {&cellStart, &cellEnd, &sortedPos, &sortedVel, &sortedTangent, &hash, &index, &pos, &vel, &tangent,
                 &n};
    return launch(K_REORDER, n, a, (uint)sizeof(uint) * (threads + 1));
}

int nwref_collideFilaments(float* force, float* sortedPos, float* sortedVel, float* sortedTangent, uint* index,
                           uint* cellStart, uint* cellEnd, uint n, uint numCells)
{
    (void)numCells;
    void* a[] = {&force, &sortedPos, &sortedVel, &sortedTangent, &index, &cellStart, &cellEnd, &n};
    return launch(K_COLLIDE_FIL, n, a);
}

/* collideSolventKernel with a given uniform buffer (the kernel half of
 * collideSolvent, particleSystem_cuda.cu:237-256). */
int nwref_collide_solvent_apply(float* pos, float* vel, float* com, float* uniform, uint n)
{
    void* a[] = {&pos, &vel, &com, &uniform, &n};
    return launch(K_COLLIDE_SOLVENT, n, a);
}

int nwref_collideSolvent(float* pos, float* vel, float* com, float* random, uint numSolventCells, uint n)
{
    int s = nwref_randomizeUniform(random, numSolventCells);
    return s ? s : nwref_collide_solvent_apply(pos, vel, com, random, n);
}

int nwref_filamentForces(float* force, float* tangent, float* pos, float numFilaments)
{
    uint m = (uint)numFilaments;
    void* a[] = {&force, &tangent, &pos, &m};
    return launch(K_FILAMENT, m, a);
}

int nwref_sortParticles(uint* hash, uint* index, uint n)
{
    thrust::sort_by_key(thrust::device_ptr<uint>(hash), thrust::device_ptr<uint>(hash + n),
                        thrust::device_ptr<uint>(index));
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : fail("thrust::sort_by_key", (int)e);
}

int nwref_reverse_apply(float* force, float* forceOld, float* vel, float* pos, float* uniform, uint m)
{
    void* a[] = {&force, &forceOld, &vel, &pos, &uniform, &m};
    return launch(K_REVERSE, m, a);
}

int nwref_reverseFilaments(float* force, float* forceOld, float* vel, float* pos, float* random, uint m)
{
    int s = nwref_randomizeUniform(random, m);
    return s ? s : nwref_reverse_apply(force, forceOld, vel, pos, random, m);
}

int nwref_langevin_apply(float* force, float* vel, float* gaussian, uint n)
{
    void* a[] = {&force, &vel, &gaussian, &n};
    return launch(K_LANGEVIN, n, a);
}

int nwref_langevinThermostat(float* force, float* vel, float* random, float gamma, float kbT, uint n)
{
    const float stddev = sqrtf(2.0f * gamma * kbT);
    int s = nwref_randomizeGaussian(random, 4 * n, 0.0f, stddev);
    return s ? s : nwref_langevin_apply(force, vel, random, n);
}

int nwref_solventCellCentorOfMomentum(float* com, float* sortedVel, uint* cellStart, uint* cellEnd, uint* index,
                                      uint numCells)
{
    void* a[] = {&com, &sortedVel, &cellStart, &cellEnd, &index, &numCells};
    return launch(K_COM, numCells, a);
}

int nwref_solventIsokineticThermostat(float* vel, float* sortedVel, uint* cellStart, uint* cellEnd, uint* index,
                                      uint numCells)
{
    void* a[] = {&vel, &sortedVel, &cellStart, &cellEnd, &index, &numCells};
    return launch(K_ISO, numCells, a);
}

/* ---- the reference's ParticleSystem buffers and update sequence ----------- */

struct nwref_system;
int nwref_copy(nwref_system* sys, int which, void* host, size_t offset, size_t bytes, int to_device);

enum {
    NWREF_POS, NWREF_VEL, NWREF_TANGENT, NWREF_FORCE, NWREF_FORCE_OLD, NWREF_RANDOM, NWREF_SORTED_POS,
    NWREF_SORTED_VEL, NWREF_SORTED_TANGENT, NWREF_HASH, NWREF_INDEX, NWREF_CELL_START, NWREF_CELL_END,
    NWREF_SOLVENT_COM, NWREF_NBUF
};

struct nwref_system {
    SimParams params;
    SolventParams solvent;
    uint numParticles, numSolvent, numFilaments, numGridCells, numSolventCells, solventGap;
    int srd;
    unsigned long long updateCount;
    void* buf[NWREF_NBUF];
    size_t bytes[NWREF_NBUF];
};

/* Buffers of ParticleSystem::_initialize (particleSystem.cpp:172-223) for a
 * system whose parameters the caller has filled in; the SRD sizes follow
 * _initSolventParams (:124-148).  Refuses SRD systems with more SRD cells
 * than 4 x beads: the reference draws the per-cell uniforms into its 4N-float
 * random buffer (particleSystem_cuda.cu:244), which they would overrun. */
nwref_system* nwref_create(const SimParams* p, const SolventParams* s, uint solventGap)
{
    if (!g_ready) {
        fail("nwref_init has not succeeded", -2);
        return nullptr;
    }
    nwref_system* sys = (nwref_system*)calloc(1, sizeof(nwref_system));
    sys->params = *p;
    sys->srd = s && s->enabled;
    if (sys->srd) sys->solvent = *s;
    sys->numParticles = p->numParticles;
    sys->numFilaments = p->numFilaments;
    sys->numGridCells = p->gridSize.x * p->gridSize.y * p->gridSize.z;
    sys->numSolvent = sys->srd ? s->numParticles : 0;
    sys->numSolventCells = sys->srd ? s->numCells : 0;
    sys->solventGap = solventGap ? solventGap : 5;
    if (sys->srd && sys->numSolventCells > 4u * sys->numParticles) {
        fail("SRD cells exceed 4 x beads: the reference's random buffer would overflow", -3);
        free(sys);
        return nullptr;
    }
    const size_t N = sys->numParticles, NT = N + sys->numSolvent;
    const size_t sz[NWREF_NBUF] = {16 * NT, 16 * NT, 16 * N, 16 * N, 16 * N, 16 * N, 16 * NT, 16 * NT, 16 * N,
                                   4 * NT, 4 * NT, 4 * (size_t)sys->numGridCells, 4 * (size_t)sys->numGridCells,
                                   16 * (size_t)sys->numSolventCells};
    for (int b = 0; b < NWREF_NBUF; ++b) {
        sys->bytes[b] = sz[b];
        if (sz[b] == 0) continue;
        cudaError_t e = cudaMalloc(&sys->buf[b], sz[b]);
        if (e == cudaSuccess) e = cudaMemset(sys->buf[b], 0, sz[b]);
        if (e != cudaSuccess) {
            fail("cudaMalloc of a system buffer", (int)e);
            for (int c = 0; c < b; ++c) cudaFree(sys->buf[c]);
            free(sys);
            return nullptr;
        }
    }
    if (sys->srd && nwref_setSolventParameters(&sys->solvent)) return nullptr;
    if (nwref_setParameters(&sys->params)) return nullptr;
    return sys;
}

/* ParticleSystem(numFilaments, filamentSize, gridSize, srd): the
 * constructor's parameter defaults (particleSystem.cpp:64-107), the SRD
 * parameters of _initSolventParams (:124-148: SRD cells of two bead cells,
 * 10 solvent per SRD cell, a collision every 5 updates) and the buffers of
 * _initialize.  The caller applies the setters main.cpp would
 * (nwref_params / nwref_solvent) before the first update. */
nwref_system* nwref_create_reference(uint numFilaments, uint filamentSize, uint gx, uint gy, uint gz, int srd)
{
    SimParams p;
    memset(&p, 0, sizeof p);
    p.numFilaments = numFilaments;
    p.filamentSize = filamentSize;
    p.numParticles = numFilaments * filamentSize;
    p.particleRadius = 0.5f;
    p.particleMass = 1.0f;
    p.gridSize = make_uint3(gx, gy, gz);
    p.numCells = gx * gy * gz;
    const float cell = p.particleRadius * 2.0f;
    p.cellSize = make_float3(cell, cell, cell);
    p.boxSize = make_float3(gx * cell, gy * cell, gz * cell);
    p.origin = make_float3(-p.boxSize.x / 2.0f, -p.boxSize.y / 2.0f, -p.boxSize.z / 2.0f);
    p.boundaryX = p.boundaryY = p.boundaryZ = PERIODIC;
    p.bondSpringK = 57.f;
    p.bondSpringL = p.particleRadius * 0.8f;
    p.bondBendingK = 0.001f;
    p.spring = 0.5f;
    p.damping = 0.02f;
    p.shear = 0.1f;
    p.attraction = 0.0f;
    p.boundaryDamping = -0.5f;
    p.activity = 0.1f;
    p.reverseProbability = 0.0f;
    p.kbT = 1.0f;
    p.gamma = 0.01f;
    p.gravity = make_float3(0.f, 0.f, 0.f);
    SolventParams sv;
    memset(&sv, 0, sizeof sv);
    if (srd) {
        sv.enabled = true;
        sv.alpha = 2.26893f;
        sv.gridSize = make_uint3(gx / 2, gy / 2, gz / 2 > 1 ? gz / 2 : 1);
        sv.cellSize = make_float3(2.0f * cell, 2.0f * cell, 2.0f * cell);
        sv.numCells = sv.gridSize.x * sv.gridSize.y * sv.gridSize.z;
        sv.randOffset = make_float3(0.f, 0.f, 0.f);
        sv.particleMass = 1.0f;
        sv.kbT = p.kbT;
        sv.numParticles = (uint)(10.0f * (float)sv.numCells);
    }
    return nwref_create(&p, srd ? &sv : nullptr, 5);
}

/* ParticleSystem::reset (particleSystem.cpp:583-678): filaments along x on
 * the lattice, every one whose draw is >= 0.5 reversed, solvent uniform in
 * the box; rand() after srand(1) (the reference never seeds it).  Uploads
 * positions and velocities of beads and solvent and the bead tangents. */
int nwref_reset(nwref_system* sys)
{
    const SimParams& P = sys->params;
    const uint L = P.filamentSize, nb = sys->numParticles, ns = sys->numSolvent;
    const float R = P.particleRadius;
    const float flen = (float)L * P.bondSpringL + 2.0f * R;
    const int xdim = (int)floorf(P.boxSize.x / flen);
    const int ydim = (int)floorf(P.boxSize.y / (2 * R));
    if (nb && (xdim <= 0 || ydim <= 0)) return fail("box too small for the reset lattice", -5);
    const uint plane = (uint)(xdim * ydim);
    float* pos = (float*)calloc(4 * (size_t)(nb + ns), sizeof(float));
    float* vel = (float*)calloc(4 * (size_t)(nb + ns), sizeof(float));
    float* tan = (float*)calloc(4 * (size_t)(nb ? nb : 1), sizeof(float));
    srand(1);
    auto frand = []() { return rand() / (float)RAND_MAX; };
    for (uint i = 0; i < nb; ++i) {
        const uint w = i / L;
        const float xh = (float)(w % (uint)xdim) * flen + R;
        pos[4 * i + 0] = xh + (float)(i % L) * P.bondSpringL + P.origin.x;
        pos[4 * i + 1] = 2.f * R * (float)((w / (uint)xdim) % (uint)ydim + 1) + P.origin.y;
        pos[4 * i + 2] = 2.f * R * (float)(w / plane + 1) + P.origin.z;
        pos[4 * i + 3] = R;
        for (int a = 0; a < 3; ++a) vel[4 * i + a] = 0.1f * (frand() * 2.0f - 1.0f);
        vel[4 * i + 3] = P.particleMass;
        tan[4 * i] = 1.0f;
    }
    for (uint w = 0; w < P.numFilaments; ++w) {
        if (frand() < 0.5f) continue;
        for (uint q = 0; q < L / 2; ++q) {
            const size_t i = (size_t)w * L + q, j = (size_t)(w + 1) * L - 1 - q;
            for (int a = 0; a < 4; ++a) {
                const float t = pos[4 * i + a];
                pos[4 * i + a] = pos[4 * j + a];
                pos[4 * j + a] = t;
                tan[4 * i + a] = -tan[4 * i + a];
                tan[4 * j + a] = -tan[4 * j + a];
            }
        }
    }
    for (uint k = 0; k < ns; ++k) {
        const size_t i = (size_t)nb + k;
        pos[4 * i + 0] = P.boxSize.x * frand() + P.origin.x;
        pos[4 * i + 1] = P.boxSize.y * frand() + P.origin.y;
        pos[4 * i + 2] = P.boxSize.z * frand() + P.origin.z;
        for (int a = 0; a < 3; ++a) vel[4 * i + a] = 5.0f * (frand() * 2.0f - 1.0f);
        vel[4 * i + 3] = sys->solvent.particleMass;
    }
    int st = nwref_copy(sys, NWREF_POS, pos, 0, 16 * (size_t)(nb + ns), 1);
    if (!st) st = nwref_copy(sys, NWREF_VEL, vel, 0, 16 * (size_t)(nb + ns), 1);
    if (!st && nb) st = nwref_copy(sys, NWREF_TANGENT, tan, 0, 16 * (size_t)nb, 1);
    free(pos);
    free(vel);
    free(tan);
    return st;
}

void nwref_destroy(nwref_system* sys)
{
    if (!sys) return;
    for (int b = 0; b < NWREF_NBUF; ++b)
        if (sys->buf[b]) cudaFree(sys->buf[b]);
    free(sys);
}

SimParams* nwref_params(nwref_system* sys) { return &sys->params; }
SolventParams* nwref_solvent(nwref_system* sys) { return &sys->solvent; }
void* nwref_buffer(nwref_system* sys, int which) { return which >= 0 && which < NWREF_NBUF ? sys->buf[which] : nullptr; }
size_t nwref_buffer_bytes(nwref_system* sys, int which) { return which >= 0 && which < NWREF_NBUF ? sys->bytes[which] : 0; }
unsigned long long nwref_update_count(nwref_system* sys) { return sys->updateCount; }

int nwref_copy(nwref_system* sys, int which, void* host, size_t offset, size_t bytes, int to_device)
{
    if (which < 0 || which >= NWREF_NBUF || offset + bytes > sys->bytes[which]) return fail("nwref_copy range", -4);
    char* d = (char*)sys->buf[which] + offset;
    cudaError_t e = to_device ? cudaMemcpy(d, host, bytes, cudaMemcpyHostToDevice)
                              : cudaMemcpy(host, d, bytes, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? 0 : fail("nwref_copy", (int)e);
}

#define NWREF_TRY(x)       \
    do {                   \
        int s_ = (x);      \
        if (s_) return s_; \
    } while (0)

/* ParticleSystem::_solventUpdate (particleSystem.cpp:341-413).  The grid
 * shift is drawn with the C library's rand() as the reference's frand()
 * does, unless the caller passes one. */
static int solvent_update(nwref_system* sys, float dt, const float* shift)
{
    if (shift) {
        sys->solvent.randOffset.x = shift[0];
        sys->solvent.randOffset.y = shift[1];
    } else {
        sys->solvent.randOffset.x = rand() / (float)RAND_MAX * sys->solvent.cellSize.x;
        sys->solvent.randOffset.y = rand() / (float)RAND_MAX * sys->solvent.cellSize.y;
    }
    NWREF_TRY(nwref_setSolventParameters(&sys->solvent));
    const uint NT = sys->numParticles + sys->numSolvent;
    float** B = (float**)sys->buf;
    uint* hash = (uint*)sys->buf[NWREF_HASH];
    uint* index = (uint*)sys->buf[NWREF_INDEX];
    uint* cs = (uint*)sys->buf[NWREF_CELL_START];
    uint* ce = (uint*)sys->buf[NWREF_CELL_END];
    NWREF_TRY(nwref_calcHash(hash, index, B[NWREF_POS], (int)NT, true));
    NWREF_TRY(nwref_sortParticles(hash, index, NT));
    NWREF_TRY(nwref_reorderDataAndFindCellStart(cs, ce, B[NWREF_SORTED_POS], B[NWREF_SORTED_VEL], nullptr, hash,
                                                index, B[NWREF_POS], B[NWREF_VEL], nullptr, NT, sys->numGridCells));
    NWREF_TRY(nwref_solventIsokineticThermostat(B[NWREF_VEL], B[NWREF_SORTED_VEL], cs, ce, index,
                                                sys->numSolventCells));
    NWREF_TRY(nwref_solventCellCentorOfMomentum(B[NWREF_SOLVENT_COM], B[NWREF_SORTED_VEL], cs, ce, index,
                                                sys->numSolventCells));
    NWREF_TRY(nwref_collideSolvent(B[NWREF_POS], B[NWREF_VEL], B[NWREF_SOLVENT_COM], B[NWREF_RANDOM],
                                   sys->numSolventCells, NT));
    NWREF_TRY(nwref_integrateSolvent(B[NWREF_POS], B[NWREF_VEL], dt, sys->numParticles, sys->numSolvent));
    return 0;
}

/* ParticleSystem::update (particleSystem.cpp:249-339). */
int nwref_update(nwref_system* sys, float dt, const float* shift)
{
    float** B = (float**)sys->buf;
    uint* hash = (uint*)sys->buf[NWREF_HASH];
    uint* index = (uint*)sys->buf[NWREF_INDEX];
    uint* cs = (uint*)sys->buf[NWREF_CELL_START];
    uint* ce = (uint*)sys->buf[NWREF_CELL_END];
    const uint N = sys->numParticles;
    NWREF_TRY(nwref_setParameters(&sys->params));
    NWREF_TRY(nwref_integrateFilaments(B[NWREF_POS], B[NWREF_VEL], B[NWREF_FORCE], B[NWREF_FORCE_OLD], dt, N));
    if (sys->params.reverseProbability > 0.0f)
        NWREF_TRY(nwref_reverseFilaments(B[NWREF_FORCE], B[NWREF_FORCE_OLD], B[NWREF_VEL], B[NWREF_POS],
                                         B[NWREF_RANDOM], sys->numFilaments));
    if (!sys->srd)
        NWREF_TRY(nwref_langevinThermostat(B[NWREF_FORCE], B[NWREF_VEL], B[NWREF_RANDOM], sys->params.gamma,
                                           sys->params.kbT, N));
    NWREF_TRY(nwref_filamentForces(B[NWREF_FORCE], B[NWREF_TANGENT], B[NWREF_POS], (float)sys->numFilaments));
    NWREF_TRY(nwref_calcHash(hash, index, B[NWREF_POS], (int)N, false));
    NWREF_TRY(nwref_sortParticles(hash, index, N));
    NWREF_TRY(nwref_reorderDataAndFindCellStart(cs, ce, B[NWREF_SORTED_POS], B[NWREF_SORTED_VEL],
                                                B[NWREF_SORTED_TANGENT], hash, index, B[NWREF_POS], B[NWREF_VEL],
                                                B[NWREF_TANGENT], N, sys->numGridCells));
    NWREF_TRY(nwref_collideFilaments(B[NWREF_FORCE], B[NWREF_SORTED_POS], B[NWREF_SORTED_VEL],
                                     B[NWREF_SORTED_TANGENT], index, cs, ce, N, sys->numGridCells));
    if (sys->srd && (sys->updateCount % sys->solventGap) == 0)
        NWREF_TRY(solvent_update(sys, dt * (float)sys->solventGap, shift));
    sys->updateCount++;
    return 0;
}

/* n updates between two events on the legacy default stream (the thrust
 * sorts synchronise the host inside, as in the reference); *ms = elapsed. */
int nwref_run(nwref_system* sys, uint n, float dt, float* ms)
{
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaDeviceSynchronize();
    cudaEventRecord(a, 0);
    int s = 0;
    for (uint k = 0; k < n && !s; ++k) s = nwref_update(sys, dt, nullptr);
    cudaEventRecord(b, 0);
    cudaEventSynchronize(b);
    float t = 0.0f;
    cudaEventElapsedTime(&t, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (ms) *ms = t;
    cudaError_t e = cudaGetLastError();
    if (!s && e != cudaSuccess) s = fail("update loop", (int)e);
    return s;
}

int nwref_sync(void)
{
    cudaError_t e = cudaDeviceSynchronize();
    return e == cudaSuccess ? 0 : fail("cudaDeviceSynchronize", (int)e);
}

}  // extern "C"
