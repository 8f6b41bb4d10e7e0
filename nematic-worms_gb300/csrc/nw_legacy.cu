// nw_legacy.cu — the reference's 20 C-ABI symbols (include/nw_legacy.h) on
// the GB300 kernels.  One process-wide parameter set, as in the reference
// (its __constant__ SimParams / SolventParams, particles_kernel_impl.cuh:29-30);
// all work on the legacy default stream.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "../../include/nw_legacy.h"
#include "nw_engine.h"
#include "nw_sort.cuh"

namespace nw {
namespace {

SimParams g_params;
SolventParams g_solvent;
bool g_have_params = false;
uint64_t g_seed = 0x5eed5eedull;
uint64_t g_calls = 0;
int g_last_status = 0;
std::mutex g_mu;
uint32_t* g_err = nullptr;
RadixScratch g_radix;

void note(cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return;
    std::fprintf(stderr, "[nwgb legacy] %s: %s\n", what, cudaGetErrorString(e));
    g_last_status = e == cudaErrorMemoryAllocation ? NW_ERR_NOMEM : NW_ERR_CUDA;
}

void check_launch(const char* what) { note(cudaGetLastError(), what); }

uint32_t* err_word()
{
    if (!g_err) {
        if (cudaMalloc(&g_err, 16) == cudaSuccess) cudaMemset(g_err, 0, 16);
        else g_err = nullptr;
    }
    return g_err;
}

// SimParams + SolventParams -> kernel parameter block (REF_DEM semantics).
DevParams legacy_params()
{
    NwConfig c;
    std::memset(&c, 0, sizeof(c));
    const SimParams& p = g_params;
    c.abi_version = NW_ABI_VERSION;
    c.model = NW_MODEL_REF_DEM;
    c.dim = 3;
    c.hash_mode = NW_HASH_MASK;
    c.num_filaments = p.numFilaments;
    c.filament_size = p.filamentSize ? p.filamentSize : 1u;
    c.grid[0] = p.gridSize.x;
    c.grid[1] = p.gridSize.y;
    c.grid[2] = p.gridSize.z;
    c.cell_size[0] = p.cellSize.x;
    c.cell_size[1] = p.cellSize.y;
    c.cell_size[2] = p.cellSize.z;
    c.origin[0] = p.origin.x;
    c.origin[1] = p.origin.y;
    c.origin[2] = p.origin.z;
    c.box[0] = p.boxSize.x;
    c.box[1] = p.boxSize.y;
    c.box[2] = p.boxSize.z;
    c.boundary[0] = p.boundaryX;
    c.boundary[1] = p.boundaryY;
    c.boundary[2] = p.boundaryZ;
    c.radius = p.particleRadius;
    c.mass = p.particleMass;
    c.bond_k = p.bondSpringK;
    c.bond_r0 = p.bondSpringL;
    c.bend_k = p.bondBendingK;
    c.spring = p.spring;
    c.damping = p.damping;
    c.shear = p.shear;
    c.attraction = p.attraction;
    c.boundary_damping = p.boundaryDamping;
    c.activity = p.activity;
    c.reverse_probability = p.reverseProbability;
    c.gamma = p.gamma;
    c.kT = p.kbT;
    c.srd_enabled = g_solvent.enabled ? 1 : 0;
    c.num_solvent = g_solvent.numParticles;
    c.srd_grid[0] = g_solvent.gridSize.x;
    c.srd_grid[1] = g_solvent.gridSize.y;
    c.srd_grid[2] = g_solvent.gridSize.z;
    c.srd_cell_size[0] = g_solvent.cellSize.x;
    c.srd_cell_size[1] = g_solvent.cellSize.y;
    c.srd_cell_size[2] = g_solvent.cellSize.z;
    c.srd_alpha = g_solvent.alpha;
    c.srd_kT = g_solvent.kbT;
    c.solvent_mass = g_solvent.particleMass;
    c.srd_thermostat = NW_SRD_THERMO_REF_LAB;
    c.srd_rotate_beads = 0;
    c.seed = g_seed;
    c.dt = 1.0f;
    DevParams P = make_dev_params(c, 1.0f);
    P.nb = p.numParticles;
    return P;
}

uint32_t blocks_for(uint64_t n, uint32_t t) { return (uint32_t)((n + t - 1) / t); }

// ---- legacy kernels ------------------------------------------------------------

__global__ void fill_uniform_kernel(float* out, uint32_t n, uint32_t seed_lo, uint32_t seed_hi, unsigned long long call)
{
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if ((uint64_t)q * 4u >= n) return;
    const uint4 x = philox4x32_10(make_uint4(q, (uint32_t)call, (uint32_t)(call >> 32), 0x4c454741u), seed_lo, seed_hi);
    const uint32_t v[4] = {x.x, x.y, x.z, x.w};
    for (int k = 0; k < 4; ++k)
        if ((uint64_t)q * 4u + k < n) out[(size_t)q * 4u + k] = u01(v[k]);
}

__global__ void fill_normal_kernel(float* out, uint32_t n, float mean, float stddev, uint32_t seed_lo, uint32_t seed_hi,
                                   unsigned long long call)
{
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if ((uint64_t)q * 4u >= n) return;
    const float4 z =
        normal4(philox4x32_10(make_uint4(q, (uint32_t)call, (uint32_t)(call >> 32), 0x4c454741u), seed_lo, seed_hi));
    const float v[4] = {z.x, z.y, z.z, z.w};
    for (int k = 0; k < 4; ++k)
        if ((uint64_t)q * 4u + k < n) out[(size_t)q * 4u + k] = mean + stddev * v[k];
}

// filament_integrator / solvent_integrator (particles_kernel_impl.cuh:71-205)
__global__ void integrate_kernel(const DevParams P, float4* pos, float4* vel, float4* f, float4* fo, float dt,
                                 uint32_t n)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 P4 = pos[i], V4 = vel[i], F4 = f[i], Fo4 = fo[i];
    float3 p = f3(P4), v = f3(V4);
    const float3 F = f3(F4), Fo = f3(Fo4);
    const float3 dv = (0.5f * (F + Fo)) * dt;
    v += dv;
    const float3 dr = v * dt + ((0.5f * F) * dt) * dt;
    p += dr;
    apply_boundaries(P, p, v, dr, P.radius);
    pos[i] = make_float4(p.x, p.y, p.z, P4.w);
    vel[i] = make_float4(v.x, v.y, v.z, V4.w);
    f[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    fo[i] = make_float4(F.x, F.y, F.z, Fo4.w);
}

__global__ void integrate_solvent_kernel(const DevParams P, float4* pos, float4* vel, float dt, uint32_t start,
                                         uint32_t count)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const uint32_t i = start + k;
    const float4 P4 = pos[i], V4 = vel[i];
    float3 p = f3(P4), v = f3(V4);
    const float3 dr = dt * v;
    p += dr;
    apply_boundaries(P, p, v, dr, 0.0f);
    pos[i] = make_float4(p.x, p.y, p.z, P4.w);
    vel[i] = make_float4(v.x, v.y, v.z, V4.w);
}

// calcHashD (particles_kernel_impl.cuh:312-342)
__global__ void hash_kernel(const DevParams P, uint32_t* hash, uint32_t* index, const float4* pos, uint32_t n, int srd,
                            float3 shift)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float3 p = f3(pos[i]);
    hash[i] = srd ? srd_hash(P, p, shift) : bead_hash(P, p);
    index[i] = i;
}

// reorderDataAndFindCellStartD (particles_kernel_impl.cuh:346-424): a cell
// starts where the sorted hash changes; only non-empty cells get an end.
__global__ void reorder_kernel(uint32_t* cellStart, uint32_t* cellEnd, float4* sPos, float4* sVel, float4* sTan,
                               const uint32_t* hash, const uint32_t* index, const float4* pos, const float4* vel,
                               const float4* tan, uint32_t n, uint32_t numCells, uint32_t* err)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t h = hash[i];
    const uint32_t prev = i > 0 ? hash[i - 1] : 0u;
    if (i == 0 || h != prev) {
        if (h < numCells) cellStart[h] = i;
        else atomicOr(err, (uint32_t)NW_EFLAG_BAD_INDEX);
        if (i > 0 && prev < numCells) cellEnd[prev] = i;
    }
    if (i == n - 1 && h < numCells) cellEnd[h] = i + 1;
    const uint32_t s = index[i];
    if (s >= n) {
        atomicOr(err, (uint32_t)NW_EFLAG_BAD_INDEX);
        return;
    }
    sPos[i] = pos[s];
    if (vel && sVel) sVel[i] = vel[s];
    if (tan && sTan) sTan[i] = tan[s];
}

// filamentKernel (particles_kernel_impl.cuh:751-818) with one thread per bead:
// the bead's (up to three) triple contributions in triple order, and its tangent.
__global__ void filament_kernel(const DevParams P, float4* force, float4* tangent, const float4* pos, uint32_t nf)
{
    const uint32_t L = P.L;
    const uint64_t gi = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gi >= (uint64_t)nf * L) return;
    const uint32_t i = (uint32_t)gi;
    const uint32_t w = i / L, c = i - w * L;
    const float4* R = pos + (size_t)w * L;
    if (L >= 3) {
        float3 fs = zero3();
        if (c >= 2) fs += bend_triple(P, f3(R[c - 2]), f3(R[c - 1]), f3(R[c])).fk;
        if (c >= 1 && c + 1 < L) fs += bend_triple(P, f3(R[c - 1]), f3(R[c]), f3(R[c + 1])).fj;
        if (c + 2 < L) fs += bend_triple(P, f3(R[c]), f3(R[c + 1]), f3(R[c + 2])).fi;
        float4 F = force[i];
        force[i] = make_float4(F.x + fs.x, F.y + fs.y, F.z + fs.z, F.w);
        float3 tg;
        bool wt = true;
        if (c == 0) tg = tangent_of(P, f3(R[0]), f3(R[1]));
        else if (c == L - 1) {
            wt = L > 3;
            tg = wt ? tangent_of(P, f3(R[L - 2]), f3(R[L - 1])) : zero3();
        } else tg = tangent_of(P, f3(R[c - 1]), f3(R[c + 1]));
        if (wt) tangent[i] = make_float4(tg.x, tg.y, tg.z, 0.f);
    }
}

__global__ void langevin_kernel(const DevParams P, float4* force, const float4* vel, const float4* gaussian, uint32_t n)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float3 f = zero3() - P.gamma * f3(vel[i]);
    f += f3(gaussian[i]);
    const float4 F = force[i];
    force[i] = make_float4(F.x + f.x, F.y + f.y, F.z + f.z, F.w + 0.f);
}

__global__ void reverse_kernel(const DevParams P, float4* force, float4* forceOld, float4* vel, float4* pos,
                               const float* uniform, uint32_t nf)
{
    const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nf) return;
    if (uniform[w] > P.reverse_p) return;
    const uint32_t L = P.L;
    const size_t head = (size_t)w * L;
    for (uint32_t q = 0; q < L / 2; ++q) {
        const size_t i = head + q, j = head + L - 1 - q;
        float4 t;
        t = pos[i]; pos[i] = pos[j]; pos[j] = t;
        t = vel[i]; vel[i] = vel[j]; vel[j] = t;
        t = force[i]; force[i] = force[j]; force[j] = t;
        t = forceOld[i]; forceOld[i] = forceOld[j]; forceOld[j] = t;
    }
}

// cellCenterOfMomentumSRD (particles_kernel_impl.cuh:560-594)
__global__ void com_kernel(float4* com, const float4* sortedVel, const uint32_t* cellStart, const uint32_t* cellEnd,
                           uint32_t numCells)
{
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= numCells) return;
    float3 u = zero3();
    const uint32_t s0 = cellStart[c];
    if (s0 != kEmpty) {
        const uint32_t s1 = cellEnd[c];
        float M = 0.f;
        for (uint32_t k = s0; k < s1; ++k) {
            const float4 V = sortedVel[k];
            u += V.w * f3(V);
            M += V.w;
        }
        if (M > 0.f) u = u * (1.0f / M);
    }
    com[c] = make_float4(u.x, u.y, u.z, 0.f);
}

// isokineticThermostatSRD (particles_kernel_impl.cuh:605-637)
__global__ void thermostat_kernel(const DevParams P, float4* vel, float4* sortedVel, const uint32_t* cellStart,
                                  const uint32_t* cellEnd, const uint32_t* index, uint32_t numCells)
{
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= numCells) return;
    const uint32_t s0 = cellStart[c];
    if (s0 == kEmpty) return;
    const uint32_t s1 = cellEnd[c];
    float E = 0.f;
    for (uint32_t k = s0; k < s1; ++k) {
        const float4 V = sortedVel[k];
        const float3 v = f3(V);
        E += (0.5f * V.w) * dot3(v, v);
    }
    const float lam = sqrtf(P.srd_kT / E);
    for (uint32_t k = s0; k < s1; ++k) {
        const uint32_t id = index[k];
        const float4 V = vel[id];
        const float4 nv = make_float4(lam * V.x, lam * V.y, lam * V.z, sortedVel[k].w);
        vel[id] = nv;
        sortedVel[k] = nv;
    }
}

// collideSolventKernel + rotate2D (particles_kernel_impl.cuh:640-691)
__global__ void collide_solvent_kernel(const DevParams P, float4* pos, float4* vel, const float4* com,
                                       const float* uniform, uint32_t n, float3 shift)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (i < P.nb) return;
    const float3 r = f3(pos[i]);
    const float4 V = vel[i];
    const uint32_t cell = srd_hash(P, r, shift);
    const float3 u = f3(com[cell]);
    const int sign = 2 * (int)(uniform[cell] > 0.5f) - 1;
    const float ang = (float)sign * P.srd_alpha;
    const float sa = sinf(ang), ca = cosf(ang);
    const float3 d = f3(V) - u;
    vel[i] = make_float4(u.x + (d.x * ca - d.y * sa), u.y + (d.x * sa + d.y * ca), u.z + d.z, V.w);
}

float3 legacy_shift() { return make_float3(g_solvent.randOffset.x, g_solvent.randOffset.y, g_solvent.randOffset.z); }

}  // namespace
}  // namespace nw

using namespace nw;

extern "C" {

void cudaInit(int argc, char** argv)
{
    int dev = 0;
    for (int k = 1; k < argc; ++k)
        if (argv[k] && std::strncmp(argv[k], "-device=", 8) == 0) dev = std::atoi(argv[k] + 8);
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        std::printf("No CUDA Capable devices found\n");
        g_last_status = NW_ERR_NO_DEVICE;
        return;
    }
    if (dev < 0 || dev >= n) dev = 0;
    note(cudaSetDevice(dev), "cudaInit");
    g_calls = 0;
}

void nw_legacy_seed(uint64_t seed)
{
    g_seed = seed;
    g_calls = 0;
}

int nw_legacy_last_status(void)
{
    int s = g_last_status;
    g_last_status = 0;
    return s;
}

void randomizeUniform(float* device, uint n)
{
    if (!n) return;
    fill_uniform_kernel<<<blocks_for((n + 3u) / 4u, 256), 256>>>(device, n, (uint32_t)g_seed, (uint32_t)(g_seed >> 32),
                                                                 g_calls++);
    check_launch("randomizeUniform");
}

void randomizeGaussian(float* device, uint n, float mean, float stddev)
{
    if (!n) return;
    fill_normal_kernel<<<blocks_for((n + 3u) / 4u, 256), 256>>>(device, n, mean, stddev, (uint32_t)g_seed,
                                                                (uint32_t)(g_seed >> 32), g_calls++);
    check_launch("randomizeGaussian");
}

void allocateArray(void** devPtr, int size) { note(cudaMalloc(devPtr, (size_t)(unsigned)size), "allocateArray"); }

void freeArray(void* devPtr) { note(cudaFree(devPtr), "freeArray"); }

void threadSync(void) { note(cudaDeviceSynchronize(), "threadSync"); }

void copyArrayToDevice(void* device, const void* host, int offset, int size)
{
    note(cudaMemcpy((char*)device + offset, host, (size_t)(unsigned)size, cudaMemcpyHostToDevice), "copyArrayToDevice");
}

void copyArrayFromDevice(void* host, const void* device, struct cudaGraphicsResource** cuda_vbo_resource, int size)
{
    (void)cuda_vbo_resource;
    note(cudaMemcpy(host, device, (size_t)(unsigned)size, cudaMemcpyDeviceToHost), "copyArrayFromDevice");
}

void setParameters(SimParams* hostParams)
{
    if (!hostParams) return;
    g_params = *hostParams;
    g_have_params = true;
}

void setSolventParameters(SolventParams* solventParams)
{
    if (!solventParams) return;
    g_solvent = *solventParams;
}

void integrateFilaments(float* pos, float* vel, float* f, float* f_old, float deltaTime, uint numParticles)
{
    if (!numParticles) return;
    const DevParams P = legacy_params();
    integrate_kernel<<<blocks_for(numParticles, 256), 256>>>(P, (float4*)pos, (float4*)vel, (float4*)f, (float4*)f_old,
                                                             deltaTime, numParticles);
    check_launch("integrateFilaments");
}

void integrateSolvent(float* pos, float* vel, float deltaTime, uint startIndex, uint numSolvent)
{
    if (!numSolvent) return;
    const DevParams P = legacy_params();
    integrate_solvent_kernel<<<blocks_for(numSolvent, 256), 256>>>(P, (float4*)pos, (float4*)vel, deltaTime, startIndex,
                                                                   numSolvent);
    check_launch("integrateSolvent");
}

void calcHash(uint* gridParticleHash, uint* gridParticleIndex, float* pos, int numParticles, bool srd)
{
    if (numParticles <= 0) return;
    const DevParams P = legacy_params();
    hash_kernel<<<blocks_for((uint32_t)numParticles, 256), 256>>>(P, gridParticleHash, gridParticleIndex,
                                                                  (const float4*)pos, (uint32_t)numParticles, srd ? 1 : 0,
                                                                  legacy_shift());
    check_launch("calcHash");
}

void reorderDataAndFindCellStart(uint* cellStart, uint* cellEnd, float* sortedPos, float* sortedVel,
                                 float* sortedTangent, uint* gridParticleHash, uint* gridParticleIndex, float* pos,
                                 float* vel, float* tangent, uint numParticles, uint numCells)
{
    note(cudaMemset(cellStart, 0xff, (size_t)numCells * sizeof(uint)), "reorderDataAndFindCellStart");
    if (!numParticles) return;
    uint32_t* err = err_word();
    reorder_kernel<<<blocks_for(numParticles, 256), 256>>>(cellStart, cellEnd, (float4*)sortedPos, (float4*)sortedVel,
                                                           (float4*)sortedTangent, gridParticleHash, gridParticleIndex,
                                                           (const float4*)pos, (const float4*)vel,
                                                           (const float4*)tangent, numParticles, numCells, err);
    check_launch("reorderDataAndFindCellStart");
}

void collideFilaments(float* force, float* sortedPos, float* sortedVel, float* sortedTangent, uint* gridParticleIndex,
                      uint* cellStart, uint* cellEnd, uint numParticles, uint numCells)
{
    (void)numCells;
    if (!numParticles) return;
    DevParams P = legacy_params();
    P.nb = numParticles;
    StepBuffers S;
    std::memset(&S, 0, sizeof(S));
    S.force = (float4*)force;
    S.sorted_pos = (float4*)sortedPos;
    S.sorted_vel = (float4*)sortedVel;
    S.sorted_tan = (float4*)sortedTangent;
    S.sorted_index = gridParticleIndex;
    S.cell_start = cellStart;
    S.cell_end = cellEnd;
    S.err = err_word();
    pair_ref_kernel<<<blocks_for(numParticles, 256), 256>>>(P, S);
    check_launch("collideFilaments");
}

void nw_legacy_collide_solvent_apply(float* pos, float* vel, const float* solventCellCOM, const float* uniform,
                                     uint numParticles)
{
    if (!numParticles) return;
    const DevParams P = legacy_params();
    collide_solvent_kernel<<<blocks_for(numParticles, 256), 256>>>(P, (float4*)pos, (float4*)vel,
                                                                   (const float4*)solventCellCOM, uniform,
                                                                   numParticles, legacy_shift());
    check_launch("collideSolvent");
}

void collideSolvent(float* pos, float* vel, float* solventCellCOM, float* random, uint numSolventCells,
                    uint numParticles)
{
    randomizeUniform(random, numSolventCells);
    nw_legacy_collide_solvent_apply(pos, vel, solventCellCOM, random, numParticles);
}

void filamentForces(float* force, float* tangent, float* pos, float numFilaments)
{
    const uint32_t nf = numFilaments > 0.0f ? (uint32_t)numFilaments : 0u;
    const DevParams P = legacy_params();
    const uint64_t n = (uint64_t)nf * P.L;
    if (!n) return;
    filament_kernel<<<blocks_for(n, 256), 256>>>(P, (float4*)force, (float4*)tangent, (const float4*)pos, nf);
    check_launch("filamentForces");
}

void sortParticles(uint* dGridParticleHash, uint* dGridParticleIndex, uint numParticles)
{
    if (numParticles < 2) return;
    std::lock_guard<std::mutex> lk(g_mu);
    if (g_radix.capacity < numParticles) {
        cudaFree(g_radix.keys_alt);
        g_radix = RadixScratch();
        uint32_t* base = nullptr;
        const size_t words = radix_scratch_layout(numParticles, nullptr, nullptr);
        if (cudaMalloc(&base, words * sizeof(uint32_t)) != cudaSuccess) {
            note(cudaErrorMemoryAllocation, "sortParticles");
            return;
        }
        radix_scratch_layout(numParticles, base, &g_radix);
    }
    radix_sort_pairs(dGridParticleHash, dGridParticleIndex, numParticles, g_radix, 0);
    check_launch("sortParticles");
}

void nw_legacy_reverse_apply(float* force, float* forceOld, float* vel, float* pos, const float* uniform,
                             uint numFilaments)
{
    if (!numFilaments) return;
    const DevParams P = legacy_params();
    reverse_kernel<<<blocks_for(numFilaments, 256), 256>>>(P, (float4*)force, (float4*)forceOld, (float4*)vel,
                                                           (float4*)pos, uniform, numFilaments);
    check_launch("reverseFilaments");
}

void reverseFilaments(float* force, float* forceOld, float* vel, float* pos, float* uniform, uint numFilaments)
{
    randomizeUniform(uniform, numFilaments);
    nw_legacy_reverse_apply(force, forceOld, vel, pos, uniform, numFilaments);
}

void nw_legacy_langevin_apply(float* force, float* vel, const float* gaussian, uint numParticles)
{
    if (!numParticles) return;
    const DevParams P = legacy_params();
    langevin_kernel<<<blocks_for(numParticles, 256), 256>>>(P, (float4*)force, (const float4*)vel,
                                                            (const float4*)gaussian, numParticles);
    check_launch("langevinThermostat");
}

void langevinThermostat(float* force, float* vel, float* random, float gamma, float kbT, uint numParticles)
{
    const float stddev = sqrtf(2.0f * gamma * kbT);
    randomizeGaussian(random, 4u * numParticles, 0.0f, stddev);
    if (!numParticles) return;
    DevParams P = legacy_params();
    P.gamma = gamma;
    langevin_kernel<<<blocks_for(numParticles, 256), 256>>>(P, (float4*)force, (const float4*)vel,
                                                            (const float4*)random, numParticles);
    check_launch("langevinThermostat");
}

void solventCellCentorOfMomentum(float* solventCellCOM, float* sortedVel, uint* cellStart, uint* cellEnd,
                                 uint* gridParticleIndex, uint numCells)
{
    (void)gridParticleIndex;
    if (!numCells) return;
    com_kernel<<<blocks_for(numCells, 256), 256>>>((float4*)solventCellCOM, (const float4*)sortedVel, cellStart,
                                                   cellEnd, numCells);
    check_launch("solventCellCentorOfMomentum");
}

void solventIsokineticThermostat(float* vel, float* sortedVel, uint* cellStart, uint* cellEnd, uint* gridParticleIndex,
                                 uint numCells)
{
    if (!numCells) return;
    const DevParams P = legacy_params();
    thermostat_kernel<<<blocks_for(numCells, 256), 256>>>(P, (float4*)vel, (float4*)sortedVel, cellStart, cellEnd,
                                                          gridParticleIndex, numCells);
    check_launch("solventIsokineticThermostat");
}

}  // extern "C"
