/*
 * ref_emu_archived.cpp — runs the reference's archived worm-force kernels
 * (archived/vs_solution/fluid_substrate/NWWormsKernel_*.h, included
 * unmodified from the reference tree at build time) on the CPU.  TEST
 * INFRASTRUCTURE ONLY: it pins the WCA_WORMS force laws of the oracle.
 *
 * Kernels run thread by thread (none of them uses shared memory or
 * barriers).  The archived code is 2D (_D_ = 2) with SoA arrays r[i + d*N].
 */
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <vector>

/* keep the CUDA builtin-variable declarations out: the emulator owns them */
#define __DEVICE_LAUNCH_PARAMETERS_H__
static uint3 nwemu_threadIdx, nwemu_blockIdx;
static dim3 nwemu_blockDim;
#define threadIdx nwemu_threadIdx
#define blockIdx nwemu_blockIdx
#define blockDim nwemu_blockDim
/* only referenced by kernels of the same headers that the emulator never runs */
static dim3 nwemu_gridDim;
#define gridDim nwemu_gridDim
static inline void __syncthreads() {}

/* the headers' parameter-upload helpers name cudaMemcpyToSymbol's C++
 * template form, which host compilers do not see; on the CPU a symbol is a
 * plain global */
template <class T>
static cudaError_t cudaMemcpyToSymbol(const T& symbol, const void* src, size_t count, size_t offset = 0,
                                      cudaMemcpyKind kind = cudaMemcpyHostToDevice)
{
    (void)kind;
    memcpy((char*)const_cast<T*>(&symbol) + offset, src, count);
    return cudaSuccess;
}

#include "NWWormsKernel_InternalForce.h"
#include "NWWormsKernel_LennardJones.h"
#include "NWWormsKernel_SetNList.h"
#include "NWWormsKernel_BondBending.h"
#include "NWWormsKernel_DriveForce.h"

#include "../../include/nwgb.h"

/* dynamic shared memory named by FastLennardJonesNListKernel (never run here) */
float f_shared[1];

/* named by the headers' error handler, which the emulation never reaches;
 * defined here so the library needs no CUDA runtime */
extern "C" const char* cudaGetErrorString(cudaError_t) { return "cuda error (emulation)"; }

template <class Fn>
static void launch(uint32_t n, uint32_t threads, Fn fn)
{
    if (n == 0) return;
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

static const int kNMax = 256;

extern "C" {

/* Total archived worm force on every bead for positions pos / velocities vel
 * (float4 AoS), in the order of NWSimulation::Run: InterForceKernel (bonds,
 * intra-worm LJ, drag, noise) -> BondBendingForces -> LennardJonesNListKernel
 * over an O(N^2) neighbour list -> DriveForceKernel.  noise is float4 AoS of
 * N(0,1) draws (x, y used) scaled by noise_scale, or NULL for none.
 * force_out is float4 AoS (z, w zero).  Returns 0, or -1 if a neighbour list
 * overflowed its capacity. */
int ref_archived_forces(const NwConfig* c, const float* pos, const float* vel, const float* noise, float noise_scale,
                        float* force_out)
{
    const int M = (int)c->num_filaments, L = (int)c->filament_size, N = M * L;
    WormsParameters wp;
    memset(&wp, 0, sizeof(wp));
    wp._XDIM = M;
    wp._YDIM = 1;
    wp._ZDIM = 1;
    wp._NP = L;
    wp._LISTSETGAP = 1;
    wp._NMAX = kNMax;
    wp._EPSILON = c->lj_epsilon;
    wp._SIGMA = c->lj_sigma;
    wp._DRIVE = c->activity;
    wp._DRIVE_ROT = 0.0f;
    wp._NOINT = false;
    wp._EXTENSILE = false;
    wp._K1 = c->bond_k;
    wp._L1 = c->bond_r0;
    wp._Ka = c->bend_k;
    wp._Ka2 = c->bend_k;
    wp._Ka_RATIO = 1.0f;
    wp._KBT = c->kT;
    wp._GAMMA = c->gamma;
    wp._BUFFER = 1.0f;
    CalculateParameters(&wp, true); /* WCA cut-off, NWWormsParameters.h:135-156 */
    dev_Params = wp;

    SimulationParameters sp;
    memset(&sp, 0, sizeof(sp));
    sp._XBOX = c->box[0];
    sp._YBOX = c->box[1];
    for (int d = 0; d < _D_; ++d) {
        sp._BOX[d] = c->box[d];
        sp._PBC[d] = c->boundary[d] == NW_PERIODIC;
    }
    dev_simParams = sp;

    std::vector<float> r(2 * N), v(2 * N), f(2 * N, 0.0f), rnd(2 * N, 0.0f);
    std::vector<int> nlist((size_t)kNMax * N, -1), cell(2 * N, 0);
    for (int i = 0; i < N; ++i)
        for (int d = 0; d < 2; ++d) {
            r[i + d * N] = pos[4 * i + d];
            v[i + d * N] = vel[4 * i + d];
            if (noise) rnd[i + d * N] = noise[4 * i + d];
        }
    const float scale = noise ? noise_scale : 0.0f;

    launch((uint32_t)N, 256, [&] { InterForceKernel(f.data(), N, v.data(), N, r.data(), N, rnd.data(), scale); });
    launch((uint32_t)M, 256, [&] { BondBendingForces(f.data(), N, r.data(), N); });
    launch((uint32_t)N, 256, [&] { SetNeighborList_N2Kernel(r.data(), N, nlist.data(), N, cell.data(), N); });
    int overflow = 0;
    for (int i = 0; i < N; ++i)
        if (nlist[(size_t)i + (size_t)(kNMax - 1) * N] != -1) overflow = 1;
    launch((uint32_t)N, 256, [&] { LennardJonesNListKernel(f.data(), N, r.data(), N, nlist.data(), N); });
    launch((uint32_t)N, 256, [&] { DriveForceKernel(f.data(), N, r.data(), N); });

    for (int i = 0; i < N; ++i) {
        force_out[4 * i] = f[i];
        force_out[4 * i + 1] = f[i + N];
        force_out[4 * i + 2] = 0.0f;
        force_out[4 * i + 3] = 0.0f;
    }
    return overflow ? -1 : 0;
}

/* The derived WCA constants of CalculateParameters (NWWormsParameters.h:135-156):
 * out = {sigma^6, 2 sigma^6, 24 eps sigma^6, r_min, r_min^2, r_cut, r_cut^2}. */
void ref_archived_lj_constants(float eps, float sigma, float out[7])
{
    WormsParameters wp;
    memset(&wp, 0, sizeof(wp));
    wp._XDIM = wp._YDIM = wp._ZDIM = 1;
    wp._NP = 1;
    wp._EPSILON = eps;
    wp._SIGMA = sigma;
    CalculateParameters(&wp, true);
    out[0] = wp._SIGMA6;
    out[1] = wp._2SIGMA6;
    out[2] = wp._LJ_AMP;
    out[3] = wp._RMIN;
    out[4] = wp._R2MIN;
    out[5] = wp._RCUT;
    out[6] = wp._R2CUT;
}

} /* extern "C" */
