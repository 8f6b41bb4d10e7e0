/*
 * nwref_kernels.cu — the reference's own device code, built for sm_103a.
 *
 * TEST INFRASTRUCTURE ONLY (the reference CUDA build used as the checker and
 * as the speed denominator); nothing in the product links or loads it.
 *
 * The reference's kernel file (simulation/particles_kernel_impl.cuh) is
 * included unmodified from the reference tree at build time; this file adds
 * only two entry points with C names for the two thrust functors that the
 * reference applies with thrust::for_each (simulation/particleSystem_cuda.cu:
 * 117-149): one thread per element calls the functor on a tuple of references
 * to that element, which is what thrust's for_each does per element.
 *
 * Compiled to a device-only fatbin (oracle/ref_cuda/Makefile); the host side
 * that loads it and issues the reference's launches is nwref_host.cu.
 */
#include <thrust/tuple.h>

#include "particles_kernel_impl.cuh"

/* particleSystem_cuda.cu:117-133: thrust::for_each over the zip of
 * (pos, vel, f, f_old) with filament_integrator(deltaTime). */
extern "C" __global__ void nwref_filament_integrator(float4* pos, float4* vel, float4* f, float4* f_old, float dt,
                                                     unsigned int n)
{
    unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    filament_integrator op(dt);
    op(thrust::tie(pos[i], vel[i], f[i], f_old[i]));
}

/* particleSystem_cuda.cu:136-149: thrust::for_each over the zip of
 * (pos + start, vel + start) with solvent_integrator(deltaTime). */
extern "C" __global__ void nwref_solvent_integrator(float4* pos, float4* vel, float dt, unsigned int start,
                                                    unsigned int n)
{
    unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    solvent_integrator op(dt);
    op(thrust::tie(pos[start + i], vel[start + i]));
}
