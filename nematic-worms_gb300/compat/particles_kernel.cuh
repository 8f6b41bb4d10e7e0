/*
 * particles_kernel.cuh — drop-in parameter ABI of the GB300 engine.
 *
 * The legacy C-ABI symbols (particleSystem.cuh) take these structs by
 * pointer, so their member types and order are those of the reference's
 * parameter structs (simulation/particles_kernel.cuh:18-73): a caller built
 * against the reference headers passes a layout-identical object.
 */
#ifndef NW_COMPAT_PARTICLES_KERNEL_H
#define NW_COMPAT_PARTICLES_KERNEL_H

#include <vector_types.h>

typedef unsigned int uint;

enum BoundaryType
{
    PERIODIC = 0,
    WALL = 1,
    WALL_NO_SLIP = 2,
};

struct SimParams
{
    float3 gravity;
    float particleRadius;
    float particleMass;

    uint3 gridSize;
    uint numCells;
    float3 origin;
    float3 boxSize;
    float3 cellSize;

    BoundaryType boundaryX;
    BoundaryType boundaryY;
    BoundaryType boundaryZ;

    uint numParticles;
    uint numFilaments;
    uint filamentSize;

    float bondSpringK;
    float bondSpringL;
    float bondBendingK;

    float activity;
    float reverseProbability;
    float kbT;
    float gamma;

    float spring;
    float damping;
    float shear;
    float attraction;
    float boundaryDamping;
};

struct SolventParams
{
    bool enabled;
    uint3 gridSize;
    uint numCells;
    float3 randOffset;   /* random grid shift of the current collision */
    float3 cellSize;
    uint numParticles;   /* solvent particles */
    float alpha;         /* rotation angle */
    float kbT;           /* solvent temperature */
    float particleMass;  /* solvent particle mass */
};

#endif
