/*
 * nwgb_adjoint.h — differentiable rollout of the WCA worm step: gradients of
 * a loss on the final state with respect to the force parameters
 * theta = (eps, k_bend, k_bond, F_act) by a hand-written adjoint.
 *
 * No reference counterpart (the reference has no gradients).  The forward
 * step is the reference's update (simulation/particleSystem.cpp:249-339:
 * velocity Verlet of particles_kernel_impl.cuh:93-97, Langevin :859-874,
 * bending :751-818) with the archived WCA_WORMS laws
 * (NWWormsKernel_LennardJones.h:38-50, NWWormsKernel_InternalForce.h:37-59,
 * NWWormsKernel_DriveForce.h:21-34), under two conventions that make the
 * rollout a smooth function of theta:
 *   - the Langevin noise realisation is fixed (Philox by seed + replica,
 *     bead and step, as in the engine);
 *   - neighbour lists are built from the positions at the start of every
 *     segment of `segment` steps (all non-excluded pairs within
 *     lj_rcut + neighbor_skin) and frozen for that segment; pairs on the
 *     list interact while closer than lj_rcut.
 * The rollout stores its state every `segment` steps and the backward pass
 * recomputes each segment from its checkpoint.
 *
 * Scope: NW_MODEL_WCA_WORMS, periodic boundaries, no reversal, no SRD;
 * n_replicas copies of one configuration with seeds cfg.seed + r.  Arrays
 * are float4[n_replicas * n_beads] on the device, replica-major.
 */
#ifndef NWGB_ADJOINT_H
#define NWGB_ADJOINT_H

#include "nwgb.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct nw_adjoint nw_adjoint;

/* precision: 32 or 64 (arithmetic and stored state of forward and adjoint). */
nw_status nw_adj_create(const NwConfig* cfg, int n_replicas, int horizon, int segment, int precision,
                        nw_adjoint** out);
nw_status nw_adj_destroy(nw_adjoint* a);
/* Stream of the rollout's work; NULL selects the handle's own stream, which
 * is ordered with the legacy default stream (work queued there before a call
 * is finished before the rollout reads its inputs). */
nw_status nw_adj_set_stream(nw_adjoint* a, void* stream);

/* Initial positions and velocities (device float4 arrays); forces start at 0. */
nw_status nw_adj_set_state(nw_adjoint* a, const float* d_pos, const float* d_vel);

/* Run `horizon` steps with theta = {eps, k_bend, k_bond, F_act}; writes the
 * final positions and velocities to device float4 arrays.  Synchronous. */
nw_status nw_adj_forward(nw_adjoint* a, const double theta[4], float* d_pos_out, float* d_vel_out);

/* The final state of the last forward as (x, y, z, 0) double quadruples
 * (device arrays of n_replicas * n_beads * 4 doubles; either may be NULL),
 * unrounded at precision 64: what finite differences of the FP64 forward
 * need, where float4 outputs would round the loss.  Synchronous. */
nw_status nw_adj_final_state_f64(nw_adjoint* a, double* d_pos_out, double* d_vel_out);

/* Given dL/d(final positions) and dL/d(final velocities) (device float4
 * arrays, w ignored), write dL/dtheta of the last forward.  Synchronous. */
nw_status nw_adj_backward(nw_adjoint* a, const float* d_grad_pos, const float* d_grad_vel, double grad_theta[4]);

/* Device time of the last forward and backward (milliseconds). */
nw_status nw_adj_timings(const nw_adjoint* a, float* forward_ms, float* backward_ms);

#ifdef __cplusplus
}
#endif

#endif /* NWGB_ADJOINT_H */
