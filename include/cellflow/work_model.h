/*
 * work_model.h - frozen algorithmic work of one CellFlow step (and of one
 * adjoint step of the differentiable rollout).
 *
 * These constants define the "algorithmic" flops and bytes that roofline
 * figures divide by a measured time.  They count the work of the reference
 * step (cuda-native/src/ParticleSimulation.cu:86-165) restricted to the
 * canonical 27-cell stencil, not the instructions a particular kernel issues.
 *
 * Force kernel (FP32 flops per step):
 *     W_step = 9 * C27 + 17 * I + 25 * N
 *   C27: directed candidate pairs (j != i) in the 27-cell stencil of the
 *        canonical grid, floor(L / r_max) cells per axis of side L / cells.
 *   I:   directed interacting pairs, the sum of the step's neighbour counts.
 *   9  per candidate: 3 subtractions, |d|^2 as 1 mul + 2 FMA (5), +1e-4 (1).
 *   17 per interacting pair: r scale 1, r^2 1, -k r^2 1, exp 1, rep* 1,
 *        attraction FMA 2, *F 1, d/dist 3, accumulate 3 FMA (6).
 *   25 per particle: density factor, scaling, integrator, wrap.
 *
 * Cell list (bytes per step): 112 per particle + 8 per cell
 *   hash 24 (read float4 16, write key 4 + index 4), sort 16 (key + value,
 *   read + write), reorder gather 68 (index 4 + pos 16 + vel 16 read,
 *   pos 16 + vel 16 written), cell start/end 4.
 *
 * Adjoint step of the differentiable rollout (FP32 flops per backward step):
 *     W_adj = 9 * C27 + 70 * I + 41 * N
 *   9  per candidate: the forward's displacement, |d|^2 and +1e-4.
 *   70 per interacting pair: 1/dist, dist, r (3), the exponent and exp (3),
 *        the force n = R e - A r (3) and its derivative n' (4), n/dist (1),
 *        the Hessian coefficient (n' dist - n)/dist^3 (5), the adjoint weight
 *        F_ji g_j - F_ij g_i (9), its projection on d (5), the position
 *        gradient phi w + h (d.w) d accumulated (13), g_i.d/dist (6), the
 *        force-table gradient (2), the repulsion, attraction and k gradients
 *        (3 + 2 + 4), the force itself for the scale gradients (7).
 *   41 per particle: the per-particle adjoint of the density scale and the
 *        integrator (26) and the warp's finish of the home (15).
 *
 * Integrator, when not fused (bytes per particle): 88.
 * Proximity graph (bytes per particle): 16 + 8 per emitted edge.
 */
#ifndef CELLFLOW_WORK_MODEL_H
#define CELLFLOW_WORK_MODEL_H

#define CF_WM_FLOPS_PER_CANDIDATE 9
#define CF_WM_FLOPS_PER_INTERACTION 17
#define CF_WM_FLOPS_PER_PARTICLE 25

#define CF_WM_ADJ_FLOPS_PER_CANDIDATE 9
#define CF_WM_ADJ_FLOPS_PER_INTERACTION 70
#define CF_WM_ADJ_FLOPS_PER_PARTICLE 41

#define CF_WM_CELL_BYTES_PER_PARTICLE 112
#define CF_WM_CELL_BYTES_PER_CELL 8
#define CF_WM_INTEGRATOR_BYTES_PER_PARTICLE 88
#define CF_WM_PROX_BYTES_PER_PARTICLE 16
#define CF_WM_PROX_BYTES_PER_EDGE 8

/* Force-kernel flops of one step. */
static inline double cf_wm_force_flops(double c27, double interacting, double n)
{
    return CF_WM_FLOPS_PER_CANDIDATE * c27 + CF_WM_FLOPS_PER_INTERACTION * interacting +
           CF_WM_FLOPS_PER_PARTICLE * n;
}

/* Adjoint flops of one backward step. */
static inline double cf_wm_adjoint_flops(double c27, double interacting, double n)
{
    return CF_WM_ADJ_FLOPS_PER_CANDIDATE * c27 + CF_WM_ADJ_FLOPS_PER_INTERACTION * interacting +
           CF_WM_ADJ_FLOPS_PER_PARTICLE * n;
}

/* Cell-list bytes of one step. */
static inline double cf_wm_cell_list_bytes(double n, double cells)
{
    return CF_WM_CELL_BYTES_PER_PARTICLE * n + CF_WM_CELL_BYTES_PER_CELL * cells;
}

#endif /* CELLFLOW_WORK_MODEL_H */
