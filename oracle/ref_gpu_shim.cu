/*
 * ref_gpu_shim.cu - the reference step and proximity kernels built for
 * sm_103a, for timing.
 *
 * TEST INFRASTRUCTURE (the benchmark's "reference kernel on this GPU" figures).
 * Includes cuda-native/src/ParticleSimulation.cu:69-166, cut unchanged into
 * oracle/_ref/ref_step_kernel.inc by build_ref.sh, and launches it the way
 * ParticleSimulation::simulate does (ParticleSimulation.cu:541-556):
 * <<<ceil(n/256), 256>>>, in place on one AoS particle buffer, with the
 * neighbour-count buffers swapped by the caller after every step.
 */
#include <cuda_runtime.h>

#include "SimulationParams.h"

#include "ref_step_kernel.inc"

extern "C" int cfref_gpu_step(void* particles, const float* force_table, const float* radio_by_type, int* cnt_in,
                              int* cnt_out, int n, float radius, float delta_t, float friction, float repulsion,
                              float attraction, float k, float balance, float w, float h, float d, int num_types,
                              float ratio_with_lfo, float force_multiplier, int max_expected_neighbors, void* stream)
{
    SimulationParams params;
    params.radius = radius;
    params.delta_t = delta_t;
    params.friction = friction;
    params.repulsion = repulsion;
    params.attraction = attraction;
    params.k = k;
    params.balance = balance;
    params.canvasWidth = w;
    params.canvasHeight = h;
    params.canvasDepth = d;
    params.numParticleTypes = num_types;
    params.ratioWithLFO = ratio_with_lfo;
    params.forceMultiplier = force_multiplier;
    params.maxExpectedNeighbors = max_expected_neighbors;
    int blocks = (n + BLOCK_SIZE - 1) / BLOCK_SIZE;
    simulateParticlesKernel<<<blocks, BLOCK_SIZE, 0, (cudaStream_t)stream>>>(
        (Particle*)particles, force_table, radio_by_type, cnt_in, cnt_out, params, n);
    return (int)cudaGetLastError();
}

/* The reference proximity kernel (ParticleSimulation.cu:188-277, cut into
 * oracle/_ref/ref_prox_kernel.inc), launched the way generateProximityGraph
 * does (:656-670): <<<ceil(n/256), 256>>> over the AoS particles, edges
 * appended through an atomicAdd on *vertex_count, which the caller zeroes.
 * `vertices` must hold n * 2 * min(max_conn, 32) * 6 floats: the kernel has
 * no capacity check. */
#include "ref_prox_kernel.inc"

extern "C" int cfref_gpu_proximity(const void* particles, int n, float distance, int max_conn, const void* colors,
                                   int num_types, float* vertices, int* vertex_count, void* stream)
{
    int blocks = (n + 255) / 256;
    generateProximityGraphKernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(
        (const Particle*)particles, n, distance * distance, max_conn, (const ParticleColor*)colors, num_types,
        vertices, vertex_count);
    return (int)cudaGetLastError();
}
