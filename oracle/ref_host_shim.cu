/*
 * ref_host_shim.cu - runs the reference's own kernel bodies on the host.
 *
 * TEST INFRASTRUCTURE.  build_ref.sh cuts three pieces of the reference
 * source by line range into oracle/_ref/ (git-ignored) and this shim
 * includes them unchanged:
 *   ref_step_kernel.inc  cuda-native/src/ParticleSimulation.cu:69-166
 *   ref_prox_kernel.inc  cuda-native/src/ParticleSimulation.cu:188-277
 *   ref_mesh_kernel.inc  cuda-native/src/ParticleSimulation.cu:280-424
 *   ref_force_table.inc  cuda-native/src/ParticleSimulation.cu:521-531
 * It is compiled by nvcc as host code (as the reference's host code was, so
 * tanh(float) resolves to the float overload) with -ffp-contract=off, which
 * rounds every float operation on its own in source order.
 *
 * The kernel bodies read blockIdx/blockDim/threadIdx; host stand-ins give
 * each call the index of one particle.  The step runs with Jacobi meaning:
 * each thread owns a private copy of the particle array, lets the kernel
 * body update slot i in that copy, moves the result out and restores the
 * slot, so every particle sees the start-of-step state of all others.
 */
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "SimulationParams.h"

struct cfref_index3 {
    unsigned int x, y, z;
};
static thread_local cfref_index3 cfref_block_idx, cfref_block_dim, cfref_thread_idx;

static int cfref_atomic_add(int* address, int value) { return __atomic_fetch_add(address, value, __ATOMIC_RELAXED); }

#define blockIdx cfref_block_idx
#define blockDim cfref_block_dim
#define threadIdx cfref_thread_idx
#define atomicAdd cfref_atomic_add
#undef __global__
#define __global__ static

#include "ref_step_kernel.inc"
#include "ref_prox_kernel.inc"
#include "ref_mesh_kernel.inc"

#undef blockIdx
#undef blockDim
#undef threadIdx
#undef atomicAdd

/* The members updateForceTable touches (ParticleSimulation.cuh:78-94). */
class ParticleSimulation {
public:
    int numParticleTypes = 0;
    std::unique_ptr<float[]> h_rawForceTable;
    float* d_forceTable = nullptr;
    void updateForceTable(float forceRange, float forceBias, float forceOffset);
};

#define CUDA_CHECK(call) (void)(call)
#define cudaMemcpy(dst, src, bytes, kind) (std::memcpy((dst), (src), (bytes)), cudaSuccess)
#include "ref_force_table.inc"
#undef cudaMemcpy

static void select_particle(int i)
{
    cfref_block_idx = {(unsigned int)i, 0u, 0u};
    cfref_block_dim = {1u, 1u, 1u};
    cfref_thread_idx = {0u, 0u, 0u};
}

extern "C" {

int cfref_sizeof_particle(void) { return (int)sizeof(Particle); }

/* One Jacobi step of the reference kernel body for i = i_begin, i_begin +
 * i_stride, ... < i_end.  `in` holds the n start-of-step particles; results
 * for the selected i are written to out[i] and cnt_out[i].  The scalar
 * arguments fill the SimulationParams fields the kernel reads; the rest keep
 * their defaults (SimulationParams.h:15-56). */
void cfref_step(int n, const Particle* in, const float* force_table, const float* radio_by_type, const int* cnt_in,
                int* cnt_out, Particle* out, int i_begin, int i_end, int i_stride, float radius, float delta_t,
                float friction, float repulsion, float attraction, float k, float balance, float w, float h, float d,
                int num_types, float ratio_with_lfo, float force_multiplier, int max_expected_neighbors)
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
    if (i_stride < 1) i_stride = 1;
    int rows = (i_end - i_begin + i_stride - 1) / i_stride;
#pragma omp parallel
    {
        std::vector<Particle> snapshot(in, in + n);
#pragma omp for schedule(dynamic, 4)
        for (int r = 0; r < rows; r++) {
            int i = i_begin + r * i_stride;
            select_particle(i);
            simulateParticlesKernel(snapshot.data(), force_table, radio_by_type, const_cast<int*>(cnt_in), cnt_out,
                                    params, n);
            out[i] = snapshot[i];
            snapshot[i] = in[i];
        }
    }
}

/* The reference proximity kernel body for every particle, in index order, on
 * one thread (so the vertex order is i order).  `vertices` needs room for
 * n * 2 * min(max_conn, 32) * 2 * 6 floats.  Returns the vertex count. */
int cfref_proximity(int n, const Particle* particles, float distance, int max_conn, const ParticleColor* colors,
                    int num_types, float* vertices)
{
    int count = 0;
    float dsq = distance * distance;
    for (int i = 0; i < n; i++) {
        select_particle(i);
        generateProximityGraphKernel(particles, n, dsq, max_conn, colors, num_types, vertices, &count);
    }
    return count;
}

/* The reference triangle-mesh kernel body for every particle, in index order,
 * on one thread (so the triangles come in i order).  The squared distance is
 * the host wrapper's, with its 1.2 hysteresis (ParticleSimulation.cu:723-724).
 * `vertices` needs room for n * 64 * 3 * 9 floats.  Returns the vertex count. */
int cfref_triangle_mesh(int n, const Particle* particles, float distance, int max_conn, const ParticleColor* colors,
                        int num_types, float* vertices)
{
    int count = 0;
    const float hysteresis = 1.2f;
    const float dsq = distance * distance * (hysteresis * hysteresis);
    for (int i = 0; i < n; i++) {
        select_particle(i);
        generateTriangleMeshKernel(particles, n, dsq, max_conn, colors, num_types, vertices, &count);
    }
    return count;
}

/* The reference force-table transform; count = T*T with T <= 10. */
int cfref_force_table(const float* raw, int num_types, float range, float bias, float offset, float* out)
{
    if (num_types < 1 || num_types > MAX_PARTICLE_TYPES) return -1;
    ParticleSimulation sim;
    sim.numParticleTypes = num_types;
    sim.h_rawForceTable = std::make_unique<float[]>(MAX_PARTICLE_TYPES * MAX_PARTICLE_TYPES);
    std::memcpy(sim.h_rawForceTable.get(), raw, sizeof(float) * num_types * num_types);
    sim.d_forceTable = out;
    sim.updateForceTable(range, bias, offset);
    return 0;
}
}
