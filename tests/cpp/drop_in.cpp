// drop_in.cpp - the caller's side of the drop-in: code written against the
// reference's ParticleSimulation (cuda-native/include/ParticleSimulation.cuh)
// compiled against include/cellflow/ParticleSimulation.hpp instead.  Steps a
// world, reads the particles back, builds the proximity graph and the
// triangle mesh into device buffers (standing in for GL VBOs) and prints one
// line of counts for the test to compare with the Python binding.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "cellflow/ParticleSimulation.hpp"

int main(int argc, char** argv)
{
    const int n = argc > 1 ? std::atoi(argv[1]) : 4096;
    const int steps = argc > 2 ? std::atoi(argv[2]) : 5;
    try {
        cellflow::ParticleSimulation sim(n, 2.0f, 2.0f, 7);
        cellflow::SimulationParams params;
        params.radius = 0.1f;
        params.delta_t = 0.01f;
        params.canvas_width = params.canvas_height = params.canvas_depth = 2.0f;
        params.num_particle_types = sim.getNumParticleTypes();
        sim.initializeParticles();  // spawn cube min(2000, extent): the whole box
        sim.updateForceTable(0.28f, -0.20f, 1.0f);
        for (int s = 0; s < steps; s++) sim.simulate(params);
        std::vector<cellflow::Particle> particles;
        sim.getParticleData(particles);
        double sx = 0.0;
        for (const auto& p : particles) sx += (double)p.pos[0] + (double)p.pos[1] + (double)p.pos[2];

        std::vector<cellflow::ParticleColor> colors(params.num_particle_types, cellflow::ParticleColor{0.5f, 0.5f, 0.5f});
        float* vbo = nullptr;
        const int cap = 6 * n;
        if (cudaMalloc(&vbo, sizeof(float) * 9 * (size_t)cap) != cudaSuccess) return 2;
        int lines = 0, tris = 0;
        sim.generateProximityGraph(vbo, cap, lines, 0.05f, 5, colors);
        sim.generateTriangleMesh(vbo, cap, tris, 0.05f, 5, colors);
        cudaFree(vbo);
        std::printf("drop_in ok n=%d types=%d steps=%d line_vertices=%d triangle_vertices=%d pos_sum=%.6f\n", n,
                    sim.getNumParticleTypes(), steps, lines, tris, sx);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}
