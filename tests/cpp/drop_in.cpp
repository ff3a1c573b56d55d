// drop_in.cpp - the caller's side of the drop-in.  A frame loop written the
// way the reference's widget drives its ParticleSimulation
// (cuda-native/src/CellFlowWidget.cpp: the LFO and step at :414-427, the
// particle log at :431-438, the canvas extent at :501, the per-type colour
// loop at :530, the vertex upload at :753-755, the arrow-key moves at
// :810-819, regenerate and rotate at :990 and :998, the raw-table edit at
// :1170-1177, the proximity graph into a GL buffer at :569-575), compiled
// against include/cellflow/ParticleSimulation.hpp with the reference's own
// type and member names: Particle with float3 members, camelCase
// SimulationParams, moveUniverse, generateProximityGraph on a buffer id.
// GL buffers are stood in for by device allocations behind the interop
// hooks.  Prints one line of results for the test to compare with the Python
// binding driven through the same calls.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <memory>
#include <vector>

#include "cellflow/ParticleSimulation.hpp"

int main(int argc, char** argv)
{
    const int n = argc > 1 ? std::atoi(argv[1]) : 4096;
    const int steps = argc > 2 ? std::atoi(argv[2]) : 5;
    try {
        SimulationParams params;
        params.radius = 0.1f;
        params.delta_t = 0.01f;
        params.canvasWidth = params.canvasHeight = params.canvasDepth = 2.0f;
        params.ratio = 0.1f;
        params.lfoA = 0.05f;
        params.lfoS = 0.5f;
        std::unique_ptr<ParticleSimulation> simulation =
            std::make_unique<ParticleSimulation>(n, params.canvasWidth, params.canvasHeight);
        simulation->initializeParticles(params.canvasWidth, params.canvasHeight);
        for (int i = 0; i < params.numParticleTypes; ++i) simulation->setRadioByTypeValue(i, 0.05f * (float)i);
        simulation->regenerateForceTable();
        float* rawForceTable = simulation->getRawForceTableValues();
        rawForceTable[0] = 0.5f;
        rawForceTable[params.numParticleTypes + 1] = -0.25f;
        simulation->updateForceTable(params.forceRange, params.forceBias, params.forceOffset);

        std::vector<Particle> particleData;
        auto frame = [&](int f) {
            if (params.lfoA != 0.0f) {
                const float t = (float)f / 60.0f;
                float lfo = params.lfoA * sin(2.0f * M_PI * params.lfoS * t);
                params.ratioWithLFO = params.ratio + lfo;
            } else {
                params.ratioWithLFO = params.ratio;
            }
            simulation->simulate(params);
            simulation->getParticleData(particleData);
        };
        int f = 0;
        for (; f < steps; f++) frame(f);
        const float moveSpeed = 0.125f;
        simulation->moveUniverse(-moveSpeed, 0);
        simulation->moveUniverse(0, moveSpeed);
        frame(f++);
        simulation->rotateRadioByType();
        frame(f++);

        std::printf("first=(%.9g,%.9g,%.9g) ", particleData[0].pos.x, particleData[0].pos.y, particleData[0].pos.z);
        const float maxUniverseSize = fmax(params.canvasWidth, fmax(params.canvasHeight, params.canvasDepth));
        std::vector<float> vertexData;
        vertexData.reserve(particleData.size() * 4);
        for (const auto& p : particleData) {
            vertexData.push_back(p.pos.x);
            vertexData.push_back(p.pos.y);
            vertexData.push_back(p.pos.z);
            vertexData.push_back(static_cast<float>(p.ptype));
        }
        double pos_sum = 0.0, type_sum = 0.0;
        for (size_t k = 0; k < vertexData.size(); k++) (k % 4 == 3 ? type_sum : pos_sum) += (double)vertexData[k];

        std::vector<ParticleColor> particleColors;
        for (int i = 0; i < params.numParticleTypes; ++i)
            particleColors.push_back({0.1f * (float)i, 0.5f, 1.0f - 0.1f * (float)i});

        // buffer id -> device allocation, standing in for registered GL buffers
        std::map<unsigned int, float*> buffers;
        const size_t cap_floats = (size_t)9 * 6 * (size_t)n;
        for (unsigned int id : {1u, 2u}) {
            float* dev = nullptr;
            if (cudaMalloc(&dev, sizeof(float) * cap_floats) != cudaSuccess) return 2;
            buffers[id] = dev;
        }
        int mapped = 0;
        simulation->setVertexBufferInterop(
            [&](unsigned int id) {
                mapped++;
                return cellflow::MappedVertexBuffer{buffers.at(id), cap_floats};
            },
            [&](unsigned int) { mapped--; });
        int gpuVertexCount = 0, triangleVertexCount = 0;
        const float proximityDistance = 0.05f;
        const int maxConnectionsPerParticle = 5;
        simulation->generateProximityGraph(1u, gpuVertexCount, proximityDistance, maxConnectionsPerParticle,
                                           particleColors);
        simulation->generateTriangleMesh(2u, triangleVertexCount, proximityDistance, maxConnectionsPerParticle,
                                         particleColors);
        for (auto& kv : buffers) cudaFree(kv.second);

        std::printf("drop_in ok n=%d types=%d frames=%d line_vertices=%d triangle_vertices=%d pos_sum=%.17g "
                    "type_sum=%.0f extent=%g mapped=%d\n",
                    n, simulation->getNumParticleTypes(), f, gpuVertexCount, triangleVertexCount, pos_sum, type_sum,
                    maxUniverseSize, mapped);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}
