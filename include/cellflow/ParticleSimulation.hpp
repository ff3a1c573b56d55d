// ParticleSimulation.hpp - drop-in C++ class over the C ABI of cellflow.h.
//
// Mirrors the public members and types of the reference class
// (cuda-native/include/ParticleSimulation.cuh:10-103) and of its parameter
// header (cuda-native/include/SimulationParams.h:6-62), so that its caller
// (CellFlowWidget) compiles against this header unchanged:
//   - Particle is the reference's 44-byte record with float3 members
//     (`p.pos.x`), byte-compatible with cf_particle;
//   - SimulationParams has the reference's camelCase fields, defaults and
//     rendering fields (`params.canvasWidth`, `params.ratioWithLFO`); the
//     physics subset is handed to cf_step by simulate();
//   - generateProximityGraph / generateTriangleMesh keep the reference's
//     GL-buffer signature.  GL interop stays with the caller: it registers a
//     pair of callbacks (setVertexBufferInterop) that map a buffer id to a
//     device pointer and unmap it again; overloads taking a device pointer are
//     there for headless use.
// Errors throw std::runtime_error with the library's message (the reference
// printed and called exit(1), cuda-native/src/ParticleSimulation.cu:10-18).
#pragma once

#include <vector_types.h>  // float3, as the reference's records use

#include <cstddef>
#include <cstdint>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#include "../cellflow.h"

// SimulationParams.h:6-12.
struct Particle {
    float3 pos;
    float3 vel;
    float3 acc;
    unsigned int ptype;
    float pad;
};
static_assert(sizeof(Particle) == sizeof(cf_particle), "Particle is the 44-byte record");
static_assert(offsetof(Particle, pos) == offsetof(cf_particle, pos) &&
                  offsetof(Particle, vel) == offsetof(cf_particle, vel) &&
                  offsetof(Particle, acc) == offsetof(cf_particle, acc) &&
                  offsetof(Particle, ptype) == offsetof(cf_particle, ptype) &&
                  offsetof(Particle, pad) == offsetof(cf_particle, pad),
              "Particle and cf_particle share one layout");

// SimulationParams.h:14-57: every field with the reference's default.
struct SimulationParams {
    float radius = 42.07f;
    float delta_t = 0.18f;
    float friction = 0.51f;
    float repulsion = 64.83f;
    float attraction = 3.06f;
    float k = 29.45f;
    float balance = 0.79f;
    float canvasWidth = 8000.0f;
    float canvasHeight = 8000.0f;
    float canvasDepth = 8000.0f;
    float spawnRegionSize = 2000.0f;
    int numParticleTypes = 6;
    float ratioWithLFO = 0.0f;
    float forceMultiplier = 2.33f;
    int maxExpectedNeighbors = 400;

    float forceRange = 0.28f;
    float forceBias = -0.20f;
    float ratio = 0.0f;
    float lfoA = 0.0f;
    float lfoS = 0.1f;
    float forceOffset = 1.0f;

    float pointSize = 10.0f;
    float depthFadeStart = 10000.0f;
    float depthFadeEnd = 15000.0f;
    float sizeAttenuationFactor = 1000.0f;
    float brightnessMin = 0.4f;
    float focusDistance = 3000.0f;
    float apertureSize = 0.0f;
    bool enableDepthFade = false;
    bool enableSizeAttenuation = true;
    bool enableBrightnessAttenuation = true;
    bool enableDOF = false;

    // The fields the step kernel reads (ParticleSimulation.cu:97-161).
    cf_step_params stepParams() const
    {
        cf_step_params p;
        p.radius = radius;
        p.delta_t = delta_t;
        p.friction = friction;
        p.repulsion = repulsion;
        p.attraction = attraction;
        p.k = k;
        p.balance = balance;
        p.canvas_width = canvasWidth;
        p.canvas_height = canvasHeight;
        p.canvas_depth = canvasDepth;
        p.num_particle_types = numParticleTypes;
        p.ratio_with_lfo = ratioWithLFO;
        p.force_multiplier = forceMultiplier;
        p.max_expected_neighbors = maxExpectedNeighbors;
        return p;
    }
};

// SimulationParams.h:60-62.
using ParticleColor = cf_color;
constexpr int MAX_PARTICLE_TYPES = CF_MAX_TYPES;  // the reference capped at 10

namespace cellflow {

inline void check(int rc)
{
    if (rc != CF_OK) throw std::runtime_error(std::string("cellflow: ") + cf_last_error());
}

// A GL (or other) vertex buffer mapped for the device: where to write, and how
// many floats fit.
struct MappedVertexBuffer {
    float* device = nullptr;
    std::size_t capacityFloats = 0;
};

class ParticleSimulation {
public:
    using MapVertexBuffer = std::function<MappedVertexBuffer(unsigned int buffer)>;
    using UnmapVertexBuffer = std::function<void(unsigned int buffer)>;

    explicit ParticleSimulation(int particleCount, std::uint64_t seed = 1)
        : ParticleSimulation(particleCount, 8000.0f, 8000.0f, seed) {}
    // The depth follows the height, as in the reference (ParticleSimulation.cu:437-439).
    ParticleSimulation(int particleCount, float canvasWidth, float canvasHeight, std::uint64_t seed = 1)
        : seed_(seed)
    {
        check(cf_create(particleCount, 6, canvasWidth, canvasHeight, canvasHeight, seed, &w_));
    }
    ~ParticleSimulation() { cf_destroy(w_); }
    ParticleSimulation(const ParticleSimulation&) = delete;
    ParticleSimulation& operator=(const ParticleSimulation&) = delete;

    void initializeParticles() { check(cf_initialize_particles(w_, ++seed_, 2000.0f)); }
    void initializeParticles(float canvasWidth, float canvasHeight)
    {
        updateCanvasDimensions(canvasWidth, canvasHeight);
        initializeParticles();
    }
    void updateCanvasDimensions(float canvasWidth, float canvasHeight)
    {
        check(cf_set_canvas(w_, canvasWidth, canvasHeight, canvasHeight));
    }
    void initializeForceTable()
    {
        raw_handed_out_ = false;
        check(cf_regenerate_force_table(w_, ++seed_));
    }
    // Edits made through getRawForceTableValues() take effect here, as in the
    // reference (loadPreset writes the raw table, then calls this).
    void updateForceTable(float forceRange, float forceBias, float forceOffset)
    {
        if (raw_handed_out_) check(cf_set_raw_force_table(w_, raw_.data(), (int)raw_.size()));
        check(cf_update_force_table(w_, forceRange, forceBias, forceOffset));
    }
    void initializeRadioByType()
    {
        std::vector<float> r(getNumParticleTypes(), 0.0f);
        check(cf_set_radio_by_type(w_, r.data(), (int)r.size()));
    }
    void simulate(const SimulationParams& params)
    {
        const cf_step_params p = params.stepParams();
        check(cf_step(w_, &p, 1));
    }
    void simulate(const cf_step_params& params) { check(cf_step(w_, &params, 1)); }
    void getParticleData(std::vector<Particle>& particles)
    {
        particles.resize(getParticleCount());
        check(cf_get_particles(w_, reinterpret_cast<cf_particle*>(particles.data()), (int)particles.size()));
    }
    // One step from and to host records (upload, step, read back); one CUDA graph
    // when both buffers are page-locked.
    void simulateHost(const SimulationParams& params, const Particle* in, Particle* out)
    {
        const cf_step_params p = params.stepParams();
        check(cf_step_host(w_, &p, reinterpret_cast<const cf_particle*>(in), reinterpret_cast<cf_particle*>(out),
                           getParticleCount()));
    }
    void setParticleCount(int count) { check(cf_set_particle_count(w_, count, ++seed_)); }
    int getParticleCount() const
    {
        int n = 0;
        check(cf_particle_count(w_, &n));
        return n;
    }
    void setNumParticleTypes(int types) { check(cf_set_num_particle_types(w_, types, ++seed_)); }
    int getNumParticleTypes() const
    {
        int t = 0;
        check(cf_num_particle_types(w_, &t));
        return t;
    }
    void regenerateForceTable() { initializeForceTable(); }
    // The reference returned a pointer into its host raw table
    // (ParticleSimulation.cuh:47); edits take effect at the next
    // updateForceTable, as there.
    float* getRawForceTableValues()
    {
        raw_.resize((size_t)getNumParticleTypes() * getNumParticleTypes());
        check(cf_get_raw_force_table(w_, raw_.data(), (int)raw_.size()));
        raw_handed_out_ = true;
        return raw_.data();
    }
    // Translate every particle and wrap into the world's box (ParticleSimulation.cuh:50).
    void moveUniverse(float dx, float dy) { check(cf_move_universe(w_, dx, dy, 0.0f)); }
    void rotateRadioByType() { check(cf_rotate_radio_by_type(w_)); }
    std::vector<float> getRadioByType() const
    {
        std::vector<float> r(getNumParticleTypes());
        check(cf_get_radio_by_type(w_, r.data(), (int)r.size()));
        return r;
    }
    void setRadioByTypeValue(int index, float value) { check(cf_set_radio_by_type_value(w_, index, value)); }

    // GL interop hooks: `map` turns a buffer id into a device pointer and its
    // capacity (e.g. cudaGraphicsGLRegisterBuffer + cudaGraphicsMapResources +
    // cudaGraphicsResourceGetMappedPointer in the caller's GL code), `unmap`
    // releases it after the vertices are written.
    void setVertexBufferInterop(MapVertexBuffer map, UnmapVertexBuffer unmap)
    {
        map_ = std::move(map);
        unmap_ = std::move(unmap);
    }
    // generateProximityGraph (ParticleSimulation.cuh:60-66): line vertices
    // [x, y, z, r, g, b] x 2 per edge into the mapped buffer.
    void generateProximityGraph(unsigned int openglVBO, int& outVertexCount, float proximityDistance,
                                int maxConnectionsPerParticle, const std::vector<ParticleColor>& particleColors)
    {
        with_buffer(openglVBO, 6, [&](float* dev, int cap) {
            generateProximityGraph(dev, cap, outVertexCount, proximityDistance, maxConnectionsPerParticle,
                                   particleColors);
        });
    }
    // generateTriangleMesh (ParticleSimulation.cuh:69-74): triangle vertices
    // [x, y, z, r, g, b, nx, ny, nz] x 3 per triangle into the mapped buffer.
    void generateTriangleMesh(unsigned int openglVBO, int& outVertexCount, float proximityDistance,
                              int maxConnectionsPerParticle, const std::vector<ParticleColor>& particleColors)
    {
        with_buffer(openglVBO, 9, [&](float* dev, int cap) {
            generateTriangleMesh(dev, cap, outVertexCount, proximityDistance, maxConnectionsPerParticle,
                                 particleColors);
        });
    }
    // Headless forms: a device buffer of capacityVertices * 6 (lines) or * 9
    // (triangles) floats.
    void generateProximityGraph(float* deviceVertices, int capacityVertices, int& outVertexCount,
                                float proximityDistance, int maxConnectionsPerParticle,
                                const std::vector<ParticleColor>& particleColors)
    {
        check(cf_proximity_vertices_device(w_, proximityDistance, maxConnectionsPerParticle, particleColors.data(),
                                           (int)particleColors.size(), deviceVertices, capacityVertices,
                                           &outVertexCount));
    }
    void generateTriangleMesh(float* deviceVertices, int capacityVertices, int& outVertexCount,
                              float proximityDistance, int maxConnectionsPerParticle,
                              const std::vector<ParticleColor>& particleColors)
    {
        check(cf_triangle_mesh_device(w_, proximityDistance, maxConnectionsPerParticle, particleColors.data(),
                                      (int)particleColors.size(), deviceVertices, capacityVertices,
                                      &outVertexCount));
    }
    cf_world* handle() const { return w_; }

private:
    template <typename Body>
    void with_buffer(unsigned int buffer, int floats_per_vertex, Body body)
    {
        if (!map_ || !unmap_)
            throw std::runtime_error(
                "cellflow: no vertex-buffer interop registered (setVertexBufferInterop); GL interop stays with the "
                "caller");
        const MappedVertexBuffer m = map_(buffer);
        try {
            body(m.device, (int)(m.capacityFloats / (std::size_t)floats_per_vertex));
        } catch (...) {
            unmap_(buffer);
            throw;
        }
        unmap_(buffer);
    }

    cf_world* w_ = nullptr;
    std::uint64_t seed_;
    std::vector<float> raw_;
    bool raw_handed_out_ = false;
    MapVertexBuffer map_;
    UnmapVertexBuffer unmap_;
};

}  // namespace cellflow

// The reference's class is in the global namespace.
using cellflow::ParticleSimulation;
