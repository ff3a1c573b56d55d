// ParticleSimulation.hpp - drop-in C++ class over the C ABI of cellflow.h.
//
// Mirrors the public members of the reference class
// (cuda-native/include/ParticleSimulation.cuh:10-103) so its caller
// (CellFlowWidget) compiles against this header unchanged except for the
// proximity graph, whose GL buffer becomes a device pointer.  Errors throw
// std::runtime_error with the library's message (the reference printed and
// called exit(1), cuda-native/src/ParticleSimulation.cu:10-18).
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../cellflow.h"

namespace cellflow {

using Particle = cf_particle;  // 44 bytes, SimulationParams.h:6-12
using ParticleColor = cf_color;

// The physics subset of SimulationParams (SimulationParams.h:15-37); the
// rendering fields of the reference struct stay with the caller.
struct SimulationParams : cf_step_params {
    float forceRange = 0.28f, forceBias = -0.20f, ratio = 0.0f, lfoA = 0.0f, lfoS = 0.1f, forceOffset = 1.0f;
    SimulationParams() { cf_default_params(this); }
};

inline void check(int rc)
{
    if (rc != CF_OK) throw std::runtime_error(std::string("cellflow: ") + cf_last_error());
}

class ParticleSimulation {
public:
    explicit ParticleSimulation(int particleCount, std::uint64_t seed = 1)
        : ParticleSimulation(particleCount, 8000.0f, 8000.0f, seed) {}
    ParticleSimulation(int particleCount, float canvasWidth, float canvasHeight, std::uint64_t seed = 1)
        : width_(canvasWidth), height_(canvasHeight), seed_(seed)
    {
        check(cf_create(particleCount, 6, canvasWidth, canvasHeight, canvasHeight, seed, &w_));
    }
    ~ParticleSimulation() { cf_destroy(w_); }
    ParticleSimulation(const ParticleSimulation&) = delete;
    ParticleSimulation& operator=(const ParticleSimulation&) = delete;

    void initializeParticles() { check(cf_initialize_particles(w_, ++seed_, 2000.0f)); }
    void initializeParticles(float canvasWidth, float canvasHeight)
    {
        width_ = canvasWidth;
        height_ = canvasHeight;
        initializeParticles();
    }
    void updateCanvasDimensions(float canvasWidth, float canvasHeight)
    {
        width_ = canvasWidth;
        height_ = canvasHeight;
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
    void simulate(const cf_step_params& params) { check(cf_step(w_, &params, 1)); }
    void getParticleData(std::vector<Particle>& particles)
    {
        particles.resize(getParticleCount());
        check(cf_get_particles(w_, particles.data(), (int)particles.size()));
    }
    // One step from and to host records (upload, step, read back); one CUDA graph
    // when both buffers are page-locked.
    void simulateHost(const cf_step_params& params, const Particle* in, Particle* out)
    {
        check(cf_step_host(w_, &params, in, out, getParticleCount()));
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
    void rotateRadioByType() { check(cf_rotate_radio_by_type(w_)); }
    std::vector<float> getRadioByType() const
    {
        std::vector<float> r(getNumParticleTypes());
        check(cf_get_radio_by_type(w_, r.data(), (int)r.size()));
        return r;
    }
    void setRadioByTypeValue(int index, float value) { check(cf_set_radio_by_type_value(w_, index, value)); }
    // generateProximityGraph with the GL VBO replaced by a device buffer of
    // capacityVertices * 6 floats.
    void generateProximityGraph(float* deviceVertices, int capacityVertices, int& outVertexCount,
                                float proximityDistance, int maxConnectionsPerParticle,
                                const std::vector<ParticleColor>& particleColors)
    {
        check(cf_proximity_vertices_device(w_, proximityDistance, maxConnectionsPerParticle, particleColors.data(),
                                           (int)particleColors.size(), deviceVertices, capacityVertices,
                                           &outVertexCount));
    }
    // generateTriangleMesh (ParticleSimulation.cuh:69-74) with the GL VBO
    // replaced by a device buffer of capacityVertices * 9 floats.
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
    cf_world* w_ = nullptr;
    float width_, height_;
    std::uint64_t seed_;
    std::vector<float> raw_;
    bool raw_handed_out_ = false;
};

}  // namespace cellflow
