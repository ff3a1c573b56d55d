// init.cu - seeded particle spawn and AoS <-> SoA conversion.
//
// Spawn follows initializeParticlesKernel (cuda-native/src/ParticleSimulation.cu:29-66):
// positions uniform in a spawn box, zero velocity and acceleration, uniform
// types.  The reference drew from a time-seeded cuRAND XORWOW state
// (:21-26, :480); here each particle draws from Philox4x32-10 (Salmon,
// Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11)
// with counter (i, 0, 0, 0) and the 64-bit seed as key, so a seed gives the
// same particles on every device and in the host generator of the tests.
#include <cuda_runtime.h>

#include "cf_internal.hpp"

namespace cf {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k)
{
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; r++) {
        if (r) {
            k.x += W0;
            k.y += W1;
        }
        const uint32_t hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
        const uint32_t hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    }
    return c;
}

// 24-bit uniform in [0, 1): exact multiples of 2^-24.
__device__ __forceinline__ float unit24(uint32_t v) { return (float)(v >> 8) * (1.0f / 16777216.0f); }

__global__ void __launch_bounds__(kThreads)
    init_particles_kernel(float4* __restrict__ pos, float4* __restrict__ vel, float4* __restrict__ acc,
                          int* __restrict__ counts, int n, int num_types, float lo_x, float lo_y, float lo_z,
                          float span_x, float span_y, float span_z, uint2 key, uint32_t world)
{
    const int i = blockIdx.x * kThreads + threadIdx.x;
    if (i >= n) return;
    const uint4 r = philox4x32_10(make_uint4((uint32_t)i, 0u, 0u, 0u), key);
    const float x = __fadd_rn(lo_x, __fmul_rn(unit24(r.x), span_x));
    const float y = __fadd_rn(lo_y, __fmul_rn(unit24(r.y), span_y));
    const float z = __fadd_rn(lo_z, __fmul_rn(unit24(r.z), span_z));
    const uint32_t type = (uint32_t)(((unsigned long long)r.w * (unsigned long long)num_types) >> 32);
    pos[i] = make_float4(x, y, z, __uint_as_float(type | (world << kWorldShift)));
    vel[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    acc[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    counts[i] = 0;
}

__global__ void __launch_bounds__(kThreads)
    aos_to_soa_kernel(const cf_particle* __restrict__ aos, float4* __restrict__ pos, float4* __restrict__ vel,
                      float4* __restrict__ acc, int n)
{
    const int i = blockIdx.x * kThreads + threadIdx.x;
    if (i >= n) return;
    const cf_particle p = aos[i];
    pos[i] = make_float4(p.pos[0], p.pos[1], p.pos[2], __uint_as_float(p.ptype));
    vel[i] = make_float4(p.vel[0], p.vel[1], p.vel[2], 0.0f);
    acc[i] = make_float4(p.acc[0], p.acc[1], p.acc[2], 0.0f);
}

__global__ void __launch_bounds__(kThreads)
    soa_to_aos_kernel(const float4* __restrict__ pos, const float4* __restrict__ vel, const float4* __restrict__ acc,
                      cf_particle* __restrict__ aos, int n)
{
    const int i = blockIdx.x * kThreads + threadIdx.x;
    if (i >= n) return;
    const float4 p = pos[i], v = vel[i], a = acc[i];
    cf_particle o;
    o.pos[0] = p.x;
    o.pos[1] = p.y;
    o.pos[2] = p.z;
    o.vel[0] = v.x;
    o.vel[1] = v.y;
    o.vel[2] = v.z;
    o.acc[0] = a.x;
    o.acc[1] = a.y;
    o.acc[2] = a.z;
    o.ptype = __float_as_uint(p.w) & kTypeMask;  // world bits stay internal
    o.pad = 0.0f;
    aos[i] = o;
}

// The same records written straight into page-locked host memory (its device
// view), one 32-bit word per thread so that consecutive threads write
// consecutive words of the 44-B records: the stores cross the CPU-GPU link as
// whole lines, with no staging buffer or separate copy.
__global__ void __launch_bounds__(kThreads)
    soa_to_aos_words_kernel(const float4* __restrict__ pos, const float4* __restrict__ vel,
                            const float4* __restrict__ acc, uint32_t* __restrict__ words, int n)
{
    constexpr int kWords = (int)(sizeof(cf_particle) / sizeof(uint32_t));
    const long long t = (long long)blockIdx.x * kThreads + threadIdx.x;
    if (t >= (long long)kWords * n) return;
    const int i = (int)(t / kWords), k = (int)(t - (long long)kWords * i);
    uint32_t v;
    if (k < 3) v = __float_as_uint(reinterpret_cast<const float*>(pos + i)[k]);
    else if (k < 6) v = __float_as_uint(reinterpret_cast<const float*>(vel + i)[k - 3]);
    else if (k < 9) v = __float_as_uint(reinterpret_cast<const float*>(acc + i)[k - 6]);
    else if (k == 9) v = __float_as_uint(pos[i].w) & kTypeMask;  // world bits stay internal
    else v = 0u;                                                // pad
    words[t] = v;
}

// The reverse: one word of the page-locked records per thread (consecutive
// threads read consecutive words), scattered into the state arrays.
__global__ void __launch_bounds__(kThreads)
    aos_words_to_soa_kernel(const uint32_t* __restrict__ words, float4* __restrict__ pos, float4* __restrict__ vel,
                            float4* __restrict__ acc, int n)
{
    constexpr int kWords = (int)(sizeof(cf_particle) / sizeof(uint32_t));
    const long long t = (long long)blockIdx.x * kThreads + threadIdx.x;
    if (t >= (long long)kWords * n) return;
    const int i = (int)(t / kWords), k = (int)(t - (long long)kWords * i);
    const uint32_t v = words[t];
    if (k < 3) reinterpret_cast<float*>(pos + i)[k] = __uint_as_float(v);
    else if (k < 6) reinterpret_cast<float*>(vel + i)[k - 3] = __uint_as_float(v);
    else if (k < 9) reinterpret_cast<float*>(acc + i)[k - 6] = __uint_as_float(v);
    else if (k == 9) pos[i].w = __uint_as_float(v);  // the type, as the per-record conversion stores it
    else {
        vel[i].w = 0.0f;
        acc[i].w = 0.0f;
    }
}

// moveParticlesKernel (cuda-native/src/ParticleSimulation.cu:169-185): every
// position translated and wrapped as fmodf((x + dx) + W, W), in that order.
__global__ void __launch_bounds__(kThreads)
    move_particles_kernel(float4* __restrict__ pos, int n, float dx, float dy, float dz, float ext_x, float ext_y,
                          float ext_z)
{
    const int i = blockIdx.x * kThreads + threadIdx.x;
    if (i >= n) return;
    float4 p = pos[i];
    p.x = fmodf(__fadd_rn(__fadd_rn(p.x, dx), ext_x), ext_x);
    p.y = fmodf(__fadd_rn(__fadd_rn(p.y, dy), ext_y), ext_y);
    p.z = fmodf(__fadd_rn(__fadd_rn(p.z, dz), ext_z), ext_z);
    pos[i] = p;
}

}  // namespace

cudaError_t launch_move_particles(float4* pos, int n, float dx, float dy, float dz, const float* ext, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    move_particles_kernel<<<(n + kThreads - 1) / kThreads, kThreads, 0, st>>>(pos, n, dx, dy, dz, ext[0], ext[1],
                                                                             ext[2]);
    note_launches(st);
    return cudaGetLastError();
}

cudaError_t launch_aos_to_soa_mapped(const cf_particle* aos_host, float4* pos, float4* vel, float4* acc, int n,
                                     cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    const long long words = 11LL * n;
    aos_words_to_soa_kernel<<<(unsigned)((words + kThreads - 1) / kThreads), kThreads, 0, st>>>(
        reinterpret_cast<const uint32_t*>(aos_host), pos, vel, acc, n);
    note_launches(st);
    return cudaGetLastError();
}

cudaError_t launch_soa_to_aos_mapped(const float4* pos, const float4* vel, const float4* acc, cf_particle* aos_host,
                                     int n, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    static_assert(sizeof(cf_particle) == 11 * sizeof(uint32_t), "44-B records");
    const long long words = 11LL * n;
    soa_to_aos_words_kernel<<<(unsigned)((words + kThreads - 1) / kThreads), kThreads, 0, st>>>(
        pos, vel, acc, reinterpret_cast<uint32_t*>(aos_host), n);
    note_launches(st);
    return cudaGetLastError();
}

cudaError_t launch_init_particles(float4* pos, float4* vel, float4* acc, int* counts, int n, int num_types,
                                  const float* lo, const float* span, uint64_t seed, cudaStream_t st, uint32_t world)
{
    if (n <= 0) return cudaSuccess;
    const uint2 key = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32));
    init_particles_kernel<<<(n + kThreads - 1) / kThreads, kThreads, 0, st>>>(
        pos, vel, acc, counts, n, num_types, lo[0], lo[1], lo[2], span[0], span[1], span[2], key, world);
    note_launches(st);
    return cudaGetLastError();
}

cudaError_t launch_aos_to_soa(const cf_particle* aos, float4* pos, float4* vel, float4* acc, int n, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    aos_to_soa_kernel<<<(n + kThreads - 1) / kThreads, kThreads, 0, st>>>(aos, pos, vel, acc, n);
    note_launches(st);
    return cudaGetLastError();
}

cudaError_t launch_soa_to_aos(const float4* pos, const float4* vel, const float4* acc, cf_particle* aos, int n,
                              cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    soa_to_aos_kernel<<<(n + kThreads - 1) / kThreads, kThreads, 0, st>>>(pos, vel, acc, aos, n);
    note_launches(st);
    return cudaGetLastError();
}

}  // namespace cf
