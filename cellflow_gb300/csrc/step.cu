// step.cu - pairwise smooth force, neighbour density and friction integrator.
//
// One thread per particle in cell order (the sorted snapshot of positions),
// fused with the integrator; results are written back to original order.
//
// Arithmetic follows cuda-native/src/ParticleSimulation.cu:86-165 operation
// by operation with round-to-nearest intrinsics, which nvcc never contracts:
//   - the neighbour test is exact: d^2 = (dx*dx + dy*dy) + dz*dz and
//     s = d^2 + 1e-4 rounded as the reference (compiled without contraction)
//     rounds them, and sqrtf(s) < eff is replaced by the equivalent s < t,
//     t the smallest float whose correctly rounded square root is >= eff, so
//     neighbour counts match bit for bit;
//   - the periodic wrap of a displacement is the reference's subtraction of
//     the extent, applied where the reference's test would fire: with at
//     least 5 cells on every axis that is exactly the stencil cells across
//     the box edge, so it is one add of a per-cell shift; with fewer cells
//     the kernel runs the reference's two tests per candidate;
//   - force terms use correctly rounded sqrt and division as the reference
//     does; only expf differs (CUDA's, within 2 ulp) and the summation order
//     (cell order instead of index order).
#include <cuda_runtime.h>

#include "cf_internal.hpp"

namespace cf {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ float wrap_ref(float d, float ext, float half)
{
    // ParticleSimulation.cu:97-102
    if (d > half) d = __fsub_rn(d, ext);
    if (d < -half) d = __fadd_rn(d, ext);
    return d;
}

template <bool kGeneric, bool kUniformR>
__global__ void __launch_bounds__(kThreads)
    step_force_kernel(StepConsts c, const PairTables* __restrict__ tables, const float4* __restrict__ pos_sorted,
                      const uint32_t* __restrict__ keys_sorted, const uint32_t* __restrict__ vals_sorted,
                      const uint32_t* __restrict__ cell_start, const uint32_t* __restrict__ cell_end,
                      float4* __restrict__ pos, float4* __restrict__ vel, float4* __restrict__ acc,
                      int* __restrict__ counts)
{
    __shared__ float s_force[kTableSize];
    __shared__ float s_eff[kTableSize];
    __shared__ float s_thr[kTableSize];
    const int T = c.num_types;
    for (int e = threadIdx.x; e < T * T; e += kThreads) {
        int a = e / T, b = e - a * T;
        int k = a * kTableStride + b;
        s_force[k] = tables->force[k];
        s_eff[k] = tables->eff[k];
        s_thr[k] = tables->threshold[k];
    }
    __syncthreads();

    const int t = blockIdx.x * kThreads + threadIdx.x;
    if (t >= c.n) return;
    const float4 h = pos_sorted[t];
    const uint32_t tp = __float_as_uint(h.w) & (kTableStride - 1);
    const uint32_t key = keys_sorted[t];
    const int mx = c.grid.m[0], my = c.grid.m[1], mz = c.grid.m[2];
    const int cx = (int)(key % (uint32_t)mx);
    const int cy = (int)((key / (uint32_t)mx) % (uint32_t)my);
    const int cz = (int)(key / (uint32_t)(mx * my));
    // stencil extent per axis: a single layer when an axis has one cell
    const int lo_x = mx > 1 ? -1 : 0, hi_x = mx > 1 ? 1 : 0;
    const int lo_y = my > 1 ? -1 : 0, hi_y = my > 1 ? 1 : 0;
    const int lo_z = mz > 1 ? -1 : 0, hi_z = mz > 1 ? 1 : 0;

    float fx = 0.0f, fy = 0.0f, fz = 0.0f;
    int count = 0;
    for (int oz = lo_z; oz <= hi_z; oz++) {
        int z = cz + oz;
        float sz = 0.0f;
        if (z < 0) { z += mz; sz = -c.ext[2]; }
        else if (z >= mz) { z -= mz; sz = c.ext[2]; }
        for (int oy = lo_y; oy <= hi_y; oy++) {
            int y = cy + oy;
            float sy = 0.0f;
            if (y < 0) { y += my; sy = -c.ext[1]; }
            else if (y >= my) { y -= my; sy = c.ext[1]; }
            for (int ox = lo_x; ox <= hi_x; ox++) {
                int x = cx + ox;
                float sx = 0.0f;
                if (x < 0) { x += mx; sx = -c.ext[0]; }
                else if (x >= mx) { x -= mx; sx = c.ext[0]; }
                const uint32_t cell = (uint32_t)((z * my + y) * mx + x);
                const uint32_t j_end = cell_end[cell];
                for (uint32_t j = cell_start[cell]; j < j_end; j++) {
                    if (j == (uint32_t)t) continue;
                    const float4 q = pos_sorted[j];
                    float dx = __fsub_rn(q.x, h.x);
                    float dy = __fsub_rn(q.y, h.y);
                    float dz = __fsub_rn(q.z, h.z);
                    if (kGeneric) {
                        dx = wrap_ref(dx, c.ext[0], c.half[0]);
                        dy = wrap_ref(dy, c.ext[1], c.half[1]);
                        dz = wrap_ref(dz, c.ext[2], c.half[2]);
                    } else {
                        dx = __fadd_rn(dx, sx);
                        dy = __fadd_rn(dy, sy);
                        dz = __fadd_rn(dz, sz);
                    }
                    const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
                    const float s = __fadd_rn(d2, 0.0001f);
                    const uint32_t to = __float_as_uint(q.w) & (kTableStride - 1);
                    const int pair = (int)(tp * kTableStride + to);
                    const float thr = kUniformR ? c.thr_uniform : s_thr[pair];
                    if (s < thr) {
                        count++;
                        const float eff = kUniformR ? c.eff_uniform : s_eff[pair];
                        const float dist = __fsqrt_rn(s);
                        const float r = __fdiv_rn(dist, eff);
                        const float rep = __fmul_rn(c.repulsion, expf(__fmul_rn(__fmul_rn(c.neg_k, r), r)));
                        const float att = __fmul_rn(c.attraction, r);
                        const float net = __fmul_rn(__fsub_rn(rep, att), s_force[pair]);
                        fx = __fadd_rn(fx, __fmul_rn(__fdiv_rn(dx, dist), net));
                        fy = __fadd_rn(fy, __fmul_rn(__fdiv_rn(dy, dist), net));
                        fz = __fadd_rn(fz, __fmul_rn(__fdiv_rn(dz, dist), net));
                    }
                }
            }
        }
    }

    // density-adaptive scale and integrator (ParticleSimulation.cu:136-161)
    const uint32_t i = vals_sorted[t];
    const int prev = counts[i];
    const float avg = __fmul_rn((float)(count + prev), 0.5f);
    const float density = fminf(__fdiv_rn(avg, (float)c.max_expected_neighbors), 1.0f);
    const float adapt = __fsub_rn(1.0f, __fmul_rn(__fsub_rn(1.0f, c.balance), density));
    const float scale = __fmul_rn(c.force_multiplier, adapt);
    fx = __fmul_rn(fx, scale);
    fy = __fmul_rn(fy, scale);
    fz = __fmul_rn(fz, scale);
    const float4 v = vel[i];
    const float vx = __fadd_rn(__fmul_rn(v.x, c.friction), __fmul_rn(fx, c.delta_t));
    const float vy = __fadd_rn(__fmul_rn(v.y, c.friction), __fmul_rn(fy, c.delta_t));
    const float vz = __fadd_rn(__fmul_rn(v.z, c.friction), __fmul_rn(fz, c.delta_t));
    float px = __fadd_rn(h.x, __fmul_rn(vx, c.delta_t));
    float py = __fadd_rn(h.y, __fmul_rn(vy, c.delta_t));
    float pz = __fadd_rn(h.z, __fmul_rn(vz, c.delta_t));
    px = fmodf(__fadd_rn(px, c.ext[0]), c.ext[0]);
    py = fmodf(__fadd_rn(py, c.ext[1]), c.ext[1]);
    pz = fmodf(__fadd_rn(pz, c.ext[2]), c.ext[2]);
    pos[i] = make_float4(px, py, pz, h.w);
    vel[i] = make_float4(vx, vy, vz, 0.0f);
    acc[i] = make_float4(fx, fy, fz, 0.0f);
    counts[i] = count;
}

}  // namespace

cudaError_t launch_step_force(const StepConsts& c, const PairTables* tables, const float4* pos_sorted,
                              const uint32_t* keys_sorted, const uint32_t* vals_sorted, const uint32_t* cell_start,
                              const uint32_t* cell_end, float4* pos, float4* vel, float4* acc, int* counts,
                              cudaStream_t st)
{
    if (c.n <= 0) return cudaSuccess;
    const int blocks = (c.n + kThreads - 1) / kThreads;
    if (c.grid.generic) {
        if (c.uniform_r)
            step_force_kernel<true, true><<<blocks, kThreads, 0, st>>>(c, tables, pos_sorted, keys_sorted,
                                                                       vals_sorted, cell_start, cell_end, pos, vel,
                                                                       acc, counts);
        else
            step_force_kernel<true, false><<<blocks, kThreads, 0, st>>>(c, tables, pos_sorted, keys_sorted,
                                                                        vals_sorted, cell_start, cell_end, pos, vel,
                                                                        acc, counts);
    } else {
        if (c.uniform_r)
            step_force_kernel<false, true><<<blocks, kThreads, 0, st>>>(c, tables, pos_sorted, keys_sorted,
                                                                        vals_sorted, cell_start, cell_end, pos, vel,
                                                                        acc, counts);
        else
            step_force_kernel<false, false><<<blocks, kThreads, 0, st>>>(c, tables, pos_sorted, keys_sorted,
                                                                         vals_sorted, cell_start, cell_end, pos,
                                                                         vel, acc, counts);
    }
    return cudaGetLastError();
}

}  // namespace cf
