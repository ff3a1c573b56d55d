// adjoint.cu - backward step of a rollout and the soft radial distribution.
//
// No counterpart in the reference: the step it differentiates is
// cuda-native/src/ParticleSimulation.cu:78-165.
//
// Backward of one step (neighbour counts held constant, the wrap taken as the
// identity, both true almost everywhere).  With d = x_j - x_i (min image),
// s = |d|^2 + 1e-4, dist = sqrt(s), r = dist / eff, e = exp(-k r^2),
// n = R e - A r and P(d) = d n / dist:
//   dP/dd = (n / dist) I + h d d^T,   h = (n' dist - n) / dist^3,
//   n'    = (R e (-2 k r) - A) / eff.
// From the adjoints (gx', gv') of the step's outputs:
//   gw = gv' + dt gx',  gv = friction gw,  ga = dt gw,  gf_i = scale_i ga_i,
//   gx_i = gx'_i + sum_{j in N(i)} dP/dd(d_ij) (F[t_j][t_i] gf_j - F[t_i][t_j] gf_i),
// and the parameter gradients
//   gF[t_i][t_j] += q n,  gR += q F e,  gA -= q F r,  gk -= q F R e r^2   (q = gf_i . d / dist),
//   gM += adapt_i (f_i . ga_i),  gb += M density_i (f_i . ga_i),  gfriction += v . gw.
//
// Kernels: adj_prep (per particle: gv, gf and ga staged in cell order) and
// adj_pair (one warp per home particle in cell order, the lanes striding over
// its 27-cell stencil, the reference's exact neighbour test on the stored
// positions so the neighbour sets are the forward's).  Table and parameter
// gradients collect in shared memory per block and are added to double
// accumulators.
//
// Soft radial distribution: bins of width D = r_max / bins, centres
// c_k = (k + 1/2) D, cubic B-spline weights B((r - c_k) / D) (support 2 bins
// each side), so a pair contributes while r < r_max + 1.5 D:
//   h[a][b][k] = sum_{i in a, j in b, j != i} B((r_ij - c_k) / D) / (N_a (N_b / V) 4 pi c_k^2 D).
#include <cuda_runtime.h>

#include <algorithm>

#include "cf_internal.hpp"

namespace cf {
namespace {

constexpr int kAdjThreads = 128;

// Streaming multiprocessors of the current device (queried once; a query,
// so also legal while a stream is being captured).
int num_sms()
{
    static int sms = 0;
    if (sms <= 0) {
        int dev = 0, v = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0)
            sms = v;
        else
            return 148;
    }
    return sms;
}

__device__ __forceinline__ float wrap_ref(float d, float ext, float half)
{
    // ParticleSimulation.cu:97-102
    if (d > half) d = __fsub_rn(d, ext);
    if (d < -half) d = __fadd_rn(d, ext);
    return d;
}

__device__ __forceinline__ uint32_t type_of(const float4& p) { return __float_as_uint(p.w) & kTypeMask; }

// Stencil offsets of one axis: {-1, 0, 1} with at least 3 cells, fewer
// distinct ones below (every cell of the axis exactly once).
__device__ __forceinline__ void axis_range(int m, int& lo, int& hi)
{
    lo = m >= 3 ? -1 : 0;
    hi = m >= 2 ? 1 : 0;
}

__device__ __forceinline__ int wrap_cell(int v, int m) { return v < 0 ? v + m : (v >= m ? v - m : v); }

__device__ __forceinline__ float warp_sum(float v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Per particle, in cell order: gv (in place), gf and (ga, density).
__global__ void adj_prep_kernel(StepConsts c, const uint32_t* __restrict__ vals, const float4* __restrict__ vel,
                                const int* __restrict__ cnt_prev, const int* __restrict__ cnt_new,
                                const float4* __restrict__ gx, float4* __restrict__ gv, float4* __restrict__ gf_sorted,
                                float4* __restrict__ ga_sorted, double* __restrict__ gacc)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    float part = 0.0f;
    if (k < c.n) {
        const uint32_t i = vals[k];
        // ParticleSimulation.cu:136-143
        const float avg = (float)(cnt_new[i] + cnt_prev[i]) * 0.5f;
        const float density = fminf(avg / (float)c.max_expected_neighbors, 1.0f);
        const float scale = c.force_multiplier * (1.0f - (1.0f - c.balance) * density);
        const float4 g = gx[i], h = gv[i], v = vel[i];
        const float wx = h.x + c.delta_t * g.x, wy = h.y + c.delta_t * g.y, wz = h.z + c.delta_t * g.z;
        part = v.x * wx + v.y * wy + v.z * wz;
        gv[i] = make_float4(c.friction * wx, c.friction * wy, c.friction * wz, 0.0f);
        const float ax = c.delta_t * wx, ay = c.delta_t * wy, az = c.delta_t * wz;
        gf_sorted[k] = make_float4(scale * ax, scale * ay, scale * az, 0.0f);
        ga_sorted[k] = make_float4(ax, ay, az, density);
    }
    part = warp_sum(part);
    if ((threadIdx.x & 31) == 0 && part != 0.0f) atomicAdd(&gacc[kTableSize + CF_GRAD_FRICTION], (double)part);
}

// The x cells cx-1..cx+1 of a stencil row (fewer on axes under 3 cells) as
// at most two runs of consecutive cells, [a0, b0] and [a1, b1] (b1 < a1: none).
__device__ __forceinline__ void x_runs(int cx, int m0, int& a0, int& b0, int& a1, int& b1)
{
    int xlo, xhi;
    axis_range(m0, xlo, xhi);
    const int lo = cx + xlo, hi = cx + xhi;
    a1 = 0;
    b1 = -1;
    if (lo < 0) {
        a0 = lo + m0;
        b0 = m0 - 1;
        b1 = hi;
    } else if (hi >= m0) {
        a0 = lo;
        b0 = m0 - 1;
        b1 = hi - m0;
    } else {
        a0 = lo;
        b0 = hi;
    }
}

constexpr int kListCap = 256;  // candidate indices staged per warp at a time

// Calls fn(q) for every particle q in the 27-cell stencil of cell `cell` (fewer
// cells on axes under 3 cells), spread over the lanes of the calling warp.  The
// stencil's rows are at most 18 runs of consecutive cells, i.e. contiguous ranges
// of the sorted snapshot; lane r < 18 describes run r, a warp prefix sum
// concatenates them, and the concatenation is staged kListCap indices at a time
// into the warp's list, so the lanes stride over the whole candidate set rather
// than over one short run at a time.  The whole warp calls it; fn must not
// synchronise the warp.
template <typename Fn>
__device__ __forceinline__ void for_stencil(int m0, int m1, int m2, uint32_t cell,
                                            const uint32_t* __restrict__ cell_off, uint32_t* list, int lane, Fn fn)
{
    const int cx = (int)(cell % (uint32_t)m0), cy = (int)((cell / (uint32_t)m0) % (uint32_t)m1),
              cz = (int)(cell / ((uint32_t)m0 * (uint32_t)m1));
    int ylo, yhi, zlo, zhi, a0, b0, a1, b1;
    axis_range(m1, ylo, yhi);
    axis_range(m2, zlo, zhi);
    x_runs(cx, m0, a0, b0, a1, b1);
    const int ny = yhi - ylo + 1, nrows = ny * (zhi - zlo + 1);
    uint32_t beg = 0u;
    int len = 0;
    if (lane < 2 * nrows) {
        const int r = lane >> 1, run = lane & 1;
        const int oy = ylo + r % ny, oz = zlo + r / ny;
        const int ra = run ? a1 : a0, rb = run ? b1 : b0;
        if (rb >= ra) {
            const int row = (wrap_cell(cz + oz, m2) * m1 + wrap_cell(cy + oy, m1)) * m0;
            beg = cell_off[row + ra];
            len = (int)(cell_off[row + rb + 1] - beg);
        }
    }
    int incl = len;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    const int pre = incl - len;
    for (int base = 0; base < total; base += kListCap) {
        // every run writes its part of [base, base + kListCap)
        const int j0 = max(0, base - pre), j1 = min(len, base + kListCap - pre);
        for (int j = j0; j < j1; j++) list[pre + j - base] = beg + (uint32_t)j;
        __syncwarp();
        const int lim = min(kListCap, total - base);
        for (int g = lane; g < lim; g += 32) fn(list[g]);
        __syncwarp();
    }
}

// One warp per home particle (grid-stride over homes in cell order): the
// lanes share the home's 27-cell stencil, nine rows of at most two runs of
// consecutive cells, i.e. contiguous ranges of the sorted snapshot, and
// stride over them; the warp then sums its partials.  The neighbour test is
// the reference's exact one on the stored positions, so the neighbour sets
// are the forward's.
__global__ void __launch_bounds__(kAdjThreads)
    adj_pair_kernel(StepConsts c, const PairTables* __restrict__ tables, const float4* __restrict__ pos_sorted,
                    const uint32_t* __restrict__ keys, const uint32_t* __restrict__ vals,
                    const uint32_t* __restrict__ cell_off, const float4* __restrict__ gf_sorted,
                    const float4* __restrict__ ga_sorted, float4* __restrict__ gx, double* __restrict__ gacc)
{
    __shared__ float s_gF[kTableSize];
    __shared__ float s_par[8];
    __shared__ float s_thr[kTableSize], s_inv_eff[kTableSize], s_F[kTableSize];
    __shared__ uint32_t s_list[kAdjThreads / 32][kListCap];
    for (int q = threadIdx.x; q < kTableSize; q += blockDim.x) {
        s_gF[q] = 0.0f;
        s_thr[q] = tables->threshold[q];
        s_inv_eff[q] = tables->eff[q] > 0.0f ? 1.0f / tables->eff[q] : 0.0f;
        s_F[q] = tables->force[q];
    }
    if (threadIdx.x < 8) s_par[threadIdx.x] = 0.0f;
    __syncthreads();

    const int lane = threadIdx.x & 31;
    const float c2 = -c.neg_k;  // k
    const float c2_log2 = c.neg_k * 1.4426950408889634f;  // -k log2(e): e = 2^(c2_log2 r^2)
    const int warps = (int)(gridDim.x * (blockDim.x >> 5));
    const float R = c.repulsion, A = c.attraction;
    const int m0 = c.grid.m[0], m1 = c.grid.m[1], m2 = c.grid.m[2];
    uint32_t* list = s_list[threadIdx.x >> 5];
    float pR = 0.0f, pA = 0.0f, pK = 0.0f, pM = 0.0f, pB = 0.0f;
    for (int k = (int)(blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)); k < c.n; k += warps) {
        const float4 h = pos_sorted[k];
        const uint32_t ti = type_of(h);
        const float4 gfi = gf_sorted[k];
        const uint32_t cell = keys[k];
        float ax = 0.0f, ay = 0.0f, az = 0.0f;  // pair part of gx_i
        float fx = 0.0f, fy = 0.0f, fz = 0.0f;  // unscaled force f_i
        for_stencil(m0, m1, m2, cell, cell_off, list, lane, [&](uint32_t q) {
                        if ((int)q == k) return;
                        const float4 o = pos_sorted[q];
                        // the reference's displacement and neighbour test (ParticleSimulation.cu:97-111)
                        const float dx = wrap_ref(__fsub_rn(o.x, h.x), c.ext[0], c.half[0]);
                        const float dy = wrap_ref(__fsub_rn(o.y, h.y), c.ext[1], c.half[1]);
                        const float dz = wrap_ref(__fsub_rn(o.z, h.z), c.ext[2], c.half[2]);
                        const float d2 =
                            __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
                        const float s = __fadd_rn(d2, 0.0001f);
                        const uint32_t tj = type_of(o);
                        const int pair = ti * kTableStride + tj;
                        if (!(s < s_thr[pair])) return;
                        // rsqrt and exp2 approximations (a few ulp): the gradient's tolerance
                        // is far wider than the forward's
                        const float inv_eff = s_inv_eff[pair];
                        const float inv_d = rsqrtf(s);
                        const float dist = s * inv_d;
                        const float r = dist * inv_eff;
                        float e;
                        asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(e) : "f"(c2_log2 * r * r));
                        const float nraw = R * e - A * r;
                        const float dn = (R * e * (-2.0f * c2 * r) - A) * inv_eff;
                        const float phi = nraw * inv_d;
                        const float hc = (dn * dist - nraw) * inv_d * inv_d * inv_d;
                        const float Fij = s_F[pair], Fji = s_F[tj * kTableStride + ti];
                        const float4 gfj = gf_sorted[q];
                        const float wx = Fji * gfj.x - Fij * gfi.x, wy = Fji * gfj.y - Fij * gfi.y,
                                    wz = Fji * gfj.z - Fij * gfi.z;
                        const float dw = dx * wx + dy * wy + dz * wz;
                        ax += phi * wx + hc * dw * dx;
                        ay += phi * wy + hc * dw * dy;
                        az += phi * wz + hc * dw * dz;
                        const float qd = (gfi.x * dx + gfi.y * dy + gfi.z * dz) * inv_d;
                        atomicAdd(&s_gF[pair], qd * nraw);
                        pR += qd * Fij * e;
                        pA -= qd * Fij * r;
                        pK -= qd * Fij * R * e * r * r;
                        const float fw = Fij * phi;
                        fx += fw * dx;
                        fy += fw * dy;
                        fz += fw * dz;
        });
        ax = warp_sum(ax);
        ay = warp_sum(ay);
        az = warp_sum(az);
        fx = warp_sum(fx);
        fy = warp_sum(fy);
        fz = warp_sum(fz);
        if (lane == 0) {
            const uint32_t i = vals[k];
            float4 g = gx[i];
            g.x += ax;
            g.y += ay;
            g.z += az;
            gx[i] = g;
            const float4 ga = ga_sorted[k];
            const float fga = fx * ga.x + fy * ga.y + fz * ga.z;
            pM += (1.0f - (1.0f - c.balance) * ga.w) * fga;
            pB += c.force_multiplier * ga.w * fga;
        }
    }
    pR = warp_sum(pR);
    pA = warp_sum(pA);
    pK = warp_sum(pK);
    if (lane == 0) {
        atomicAdd(&s_par[CF_GRAD_REPULSION], pR);
        atomicAdd(&s_par[CF_GRAD_ATTRACTION], pA);
        atomicAdd(&s_par[CF_GRAD_K], pK);
        atomicAdd(&s_par[CF_GRAD_FORCE_MULTIPLIER], pM);
        atomicAdd(&s_par[CF_GRAD_BALANCE], pB);
    }
    __syncthreads();
    const int T = c.num_types;
    for (int q = threadIdx.x; q < T * T; q += blockDim.x) {
        const int a = q / T, b = q - a * T;
        const float v = s_gF[a * kTableStride + b];
        if (v != 0.0f) atomicAdd(&gacc[a * kTableStride + b], (double)v);
    }
    if (threadIdx.x < CF_GRAD_FRICTION && s_par[threadIdx.x] != 0.0f)
        atomicAdd(&gacc[kTableSize + threadIdx.x], (double)s_par[threadIdx.x]);
}

// ---- soft radial distribution

struct RdfConsts {
    float ext[3], half[3];
    int m[3];
    int n, T, bins;
    float inv_bin;  // 1 / D
    float r_cut;    // r_max + 1.5 D
};

__device__ __forceinline__ float bspline3(float t)
{
    const float a = fabsf(t);
    if (a < 1.0f) return 2.0f / 3.0f - a * a + 0.5f * a * a * a;
    if (a < 2.0f) {
        const float u = 2.0f - a;
        return u * u * u * (1.0f / 6.0f);
    }
    return 0.0f;
}

__device__ __forceinline__ float bspline3_d(float t)
{
    const float a = fabsf(t);
    float g = 0.0f;
    if (a < 1.0f)
        g = -2.0f * a + 1.5f * a * a;
    else if (a < 2.0f) {
        const float u = 2.0f - a;
        g = -0.5f * u * u;
    }
    return t < 0.0f ? -g : g;
}

// Calls fn(q, o, dx, dy, dz, r) for every other particle q (position o) within r_cut of
// home k, spread over the lanes of the calling warp (for_stencil).
template <typename Fn>
__device__ __forceinline__ void rdf_neighbours_warp(const RdfConsts& c, const float4* __restrict__ pos_sorted,
                                                    const uint32_t* __restrict__ keys,
                                                    const uint32_t* __restrict__ cell_off, uint32_t* list, int k,
                                                    const float4& h, int lane, Fn fn)
{
    for_stencil(c.m[0], c.m[1], c.m[2], keys[k], cell_off, list, lane, [&](uint32_t q) {
        if ((int)q == k) return;
        const float4 o = pos_sorted[q];
        const float dx = wrap_ref(o.x - h.x, c.ext[0], c.half[0]);
        const float dy = wrap_ref(o.y - h.y, c.ext[1], c.half[1]);
        const float dz = wrap_ref(o.z - h.z, c.ext[2], c.half[2]);
        const float r = sqrtf(dx * dx + dy * dy + dz * dz);
        if (r < c.r_cut) fn(q, o, dx, dy, dz, r);
    });
}

// One warp per home (grid-stride), the histogram in shared memory per block.
__global__ void rdf_kernel(RdfConsts c, const float4* __restrict__ pos_sorted, const uint32_t* __restrict__ keys,
                           const uint32_t* __restrict__ cell_off, double* __restrict__ acc,
                           unsigned long long* __restrict__ type_count)
{
    extern __shared__ float s_hist[];
    __shared__ unsigned int s_count[CF_MAX_TYPES];
    __shared__ uint32_t s_list[kAdjThreads / 32][kListCap];
    const int H = c.T * c.T * c.bins;
    for (int q = threadIdx.x; q < H; q += blockDim.x) s_hist[q] = 0.0f;
    if (threadIdx.x < CF_MAX_TYPES) s_count[threadIdx.x] = 0u;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int warps = (int)(gridDim.x * (blockDim.x >> 5));
    for (int k = (int)(blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)); k < c.n; k += warps) {
        const float4 h = pos_sorted[k];
        const uint32_t ti = type_of(h);
        // a type outside [0, T) is reported by the cell list's hash; skip it here
        if (ti >= (uint32_t)c.T) continue;
        if (lane == 0) atomicAdd(&s_count[ti], 1u);
        rdf_neighbours_warp(c, pos_sorted, keys, cell_off, s_list[threadIdx.x >> 5], k, h, lane,
                            [&](uint32_t, const float4& o, float, float, float, float r) {
                                if (type_of(o) >= (uint32_t)c.T) return;
                                const float t0 = r * c.inv_bin - 0.5f;
                                const int k0 = max(0, (int)ceilf(t0 - 2.0f));
                                const int k1 = min(c.bins - 1, (int)floorf(t0 + 2.0f));
                                float* row = s_hist + ((int)ti * c.T + (int)type_of(o)) * c.bins;
                                for (int b = k0; b <= k1; b++) atomicAdd(&row[b], bspline3(t0 - (float)b));
                            });
    }
    __syncthreads();
    for (int q = threadIdx.x; q < H; q += blockDim.x)
        if (s_hist[q] != 0.0f) atomicAdd(&acc[q], (double)s_hist[q]);
    if (threadIdx.x < c.T && s_count[threadIdx.x]) atomicAdd(&type_count[threadIdx.x], s_count[threadIdx.x]);
}

__global__ void type_count_kernel(const float4* __restrict__ pos, int n, unsigned long long* __restrict__ type_count)
{
    __shared__ unsigned int s_count[CF_MAX_TYPES];
    if (threadIdx.x < CF_MAX_TYPES) s_count[threadIdx.x] = 0u;
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) atomicAdd(&s_count[type_of(pos[i])], 1u);
    __syncthreads();
    if (threadIdx.x < CF_MAX_TYPES && s_count[threadIdx.x]) atomicAdd(&type_count[threadIdx.x], s_count[threadIdx.x]);
}

// Normalisation N_a (N_b / V) 4 pi c_k^2 D of bin (a, b, k); 0 where a type is absent.
__device__ __forceinline__ double rdf_den(const RdfConsts& c, const unsigned long long* type_count, int q)
{
    const int b = q % c.bins, ab = q / c.bins, tb = ab % c.T, ta = ab / c.T;
    const double V = (double)c.ext[0] * (double)c.ext[1] * (double)c.ext[2];
    const double D = 1.0 / (double)c.inv_bin, ck = ((double)b + 0.5) * D;
    return (double)type_count[ta] * ((double)type_count[tb] / V) * 4.0 * 3.14159265358979323846 * ck * ck * D;
}

__global__ void rdf_finish_kernel(RdfConsts c, const double* __restrict__ acc,
                                  const unsigned long long* __restrict__ type_count, float* __restrict__ hist)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= c.T * c.T * c.bins) return;
    const double den = rdf_den(c, type_count, q);
    hist[q] = den > 0.0 ? (float)(acc[q] / den) : 0.0f;
}

__global__ void rdf_grad_kernel(RdfConsts c, const float4* __restrict__ pos_sorted, const uint32_t* __restrict__ keys,
                                const uint32_t* __restrict__ vals, const uint32_t* __restrict__ cell_off,
                                const float* __restrict__ ghist, const unsigned long long* __restrict__ type_count,
                                float4* __restrict__ gpos)
{
    extern __shared__ float s_g[];  // ghist / den
    __shared__ uint32_t s_list[kAdjThreads / 32][kListCap];
    const int H = c.T * c.T * c.bins;
    for (int q = threadIdx.x; q < H; q += blockDim.x) {
        const double den = rdf_den(c, type_count, q);
        s_g[q] = den > 0.0 ? (float)((double)ghist[q] / den) : 0.0f;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int warps = (int)(gridDim.x * (blockDim.x >> 5));
    for (int k = (int)(blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)); k < c.n; k += warps) {
        const float4 h = pos_sorted[k];
        const uint32_t ti = type_of(h);
        float ax = 0.0f, ay = 0.0f, az = 0.0f;
        // a type outside [0, T) is reported by the cell list's hash; it contributes nothing here
        if (ti < (uint32_t)c.T)
            rdf_neighbours_warp(c, pos_sorted, keys, cell_off, s_list[threadIdx.x >> 5], k, h, lane,
                                [&](uint32_t, const float4& o, float dx, float dy, float dz, float r) {
                                    const uint32_t tj = type_of(o);
                                    if (!(r > 0.0f) || tj >= (uint32_t)c.T) return;
                                    const float t0 = r * c.inv_bin - 0.5f;
                                    const int k0 = max(0, (int)ceilf(t0 - 2.0f));
                                    const int k1 = min(c.bins - 1, (int)floorf(t0 + 2.0f));
                                    const float* gij = s_g + ((int)ti * c.T + (int)tj) * c.bins;
                                    const float* gji = s_g + ((int)tj * c.T + (int)ti) * c.bins;
                                    float G = 0.0f;
                                    for (int b = k0; b <= k1; b++) G += (gij[b] + gji[b]) * bspline3_d(t0 - (float)b);
                                    const float s = G * c.inv_bin / r;
                                    ax -= s * dx;
                                    ay -= s * dy;
                                    az -= s * dz;
                                });
        ax = warp_sum(ax);
        ay = warp_sum(ay);
        az = warp_sum(az);
        if (lane == 0) gpos[vals[k]] = make_float4(ax, ay, az, 0.0f);
    }
}

// dst.xyz = src.xyz, dst.w = typesrc.w (the particle's type bits).
__global__ void pack_pos_kernel(const float4* __restrict__ src, const float4* typesrc, float4* dst, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 s = src[i];
    dst[i] = make_float4(s.x, s.y, s.z, typesrc[i].w);
}

RdfConsts rdf_consts(const float* ext, const Grid& g, int n, int T, int bins, float r_max)
{
    RdfConsts c;
    for (int a = 0; a < 3; a++) {
        c.ext[a] = ext[a];
        c.half[a] = ext[a] * 0.5f;
        c.m[a] = g.m[a];
    }
    c.n = n;
    c.T = T;
    c.bins = bins;
    c.inv_bin = (float)bins / r_max;
    c.r_cut = rdf_cutoff(bins, r_max);
    return c;
}

}  // namespace

float rdf_cutoff(int bins, float r_max) { return r_max + 1.5f * (r_max / (float)bins); }

size_t rdf_smem_bytes(int T, int bins) { return sizeof(float) * (size_t)T * T * bins; }

cudaError_t configure_adjoint()
{
    cudaError_t e = cudaFuncSetAttribute(rdf_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kRdfMaxSmem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(rdf_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kRdfMaxSmem);
    return e;
}

cudaError_t launch_adjoint_step(const StepConsts& c, const PairTables* tables, const float4* pos_sorted,
                                const uint32_t* keys_sorted, const uint32_t* vals_sorted, const uint32_t* cell_off,
                                const float4* vel, const int* cnt_prev, const int* cnt_new, float4* gx, float4* gv,
                                float4* gf_sorted, float4* ga_sorted, double* gacc, cudaStream_t st)
{
    if (c.n == 0) return cudaSuccess;
    const int blocks = (c.n + kAdjThreads - 1) / kAdjThreads;
    adj_prep_kernel<<<blocks, kAdjThreads, 0, st>>>(c, vals_sorted, vel, cnt_prev, cnt_new, gx, gv, gf_sorted,
                                                     ga_sorted, gacc);
    note_launches(st);
    // one warp per home, grid-stride: eight blocks of four warps per SM
    const int pair_blocks = std::min((c.n + kAdjThreads / 32 - 1) / (kAdjThreads / 32), 8 * num_sms());
    adj_pair_kernel<<<pair_blocks, kAdjThreads, 0, st>>>(c, tables, pos_sorted, keys_sorted, vals_sorted, cell_off,
                                                          gf_sorted, ga_sorted, gx, gacc);
    note_launches(st);
    return cudaGetLastError();
}

cudaError_t launch_pack_pos(const float4* src, const float4* typesrc, float4* dst, int n, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    pack_pos_kernel<<<(n + 255) / 256, 256, 0, st>>>(src, typesrc, dst, n);
    note_launches(st);
    return cudaGetLastError();
}

cudaError_t launch_rdf(const float* ext, const Grid& g, int n, int T, int bins, float r_max, const float4* pos_sorted,
                       const uint32_t* keys_sorted, const uint32_t* cell_off, double* acc,
                       unsigned long long* type_count, float* hist, cudaStream_t st)
{
    const RdfConsts c = rdf_consts(ext, g, n, T, bins, r_max);
    const int H = T * T * bins;
    cudaError_t e = cudaMemsetAsync(acc, 0, sizeof(double) * H, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(type_count, 0, sizeof(unsigned long long) * CF_MAX_TYPES, st);
    if (e != cudaSuccess) return e;
    // one warp per home, grid-stride; up to eight blocks per SM while their histograms
    // stay within 48 KB of shared memory (every block flushes its histogram once)
    const int warps_per_block = kAdjThreads / 32;
    const int per_sm = (int)std::max<size_t>(1, std::min<size_t>(8, (48u << 10) / rdf_smem_bytes(T, bins)));
    if (n > 0) {
        rdf_kernel<<<std::min((n + warps_per_block - 1) / warps_per_block, per_sm * num_sms()), kAdjThreads,
                     rdf_smem_bytes(T, bins), st>>>(c, pos_sorted, keys_sorted, cell_off, acc, type_count);
        note_launches(st);
    }
    rdf_finish_kernel<<<(H + 255) / 256, 256, 0, st>>>(c, acc, type_count, hist);
    note_launches(st);
    return cudaGetLastError();
}

cudaError_t launch_rdf_grad(const float* ext, const Grid& g, int n, int T, int bins, float r_max,
                            const float4* pos, const float4* pos_sorted, const uint32_t* keys_sorted,
                            const uint32_t* vals_sorted, const uint32_t* cell_off, const float* ghist,
                            unsigned long long* type_count, float4* gpos, cudaStream_t st)
{
    const RdfConsts c = rdf_consts(ext, g, n, T, bins, r_max);
    cudaError_t e = cudaMemsetAsync(type_count, 0, sizeof(unsigned long long) * CF_MAX_TYPES, st);
    if (e != cudaSuccess || n == 0) return e;
    type_count_kernel<<<(n + 255) / 256, 256, 0, st>>>(pos, n, type_count);
    note_launches(st);
    const int warps_per_block = kAdjThreads / 32;
    rdf_grad_kernel<<<std::min((n + warps_per_block - 1) / warps_per_block, 8 * num_sms()), kAdjThreads,
                      rdf_smem_bytes(T, bins), st>>>(c, pos_sorted, keys_sorted, vals_sorted, cell_off, ghist,
                                                     type_count, gpos);
    note_launches(st);
    return cudaGetLastError();
}

}  // namespace cf
