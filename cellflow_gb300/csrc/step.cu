// step.cu - pairwise smooth force, neighbour density and friction integrator.
//
// Work decomposition.  Particles are in cell order (the sorted snapshot of
// positions).  An item is up to 32 consecutive particles of one row of cells
// (same y and z cell): one warp, one particle per lane.  The candidates of
// an item are the particles of the union of its homes' 27-cell stencils:
// 9 rows, each a run of consecutive cells, i.e. one contiguous range of the
// sorted snapshot (two where the run wraps around the box in x).  The warp
// copies those ranges into shared memory, 256, 384 or 512 at a time (chosen
// by the autotuner), with their periodic shift already applied, and every
// lane tests every staged candidate (broadcast reads).  For worlds too small
// to fill the GPU, 2 or 4 warps share an item, each taking an equal share of
// its candidates; the first adds the others' partial sums in a fixed order.
// Items are 16-B records (first particle, count, the row's y/z, world)
// written by the cell list, so no per-item integer division is needed.
//
// Coordinates are staged relative to an origin per pass (the centre of the
// stencil box where that keeps c - o exact, else 0), periodic shift folded
// in, with |c|^2 beside them; an unshifted displacement is then the
// reference's fl(c - h) bit for bit.
//
// Per batch of staged candidates, two phases per lane:
//   Filter: |c - h|^2 - bound = |c|^2 + (|h|^2 - bound) - 2 h.c for two
//     candidates per instruction chain (packed f32x2 add/fma of sm_100+: one
//     add and three fma per pair of candidates), the sign bit of each result
//     shifted into a 32-bit mask per 32 candidates.  The bound is >= the
//     exact test for every pair plus the expansion's rounding, which the
//     origin keeps at the scale of the stencil box.  ~85% of pairs stop here.
//   Drain: for every set bit (two per trip, three with lane pairing; a
//     warp-uniform trip count from the filter's per-lane hit counts), the
//     contracted distance of the displacement; pairs below a second bound
//     (<= the exact test for every pair) interact for certain, and only the
//     rare pairs between the two bounds (a band ~1e-6 wide) take the
//     reference's exact test on the unshifted coordinates, in the trips where
//     a warp vote finds one (written inline, its instructions ran predicated
//     for every pair).  Interacting pairs add their force term.  In
//     the lane-paired variant the lanes are sorted by hit count and paired
//     busiest with idlest; the idler lane of a pair, after its own hits,
//     walks the top part of its partner's with its partner's home and hands
//     the partial sums over, so the trip count falls towards the mean.
//
// Exactness (cuda-native/src/ParticleSimulation.cu:86-165):
//   - the neighbour test is the reference's: d^2 = (dx*dx + dy*dy) + dz*dz and
//     s = d^2 + 1e-4 rounded as the reference (compiled without contraction)
//     rounds them, and sqrtf(s) < eff is replaced by the equivalent s < t,
//     t the smallest float whose correctly rounded square root is >= eff.
//     The two bounds bracket that test, so neighbour counts match bit for bit;
//   - a displacement is wrapped like the reference (subtract the extent where
//     its test fires).  With at least 5 cells per axis that is exactly the
//     stencil cells across the box edge: the union of an item spans at most
//     the box width in x, so every staged range has one shift for every lane,
//     added after the subtraction (exact path) as the reference does.  With
//     fewer cells both phases run the reference's tests per candidate;
//   - force terms use rsqrt and exp approximations (a few ulp) and the
//     contracted distance; the sum runs in cell order.
//   The density factor, integrator and wrap are the reference's operations.
#include <type_traits>
#include <cuda_runtime.h>

#include "cf_internal.hpp"

namespace cf {
namespace {

constexpr int kWarps = 4;
constexpr int kThreads = 32 * kWarps;
constexpr float kFar = 1e30f;  // padding slots sit at +kFar, idle homes at -kFar
constexpr int kTypeShift = 27; // staged meta: sorted index | type << 27
constexpr uint32_t kIndexMask = (1u << kTypeShift) - 1u;

__device__ __forceinline__ float wrap_ref(float d, float ext, float half)
{
    // ParticleSimulation.cu:97-102
    if (d > half) d = __fsub_rn(d, ext);
    if (d < -half) d = __fadd_rn(d, ext);
    return d;
}

// Shift code per axis: 0 none, 1 subtract the extent, 2 add it.
__device__ __forceinline__ float code_shift(uint32_t code, float ext)
{
    return code == 1u ? -ext : (code == 2u ? ext : 0.0f);
}

// The shift that was added to a raw coordinate to give its staged value.
__device__ __forceinline__ float staged_shift(float staged, float raw, float ext)
{
    const float d = staged - raw;
    return d > 0.5f * ext ? ext : (d < -0.5f * ext ? -ext : 0.0f);
}

__device__ __forceinline__ int wrap_index(int v, int m) { return v < 0 ? v + m : (v >= m ? v - m : v); }

// fmodf(x, W) of the integrator's wrap (ParticleSimulation.cu:159-161), exact:
// for x in [0, 2W) it is x or x - W, and x - W is exact there (Sterbenz).
__device__ __forceinline__ float wrap_pos(float x, float W)
{
    if (x >= 0.0f && x < 2.0f * W) return x >= W ? __fsub_rn(x, W) : x;
    return fmodf(x, W);
}

// Staging origin on one axis for stencil cells [clo, chi] (shifted cell
// coordinates, cell size cs) and the radius r of the box around it.  The
// centre is used only where it is at least twice the half-width: then every
// raw coordinate c in the box satisfies o/2 <= c <= 2o, so c - o is exact
// (Sterbenz) and an unshifted displacement (c - o) - (h - o) rounds to the
// reference's fl(c - h).  Otherwise the origin is 0 (also exact).
__device__ __forceinline__ void stencil_origin(int clo, int chi, float cs, float& o, float& r)
{
    const float lo = (float)clo * cs, hi = (float)(chi + 1) * cs, mg = 0.05f * cs;
    const float ctr = 0.5f * (lo + hi), half = 0.5f * (hi - lo) + mg;
    if (ctr >= 2.0f * half) {
        o = ctr;
        r = half;
    } else {
        o = 0.0f;
        r = fmaxf(fabsf(lo), fabsf(hi)) + mg;
    }
}

// Lane pairing scratch of the drain (the variants that pair lanes):
// each lane's home and filter operands for the pass, its group bitmap for the
// batch, its partner, and its own partial sums while it works on its partner's hits.
struct PairScratch {
    float4 home_h[32];
    float4 home_m2[32];
    float4 saved[32];
    uint32_t nzw[32];
    uint32_t pairing[32];
};
struct NoScratch {};
// Balanced drain: each lane's home and filter operands, group bitmap and hit
// count for the batch, and the partial sums of the (lane, home) pieces of the
// task line, at index lane + rank of the home among the homes with hits.
struct BalScratch {
    float4 home_h[32];
    float4 home_m2[32];
    uint32_t nzw[32];
    int hits[32];
    float4 part[64];
};

// Per-warp staging area, kStage candidates (a multiple of 32) per batch.
// Drain modes: 0 one lane per home, 1 lanes paired (busiest with idlest),
// 2 balanced (the batch's hits split evenly over the lanes).
template <int kMode>
using DrainScratch = typename std::conditional<kMode == 1, PairScratch,
                                               typename std::conditional<kMode == 2, BalScratch, NoScratch>::type>::type;

template <int kStage, int kMode>
struct WarpSmem {
    float4 xy[kStage / 2];              // staged (x_a, x_b, y_a, y_b) of slots 2p, 2p+1
    float4 zc[kStage / 2];              // staged (z_a, z_b, |c_a|^2, |c_b|^2)
    uint32_t meta[kStage];              // sorted index | type << 27
    uint32_t mask[(kStage / 32) * 32];  // [group][lane]
    float origin[4];                    // the pass's staging origin (x, y, z)
    DrainScratch<kMode> pr;
};

// Named barrier of the warps sharing an item: id 1 + slot (slot < kWarps),
// immediate ids so only five hardware barriers are reserved.
__device__ __forceinline__ void item_barrier(int slot, int threads)
{
    switch (slot) {
    case 0: asm volatile("bar.sync 1, %0;" ::"r"(threads) : "memory"); break;
    case 1: asm volatile("bar.sync 2, %0;" ::"r"(threads) : "memory"); break;
    case 2: asm volatile("bar.sync 3, %0;" ::"r"(threads) : "memory"); break;
    default: asm volatile("bar.sync 4, %0;" ::"r"(threads) : "memory"); break;
    }
}

struct Lane {
    float4 h;     // home position (raw)
    uint32_t tp;  // home type
    float fx, fy, fz;
    int count;
};

// The origin-relative home of a pass as the filter's packed operands:
// (-2 h', -2 h') per axis and (|h'|^2 - bound) twice.  h' itself is
// -0.5 * m2h exactly, so the drain's displacement fl(c' - h') is
// fmaf(0.5, m2h, c').
struct HomeOps {
    float2 m2x, m2y, m2z, k;
};

// Per type pair of the item's world, T-stride: (R F, A F / eff).  With
// s = d^2 + 1e-4, dist = sqrt(s) and rs = 1/dist, the reference's term
//   (d / dist) F (R exp(-k r^2) - A r),  r = dist / eff   (ParticleSimulation.cu:113-124)
// is  d * (R F * exp2(c1 s) * rs - A F / eff),  c1 = -k log2(e) / eff^2.
struct Tables {
    const float2* coef;  // (R F, A F / eff), T-stride
    const float* c1;     // 32-stride (unused with a uniform radius)
    const float* thr;
    const float* thr_lo;
    int T;
};

constexpr float kLog2e = 1.4426950408889634f;

// Displacement from the home to a staged candidate.  Generic grids stage raw
// coordinates and wrap per candidate; otherwise both ends are origin-relative
// and the shift is already in the staged value.
template <bool kGeneric>
__device__ __forceinline__ void staged_delta(const StepConsts& c, float cx, float cy, float cz, const float4& h,
                                             const HomeOps& H, float& dx, float& dy, float& dz)
{
    if (kGeneric) {
        dx = wrap_ref(cx - h.x, c.ext[0], c.half[0]);
        dy = wrap_ref(cy - h.y, c.ext[1], c.half[1]);
        dz = wrap_ref(cz - h.z, c.ext[2], c.half[2]);
    } else {
        dx = fmaf(0.5f, H.m2x.x, cx);
        dy = fmaf(0.5f, H.m2y.x, cy);
        dz = fmaf(0.5f, H.m2z.x, cz);
    }
}

// One queued pair's interaction test: certain-interaction bound, exact
// fallback.  Returns the staged displacement and its contracted d^2.
// `origin` is the pass's staging origin (unused on generic grids).
template <bool kGeneric, bool kUniformR>
__device__ __forceinline__ bool pair_fast(const StepConsts& c, const Lane& L, const HomeOps& H, float cx, float cy,
                                          float cz, uint32_t meta, const Tables& tb, float& dx, float& dy, float& dz,
                                          float& d2)
{
    staged_delta<kGeneric>(c, cx, cy, cz, L.h, H, dx, dy, dz);
    d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
    const uint32_t other = meta >> kTypeShift;
    const uint32_t pair = L.tp * kTableStride + other;
    return d2 < (kUniformR ? c.thr_lo_uniform : tb.thr_lo[pair]);
}

// The reference's exact test for a pair the certain-interaction bound left
// open (within rounding of the threshold), on the unshifted coordinates.
template <bool kGeneric, bool kUniformR>
__device__ __forceinline__ bool pair_exact(const StepConsts& c, const Lane& L, const float* origin, float cx, float cy,
                                           float cz, uint32_t meta, const float4* __restrict__ pos_sorted,
                                           const Tables& tb)
{
    if (!CF_IN_BOUNDS(meta & kIndexMask, c.n)) return false;
    const float4 o = pos_sorted[meta & kIndexMask];
    float ex = __fsub_rn(o.x, L.h.x), ey = __fsub_rn(o.y, L.h.y), ez = __fsub_rn(o.z, L.h.z);
    if (kGeneric) {
        ex = wrap_ref(ex, c.ext[0], c.half[0]);
        ey = wrap_ref(ey, c.ext[1], c.half[1]);
        ez = wrap_ref(ez, c.ext[2], c.half[2]);
    } else {
        ex = __fadd_rn(ex, staged_shift(cx + origin[0], o.x, c.ext[0]));
        ey = __fadd_rn(ey, staged_shift(cy + origin[1], o.y, c.ext[1]));
        ez = __fadd_rn(ez, staged_shift(cz + origin[2], o.z, c.ext[2]));
    }
    const float e2 = __fadd_rn(__fadd_rn(__fmul_rn(ex, ex), __fmul_rn(ey, ey)), __fmul_rn(ez, ez));
    const uint32_t pair = L.tp * kTableStride + (meta >> kTypeShift);
    return __fadd_rn(e2, 0.0001f) < (kUniformR ? c.thr_uniform : tb.thr[pair]);
}

template <bool kGeneric, bool kUniformR>
__device__ __forceinline__ bool pair_test(const StepConsts& c, const Lane& L, const HomeOps& H,
                                          const float* origin, float cx, float cy, float cz, uint32_t meta,
                                          const float4* __restrict__ pos_sorted, const Tables& tb, float& dx,
                                          float& dy, float& dz, float& d2)
{
    staged_delta<kGeneric>(c, cx, cy, cz, L.h, H, dx, dy, dz);
    d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
    const uint32_t other = meta >> kTypeShift;
    const uint32_t pair = L.tp * kTableStride + other;
    bool inter = d2 < (kUniformR ? c.thr_lo_uniform : tb.thr_lo[pair]);
    if (!inter) {
        // within rounding of the threshold: the reference's exact test
        if (!CF_IN_BOUNDS(meta & kIndexMask, c.n)) return false;
        const float4 o = pos_sorted[meta & kIndexMask];
        float ex = __fsub_rn(o.x, L.h.x), ey = __fsub_rn(o.y, L.h.y), ez = __fsub_rn(o.z, L.h.z);
        if (kGeneric) {
            ex = wrap_ref(ex, c.ext[0], c.half[0]);
            ey = wrap_ref(ey, c.ext[1], c.half[1]);
            ez = wrap_ref(ez, c.ext[2], c.half[2]);
        } else {
            ex = __fadd_rn(ex, staged_shift(cx + origin[0], o.x, c.ext[0]));
            ey = __fadd_rn(ey, staged_shift(cy + origin[1], o.y, c.ext[1]));
            ez = __fadd_rn(ez, staged_shift(cz + origin[2], o.z, c.ext[2]));
        }
        const float e2 = __fadd_rn(__fadd_rn(__fmul_rn(ex, ex), __fmul_rn(ey, ey)), __fmul_rn(ez, ez));
        inter = __fadd_rn(e2, 0.0001f) < (kUniformR ? c.thr_uniform : tb.thr[pair]);
    }
    return inter;
}

// The force weight of an interacting pair (multiplies the displacement).
template <bool kUniformR>
__device__ __forceinline__ float pair_weight(float d2, uint32_t meta, const Lane& L, const Tables& tb, float c1u)
{
    const uint32_t other = meta >> kTypeShift;
    const float2 k = tb.coef[L.tp * tb.T + other];
    const float s = d2 + 0.0001f;
    const float rs = rsqrtf(s);
    const float c1 = kUniformR ? c1u : tb.c1[L.tp * kTableStride + other];
    float e;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(e) : "f"(c1 * s));
    return fmaf(k.x * e, rs, -k.y);
}

// The staged coordinates of a slot.
__device__ __forceinline__ void staged_xyz(const float* xyf, const float* zcf, int slot, float& x, float& y, float& z)
{
    const int pb = (slot >> 1) * 4 + (slot & 1);
    x = xyf[pb];
    y = xyf[pb + 2];
    z = zcf[pb];
}

template <int kStage, int kMinBlocks, int kMode, bool kGeneric, bool kUniformR>
__global__ void __launch_bounds__(kThreads, kMinBlocks)
    step_force_kernel(StepConsts c, const PairTables* __restrict__ tables, const float4* __restrict__ pos_sorted,
                      const uint32_t* __restrict__ keys_sorted, const uint32_t* __restrict__ vals_sorted,
                      const uint32_t* __restrict__ cell_off, const Item* __restrict__ items,
                      const int* __restrict__ n_items, float4* __restrict__ pos, float4* __restrict__ vel,
                      float4* __restrict__ acc, int* __restrict__ counts)
{
    __shared__ float s_inv_eff[kUniformR ? 1 : kTableSize];
    __shared__ float s_c1[kUniformR ? 1 : kTableSize];
    __shared__ float s_thr[kUniformR ? 1 : kTableSize];
    __shared__ float s_thr_lo[kUniformR ? 1 : kTableSize];
    __shared__ float4 s_part[kWarps][32];  // partial sums of the item's other warps (split > 1)
    extern __shared__ __align__(16) unsigned char s_dyn[];
    const int T = c.num_types;
    // force coefficients, compact T-stride: one copy per block for a single
    // world, one per warp (filled once its item's world is known) for a batch
    const bool one_world = c.grid.worlds == 1;
    float2* coef_base = reinterpret_cast<float2*>(s_dyn + sizeof(WarpSmem<kStage, kMode>) * kWarps);
    if (!kUniformR) {
        for (int e = threadIdx.x; e < T * T; e += kThreads) {
            const int a = e / T, b = e - a * T;
            const int k = a * kTableStride + b;
            const float inv = 1.0f / tables->eff[k];
            s_inv_eff[k] = inv;
            s_c1[k] = c.neg_k * kLog2e * inv * inv;
            s_thr[k] = tables->threshold[k];
            s_thr_lo[k] = tables->threshold_lo[k];
        }
    }
    if (one_world) {
        for (int e = threadIdx.x; e < T * T; e += kThreads) {
            const int a = e / T, b = e - a * T;
            const float F = c.world_force[a * kTableStride + b];
            const float inv = kUniformR ? c.inv_eff_uniform : 1.0f / tables->eff[a * kTableStride + b];
            coef_base[e] = make_float2(c.repulsion * F, c.attraction * F * inv);
        }
    }
    __syncthreads();
    const float c1u = c.neg_k * kLog2e * c.inv_eff_uniform * c.inv_eff_uniform;
    // pairs per drain trip: two side by side where the register budget allows,
    // three with lane pairing (more of the lanes stay busy, so more independent
    // work per trip pays there; it does not without pairing)
    constexpr int kPer = kMinBlocks >= 8 ? 1 : (kMode != 0 && !kGeneric ? 3 : 2);
    // lane pairing or the balanced drain (regular grids)
    constexpr bool kBalance = kMode == 1 && !kGeneric;
    constexpr bool kBal = kMode == 2 && !kGeneric;

    // c.split warps (1, 2 or 4) share an item, each taking an equal share of its
    // candidates; part 0 adds the others' partial sums and integrates
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int split = c.split;
    const int part = warp & (split - 1);
    const int item = blockIdx.x * (kWarps / split) + warp / split;
    if (item >= *n_items) return;  // the item's other warps leave too: no barrier is pending
    using Smem = WarpSmem<kStage, kMode>;
    Smem& w = reinterpret_cast<Smem*>(s_dyn)[warp];
    float2* wcoef = coef_base + (one_world ? 0 : warp * T * T);
    const float* xyf = reinterpret_cast<const float*>(w.xy);
    const float* zcf = reinterpret_cast<const float*>(w.zc);
    const Item it = items[item];
    // (bounds-checked build) the item's particles lie in [0, n): else the item's warps skip it
    if (!CF_IN_BOUNDS(it.count - 1, 32) || !CF_IN_BOUNDS(it.first, c.n) || !CF_IN_BOUNDS(it.first + it.count - 1, c.n))
        return;
    const bool active = lane < it.count;
    const int t = it.first + (active ? lane : 0);
    Lane L;
    L.h = pos_sorted[t];
    L.tp = __float_as_uint(L.h.w) & kTypeMask;
    L.fx = L.fy = L.fz = 0.0f;
    L.count = 0;

    // cell coordinates inside the item's world (items never straddle worlds or rows)
    const int mx = c.grid.m[0], my = c.grid.m[1], mz = c.grid.m[2];
    const uint32_t world = (uint32_t)it.world;
    const uint32_t world_base = world * (uint32_t)c.grid.cells_w;
    const int yc = it.yz & 0xffff, zc = it.yz >> 16;
    const uint32_t row_base = world_base + (uint32_t)((zc * my + yc) * mx);
    const int x0 = (int)(keys_sorted[it.first] - row_base);
    const int x1 = (int)(keys_sorted[it.first + it.count - 1] - row_base);
    const int hx = (int)(keys_sorted[t] - row_base);
    if (!one_world) {
        for (int e = lane; e < T * T; e += 32) {
            const int a = e / T, b = e - a * T;
            const float F = c.world_force[(size_t)world * kTableSize + a * kTableStride + b];
            const float inv = kUniformR ? c.inv_eff_uniform : s_inv_eff[a * kTableStride + b];
            wcoef[e] = make_float2(c.repulsion * F, c.attraction * F * inv);
        }
        __syncwarp();
    }
    const Tables tb{wcoef, s_c1, s_thr, s_thr_lo, T};
    // x sub-ranges whose union (range plus one cell each side) fits in the box
    const int width = kGeneric ? mx : (mx - 2);
    const int passes = kGeneric ? 1 : (x1 - x0 + width) / width;
    const float thr_f = c.thr_filter;

    for (int pass = 0; pass < passes; pass++) {
        const int px0 = kGeneric ? x0 : x0 + pass * width;
        const int px1 = kGeneric ? x1 : min(x1, px0 + width - 1);
        const bool mine = active && (kGeneric || (hx >= px0 && hx <= px1));
        // generic grids: an idle home sits at -kFar, 2e30 from every candidate and from the
        // +kFar padding slots
        const float hxf = mine ? L.h.x : -kFar, hyf = mine ? L.h.y : -kFar, hzf = mine ? L.h.z : -kFar;

        const int xlo = mx > 1 ? px0 - 1 : 0;
        const int xhi = mx > 1 ? min(px1 + 1, xlo + mx - 1) : 0;  // inclusive, at most mx cells

        // Staging origin per axis (stencil_origin) for the stencil box (cells xlo..xhi,
        // yc-1..yc+1, zc-1..zc+1 in shifted coordinates).  Every staged candidate and the
        // homes lie within (rx, ry, rz) of it, so |c'|, |h'| <= R.  The expanded filter value
        // |c'|^2 + (|h'|^2 - B) - 2 h'.c' carries at most 2^-24 (21 R^2 + 5 B) of rounding
        // (three roundings in each square, one in the constant, four in the chain); the
        // bound B = (thr_f (1 + 2^-18) + 2^-19 R^2)(1 + 2^-18) exceeds thr_f by more, so
        // every pair whose staged d^2 is within thr_f stays negative.
        HomeOps H;
        float ox = 0.0f, oy = 0.0f, oz = 0.0f;
        if (!kGeneric) {
            float rx, ry, rz;
            stencil_origin(xlo, xhi, c.ext[0] / (float)mx, ox, rx);
            stencil_origin(yc - 1, yc + 1, c.ext[1] / (float)my, oy, ry);
            stencil_origin(zc - 1, zc + 1, c.ext[2] / (float)mz, oz, rz);
            const float r2 = fmaf(rz, rz, fmaf(ry, ry, rx * rx));
            const float bnd = (thr_f * (1.0f + 0x1p-18f) + r2 * 0x1p-19f) * (1.0f + 0x1p-18f);
            const float hpx = mine ? L.h.x - ox : 0.0f, hpy = mine ? L.h.y - oy : 0.0f,
                        hpz = mine ? L.h.z - oz : 0.0f;
            const float kk = mine ? fmaf(hpz, hpz, fmaf(hpy, hpy, hpx * hpx)) - bnd : kFar;
            H.m2x = make_float2(-2.0f * hpx, -2.0f * hpx);
            H.m2y = make_float2(-2.0f * hpy, -2.0f * hpy);
            H.m2z = make_float2(-2.0f * hpz, -2.0f * hpz);
            H.k = make_float2(kk, kk);
            if (lane == 0) {
                w.origin[0] = ox;
                w.origin[1] = oy;
                w.origin[2] = oz;
            }
            if constexpr (kBalance || kBal) {
                w.pr.home_h[lane] = L.h;
                w.pr.home_m2[lane] = make_float4(H.m2x.x, H.m2y.x, H.m2z.x, 0.0f);
            }
        } else {
            H.m2x = H.m2y = H.m2z = H.k = make_float2(0.0f, 0.0f);
        }
        // segments: lane 2*row + half describes one contiguous range of the snapshot and
        // its periodic shift less the origin (zero on generic grids)
        int seg_beg = 0, seg_len = 0;
        float seg_sx = 0.0f, seg_sy = 0.0f, seg_sz = 0.0f;
        const int ny = my > 1 ? 3 : 1, nz = mz > 1 ? 3 : 1;
        const int nseg = 2 * ny * nz;
        {
            const int row = lane >> 1, half = lane & 1;
            const int dy_row = ny > 1 ? (row % ny) - 1 : 0, dz_row = nz > 1 ? (row / ny) - 1 : 0;
            const int yy = wrap_index(yc + dy_row, my), zz = wrap_index(zc + dz_row, mz);
            const uint32_t cy = (yc + dy_row < 0) ? 1u : (yc + dy_row >= my ? 2u : 0u);
            const uint32_t cz = (zc + dz_row < 0) ? 1u : (zc + dz_row >= mz ? 2u : 0u);
            // split [xlo, xhi] at the box edge: half 0 is the in-box part, half 1 the wrapped part
            int a = xlo, b = xhi;
            uint32_t cx = 0u;
            if (xlo < 0) {
                if (half == 0) a = 0;
                else { a = xlo + mx; b = mx - 1; cx = 1u; }
            } else if (xhi >= mx) {
                if (half == 0) b = mx - 1;
                else { a = 0; b = xhi - mx; cx = 2u; }
            } else if (half == 1) {
                b = a - 1;
            }
            if (row < ny * nz && b >= a && CF_IN_BOUNDS(world_base + (uint32_t)((zz * my + yy) * mx) + b + 1,
                                                        c.grid.cells + 1)) {
                const uint32_t base = world_base + (uint32_t)((zz * my + yy) * mx);
                seg_beg = (int)cell_off[base + a];
                seg_len = (int)cell_off[base + b + 1] - seg_beg;
                if (!CF_IN_BOUNDS(seg_len, c.n + 1) || !CF_IN_BOUNDS(seg_beg + seg_len, c.n + 1)) seg_len = 0;
                if (!kGeneric) {
                    seg_sx = code_shift(cx, c.ext[0]) - ox;
                    seg_sy = code_shift(cy, c.ext[1]) - oy;
                    seg_sz = code_shift(cz, c.ext[2]) - oz;
                }
            }
        }
        int seg_pre = seg_len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, seg_pre, o);
            if (lane >= o) seg_pre += v;
        }
        const int total = __shfl_sync(0xffffffffu, seg_pre, 31);
        seg_pre -= seg_len;
        // the home's place in the concatenation: its cell is in the centre row's in-box part
        const int seg_c = 2 * ((nz > 1 ? ny : 0) + (ny > 1 ? 1 : 0));
        const int beg_c = __shfl_sync(0xffffffffu, seg_beg, seg_c);
        const int len_c = __shfl_sync(0xffffffffu, seg_len, seg_c);
        const int pre_c = __shfl_sync(0xffffffffu, seg_pre, seg_c);
        const int g_own = (t >= beg_c && t < beg_c + len_c) ? pre_c + (t - beg_c) : -1;

        const int share_lo = (int)((long long)total * part / split);
        const int share_hi = (int)((long long)total * (part + 1) / split);
        for (int base = share_lo; base < share_hi; base += kStage) {
            const int lim = min(kStage, share_hi - base);
            const int ngroups = (lim + 31) >> 5;
            // this lane's own slot in the batch (self exclusion), -1 when elsewhere
            const int own = (g_own >= base && g_own < base + lim) ? g_own - base : -1;
            // ---- stage [base, base + lim) of the concatenated segments: only the segments
            // that overlap it (a warp-uniform ballot over the segment lanes)
            uint32_t overlap = __ballot_sync(0xffffffffu, lane < nseg && seg_len > 0 && seg_pre < base + lim &&
                                                              seg_pre + seg_len > base);
            while (overlap) {
                const int sg = __ffs(overlap) - 1;
                overlap &= overlap - 1u;
                const int pre = __shfl_sync(0xffffffffu, seg_pre, sg);
                const int len = __shfl_sync(0xffffffffu, seg_len, sg);
                const int beg = __shfl_sync(0xffffffffu, seg_beg, sg);
                const float sx = __shfl_sync(0xffffffffu, seg_sx, sg);
                const float sy = __shfl_sync(0xffffffffu, seg_sy, sg);
                const float sz = __shfl_sync(0xffffffffu, seg_sz, sg);
                const int lo = max(pre, base), hi = min(pre + len, base + lim);
                for (int g = lo + lane; g < hi; g += 32) {
                    const int slot = g - base;
                    const int j = beg + (g - pre);
                    const float4 p = CF_IN_BOUNDS(j, c.n) ? pos_sorted[j] : make_float4(kFar, kFar, kFar, 0.0f);
                    float* xy = reinterpret_cast<float*>(&w.xy[slot >> 1]);
                    float* zc = reinterpret_cast<float*>(&w.zc[slot >> 1]);
                    const float x = p.x + sx, y = p.y + sy, z = p.z + sz;
                    xy[slot & 1] = x;
                    xy[2 + (slot & 1)] = y;
                    zc[slot & 1] = z;
                    zc[2 + (slot & 1)] = fmaf(z, z, fmaf(y, y, x * x));
                    w.meta[slot] = (uint32_t)j | ((__float_as_uint(p.w) & (kTableStride - 1)) << kTypeShift);
                }
            }
            // padding up to a whole group: never passes the filter (at +kFar on generic
            // grids, |c|^2 = kFar otherwise)
            for (int slot = lim + lane; slot < ngroups * 32; slot += 32) {
                float* xy = reinterpret_cast<float*>(&w.xy[slot >> 1]);
                float* zc = reinterpret_cast<float*>(&w.zc[slot >> 1]);
                const float far = kGeneric ? kFar : 0.0f;
                xy[slot & 1] = far;
                xy[2 + (slot & 1)] = far;
                zc[slot & 1] = far;
                zc[2 + (slot & 1)] = kFar;
            }
            __syncwarp();
            const int own_g = own >> 5;  // -1 when the home is not in this batch
            const uint32_t own_keep = ~(1u << (own & 31));
            int hits = 0;      // set bits of this lane in the batch
            uint32_t nz = 0u;  // bit g: group g has a set bit

            // ---- filter: one bit per candidate
            if (kGeneric) {
                const float4 hh = make_float4(hxf, hyf, hzf, 0.0f);
                for (int gi = 0; gi < ngroups; gi++) {
                    uint32_t m = 0;
                    for (int q = 0; q < 32; q++) {
                        const int slot = gi * 32 + q;
                        if (slot >= lim) break;
                        float dx, dy, dz;
                        const int pb = (slot >> 1) * 4 + (slot & 1);
                        staged_delta<true>(c, xyf[pb], xyf[pb + 2], zcf[pb], hh, H, dx, dy, dz);
                        const float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
                        if (d2 < thr_f) m |= 1u << q;
                    }
                    const uint32_t mm = gi == own_g ? (m & own_keep) : m;
                    w.mask[gi * 32 + lane] = mm;
                    hits += __popc(mm);
                    nz |= (mm != 0u ? 1u : 0u) << gi;
                }
            } else {
                for (int gi = 0; gi < ngroups; gi++) {
                    // |c'|^2 + (|h'|^2 - bound) - 2 h'.c', two candidates per chain; the sign
                    // bit of each result is shifted into the mask (last pair first, so pair p
                    // lands on bits 2p, 2p + 1)
                    uint32_t m = 0;
#pragma unroll
                    for (int p = 15; p >= 0; p--) {
                        const float4 a = w.xy[gi * 16 + p];
                        const float4 b = w.zc[gi * 16 + p];
                        float2 q = __fadd2_rn(make_float2(b.z, b.w), H.k);
                        q = __ffma2_rn(make_float2(a.x, a.y), H.m2x, q);
                        q = __ffma2_rn(make_float2(a.z, a.w), H.m2y, q);
                        q = __ffma2_rn(make_float2(b.x, b.y), H.m2z, q);
                        m = __funnelshift_l(__float_as_uint(q.y), m, 1);
                        m = __funnelshift_l(__float_as_uint(q.x), m, 1);
                    }
                    const uint32_t mm = gi == own_g ? (m & own_keep) : m;
                    w.mask[gi * 32 + lane] = mm;
                    hits += __popc(mm);
                    nz |= (mm != 0u ? 1u : 0u) << gi;
                }
            }

            // ---- drain: every set bit of this lane in slot order, kPer per trip.  The trip
            // count is uniform over the warp (the largest hit count over kPer), and a lane
            // whose current group mask runs out moves to the next non-empty group (the
            // lowest remaining bit of nz) with one load: no nested loop, no vote per trip.
            // A lane with fewer than kPer hits left repeats its first pair of the trip
            // without accumulating it.
            //
            // Lane pairing (kBalance): the trip count is the busiest lane's, so lanes are
            // paired heaviest with lightest (a bitonic sort of the hit counts) and the light
            // lane of a pair, once its own hits are done (rounded up to a whole trip), takes
            // the top part of its partner's hits with its partner's home, accumulating them
            // apart; the partner adds that partial after the trips.  Each pair's work is then
            // about half its total.
            if constexpr (kBal) {
                // ---- balanced drain: the batch's H hits, home by home in lane order, form a
                // task line; lane l takes tasks [l H / 32, (l + 1) H / 32), walking each home's
                // set bits with that home's position (a new home starts a new trip), and
                // writes the partial sums of each (lane, home) piece to part[lane + rank of
                // the home]; each home then adds its pieces in lane order (deterministic).
                w.pr.nzw[lane] = nz;
                w.pr.hits[lane] = hits;
                int pre = hits;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int v = __shfl_up_sync(0xffffffffu, pre, o);
                    if (lane >= o) pre += v;
                }
                const int H_all = __shfl_sync(0xffffffffu, pre, 31);
                pre -= hits;  // exclusive prefix: where this lane's home starts on the task line
                const uint32_t has = __ballot_sync(0xffffffffu, hits > 0);
                const int t0 = (lane * H_all) >> 5, t1 = ((lane + 1) * H_all) >> 5;
                int left = t1 - t0;
                // the home of task t0: the last home whose start is <= t0 (a home with hits)
                int hm = 0;
#pragma unroll
                for (int step = 16; step >= 1; step >>= 1) {
                    const int cand = hm + step;
                    if (__shfl_sync(0xffffffffu, pre, cand) <= t0) hm = cand;
                }
                const int rank0 = t0 - __shfl_sync(0xffffffffu, pre, hm);
                __syncwarp();
                uint32_t m = 0u;
                int gi = 0, inh = 0;
                if (left > 0) {
                    // skip the first rank0 set bits of home hm
                    int r = rank0;
                    nz = w.pr.nzw[hm];
                    for (;;) {
                        gi = __ffs(nz) - 1;
                        m = w.mask[gi * 32 + hm];
                        const int cnt = __popc(m);
                        if (r < cnt) break;
                        r -= cnt;
                        nz &= nz - 1u;
                    }
                    for (; r > 0; r--) m &= m - 1u;
                    inh = min(left, w.pr.hits[hm] - rank0);
                    const float4 ph = w.pr.home_h[hm];
                    const float4 pm = w.pr.home_m2[hm];
                    L.h = ph;
                    L.tp = __float_as_uint(ph.w) & kTypeMask;
                    H.m2x.x = pm.x;
                    H.m2y.x = pm.y;
                    H.m2z.x = pm.z;
                }
                const bool worked = left > 0;
                // running sums of this lane's own home stay in (sx, sy, sz, sc); L accumulates pieces
                const float sx = L.fx, sy = L.fy, sz = L.fz;
                const int sc = L.count;
                L.fx = L.fy = L.fz = 0.0f;
                L.count = 0;
                while (__any_sync(0xffffffffu, left > 0)) {
                    if (left > 0 && inh == 0) {
                        // this home's tasks are done: its piece goes to part[], the next home starts
                        w.pr.part[lane + __popc(has & ((1u << hm) - 1u))] =
                            make_float4(L.fx, L.fy, L.fz, __int_as_float(L.count));
                        L.fx = L.fy = L.fz = 0.0f;
                        L.count = 0;
                        hm = __ffs(has & (0xfffffffeu << hm)) - 1;
                        nz = w.pr.nzw[hm];
                        gi = __ffs(nz) - 1;
                        m = w.mask[gi * 32 + hm];
                        inh = min(left, w.pr.hits[hm]);
                        const float4 ph = w.pr.home_h[hm];
                        const float4 pm = w.pr.home_m2[hm];
                        L.h = ph;
                        L.tp = __float_as_uint(ph.w) & kTypeMask;
                        H.m2x.x = pm.x;
                        H.m2y.x = pm.y;
                        H.m2z.x = pm.z;
                    }
                    const int nq = min(kPer, inh);
                    int slot[kPer];
                    bool valid[kPer];
#pragma unroll
                    for (int q = 0; q < kPer; q++) {
                        valid[q] = q < nq;
                        if (valid[q] && m == 0u) {
                            nz &= nz - 1u;
                            gi = __ffs(nz) - 1;
                            m = w.mask[gi * 32 + hm];
                        }
                        slot[q] = valid[q] ? gi * 32 + (__ffs(m) - 1) : 0;
                        if (valid[q]) m &= m - 1u;
                    }
                    float dx[kPer], dy[kPer], dz[kPer], d2[kPer], wgt[kPer];
                    uint32_t meta[kPer];
                    bool inter[kPer];
                    // (every lane runs this body in every pass of the loop, so the vote is warp-wide)
                    float sx[kPer], sy[kPer], sz[kPer];
                    bool band = false;
#pragma unroll
                    for (int q = 0; q < kPer; q++) {
                        staged_xyz(xyf, zcf, slot[q], sx[q], sy[q], sz[q]);
                        meta[q] = w.meta[slot[q]];
                        const bool fast = pair_fast<kGeneric, kUniformR>(c, L, H, sx[q], sy[q], sz[q], meta[q], tb,
                                                                        dx[q], dy[q], dz[q], d2[q]);
                        inter[q] = fast && valid[q];
                        band |= valid[q] && !fast;
                    }
                    if (__any_sync(0xffffffffu, band)) {
#pragma unroll
                        for (int q = 0; q < kPer; q++)
                            if (valid[q] && !inter[q])
                                inter[q] = pair_exact<kGeneric, kUniformR>(c, L, w.origin, sx[q], sy[q], sz[q],
                                                                           meta[q], pos_sorted, tb);
                    }
#pragma unroll
                    for (int q = 0; q < kPer; q++) wgt[q] = pair_weight<kUniformR>(d2[q], meta[q], L, tb, c1u);
#pragma unroll
                    for (int q = 0; q < kPer; q++) {
                        if (inter[q]) {
                            L.count++;
                            L.fx = fmaf(dx[q], wgt[q], L.fx);
                            L.fy = fmaf(dy[q], wgt[q], L.fy);
                            L.fz = fmaf(dz[q], wgt[q], L.fz);
                        }
                    }
                    inh -= nq;
                    left -= nq;
                }
                if (worked)
                    w.pr.part[lane + __popc(has & ((1u << hm) - 1u))] =
                        make_float4(L.fx, L.fy, L.fz, __int_as_float(L.count));
                __syncwarp();
                // each home adds its pieces in lane order; back to the lane's own home
                L.fx = sx;
                L.fy = sy;
                L.fz = sz;
                L.count = sc;
                if (hits > 0) {
                    // lanes la..lb hold the home's tasks (those with an empty range, when the
                    // batch has fewer hits than lanes, hold none)
                    const int rk = __popc(has & ((1u << lane) - 1u));
                    const int la = (32 * (pre + 1) - 1) / H_all;
                    const int lb = (32 * (pre + hits) - 1) / H_all;
                    for (int l2 = la; l2 <= lb; l2++) {
                        if (((l2 + 1) * H_all) >> 5 == (l2 * H_all) >> 5) continue;
                        const float4 v = w.pr.part[l2 + rk];
                        L.fx += v.x;
                        L.fy += v.y;
                        L.fz += v.z;
                        L.count += __float_as_int(v.w);
                    }
                }
                const float4 oh = w.pr.home_h[lane];
                const float4 om = w.pr.home_m2[lane];
                L.h = oh;
                L.tp = __float_as_uint(oh.w) & kTypeMask;
                H.m2x.x = om.x;
                H.m2y.x = om.y;
                H.m2z.x = om.z;
            } else {
            int upto = hits;         // pair indices below upto are valid in the current phase
            int work = hits;         // pairs this lane walks in the batch
            int switch_trip = -1;    // trip at which a light lane turns to its partner's hits
            int partner = lane, fw = 0, src = lane;
            bool light = false;
            int fgi = 0;             // where a light lane's share of its partner's hits starts
            uint32_t fm = 0u, fnz = 0u;
            if constexpr (kBalance) {
                uint32_t key = ((uint32_t)hits << 5) | (uint32_t)lane;
#pragma unroll
                for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
                    for (int j = k >> 1; j > 0; j >>= 1) {
                        const uint32_t o = __shfl_xor_sync(0xffffffffu, key, j);
                        key = (((lane & j) == 0) == ((lane & k) == 0)) ? min(key, o) : max(key, o);
                    }
                }
                // sorted position lane holds key; it pairs with position 31 - lane
                const uint32_t mate = __shfl_sync(0xffffffffu, key, 31 - lane);
                w.pr.pairing[key & 31u] = (mate & 31u) | (lane < 16 ? 0x100u : 0u);
                w.pr.nzw[lane] = nz;
                __syncwarp();
                const uint32_t pr = w.pr.pairing[lane];
                partner = (int)(pr & 31u);
                light = (pr & 0x100u) != 0u;
                const int hp = __shfl_sync(0xffffffffu, hits, partner);
                if (light) {
                    const int padded = (hits + kPer - 1) / kPer * kPer;
                    fw = max(0, (hp - padded) >> 1);
                    work = padded + fw;
                    if (fw > 0) {
                        switch_trip = padded / kPer;
                        // skip the partner's own share, its first hp - fw set bits; the group
                        // bitmap keeps the current group as its lowest bit, like nz
                        int skip = hp - fw;
                        fnz = w.pr.nzw[partner];
                        while (fnz) {
                            fgi = __ffs(fnz) - 1;
                            fm = w.mask[fgi * 32 + partner];
                            const int cnt = __popc(fm);
                            if (skip < cnt) break;
                            skip -= cnt;
                            fnz &= fnz - 1u;
                        }
                        for (; skip > 0; skip--) fm &= fm - 1u;
                    }
                } else {
                    fw = max(0, (hits - (hp + kPer - 1) / kPer * kPer) >> 1);
                    upto = work = hits - fw;
                }
            }
            const int trips = (__reduce_max_sync(0xffffffffu, work) + kPer - 1) / kPer;
            int gi = nz ? __ffs(nz) - 1 : 0;
            uint32_t m = w.mask[gi * 32 + lane];
            for (int it = 0; it < trips; it++) {
                if constexpr (kBalance) {
                    if (it == switch_trip) {
                        // own hits done: keep their sums, take the partner's home and its top fw hits
                        w.pr.saved[lane] = make_float4(L.fx, L.fy, L.fz, __int_as_float(L.count));
                        L.fx = L.fy = L.fz = 0.0f;
                        L.count = 0;
                        const float4 ph = w.pr.home_h[partner];
                        const float4 pm = w.pr.home_m2[partner];
                        L.h = ph;
                        L.tp = __float_as_uint(ph.w) & kTypeMask;
                        H.m2x.x = pm.x;
                        H.m2y.x = pm.y;
                        H.m2z.x = pm.z;
                        src = partner;
                        gi = fgi;
                        m = fm;
                        nz = fnz;
                        upto = kPer * it + fw;
                    }
                }
                // every lane runs the trip (a lane whose pairs are done has none valid), so the
                // warp-wide vote below is reached by all 32 lanes in every trip
                {
                    int slot[kPer];
                    bool valid[kPer];
#pragma unroll
                    for (int q = 0; q < kPer; q++) {
                        valid[q] = kPer * it + q < upto;
                        if (valid[q] && m == 0u) {
                            nz &= nz - 1u;
                            gi = __ffs(nz) - 1;  // a later group holds a hit
                            m = w.mask[gi * 32 + src];
                        }
                        slot[q] = valid[q] ? gi * 32 + (__ffs(m) - 1) : (q == 0 ? 0 : slot[0]);
                        if (valid[q]) m &= m - 1u;
                    }
                    float dx[kPer], dy[kPer], dz[kPer], d2[kPer], wgt[kPer];
                    uint32_t meta[kPer];
                    bool inter[kPer];
                    float sx[kPer], sy[kPer], sz[kPer];
                    bool band = false;
#pragma unroll
                    for (int q = 0; q < kPer; q++) {
                        staged_xyz(xyf, zcf, slot[q], sx[q], sy[q], sz[q]);
                        meta[q] = w.meta[slot[q]];
                        const bool fast = pair_fast<kGeneric, kUniformR>(c, L, H, sx[q], sy[q], sz[q], meta[q], tb,
                                                                        dx[q], dy[q], dz[q], d2[q]);
                        inter[q] = fast && valid[q];
                        band |= valid[q] && !fast;
                    }
                    // pairs within rounding of the threshold are rare: the exact test runs only in
                    // the trips where some lane of the warp holds one
                    if (__any_sync(0xffffffffu, band)) {
#pragma unroll
                        for (int q = 0; q < kPer; q++)
                            if (valid[q] && !inter[q])
                                inter[q] = pair_exact<kGeneric, kUniformR>(c, L, w.origin, sx[q], sy[q], sz[q],
                                                                           meta[q], pos_sorted, tb);
                    }
#pragma unroll
                    for (int q = 0; q < kPer; q++) wgt[q] = pair_weight<kUniformR>(d2[q], meta[q], L, tb, c1u);
#pragma unroll
                    for (int q = 0; q < kPer; q++) {
                        if (inter[q]) {
                            L.count++;
                            L.fx = fmaf(dx[q], wgt[q], L.fx);
                            L.fy = fmaf(dy[q], wgt[q], L.fy);
                            L.fz = fmaf(dz[q], wgt[q], L.fz);
                        }
                    }
                }
            }
            if constexpr (kBalance) {
                // a light lane that switched holds its partner's partial: hand it over and
                // take back its own sums and home
                const float px = __shfl_sync(0xffffffffu, L.fx, partner);
                const float py = __shfl_sync(0xffffffffu, L.fy, partner);
                const float pz = __shfl_sync(0xffffffffu, L.fz, partner);
                const int pc = __shfl_sync(0xffffffffu, L.count, partner);
                if (switch_trip >= 0) {
                    const float4 sv = w.pr.saved[lane];
                    L.fx = sv.x;
                    L.fy = sv.y;
                    L.fz = sv.z;
                    L.count = __float_as_int(sv.w);
                    const float4 oh = w.pr.home_h[lane];
                    const float4 om = w.pr.home_m2[lane];
                    L.h = oh;
                    L.tp = __float_as_uint(oh.w) & kTypeMask;
                    H.m2x.x = om.x;
                    H.m2y.x = om.y;
                    H.m2z.x = om.z;
                } else if (!light && fw > 0) {
                    L.fx += px;
                    L.fy += py;
                    L.fz += pz;
                    L.count += pc;
                }
            }
            }
            __syncwarp();
        }
    }
    if (split > 1) {
        // the item's warps meet at a named barrier (id 1 + item slot, 32 * split threads);
        // part 0 adds the partial sums in part order, so the result is deterministic
        if (part != 0) s_part[warp][lane] = make_float4(L.fx, L.fy, L.fz, __int_as_float(L.count));
        item_barrier(warp / split, 32 * split);
        if (part != 0) return;
        for (int q = 1; q < split; q++) {
            const float4 v = s_part[warp + q][lane];
            L.fx += v.x;
            L.fy += v.y;
            L.fz += v.z;
            L.count += __float_as_int(v.w);
        }
    }
    if (!active) return;

    // density-adaptive scale and integrator (ParticleSimulation.cu:136-161)
    const uint32_t i = vals_sorted[t];
    if (!CF_IN_BOUNDS(i, c.n)) return;
    const int prev = counts[i];
    const float avg = __fmul_rn((float)(L.count + prev), 0.5f);
    const float density = fminf(__fdiv_rn(avg, (float)c.max_expected_neighbors), 1.0f);
    const float adapt = __fsub_rn(1.0f, __fmul_rn(__fsub_rn(1.0f, c.balance), density));
    const float scale = __fmul_rn(c.force_multiplier, adapt);
    const float fx = __fmul_rn(L.fx, scale);
    const float fy = __fmul_rn(L.fy, scale);
    const float fz = __fmul_rn(L.fz, scale);
    const float4 v = vel[i];
    const float vx = __fadd_rn(__fmul_rn(v.x, c.friction), __fmul_rn(fx, c.delta_t));
    const float vy = __fadd_rn(__fmul_rn(v.y, c.friction), __fmul_rn(fy, c.delta_t));
    const float vz = __fadd_rn(__fmul_rn(v.z, c.friction), __fmul_rn(fz, c.delta_t));
    float px = __fadd_rn(L.h.x, __fmul_rn(vx, c.delta_t));
    float py = __fadd_rn(L.h.y, __fmul_rn(vy, c.delta_t));
    float pz = __fadd_rn(L.h.z, __fmul_rn(vz, c.delta_t));
    px = wrap_pos(__fadd_rn(px, c.ext[0]), c.ext[0]);
    py = wrap_pos(__fadd_rn(py, c.ext[1]), c.ext[1]);
    pz = wrap_pos(__fadd_rn(pz, c.ext[2]), c.ext[2]);
    pos[i] = make_float4(px, py, pz, L.h.w);
    vel[i] = make_float4(vx, vy, vz, 0.0f);
    acc[i] = make_float4(fx, fy, fz, 0.0f);
    counts[i] = L.count;
}

// The filter's work of one step, from the cell list alone: per item and pass
// the candidates staged (the union of its homes' stencils, as the force
// kernel concatenates them) and the tests of them by the item's particles.
// One thread per item; out[0] += staged, out[1] += staged * particles.
__global__ void __launch_bounds__(256)
    force_work_kernel(StepConsts c, const uint32_t* __restrict__ keys_sorted, const uint32_t* __restrict__ cell_off,
                      const Item* __restrict__ items, const int* __restrict__ n_items,
                      unsigned long long* __restrict__ out)
{
    const int k = blockIdx.x * 256 + threadIdx.x;
    unsigned long long staged = 0, tested = 0;
    if (k < *n_items) {
        const Item it = items[k];
        const int mx = c.grid.m[0], my = c.grid.m[1], mz = c.grid.m[2];
        const uint32_t world_base = (uint32_t)it.world * (uint32_t)c.grid.cells_w;
        const int yc = it.yz & 0xffff, zc = it.yz >> 16;
        const uint32_t row_base = world_base + (uint32_t)((zc * my + yc) * mx);
        const int x0 = (int)(keys_sorted[it.first] - row_base);
        const int x1 = (int)(keys_sorted[it.first + it.count - 1] - row_base);
        const bool generic = c.grid.generic != 0;
        const int width = generic ? mx : (mx - 2);
        const int passes = generic ? 1 : (x1 - x0 + width) / width;
        const int ny = my > 1 ? 3 : 1, nz = mz > 1 ? 3 : 1;
        for (int pass = 0; pass < passes; pass++) {
            const int px0 = generic ? x0 : x0 + pass * width;
            const int px1 = generic ? x1 : min(x1, px0 + width - 1);
            const int xlo = mx > 1 ? px0 - 1 : 0;
            const int xhi = mx > 1 ? min(px1 + 1, xlo + mx - 1) : 0;
            unsigned long long total = 0;
            for (int row = 0; row < ny * nz; row++) {
                const int dy_row = ny > 1 ? (row % ny) - 1 : 0, dz_row = nz > 1 ? (row / ny) - 1 : 0;
                const int yy = wrap_index(yc + dy_row, my), zz = wrap_index(zc + dz_row, mz);
                const uint32_t base = world_base + (uint32_t)((zz * my + yy) * mx);
                for (int half = 0; half < 2; half++) {
                    int a = xlo, b = xhi;
                    if (xlo < 0) {
                        if (half == 0) a = 0;
                        else { a = xlo + mx; b = mx - 1; }
                    } else if (xhi >= mx) {
                        if (half == 0) b = mx - 1;
                        else { a = 0; b = xhi - mx; }
                    } else if (half == 1) {
                        b = a - 1;
                    }
                    if (b >= a) total += cell_off[base + b + 1] - cell_off[base + a];
                }
            }
            // the homes of this pass: those whose cell lies in [px0, px1]
            int homes = 0;
            for (int q = 0; q < it.count; q++) {
                const int hx = (int)(keys_sorted[it.first + q] - row_base);
                homes += (generic || (hx >= px0 && hx <= px1)) ? 1 : 0;
            }
            staged += total;
            tested += total * (unsigned long long)homes;
        }
    }
    // one atomic per warp
    for (int o = 16; o > 0; o >>= 1) {
        staged += __shfl_down_sync(0xffffffffu, staged, o);
        tested += __shfl_down_sync(0xffffffffu, tested, o);
    }
    if ((threadIdx.x & 31) == 0 && (staged | tested)) {
        atomicAdd(&out[0], staged);
        atomicAdd(&out[1], tested);
    }
}

// Items: each row of cells (rows = (y, z) pairs) cut into chunks of at most
// 32 sorted particles.  One block; rows are split into contiguous segments.
__global__ void __launch_bounds__(1024)
    plan_kernel(const uint32_t* __restrict__ cell_off, int mx, int my, int mz, int rows, Item* __restrict__ items,
                int* __restrict__ n_items)
{
    __shared__ uint32_t s_chunk[1024];
    const int tid = threadIdx.x;
    const int per = (rows + 1023) / 1024;
    const int r0 = min(tid * per, rows), r1 = min(r0 + per, rows);
    uint32_t chunks = 0;
    for (int r = r0; r < r1; r++) {
        const uint32_t cnt = cell_off[(r + 1) * mx] - cell_off[r * mx];
        chunks += (cnt + 31u) / 32u;
    }
    s_chunk[tid] = chunks;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const uint32_t b = tid >= o ? s_chunk[tid - o] : 0u;
        __syncthreads();
        s_chunk[tid] += b;
        __syncthreads();
    }
    uint32_t item = s_chunk[tid] - chunks;
    for (int r = r0; r < r1; r++) {
        const uint32_t start = cell_off[r * mx];
        const uint32_t cnt = cell_off[(r + 1) * mx] - start;
        const int yz_w = r / my;
        const int yz = (r - yz_w * my) | ((yz_w % mz) << 16), world = yz_w / mz;
        for (uint32_t k = 0; k < cnt; k += 32u) items[item++] = Item{(int)(start + k), (int)min(32u, cnt - k), yz, world};
    }
    if (tid == 1023) *n_items = (int)s_chunk[1023];
}

template <int S, int B, int P, bool G, bool U>
cudaError_t configure_one()
{
    return cudaFuncSetAttribute(step_force_kernel<S, B, P, G, U>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)((sizeof(WarpSmem<S, P>) + sizeof(float2) * kTableSize) * kWarps));
}

template <int S, int B, int P>
cudaError_t configure_variant()
{
    cudaError_t e = configure_one<S, B, P, false, false>();
    if (e == cudaSuccess) e = configure_one<S, B, P, false, true>();
    if (e == cudaSuccess) e = configure_one<S, B, P, true, false>();
    if (e == cudaSuccess) e = configure_one<S, B, P, true, true>();
    return e;
}

// Variant S = staged candidates per batch, B = resident blocks per SM the
// register budget is sized for, P = lanes paired in the drain.
template <int S, int B, int P>
cudaError_t launch_variant(const StepConsts& c, const PairTables* tables, const float4* pos_sorted,
                           const uint32_t* keys_sorted, const uint32_t* vals_sorted, const uint32_t* cell_off,
                           const Item* items, const int* n_items, int blocks, float4* pos, float4* vel, float4* acc,
                           int* counts, cudaStream_t st)
{
    // staging per warp; force coefficients per block (one world) or per warp (a batch)
    const size_t smem = sizeof(WarpSmem<S, P>) * kWarps +
                        sizeof(float2) * c.num_types * c.num_types * (c.grid.worlds == 1 ? 1 : kWarps);
#define CF_FORCE_LAUNCH(G, U)                                                                                        \
    step_force_kernel<S, B, P, G, U><<<blocks, kThreads, smem, st>>>(c, tables, pos_sorted, keys_sorted, vals_sorted,   \
                                                                  cell_off, items, n_items, pos, vel, acc, counts)
    if (c.grid.generic) {
        if (c.uniform_r)
            CF_FORCE_LAUNCH(true, true);
        else
            CF_FORCE_LAUNCH(true, false);
    } else {
        if (c.uniform_r)
            CF_FORCE_LAUNCH(false, true);
        else
            CF_FORCE_LAUNCH(false, false);
    }
#undef CF_FORCE_LAUNCH
    note_launches(st);
    return cudaGetLastError();
}

}  // namespace

CF_BOUNDS_READER(step)

cudaError_t launch_force_work(const StepConsts& c, const uint32_t* keys_sorted, const uint32_t* cell_off,
                              const Item* items, const int* n_items, int max_items, unsigned long long* out,
                              cudaStream_t st)
{
    cudaError_t e = cudaMemsetAsync(out, 0, 2 * sizeof(unsigned long long), st);
    if (e != cudaSuccess || max_items <= 0) return e;
    force_work_kernel<<<(max_items + 255) / 256, 256, 0, st>>>(c, keys_sorted, cell_off, items, n_items, out);
    note_launches(st);
    return cudaGetLastError();
}

int max_step_items(int n, const Grid& g) { return (n + 31) / 32 + g.worlds * g.m[1] * g.m[2]; }

int step_launches(int n) { return n > 0 ? 1 : 0; }  // the force kernel (the plan is part of the cell list)

cudaError_t launch_step_plan(const uint32_t* cell_off, int n, const Grid& g, Item* items, int* n_items,
                             cudaStream_t st)
{
    if (n <= 0) return cudaMemsetAsync(n_items, 0, sizeof(int), st);
    plan_kernel<<<1, 1024, 0, st>>>(cell_off, g.m[0], g.m[1], g.m[2], g.worlds * g.m[1] * g.m[2], items, n_items);
    note_launches(st);
    return cudaGetLastError();
}

// Opt the force kernels into their dynamic shared memory (outside any
// stream capture).
cudaError_t configure_step_force()
{
    cudaError_t e = configure_variant<256, 8, 0>();
    if (e == cudaSuccess) e = configure_variant<256, 6, 0>();
    if (e == cudaSuccess) e = configure_variant<256, 6, 1>();
    if (e == cudaSuccess) e = configure_variant<384, 6, 0>();
    if (e == cudaSuccess) e = configure_variant<256, 6, 2>();
    return e;
}

cudaError_t launch_step_force(const StepConsts& c, const PairTables* tables, const float4* pos_sorted,
                              const uint32_t* keys_sorted, const uint32_t* vals_sorted, const uint32_t* cell_off,
                              const Item* items, const int* n_items, int max_items, float4* pos, float4* vel,
                              float4* acc, int* counts, cudaStream_t st)
{
    if (c.n <= 0 || max_items <= 0) return cudaSuccess;
    if (c.split != 1 && c.split != 2 && c.split != 4) return cudaErrorInvalidValue;
    const int blocks = (int)(((long long)max_items * c.split + kWarps - 1) / kWarps);
    switch (c.variant) {
    case 1:
        return launch_variant<256, 6, 0>(c, tables, pos_sorted, keys_sorted, vals_sorted, cell_off, items, n_items,
                                      blocks, pos, vel, acc, counts, st);
    case 2:
        return launch_variant<256, 6, 1>(c, tables, pos_sorted, keys_sorted, vals_sorted, cell_off, items, n_items,
                                      blocks, pos, vel, acc, counts, st);
    case 4:
        return launch_variant<256, 6, 2>(c, tables, pos_sorted, keys_sorted, vals_sorted, cell_off, items, n_items,
                                         blocks, pos, vel, acc, counts, st);
    case 3:
        return launch_variant<384, 6, 0>(c, tables, pos_sorted, keys_sorted, vals_sorted, cell_off, items, n_items,
                                      blocks, pos, vel, acc, counts, st);
    default:
        return launch_variant<256, 8, 0>(c, tables, pos_sorted, keys_sorted, vals_sorted, cell_off, items, n_items,
                                      blocks, pos, vel, acc, counts, st);
    }
}

}  // namespace cf
