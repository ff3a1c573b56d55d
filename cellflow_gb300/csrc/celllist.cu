// celllist.cu - uniform-grid cell list: cell hash, stable LSD radix sort,
// cell start/end with the sorted position snapshot, device-wide scan, and
// the work-model counters.
//
// The reference has no spatial structure (its step is O(N^2),
// cuda-native/src/ParticleSimulation.cu:86); this list is what makes a step
// O(N * neighbours).  Its order is fixed: particles sorted by cell id with
// ties in index order, the result a stable sort gives, so the order and every
// per-cell range are reproducible bit for bit.
#include <cuda_runtime.h>

#include <algorithm>

#include "cf_internal.hpp"

namespace cf {
namespace {

constexpr int kThreads = 256;
constexpr int kRadix = 256;
constexpr int kWarps = kThreads / 32;

__device__ __forceinline__ int cell_coord(float x, float inv, int m)
{
    int c = __float2int_rd(__fmul_rn(x, inv));
    return min(max(c, 0), m - 1);
}

// Cell id of every particle; flags positions outside [0, extent) or not
// finite, and types outside [0, T).
__global__ void __launch_bounds__(kThreads)
    cell_hash_kernel(const float4* __restrict__ pos, int n, Grid g, float ex, float ey, float ez, int num_types,
                     uint32_t* __restrict__ keys, int* __restrict__ err)
{
    int i = blockIdx.x * kThreads + threadIdx.x;
    if (i >= n) return;
    float4 p = pos[i];
    bool inside = (p.x >= 0.0f && p.x < ex) && (p.y >= 0.0f && p.y < ey) && (p.z >= 0.0f && p.z < ez);
    if (!inside) atomicOr(err, kDevErrDomain);
    if (__float_as_uint(p.w) >= (uint32_t)num_types) atomicOr(err, kDevErrType);
    int cx = cell_coord(p.x, g.inv[0], g.m[0]);
    int cy = cell_coord(p.y, g.inv[1], g.m[1]);
    int cz = cell_coord(p.z, g.inv[2], g.m[2]);
    keys[i] = (uint32_t)((cz * g.m[1] + cy) * g.m[0] + cx);
}

// Cell id of every particle (world * cells_w + cell) and the population of
// every cell (counts must be zero on entry); flags positions outside the box,
// types outside [0, T) and world indices outside the batch.  With slot, the
// particle's arrival slot in its cell (unordered: it only places the
// particle for the stable ranking that follows).
__global__ void __launch_bounds__(kThreads)
    cell_hash_count_kernel(const float4* __restrict__ pos, int n, Grid g, float ex, float ey, float ez, int num_types,
                           uint32_t* __restrict__ keys, uint32_t* __restrict__ counts, uint32_t* __restrict__ slot,
                           int* __restrict__ err)
{
    int i = blockIdx.x * kThreads + threadIdx.x;
    if (i >= n) return;
    float4 p = pos[i];
    bool inside = (p.x >= 0.0f && p.x < ex) && (p.y >= 0.0f && p.y < ey) && (p.z >= 0.0f && p.z < ez);
    if (!inside) atomicOr(err, kDevErrDomain);
    const uint32_t bits = __float_as_uint(p.w);
    uint32_t world = bits >> kWorldShift;
    if ((bits & kTypeMask) >= (uint32_t)num_types || world >= (uint32_t)g.worlds) atomicOr(err, kDevErrType);
    if (world >= (uint32_t)g.worlds) world = 0;
    int cx = cell_coord(p.x, g.inv[0], g.m[0]);
    int cy = cell_coord(p.y, g.inv[1], g.m[1]);
    int cz = cell_coord(p.z, g.inv[2], g.m[2]);
    const uint32_t key = world * (uint32_t)g.cells_w + (uint32_t)((cz * g.m[1] + cy) * g.m[0] + cx);
    keys[i] = key;
    if (!CF_IN_BOUNDS(key, g.cells)) return;
    const uint32_t s = atomicAdd(&counts[key], 1u);
    if (slot) slot[i] = s;
}

// The position snapshot in sorted (cell) order.
__global__ void __launch_bounds__(kThreads)
    gather_sorted_kernel(const uint32_t* __restrict__ vals, int n, const float4* __restrict__ pos,
                         float4* __restrict__ pos_sorted)
{
    int t = blockIdx.x * kThreads + threadIdx.x;
    if (t < n) pos_sorted[t] = pos[vals[t]];
}

// Digit histogram of one tile of kThreads*ITEMS keys, written digit-major:
// hist[digit * nblocks + block].
template <int ITEMS>
__global__ void __launch_bounds__(kThreads)
    radix_hist_kernel(const uint32_t* __restrict__ keys, int n, int shift, uint32_t* __restrict__ hist, int nblocks)
{
    __shared__ uint32_t h[kRadix];
    h[threadIdx.x] = 0;
    __syncthreads();
    int base = blockIdx.x * (kThreads * ITEMS);
#pragma unroll
    for (int it = 0; it < ITEMS; it++) {
        int i = base + it * kThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & (kRadix - 1)], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter of one tile.  Keys are visited in index order, kThreads at a
// time; within a round a key's rank among equal digits is the count of equal
// digits in lower lanes (__match_any_sync), in lower warps (shared counts),
// and in earlier rounds (running offsets).  vals_in == nullptr means the
// identity permutation (first pass).
template <int ITEMS>
__global__ void __launch_bounds__(kThreads)
    radix_scatter_kernel(const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
                         uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out, int n, int shift,
                         const uint32_t* __restrict__ offsets, int nblocks)
{
    __shared__ uint32_t running[kRadix];
    __shared__ uint32_t warp_cnt[kWarps][kRadix];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    running[tid] = offsets[tid * nblocks + blockIdx.x];
#pragma unroll
    for (int w = 0; w < kWarps; w++) warp_cnt[w][tid] = 0;
    __syncthreads();
    const int base = blockIdx.x * (kThreads * ITEMS);
    for (int it = 0; it < ITEMS; it++) {
        int i = base + it * kThreads + tid;
        bool valid = i < n;
        uint32_t key = valid ? keys_in[i] : 0u;
        uint32_t val = valid ? (vals_in ? vals_in[i] : (uint32_t)i) : 0u;
        uint32_t digit = valid ? ((key >> shift) & (kRadix - 1)) : (uint32_t)(kRadix + lane);
        uint32_t peers = __match_any_sync(0xffffffffu, digit);
        uint32_t lower = peers & ((1u << lane) - 1u);
        if (valid && lower == 0u) warp_cnt[warp][digit] = __popc(peers);
        __syncthreads();
        if (valid) {
            uint32_t dst = running[digit] + __popc(lower);
            for (int w = 0; w < warp; w++) dst += warp_cnt[w][digit];
            keys_out[dst] = key;
            vals_out[dst] = val;
        }
        __syncthreads();
        uint32_t add = 0;
#pragma unroll
        for (int w = 0; w < kWarps; w++) {
            add += warp_cnt[w][tid];
            warp_cnt[w][tid] = 0;
        }
        running[tid] += add;
        __syncthreads();
    }
}

// ---- device-wide exclusive scan (three phases) -----------------------------

constexpr int kScanItems = 8;
constexpr int kScanTile = kThreads * kScanItems;

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total)
{
    __shared__ uint32_t warp_sums[kWarps];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t s = lane < kWarps ? warp_sums[lane] : 0u;
#pragma unroll
        for (int o = 1; o < kWarps; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < kWarps) warp_sums[lane] = s;
    }
    __syncthreads();
    uint32_t before = warp ? warp_sums[warp - 1] : 0u;
    *total = warp_sums[kWarps - 1];
    __syncthreads();
    return before + x - v;
}

__global__ void __launch_bounds__(kThreads) scan_tile_sums(const uint32_t* __restrict__ in, int n, uint32_t* sums)
{
    int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++)
        if (base + k < n) s += in[base + k];
    uint32_t total;
    block_exclusive_scan(s, &total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// Exclusive scan of count values in one block, in place.
__global__ void __launch_bounds__(kThreads) scan_single_block(uint32_t* data, int count)
{
    uint32_t carry = 0;
    for (int base = 0; base < count; base += kScanTile) {
        int idx = base + threadIdx.x * kScanItems;
        uint32_t v[kScanItems];
        uint32_t s = 0;
#pragma unroll
        for (int k = 0; k < kScanItems; k++) {
            v[k] = idx + k < count ? data[idx + k] : 0u;
            s += v[k];
        }
        uint32_t total;
        uint32_t run = carry + block_exclusive_scan(s, &total);
#pragma unroll
        for (int k = 0; k < kScanItems; k++) {
            if (idx + k < count) data[idx + k] = run;
            run += v[k];
        }
        carry += total;
    }
}

__global__ void __launch_bounds__(kThreads)
    scan_apply(const uint32_t* in, uint32_t* out, int n, const uint32_t* __restrict__ sums)
{
    int idx = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        v[k] = idx + k < n ? in[idx + k] : 0u;
        s += v[k];
    }
    uint32_t total;
    uint32_t run = sums[blockIdx.x] + block_exclusive_scan(s, &total);
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        if (idx + k < n) out[idx + k] = run;
        run += v[k];
    }
}

// Cell start/end from the sorted keys, and the snapshot of positions in
// sorted order.  Empty cells keep the 0/0 written before the launch.
__global__ void __launch_bounds__(kThreads)
    cell_bounds_kernel(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ vals, int n,
                       const float4* __restrict__ pos, uint32_t* __restrict__ start, uint32_t* __restrict__ end,
                       float4* __restrict__ pos_sorted)
{
    int t = blockIdx.x * kThreads + threadIdx.x;
    if (t >= n) return;
    uint32_t k = keys[t];
    if (t == 0 || keys[t - 1] != k) start[k] = (uint32_t)t;
    if (t == n - 1 || keys[t + 1] != k) end[k] = (uint32_t)(t + 1);
    pos_sorted[t] = pos[vals[t]];
}

// ---- CSR cell list with the force kernel's plan ------------------------------
//
// After the hash (populations by atomics, each particle's arrival slot):
//   tile_reduce  per tile of whole cell rows: its particles and its items
//                (32-particle chunks of each row, the force kernel's work units)
//   tile_apply   per tile: the totals of the tiles before it (summed by the
//                block, a few hundred values at most), then the tile's CSR
//                offsets and its rows' items
//   place        particle i to offset[cell] + slot (unordered within a cell)
//   rank_gather  the stable position of every particle: its cell's start plus
//                the number of particles of that cell with a smaller index;
//                writes sorted values, keys and the position snapshot
// No kernel waits on another block.

constexpr int kTileThreads = 512;
constexpr int kTileItems = kTileCellsMax / kTileThreads;  // cells (and rows) per thread at most
constexpr int kTileWarps = kTileThreads / 32;
constexpr int kTileTarget = 256;  // tiles a grid is spread over at least, row count permitting

struct TileGeom {
    int m0;             // cells per row
    int m1, m2;         // cells along y and z (a row r is y = r % m1, z = r / m1 % m2, world = r / (m1 m2))
    int rows;           // rows of the whole grid (all worlds)
    int rows_per_tile;  // whole rows per tile (tile_rows): 1 .. floor(kTileCellsMax / m0)
    int tiles;
};

// Exclusive scan of one value per thread over a kTileThreads block.
__device__ __forceinline__ uint32_t tile_block_scan(uint32_t v, uint32_t* total, uint32_t* warp_sums)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t s = lane < kTileWarps ? warp_sums[lane] : 0u;
#pragma unroll
        for (int o = 1; o < kTileWarps; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < kTileWarps) warp_sums[lane] = s;
    }
    __syncthreads();
    const uint32_t before = warp ? warp_sums[warp - 1] : 0u;
    *total = warp_sums[kTileWarps - 1];
    __syncthreads();
    return before + x - v;
}

// The tile's local CSR offsets (s_off[0..tc], s_off[tc] = its particles) and
// each thread's first local item with the tile's item total.
struct TileLocal {
    int c0, tc, r0, nr;   // first cell, cells, first row, rows
    uint32_t particles;   // of the tile
    uint32_t items;       // of the tile
    uint32_t item_before; // local items before this thread's rows
    int rk;               // rows per thread
};

__device__ __forceinline__ TileLocal tile_local(const uint32_t* __restrict__ counts, const TileGeom& tg, int t,
                                                uint32_t* s_off, uint32_t* warp_sums)
{
    TileLocal L;
    L.r0 = t * tg.rows_per_tile;
    L.nr = min(tg.rows_per_tile, tg.rows - L.r0);
    L.c0 = L.r0 * tg.m0;
    L.tc = L.nr * tg.m0;
    const int j0 = threadIdx.x * kTileItems;
    uint32_t v[kTileItems];
    uint32_t sum = 0;
#pragma unroll
    for (int k = 0; k < kTileItems; k++) {
        v[k] = j0 + k < L.tc ? counts[L.c0 + j0 + k] : 0u;
        sum += v[k];
    }
    uint32_t run = tile_block_scan(sum, &L.particles, warp_sums);
#pragma unroll
    for (int k = 0; k < kTileItems; k++) {
        if (j0 + k < L.tc) s_off[j0 + k] = run;
        run += v[k];
    }
    if (threadIdx.x == 0) s_off[L.tc] = L.particles;
    __syncthreads();
    L.rk = (L.nr + kTileThreads - 1) / kTileThreads;
    uint32_t chunks = 0;
    for (int q = 0; q < L.rk; q++) {
        const int r = threadIdx.x * L.rk + q;
        if (r < L.nr) chunks += (s_off[(r + 1) * tg.m0] - s_off[r * tg.m0] + 31u) / 32u;
    }
    L.item_before = tile_block_scan(chunks, &L.items, warp_sums);
    return L;
}

__global__ void __launch_bounds__(kTileThreads)
    tile_reduce_kernel(const uint32_t* __restrict__ counts, TileGeom tg, uint2* __restrict__ tile_sums)
{
    __shared__ uint32_t s_off[kTileCellsMax + 1];
    __shared__ uint32_t warp_sums[kTileWarps];
    const TileLocal L = tile_local(counts, tg, blockIdx.x, s_off, warp_sums);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = make_uint2(L.particles, L.items);
}

__global__ void __launch_bounds__(kTileThreads)
    tile_apply_kernel(uint32_t* cell_off, TileGeom tg, const uint2* __restrict__ tile_sums, Item* __restrict__ items,
                      int* __restrict__ n_items)
{
    __shared__ uint32_t s_off[kTileCellsMax + 1];
    __shared__ uint32_t warp_sums[kTileWarps];
    __shared__ uint32_t s_prefix[2][kTileWarps];
    // totals of the tiles before this one
    uint32_t pp = 0, pi = 0;
    for (int q = threadIdx.x; q < (int)blockIdx.x; q += kTileThreads) {
        const uint2 s = tile_sums[q];
        pp += s.x;
        pi += s.y;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        pp += __shfl_xor_sync(0xffffffffu, pp, o);
        pi += __shfl_xor_sync(0xffffffffu, pi, o);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        s_prefix[0][warp] = pp;
        s_prefix[1][warp] = pi;
    }
    // cell_off holds the populations on entry: this tile reads its own cells
    // (into shared memory) before any block writes offsets over them, and no
    // block reads another tile's cells
    const TileLocal L = tile_local(cell_off, tg, blockIdx.x, s_off, warp_sums);
    uint32_t prefix_p = 0, prefix_i = 0;
#pragma unroll
    for (int w = 0; w < kTileWarps; w++) {
        prefix_p += s_prefix[0][w];
        prefix_i += s_prefix[1][w];
    }
    for (int k = threadIdx.x; k < L.tc; k += kTileThreads) cell_off[L.c0 + k] = prefix_p + s_off[k];
    const bool last = (int)blockIdx.x == tg.tiles - 1;
    if (last && threadIdx.x == 0) cell_off[L.c0 + L.tc] = prefix_p + L.particles;
    if (!items) return;
    uint32_t item = prefix_i + L.item_before;
    for (int q = 0; q < L.rk; q++) {
        const int r = threadIdx.x * L.rk + q;
        if (r >= L.nr) break;
        const uint32_t start = prefix_p + s_off[r * tg.m0];
        const uint32_t cnt = s_off[(r + 1) * tg.m0] - s_off[r * tg.m0];
        const int gr = L.r0 + r, yz_w = gr / tg.m1;
        const int yz = (gr - yz_w * tg.m1) | ((yz_w % tg.m2) << 16), world = yz_w / tg.m2;
        for (uint32_t k = 0; k < cnt; k += 32u) items[item++] = Item{(int)(start + k), (int)min(32u, cnt - k), yz, world};
    }
    if (last && threadIdx.x == 0) *n_items = (int)(prefix_i + L.items);
}

__global__ void __launch_bounds__(kThreads)
    place_kernel(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ slot,
                 const uint32_t* __restrict__ cell_off, int n, int cells, uint32_t* __restrict__ unsorted)
{
    const int i = blockIdx.x * kThreads + threadIdx.x;
    if (i >= n) return;
    const uint32_t key = keys[i];
    if (!CF_IN_BOUNDS(key, cells)) return;
    const uint32_t dst = cell_off[key] + slot[i];
    if (CF_IN_BOUNDS(dst, n)) unsorted[dst] = (uint32_t)i;
}

// Unordered cell list: particle i straight to offset[cell] + arrival slot,
// with its value, key and position (callers that do not depend on the order
// within a cell).
__global__ void __launch_bounds__(kThreads)
    place_gather_kernel(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ slot,
                        const uint32_t* __restrict__ cell_off, const float4* __restrict__ pos, int n, int cells,
                        uint32_t* __restrict__ vals_sorted, uint32_t* __restrict__ keys_sorted,
                        float4* __restrict__ pos_sorted)
{
    const int i = blockIdx.x * kThreads + threadIdx.x;
    if (i >= n) return;
    const uint32_t key = keys[i];
    if (!CF_IN_BOUNDS(key, cells)) return;
    const uint32_t dst = cell_off[key] + slot[i];
    if (!CF_IN_BOUNDS(dst, n)) return;
    vals_sorted[dst] = (uint32_t)i;
    keys_sorted[dst] = key;
    pos_sorted[dst] = pos[i];
}

// Cells of more than this many particles are ranked by the warp-wide method
// below when a warp's 32 positions all lie in one of them.
constexpr uint32_t kRankWarpMin = 64;

__global__ void __launch_bounds__(kThreads)
    rank_gather_kernel(const uint32_t* __restrict__ unsorted, const uint32_t* __restrict__ keys,
                       const uint32_t* __restrict__ cell_off, const float4* __restrict__ pos, int n, int cells,
                       uint32_t* __restrict__ vals_sorted, uint32_t* __restrict__ keys_sorted,
                       float4* __restrict__ pos_sorted)
{
    __shared__ uint32_t s_hist[kWarps][33];
    const int p = blockIdx.x * kThreads + threadIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    bool valid = p < n;
    uint32_t i = valid ? unsorted[p] : 0u;
    valid = valid && CF_IN_BOUNDS(i, n);
    uint32_t key = valid ? keys[i] : 0xffffffffu;
    valid = valid && CF_IN_BOUNDS(key, cells);
    uint32_t b = valid ? cell_off[key] : 0u, e = valid ? cell_off[key + 1] : 0u;
    valid = valid && CF_IN_BOUNDS(e, n + 1) && b <= e;
    if (!valid) key = 0xffffffffu;
    const uint32_t key0 = __shfl_sync(0xffffffffu, key, 0);
    if (__all_sync(0xffffffffu, valid && key == key0) && e - b > kRankWarpMin) {
        // The warp's 32 positions lie in one large cell [b, e).  Sort the warp's own
        // particle indices (bitonic over shuffles: lane j then holds the j-th smallest,
        // s_j).  For every entry x of the cell, c(x) = #{j : s_j <= x} by a binary
        // search over the lanes; x < s_j exactly when c(x) <= j, so the rank of s_j in
        // the cell is the number of entries with c(x) <= j: a histogram of c, summed.
        uint32_t v = i;
#pragma unroll
        for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
            for (int j = k >> 1; j > 0; j >>= 1) {
                const uint32_t o = __shfl_xor_sync(0xffffffffu, v, j);
                v = (((lane & j) == 0) == ((lane & k) == 0)) ? min(v, o) : max(v, o);
            }
        }
        s_hist[warp][lane] = 0u;
        if (lane == 0) s_hist[warp][32] = 0u;
        __syncwarp();
        for (uint32_t q0 = b; q0 < e; q0 += 32u) {
            const uint32_t q = q0 + (uint32_t)lane;
            const uint32_t x = q < e ? unsorted[q] : 0u;
            int c = 0;
#pragma unroll
            for (int step = 16; step >= 1; step >>= 1)
                if (__shfl_sync(0xffffffffu, v, c + step - 1) <= x) c += step;
            if (__shfl_sync(0xffffffffu, v, c) <= x && c == 31) c = 32;  // x >= s_31
            if (q < e) atomicAdd(&s_hist[warp][c], 1u);
        }
        __syncwarp();
        uint32_t rank = s_hist[warp][lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, rank, o);
            if (lane >= o) rank += y;
        }
        i = v;
        const uint32_t dst = b + rank;
        if (!CF_IN_BOUNDS(i, n) || !CF_IN_BOUNDS(dst, n)) return;
        vals_sorted[dst] = i;
        keys_sorted[dst] = key;
        pos_sorted[dst] = pos[i];
        return;
    }
    if (!valid) return;
    uint32_t rank = 0;
    for (uint32_t q = b; q < e; q++) rank += unsorted[q] < i ? 1u : 0u;
    const uint32_t dst = b + rank;
    if (!CF_IN_BOUNDS(dst, n)) return;
    vals_sorted[dst] = i;
    keys_sorted[dst] = key;
    pos_sorted[dst] = pos[i];
}

// ---- work counters ---------------------------------------------------------

// Cell of a particle in the work-model grid of its own world (world-major).
__device__ __forceinline__ uint32_t canon_cell(float4 p, const Grid& g)
{
    int cx = cell_coord(p.x, g.inv[0], g.m[0]);
    int cy = cell_coord(p.y, g.inv[1], g.m[1]);
    int cz = cell_coord(p.z, g.inv[2], g.m[2]);
    uint32_t world = __float_as_uint(p.w) >> kWorldShift;
    if (world >= (uint32_t)g.worlds) world = 0;
    return world * (uint32_t)g.cells_w + (uint32_t)((cz * g.m[1] + cy) * g.m[0] + cx);
}

__global__ void __launch_bounds__(kThreads)
    population_kernel(const float4* __restrict__ pos, int n, Grid g, uint32_t* __restrict__ pop)
{
    int i = blockIdx.x * kThreads + threadIdx.x;
    if (i < n) atomicAdd(&pop[canon_cell(pos[i], g)], 1u);
}

// Distinct stencil coordinates along one periodic axis.
__device__ __forceinline__ int stencil_axis(int c, int m, int* out)
{
    int k = 0;
    for (int o = -1; o <= 1; o++) {
        int v = c + o;
        v = v < 0 ? v + m : (v >= m ? v - m : v);
        bool dup = false;
        for (int q = 0; q < k; q++) dup |= out[q] == v;
        if (!dup) out[k++] = v;
    }
    return k;
}

__global__ void __launch_bounds__(kThreads)
    c27_kernel(const float4* __restrict__ pos, const int* __restrict__ counts, int n, Grid g,
               const uint32_t* __restrict__ pop, unsigned long long* __restrict__ out)
{
    int i = blockIdx.x * kThreads + threadIdx.x;
    unsigned long long cand = 0, inter = 0;
    if (i < n) {
        const uint32_t key = canon_cell(pos[i], g);
        const uint32_t world = key / (uint32_t)g.cells_w;
        const uint32_t c = key - world * (uint32_t)g.cells_w;
        const uint32_t base = world * (uint32_t)g.cells_w;
        int cx = (int)(c % (uint32_t)g.m[0]);
        int cy = (int)((c / (uint32_t)g.m[0]) % (uint32_t)g.m[1]);
        int cz = (int)(c / (uint32_t)(g.m[0] * g.m[1]));
        int ox[3], oy[3], oz[3];
        int nx = stencil_axis(cx, g.m[0], ox), ny = stencil_axis(cy, g.m[1], oy), nz = stencil_axis(cz, g.m[2], oz);
        for (int a = 0; a < nz; a++)
            for (int b = 0; b < ny; b++)
                for (int e = 0; e < nx; e++) cand += pop[base + (oz[a] * g.m[1] + oy[b]) * g.m[0] + ox[e]];
        cand -= 1;
        inter = (unsigned long long)counts[i];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        cand += __shfl_down_sync(0xffffffffu, cand, o);
        inter += __shfl_down_sync(0xffffffffu, inter, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&out[0], cand);
        atomicAdd(&out[1], inter);
    }
}

inline int blocks_for(int n, int per_block) { return (n + per_block - 1) / per_block; }

constexpr int kSortItemsSmall = 4;
constexpr int kSortItemsLarge = 16;

inline int sort_items(int n) { return n <= (1 << 18) ? kSortItemsSmall : kSortItemsLarge; }

}  // namespace

CF_BOUNDS_READER(celllist)

size_t radix_hist_entries(int n)
{
    int items = sort_items(n);
    size_t nblocks = (size_t)blocks_for(n > 0 ? n : 1, kThreads * items);
    return nblocks * kRadix;
}

size_t scan_tmp_entries(int n) { return (size_t)blocks_for(n > 0 ? n : 1, kScanTile) + 1; }

// Kernel launches of one cell-list build: hash, per radix pass histogram +
// scan (1 or 3 kernels) + scatter, and start/end.
int cell_list_launches(int n, int key_bits)
{
    if (n <= 0) return 0;
    int passes = (key_bits + 7) / 8;
    if (passes < 1) passes = 1;
    int entries = (int)radix_hist_entries(n);
    int scan = blocks_for(entries, kScanTile) == 1 ? 1 : 3;
    return 1 + passes * (2 + scan) + 1;
}

cudaError_t launch_cell_hash(const float4* pos, int n, const Grid& g, const float* ext, int num_types,
                             uint32_t* keys, int* err, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    cell_hash_kernel<<<blocks_for(n, kThreads), kThreads, 0, st>>>(pos, n, g, ext[0], ext[1], ext[2], num_types,
                                                                  keys, err);
    note_launches(st);
    return cudaGetLastError();
}

cudaError_t launch_scan_exclusive(const uint32_t* in, uint32_t* out, int n, uint32_t* tmp, size_t tmp_cap,
                                  cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    int tiles = blocks_for(n, kScanTile);
    if ((size_t)tiles > tmp_cap) return cudaErrorInvalidValue;
    if (tiles == 1) {
        if (in != out) {
            cudaError_t e = cudaMemcpyAsync(out, in, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, st);
            if (e != cudaSuccess) return e;
        }
        scan_single_block<<<1, kThreads, 0, st>>>(out, n);
        note_launches(st);
        return cudaGetLastError();
    }
    scan_tile_sums<<<tiles, kThreads, 0, st>>>(in, n, tmp);
    note_launches(st);
    scan_single_block<<<1, kThreads, 0, st>>>(tmp, tiles);
    note_launches(st);
    scan_apply<<<tiles, kThreads, 0, st>>>(in, out, n, tmp);
    note_launches(st);
    return cudaGetLastError();
}

cudaError_t launch_radix_sort(Scratch& s, int n, int key_bits, int* which, cudaStream_t st)
{
    *which = 0;
    if (n <= 0) return cudaSuccess;
    int items = sort_items(n);
    int nblocks = blocks_for(n, kThreads * items);
    int passes = (key_bits + 7) / 8;
    if (passes < 1) passes = 1;
    size_t entries = (size_t)nblocks * kRadix;
    if (entries > s.hist_cap) return cudaErrorInvalidValue;
    int cur = 0;
    for (int p = 0; p < passes; p++) {
        int shift = 8 * p;
        const uint32_t* vals_in = p == 0 ? nullptr : s.vals[cur];
        if (items == kSortItemsSmall) {
            radix_hist_kernel<kSortItemsSmall><<<nblocks, kThreads, 0, st>>>(s.keys[cur], n, shift, s.hist, nblocks);
            note_launches(st);
        } else {
            radix_hist_kernel<kSortItemsLarge><<<nblocks, kThreads, 0, st>>>(s.keys[cur], n, shift, s.hist, nblocks);
            note_launches(st);
        }
        cudaError_t e = launch_scan_exclusive(s.hist, s.hist, (int)entries, s.scan_tmp, s.scan_tmp_cap, st);
        if (e != cudaSuccess) return e;
        if (items == kSortItemsSmall) {
            radix_scatter_kernel<kSortItemsSmall><<<nblocks, kThreads, 0, st>>>(
                s.keys[cur], vals_in, s.keys[cur ^ 1], s.vals[cur ^ 1], n, shift, s.hist, nblocks);
            note_launches(st);
        } else {
            radix_scatter_kernel<kSortItemsLarge><<<nblocks, kThreads, 0, st>>>(
                s.keys[cur], vals_in, s.keys[cur ^ 1], s.vals[cur ^ 1], n, shift, s.hist, nblocks);
            note_launches(st);
        }
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        cur ^= 1;
    }
    *which = cur;
    return cudaSuccess;
}

cudaError_t launch_cell_bounds(const uint32_t* keys, const uint32_t* vals, int n, const float4* pos, uint32_t* start,
                               uint32_t* end, int cells, float4* pos_sorted, cudaStream_t st)
{
    cudaError_t e = cudaMemsetAsync(start, 0, sizeof(uint32_t) * (size_t)cells, st);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(end, 0, sizeof(uint32_t) * (size_t)cells, st);
    if (e != cudaSuccess) return e;
    if (n <= 0) return cudaSuccess;
    cell_bounds_kernel<<<blocks_for(n, kThreads), kThreads, 0, st>>>(keys, vals, n, pos, start, end, pos_sorted);
    note_launches(st);
    return cudaGetLastError();
}

// Cell list in CSR form for the step: keys[0] = cell ids, radix-sorted
// (keys, vals)[*which], cell_off[c] = particles in cells < c (cells + 1
// entries), pos_sorted = positions in sorted order.
// Whole rows per tile: as many as fit in kTileCellsMax cells, fewer when that
// would leave under kTileTarget tiles (small grids: more blocks, shorter scans).
int tile_rows(const Grid& g)
{
    const int rows = g.cells / g.m[0];
    const int fit = kTileCellsMax / g.m[0];
    const int spread = (rows + kTileTarget - 1) / kTileTarget;
    return std::max(1, std::min(fit, spread));
}

int cell_list_tiles(const Grid& g)
{
    if (g.m[0] > kTileCellsMax) return 0;
    const int rows = g.cells / g.m[0];
    const int per = tile_rows(g);
    return (rows + per - 1) / per;
}

cudaError_t launch_cell_list_csr(const float4* pos, int n, const Grid& g, const float* ext, int num_types,
                                 Scratch& s, uint32_t* cell_off, Item* items, int* n_items, int* err, int* which,
                                 cudaStream_t st, bool stable)
{
    cudaError_t e = cudaMemsetAsync(cell_off, 0, sizeof(uint32_t) * ((size_t)g.cells + 1), st);
    if (e != cudaSuccess) return e;
    const int tiles = cell_list_tiles(g);
    if (n > 0) {
        cell_hash_count_kernel<<<blocks_for(n, kThreads), kThreads, 0, st>>>(
            pos, n, g, ext[0], ext[1], ext[2], num_types, s.keys[0], cell_off, tiles ? s.aux : nullptr, err);
        note_launches(st);
    }
    if (!tiles) {
        // rows longer than a tile: stable radix sort of the cell ids, device-wide scan
        e = launch_radix_sort(s, n, g.key_bits, which, st);
        if (e == cudaSuccess) e = launch_scan_exclusive(cell_off, cell_off, g.cells + 1, s.scan_tmp, s.scan_tmp_cap, st);
        if (e == cudaSuccess && n > 0) {
            gather_sorted_kernel<<<blocks_for(n, kThreads), kThreads, 0, st>>>(s.vals[*which], n, pos, s.pos_sorted);
            note_launches(st);
        }
        if (e == cudaSuccess && items) e = launch_step_plan(cell_off, n, g, items, n_items, st);
        return e == cudaSuccess ? cudaGetLastError() : e;
    }
    TileGeom tg;
    tg.m0 = g.m[0];
    tg.m1 = g.m[1];
    tg.m2 = g.m[2];
    tg.rows = g.cells / g.m[0];
    tg.rows_per_tile = tile_rows(g);
    tg.tiles = tiles;
    tile_reduce_kernel<<<tiles, kTileThreads, 0, st>>>(cell_off, tg, s.tile_sums);
    note_launches(st);
    tile_apply_kernel<<<tiles, kTileThreads, 0, st>>>(cell_off, tg, s.tile_sums, items, n_items);
    note_launches(st);
    *which = 1;
    if (n > 0 && !stable) {
        place_gather_kernel<<<blocks_for(n, kThreads), kThreads, 0, st>>>(s.keys[0], s.aux, cell_off, pos, n, g.cells,
                                                                          s.vals[1], s.keys[1], s.pos_sorted);
        note_launches(st);
    } else if (n > 0) {
        place_kernel<<<blocks_for(n, kThreads), kThreads, 0, st>>>(s.keys[0], s.aux, cell_off, n, g.cells, s.vals[0]);
        note_launches(st);
        rank_gather_kernel<<<blocks_for(n, kThreads), kThreads, 0, st>>>(s.vals[0], s.keys[0], cell_off, pos, n,
                                                                         g.cells, s.vals[1], s.keys[1], s.pos_sorted);
        note_launches(st);
    }
    return cudaGetLastError();
}

// The buffer of the scratch pair (keys, vals)[k] that launch_cell_list_csr
// leaves the sorted order in: a function of the grid and the count alone.
int cell_list_csr_buffer(int n, const Grid& g)
{
    if (cell_list_tiles(g) != 0) return 1;
    if (n <= 0) return 0;
    const int passes = std::max(1, (g.key_bits + 7) / 8);
    return passes & 1;
}

int cell_list_csr_launches(int n, const Grid& g, bool with_plan)
{
    if (cell_list_tiles(g) == 0) {
        if (n <= 0) return with_plan ? 0 : 0;
        int passes = (g.key_bits + 7) / 8;
        if (passes < 1) passes = 1;
        int entries = (int)radix_hist_entries(n);
        int scan = blocks_for(entries, kScanTile) == 1 ? 1 : 3;
        int cscan = blocks_for(g.cells + 1, kScanTile) == 1 ? 1 : 3;
        return 1 + passes * (2 + scan) + cscan + 1 + (with_plan ? 1 : 0);
    }
    return 2 + (n > 0 ? 3 : 0);  // tile reduce and apply; hash, place, rank
}

cudaError_t launch_work_counters(const float4* pos, const int* counts, int n, const Grid& canon, uint32_t* pop,
                                 unsigned long long* out, cudaStream_t st)
{
    cudaError_t e = cudaMemsetAsync(pop, 0, sizeof(uint32_t) * (size_t)canon.cells, st);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(out, 0, 2 * sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    if (n <= 0) return cudaSuccess;
    population_kernel<<<blocks_for(n, kThreads), kThreads, 0, st>>>(pos, n, canon, pop);
    note_launches(st);
    c27_kernel<<<blocks_for(n, kThreads), kThreads, 0, st>>>(pos, counts, n, canon, pop, out);
    note_launches(st);
    return cudaGetLastError();
}

}  // namespace cf
