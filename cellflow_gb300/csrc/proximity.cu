// proximity.cu - proximity-graph edges on the cell list.
//
// The reference kernel (cuda-native/src/ParticleSimulation.cu:188-277) scans
// j = i+1 .. N-1 in index order, keeps same-type particles with non-periodic
// squared distance below distance^2 until it holds 2*maxConn of them
// (:215), insertion-sorts them by squared distance (:235-243, stable) and
// emits the first maxConn (:246-275) through an atomicAdd offset (:250).
//
// Here each particle scans only the cells within the distance and keeps the
// 2*maxConn smallest qualifying indices, which is the same candidate set;
// the same stable sort by squared distance then picks the same edges.  For
// the edge list, edges are placed by an exclusive scan of per-particle counts,
// so its order is deterministic: by i, then by distance.  The line vertices
// are written by the selection pass itself at places reserved by one atomic
// per particle: arbitrary order, as the reference's append.
#include <cuda_runtime.h>

#include "cf_internal.hpp"

namespace cf {
namespace {

constexpr int kThreads = 128;
constexpr int kMaxHeld = 2 * CF_MAX_PROX_CONN;

// A particle's cell along one axis, computed from its position exactly as the
// cell list's hash computed it (three multiplies instead of dividing the cell
// id back into coordinates).
__device__ __forceinline__ int axis_cell(float x, float inv, int m)
{
    const int c = __float2int_rd(__fmul_rn(x, inv));
    return min(max(c, 0), m - 1);
}

// Calls fn(u) for every sorted slot u in the cells within one cell of (cx, cy,
// cz), clipped at the box (the proximity grid is not periodic), in cell order.
// kCsr: cell_start = CSR offsets, cell_end = offsets + 1, so each of the
// (at most) nine rows of the stencil is one contiguous range, read up front;
// otherwise per-cell start/end arrays (zeros for empty cells).
template <bool kCsr, typename Fn>
__device__ __forceinline__ void for_each_candidate(const uint32_t* __restrict__ cell_start,
                                                   const uint32_t* __restrict__ cell_end, const Grid& g, int cx,
                                                   int cy, int cz, Fn fn)
{
    const int mx = g.m[0], my = g.m[1], mz = g.m[2];
    const int xlo = max(cx - 1, 0), xhi = min(cx + 1, mx - 1);
    if (kCsr) {
        uint32_t rb[9], re[9];
        int nr = 0;
        for (int z = max(cz - 1, 0); z <= min(cz + 1, mz - 1); z++)
            for (int y = max(cy - 1, 0); y <= min(cy + 1, my - 1); y++) {
                const uint32_t row = (uint32_t)((z * my + y) * mx);
                rb[nr] = cell_start[row + xlo];
                re[nr] = cell_end[row + xhi];
                nr++;
            }
        for (int r = 0; r < nr; r++)
            for (uint32_t u = rb[r]; u < re[r]; u++) fn(u);
    } else {
        for (int z = max(cz - 1, 0); z <= min(cz + 1, mz - 1); z++)
            for (int y = max(cy - 1, 0); y <= min(cy + 1, my - 1); y++)
                for (int x = xlo; x <= xhi; x++) {
                    const uint32_t cell = (uint32_t)((z * my + y) * mx + x);
                    const uint32_t u_end = cell_end[cell];
                    for (uint32_t u = cell_start[cell]; u < u_end; u++) fn(u);
                }
    }
}

template <bool kCsr>
__global__ void __launch_bounds__(kThreads)
    proximity_select_kernel(const float4* __restrict__ pos_sorted, const uint32_t* __restrict__ keys_sorted,
                            const uint32_t* __restrict__ vals_sorted, const uint32_t* __restrict__ cell_start,
                            const uint32_t* __restrict__ cell_end, Grid g, int n, float dsq, int max_conn,
                            int32_t* __restrict__ slots, uint32_t* __restrict__ count)
{
    const int t = blockIdx.x * kThreads + threadIdx.x;
    if (t >= n) return;
    const float4 h = pos_sorted[t];
    const uint32_t i = vals_sorted[t];
    const int mx = g.m[0], my = g.m[1], mz = g.m[2];
    const int cx = axis_cell(h.x, g.inv[0], mx);
    const int cy = axis_cell(h.y, g.inv[1], my);
    const int cz = axis_cell(h.z, g.inv[2], mz);
    const int cap = 2 * max_conn;
    if (cap <= 0) {
        count[i] = 0;
        return;
    }

    int held = 0;
    int hj[kMaxHeld];
    float hd[kMaxHeld];
    for_each_candidate<kCsr>(cell_start, cell_end, g, cx, cy, cz, [&](uint32_t u) {
        const float4 q = pos_sorted[u];
        if (__float_as_uint(q.w) != __float_as_uint(h.w)) return;
        const int j = (int)vals_sorted[u];
        if (j <= (int)i) return;
        if (held == cap && j >= hj[cap - 1]) return;
        const float dx = __fsub_rn(q.x, h.x);
        const float dy = __fsub_rn(q.y, h.y);
        const float dz = __fsub_rn(q.z, h.z);
        const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
        if (!(d2 < dsq)) return;
        // insert into the index-ordered set, dropping the largest when full
        int p = held < cap ? held : cap - 1;
        while (p > 0 && hj[p - 1] > j) {
            hj[p] = hj[p - 1];
            hd[p] = hd[p - 1];
            p--;
        }
        hj[p] = j;
        hd[p] = d2;
        if (held < cap) held++;
    });
    // stable insertion sort by squared distance (ParticleSimulation.cu:235-243)
    for (int a = 1; a < held; a++) {
        const float kd = hd[a];
        const int kj = hj[a];
        int b = a - 1;
        while (b >= 0 && hd[b] > kd) {
            hd[b + 1] = hd[b];
            hj[b + 1] = hj[b];
            b--;
        }
        hd[b + 1] = kd;
        hj[b + 1] = kj;
    }
    const int emit = held < max_conn ? held : max_conn;
    for (int e = 0; e < emit; e++) slots[(size_t)i * CF_MAX_PROX_CONN + e] = hj[e];
    count[i] = (uint32_t)emit;
}

// The CSR cell list's selection with one warp per particle (grid-stride): the
// warp stages the particle's clipped stencil (at most nine rows, one contiguous
// range each, one lane per row, concatenated by a prefix sum) as a list of
// sorted slots and its lanes test 32 candidates at a time.  Qualifying
// candidates join the held set one at a time in ballot order; the set lives in
// lanes 0 .. held-1, ordered by index, and keeps the 2*maxConn smallest indices,
// as the per-thread kernel does.  The final order is the stable sort by squared
// distance of that index-ordered set, i.e. by (distance, index): each held lane
// counts the entries before it.
constexpr int kSelWarps = kThreads / 32;
constexpr int kSelListCap = 256;

// kEmit: instead of the per-particle slots and counts, each particle's warp
// reserves its edges' places with one atomic on *count (the running total) and
// writes their line vertices itself (ParticleSimulation.cu:253-275: per edge the
// vertex of i then of j, each x, y, z, r, g, b with the colour of i's type).
template <bool kEmit>
__global__ void __launch_bounds__(kThreads)
    proximity_select_warp_kernel(const float4* __restrict__ pos_sorted, const uint32_t* __restrict__ keys_sorted,
                                 const uint32_t* __restrict__ vals_sorted, const uint32_t* __restrict__ cell_off,
                                 Grid g, int n, float dsq, int max_conn, int32_t* __restrict__ slots,
                                 uint32_t* __restrict__ count, const float4* __restrict__ pos, ColorTable colors,
                                 int n_colors, float* __restrict__ vertices, int cap_vertices)
{
    __shared__ uint32_t s_list[kSelWarps][kSelListCap];
    const int lane = threadIdx.x & 31;
    uint32_t* list = s_list[threadIdx.x >> 5];
    const int warps = (int)gridDim.x * kSelWarps;
    const int mx = g.m[0], my = g.m[1], mz = g.m[2];
    const int cap = 2 * max_conn;
    for (int t = (int)blockIdx.x * kSelWarps + (threadIdx.x >> 5); t < n; t += warps) {
        const float4 h = pos_sorted[t];
        const uint32_t i = vals_sorted[t];
        const uint32_t key = keys_sorted[t];
        if (!CF_IN_BOUNDS(i, n) || !CF_IN_BOUNDS(key, g.cells)) continue;  // (bounds-checked build)
        if (cap <= 0) {
            if (!kEmit && lane == 0) count[i] = 0;
            continue;
        }
        const int cx = axis_cell(h.x, g.inv[0], mx);
        const int cy = axis_cell(h.y, g.inv[1], my);
        const int cz = axis_cell(h.z, g.inv[2], mz);
        const int xlo = max(cx - 1, 0), xhi = min(cx + 1, mx - 1);
        const int ylo = max(cy - 1, 0), yhi = min(cy + 1, my - 1);
        const int zlo = max(cz - 1, 0), zhi = min(cz + 1, mz - 1);
        const int ny = yhi - ylo + 1, nrows = ny * (zhi - zlo + 1);
        uint32_t beg = 0u;
        int len = 0;
        if (lane < nrows) {
            // lane / ny for lane < 9 and ny in {1, 2, 3} without a division: (lane * 11) >> 5 = lane / 3
            const int zq = ny == 3 ? (lane * 11) >> 5 : (ny == 2 ? lane >> 1 : lane);
            const int y = ylo + (lane - zq * ny), z = zlo + zq;
            const uint32_t row = (uint32_t)((z * my + y) * mx);
            beg = cell_off[row + xlo];
            len = (int)(cell_off[row + xhi + 1] - beg);
            if (!CF_IN_BOUNDS(len, n + 1) || !CF_IN_BOUNDS(beg + len, n + 1)) len = 0;
        }
        int incl = len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        const int pre = incl - len;
        int held = 0;
        int hj = 0;
        float hd = 0.0f;
        for (int base = 0; base < total; base += kSelListCap) {
            const int j0 = max(0, base - pre), j1 = min(len, base + kSelListCap - pre);
            for (int j = j0; j < j1; j++) list[pre + j - base] = beg + (uint32_t)j;
            __syncwarp();
            const int lim = min(kSelListCap, total - base);
            for (int g0 = 0; g0 < lim; g0 += 32) {
                const int gg = g0 + lane;
                bool ok = false;
                int cj = 0;
                float cd = 0.0f;
                if (gg < lim && CF_IN_BOUNDS(list[gg], n)) {
                    const uint32_t u = list[gg];
                    const float4 q = pos_sorted[u];
                    if (__float_as_uint(q.w) == __float_as_uint(h.w)) {
                        cj = (int)vals_sorted[u];
                        if (cj > (int)i) {
                            const float dx = __fsub_rn(q.x, h.x);
                            const float dy = __fsub_rn(q.y, h.y);
                            const float dz = __fsub_rn(q.z, h.z);
                            cd = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
                            ok = cd < dsq;
                        }
                    }
                }
                uint32_t qm = __ballot_sync(0xffffffffu, ok);
                while (qm) {
                    const int src = __ffs(qm) - 1;
                    qm &= qm - 1u;
                    const int j = __shfl_sync(0xffffffffu, cj, src);
                    const float d2 = __shfl_sync(0xffffffffu, cd, src);
                    // its place in the index-ordered set; past the end of a full set it is dropped
                    const int pos = __popc(__ballot_sync(0xffffffffu, lane < held && hj < j));
                    if (pos >= cap) continue;
                    const int uj = __shfl_up_sync(0xffffffffu, hj, 1);
                    const float ud = __shfl_up_sync(0xffffffffu, hd, 1);
                    if (lane > pos && lane < cap) {
                        hj = uj;
                        hd = ud;
                    }
                    if (lane == pos) {
                        hj = j;
                        hd = d2;
                    }
                    held = min(held + 1, cap);
                }
            }
            __syncwarp();
        }
        // stable sort by squared distance (ParticleSimulation.cu:235-243): rank by (distance, index)
        int rank = 0;
        for (int r = 0; r < held; r++) {
            const float od = __shfl_sync(0xffffffffu, hd, r);
            const int oj = __shfl_sync(0xffffffffu, hj, r);
            rank += (od < hd || (od == hd && oj < hj)) ? 1 : 0;
        }
        const int emit = min(held, max_conn);
        if constexpr (kEmit) {
            uint32_t base = 0u;
            if (lane == 0 && emit > 0) base = atomicAdd(count, (uint32_t)emit);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (lane < held && rank < emit && CF_IN_BOUNDS(hj, n)) {
                const size_t k = (size_t)base + (size_t)rank;
                if (2 * k + 1 < (size_t)cap_vertices) {
                    // ParticleSimulation.cu:253-275: i then j, each x, y, z, r, g, b with i's colour
                    const float4 q = pos[hj];
                    const uint32_t c = (__float_as_uint(h.w) & kTypeMask) % (uint32_t)n_colors;
                    const float r = colors.c[3 * c], gg = colors.c[3 * c + 1], b = colors.c[3 * c + 2];
                    float* v = vertices + k * 12;
                    v[0] = h.x; v[1] = h.y; v[2] = h.z; v[3] = r; v[4] = gg; v[5] = b;
                    v[6] = q.x; v[7] = q.y; v[8] = q.z; v[9] = r; v[10] = gg; v[11] = b;
                }
            }
        } else {
            if (lane < held && rank < emit) slots[(size_t)i * CF_MAX_PROX_CONN + rank] = hj;
            if (lane == 0) count[i] = (uint32_t)emit;
        }
    }
}

__global__ void __launch_bounds__(256)
    proximity_edges_kernel(const int32_t* __restrict__ slots, const uint32_t* __restrict__ offsets, int n,
                           int32_t* __restrict__ edges, int cap)
{
    const int i = blockIdx.x * 256 + threadIdx.x;
    if (i >= n) return;
    const uint32_t o = offsets[i], e_count = offsets[i + 1] - o;
    for (uint32_t e = 0; e < e_count; e++) {
        const uint32_t k = o + e;
        if (k < (uint32_t)cap) {
            edges[2 * (size_t)k] = i;
            edges[2 * (size_t)k + 1] = slots[(size_t)i * CF_MAX_PROX_CONN + e];
        }
    }
}

// ---- triangle mesh (ParticleSimulation.cu:280-424) ----------------------------
//
// The reference scans j != i in index order and keeps the first
// min(maxConn, 32) same-type particles with non-periodic squared distance
// below distance^2 * 1.2^2 (the host wrapper's hysteresis, :723-724); every
// pair of them whose indices both exceed i is a triangle (i, a, b), at most 64
// per particle, in pair order (:333-349).  Here each particle keeps the
// min(maxConn, 32) smallest qualifying indices over the cells within range
// (the same list), counts its triangles, and an exclusive scan places them:
// output in i order, then pair order.

constexpr int kMeshHeld = CF_MESH_MAX_CONN;
constexpr int kMeshMaxTriangles = 64;

__global__ void __launch_bounds__(kThreads)
    mesh_select_kernel(const float4* __restrict__ pos_sorted, const uint32_t* __restrict__ keys_sorted,
                       const uint32_t* __restrict__ vals_sorted, const uint32_t* __restrict__ cell_start,
                       const uint32_t* __restrict__ cell_end, Grid g, int n, float dsq, int max_conn,
                       int32_t* __restrict__ slots, uint32_t* __restrict__ count)
{
    const int t = blockIdx.x * kThreads + threadIdx.x;
    if (t >= n) return;
    const float4 h = pos_sorted[t];
    const uint32_t i = vals_sorted[t];
    const int mx = g.m[0], my = g.m[1], mz = g.m[2];
    const int cx = axis_cell(h.x, g.inv[0], mx);
    const int cy = axis_cell(h.y, g.inv[1], my);
    const int cz = axis_cell(h.z, g.inv[2], mz);
    const int cap = min(max_conn, kMeshHeld);
    int held = 0;
    int hj[kMeshHeld];
    if (cap > 0) {
        for_each_candidate<true>(cell_start, cell_end, g, cx, cy, cz, [&](uint32_t u) {
            const float4 q = pos_sorted[u];
            if (__float_as_uint(q.w) != __float_as_uint(h.w)) return;
            const int j = (int)vals_sorted[u];
            if (j == (int)i) return;
            if (held == cap && j >= hj[cap - 1]) return;
            // ParticleSimulation.cu:314-317, rounded on its own in source order
            const float dx = __fsub_rn(q.x, h.x);
            const float dy = __fsub_rn(q.y, h.y);
            const float dz = __fsub_rn(q.z, h.z);
            const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
            if (!(d2 < dsq)) return;
            int p = held < cap ? held : cap - 1;
            while (p > 0 && hj[p - 1] > j) {
                hj[p] = hj[p - 1];
                p--;
            }
            hj[p] = j;
            if (held < cap) held++;
        });
    }
    // the held list is in index order: the ones above i form its tail
    int above = 0;
    for (int e = 0; e < held; e++) {
        slots[(size_t)i * kMeshHeld + e] = hj[e];
        above += hj[e] > (int)i ? 1 : 0;
    }
    if (held < kMeshHeld) slots[(size_t)i * kMeshHeld + held] = -1;
    count[i] = (uint32_t)min(above * (above - 1) / 2, kMeshMaxTriangles);
}

// Triangles of particle i in the reference's pair order, placed at offsets[i];
// index triples and / or vertices of 9 floats (position, flat normal, colour).
__global__ void __launch_bounds__(256)
    mesh_emit_kernel(const int32_t* __restrict__ slots, const uint32_t* __restrict__ offsets, int n,
                     const float4* __restrict__ pos, ColorTable colors, int n_colors,
                     int32_t* __restrict__ tris, float* __restrict__ vertices, long long cap_tris)
{
    const int i = blockIdx.x * 256 + threadIdx.x;
    if (i >= n) return;
    const uint32_t o = offsets[i], total = offsets[i + 1] - o;
    if (total == 0) return;
    int list[kMeshHeld];
    int m = 0;
    for (int e = 0; e < kMeshHeld; e++) {
        const int j = slots[(size_t)i * kMeshHeld + e];
        if (j < 0) break;
        if (j > i) list[m++] = j;
    }
    const float4 v1 = pos[i];
    float cr = 0.0f, cg = 0.0f, cb = 0.0f;
    if (vertices) {  // colours are given only with a vertex buffer
        const uint32_t c = (__float_as_uint(v1.w) & kTypeMask) % (uint32_t)n_colors;
        cr = colors.c[3 * c];
        cg = colors.c[3 * c + 1];
        cb = colors.c[3 * c + 2];
    }
    uint32_t made = 0;
    for (int a = 0; a < m && made < total; a++)
        for (int b = a + 1; b < m && made < total; b++, made++) {
            const long long k = (long long)o + made;
            if (k >= cap_tris) return;
            if (tris) {
                tris[3 * k] = i;
                tris[3 * k + 1] = list[a];
                tris[3 * k + 2] = list[b];
            }
            if (!vertices) continue;
            const float4 v2 = pos[list[a]], v3 = pos[list[b]];
            // ParticleSimulation.cu:365-382, each operation rounded on its own
            const float e1x = __fsub_rn(v2.x, v1.x), e1y = __fsub_rn(v2.y, v1.y), e1z = __fsub_rn(v2.z, v1.z);
            const float e2x = __fsub_rn(v3.x, v1.x), e2y = __fsub_rn(v3.y, v1.y), e2z = __fsub_rn(v3.z, v1.z);
            float nx = __fsub_rn(__fmul_rn(e1y, e2z), __fmul_rn(e1z, e2y));
            float ny = __fsub_rn(__fmul_rn(e1z, e2x), __fmul_rn(e1x, e2z));
            float nz = __fsub_rn(__fmul_rn(e1x, e2y), __fmul_rn(e1y, e2x));
            const float len =
                __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(nx, nx), __fmul_rn(ny, ny)), __fmul_rn(nz, nz)));
            if (len > 0.0001f) {
                nx = __fdiv_rn(nx, len);
                ny = __fdiv_rn(ny, len);
                nz = __fdiv_rn(nz, len);
            }
            float* v = vertices + k * 27;
            const float4* vs[3] = {&v1, &v2, &v3};
            for (int q = 0; q < 3; q++) {
                v[9 * q + 0] = vs[q]->x;
                v[9 * q + 1] = vs[q]->y;
                v[9 * q + 2] = vs[q]->z;
                v[9 * q + 3] = nx;
                v[9 * q + 4] = ny;
                v[9 * q + 5] = nz;
                v[9 * q + 6] = cr;
                v[9 * q + 7] = cg;
                v[9 * q + 8] = cb;
            }
        }
}

}  // namespace

CF_BOUNDS_READER(proximity)

cudaError_t launch_mesh_select(const float4* pos_sorted, const uint32_t* keys_sorted, const uint32_t* vals_sorted,
                               const uint32_t* cell_start, const uint32_t* cell_end, const Grid& g, int n, float dsq,
                               int max_conn, int32_t* slots, uint32_t* count, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    mesh_select_kernel<<<(n + kThreads - 1) / kThreads, kThreads, 0, st>>>(pos_sorted, keys_sorted, vals_sorted,
                                                                          cell_start, cell_end, g, n, dsq, max_conn,
                                                                          slots, count);
    note_launches(st);
    return cudaGetLastError();
}

cudaError_t launch_mesh_emit(const int32_t* slots, const uint32_t* offsets, int n, const float4* pos,
                             const ColorTable& colors, int n_colors, int32_t* tris, float* vertices, long long cap_tris,
                             cudaStream_t st)
{
    if (n <= 0 || cap_tris <= 0) return cudaSuccess;
    mesh_emit_kernel<<<(n + 255) / 256, 256, 0, st>>>(slots, offsets, n, pos, colors, n_colors, tris, vertices,
                                                      cap_tris);
    note_launches(st);
    return cudaGetLastError();
}

cudaError_t launch_proximity_select(const float4* pos_sorted, const uint32_t* keys_sorted,
                                    const uint32_t* vals_sorted, const uint32_t* cell_start,
                                    const uint32_t* cell_end, bool csr, const Grid& g, int n, float dsq,
                                    int max_conn, int32_t* slots, uint32_t* count, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    const int blocks = (n + kThreads - 1) / kThreads;
    if (csr) {
        // a warp per particle: on clustered states (hundreds of candidates) it is up to 1.6x
        // faster than a thread per particle, which wins only on near-uniform ones (0.081 against
        // 0.093 ms per call at 100k)
        const int warp_blocks = (n + kSelWarps - 1) / kSelWarps;
        proximity_select_warp_kernel<false><<<warp_blocks, kThreads, 0, st>>>(
            pos_sorted, keys_sorted, vals_sorted, cell_start, g, n, dsq, max_conn, slots, count, nullptr,
            ColorTable{}, 1, nullptr, 0);
        note_launches(st);
    } else {
        proximity_select_kernel<false><<<blocks, kThreads, 0, st>>>(pos_sorted, keys_sorted, vals_sorted, cell_start,
                                                                   cell_end, g, n, dsq, max_conn, slots, count);
        note_launches(st);
    }
    return cudaGetLastError();
}

cudaError_t launch_proximity_select_vertices(const float4* pos_sorted, const uint32_t* keys_sorted,
                                             const uint32_t* vals_sorted, const uint32_t* cell_off, const Grid& g,
                                             int n, float dsq, int max_conn, const float4* pos,
                                             const ColorTable& colors, int n_colors, float* vertices,
                                             int cap_vertices, uint32_t* total, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    const int warp_blocks = (n + kSelWarps - 1) / kSelWarps;
    proximity_select_warp_kernel<true><<<warp_blocks, kThreads, 0, st>>>(pos_sorted, keys_sorted, vals_sorted,
                                                                         cell_off, g, n, dsq, max_conn, nullptr,
                                                                         total, pos, colors, n_colors, vertices,
                                                                         cap_vertices);
    note_launches(st);
    return cudaGetLastError();
}

cudaError_t launch_proximity_emit_edges(const int32_t* slots, const uint32_t* offsets, int n, int max_conn,
                                        int32_t* edges, int cap, cudaStream_t st)
{
    (void)max_conn;
    if (n <= 0 || cap <= 0) return cudaSuccess;
    proximity_edges_kernel<<<(n + 255) / 256, 256, 0, st>>>(slots, offsets, n, edges, cap);
    note_launches(st);
    return cudaGetLastError();
}


}  // namespace cf
