// noalloc.cu - proximity edges from caller-owned device buffers, with all
// scratch in one fixed file-scope device array: the entry point allocates
// nothing.
//
// Who needs it: a renderer's frame loop that builds the graph every frame
// and may not allocate per frame (cudaMalloc/cudaFree can stall the device,
// and the frame budget has no room for that), and host applications whose
// device memory belongs to their own pool or allocator, so a library may not
// take more.  The reference wrapper allocated and freed two buffers on every
// call (cuda-native/src/ParticleSimulation.cu:646-654, 681-682).
//
// The array below is reserved on every device that loads the library, for as
// long as the process lives (kNoAllocBytes, about 6.9 MB).  Host code cannot
// use its name as a device address: the first call on each device looks the
// address up with cudaGetSymbolAddress while that device is current and keeps
// it.  Every call shares the array; calls whose work overlaps on the GPU
// (different streams, or different threads on one device) race on it.
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <mutex>

#include "cf_internal.hpp"

namespace cf {
namespace {

constexpr int kNoAllocMaxParticles = 1 << 16;  // 65,536 particles
constexpr int kNoAllocMaxCells = 1 << 16;      // 65,536 cells (the grid is coarsened to fit)
constexpr int kMaxDevices = 64;

constexpr size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// Layout of the scratch array (byte offsets).
constexpr size_t kKeysBytes = align256(sizeof(uint32_t) * kNoAllocMaxParticles);
constexpr size_t kPosBytes = align256(sizeof(float4) * kNoAllocMaxParticles);
constexpr size_t kSlotsBytes = align256(sizeof(int32_t) * kNoAllocMaxParticles * CF_MAX_PROX_CONN);
constexpr size_t kCountBytes = align256(sizeof(uint32_t) * (kNoAllocMaxParticles + 1));
constexpr size_t kHistEntries = 256 * ((kNoAllocMaxParticles + 1023) / 1024);  // radix tiles of 1024 keys
constexpr size_t kHistBytes = align256(sizeof(uint32_t) * kHistEntries);
constexpr size_t kScanEntries = 64;
constexpr size_t kScanBytes = align256(sizeof(uint32_t) * kScanEntries);
constexpr size_t kCellBytes = align256(sizeof(uint32_t) * kNoAllocMaxCells);
constexpr size_t kErrBytes = 256;

constexpr size_t kOffKeys0 = 0;
constexpr size_t kOffKeys1 = kOffKeys0 + kKeysBytes;
constexpr size_t kOffVals0 = kOffKeys1 + kKeysBytes;
constexpr size_t kOffVals1 = kOffVals0 + kKeysBytes;
constexpr size_t kOffPos = kOffVals1 + kKeysBytes;
constexpr size_t kOffSlots = kOffPos + kPosBytes;
constexpr size_t kOffCount = kOffSlots + kSlotsBytes;
constexpr size_t kOffHist = kOffCount + kCountBytes;
constexpr size_t kOffScan = kOffHist + kHistBytes;
constexpr size_t kOffStart = kOffScan + kScanBytes;
constexpr size_t kOffEnd = kOffStart + kCellBytes;
constexpr size_t kOffErr = kOffEnd + kCellBytes;
constexpr size_t kNoAllocBytes = kOffErr + kErrBytes;

static_assert(kHistEntries >= 256 * 64, "radix histogram capacity");

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

std::mutex g_symbol_mutex;
void* g_symbol_address[kMaxDevices] = {};

// Device address of the scratch array on the current device (looked up once
// per device, with that device current).
int scratch_address(unsigned char** out)
{
    int dev = 0;
    CF_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(CF_ERR_INVALID, "device index out of range");
    std::lock_guard<std::mutex> lock(g_symbol_mutex);
    if (!g_symbol_address[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_symbol_address[dev] = p;
    }
    *out = static_cast<unsigned char*>(g_symbol_address[dev]);
    return CF_OK;
}

}  // namespace
}  // namespace cf

extern "C" int cf_proximity_edges_noalloc(const void* d_pos4, int n, float width, float height, float depth,
                                          float distance, int max_conn, int32_t* d_edges, int cap, int* n_edges,
                                          void* stream)
{
    using namespace cf;
    if (n < 0 || n > kNoAllocMaxParticles)
        return fail(CF_ERR_INVALID, "cf_proximity_edges_noalloc: n must be in [0, 65536]");
    if (n > 0 && !d_pos4) return fail(CF_ERR_INVALID, "cf_proximity_edges_noalloc: null positions");
    if (!(std::isfinite(width) && width > 0.0f && std::isfinite(height) && height > 0.0f && std::isfinite(depth) &&
          depth > 0.0f))
        return fail(CF_ERR_INVALID, "cf_proximity_edges_noalloc: box extents must be finite and positive");
    if (!(distance >= 0.0f) || !std::isfinite(distance))
        return fail(CF_ERR_INVALID, "cf_proximity_edges_noalloc: distance must be finite, >= 0");
    if (max_conn < 0 || max_conn > CF_MAX_PROX_CONN)
        return fail(CF_ERR_INVALID, "cf_proximity_edges_noalloc: max_conn must be in [0, 16]");
    if (cap < 0 || (cap > 0 && !d_edges)) return fail(CF_ERR_INVALID, "cf_proximity_edges_noalloc: bad edge buffer");
    if (!n_edges) return fail(CF_ERR_INVALID, "cf_proximity_edges_noalloc: null edge count");

    unsigned char* base = nullptr;
    int rc = scratch_address(&base);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const float ext[3] = {width, height, depth};
    const Grid g = choose_prox_grid(ext, distance, kNoAllocMaxCells);
    if (g.cells > kNoAllocMaxCells) return fail(CF_ERR_INVALID, "cf_proximity_edges_noalloc: grid too large");

    Scratch s;
    s.keys[0] = reinterpret_cast<uint32_t*>(base + kOffKeys0);
    s.keys[1] = reinterpret_cast<uint32_t*>(base + kOffKeys1);
    s.vals[0] = reinterpret_cast<uint32_t*>(base + kOffVals0);
    s.vals[1] = reinterpret_cast<uint32_t*>(base + kOffVals1);
    s.pos_sorted = reinterpret_cast<float4*>(base + kOffPos);
    s.prox_slots = reinterpret_cast<int32_t*>(base + kOffSlots);
    s.prox_count = reinterpret_cast<uint32_t*>(base + kOffCount);
    s.hist = reinterpret_cast<uint32_t*>(base + kOffHist);
    s.hist_cap = kHistEntries;
    s.scan_tmp = reinterpret_cast<uint32_t*>(base + kOffScan);
    s.scan_tmp_cap = kScanEntries;
    s.cell_start = reinterpret_cast<uint32_t*>(base + kOffStart);
    s.cell_end = reinterpret_cast<uint32_t*>(base + kOffEnd);
    s.cells_cap = kNoAllocMaxCells;
    s.n_cap = kNoAllocMaxParticles;
    int* err = reinterpret_cast<int*>(base + kOffErr);
    if (radix_hist_entries(n) > s.hist_cap || scan_tmp_entries(n + 1) > s.scan_tmp_cap ||
        scan_tmp_entries((int)radix_hist_entries(n)) > s.scan_tmp_cap)
        return fail(CF_ERR_INVALID, "cf_proximity_edges_noalloc: scratch layout too small");

    // The array keeps the previous call's contents: clear what must start at zero.
    CF_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
    CF_CUDA(cudaMemsetAsync(s.prox_count + n, 0, sizeof(uint32_t), st));

    const float4* pos = static_cast<const float4*>(d_pos4);
    CF_CUDA(launch_cell_hash(pos, n, g, ext, INT_MAX, s.keys[0], err, st));
    int which = 0;
    CF_CUDA(launch_radix_sort(s, n, g.key_bits, &which, st));
    CF_CUDA(launch_cell_bounds(s.keys[which], s.vals[which], n, pos, s.cell_start, s.cell_end, g.cells, s.pos_sorted,
                               st));
    const float dsq = distance * distance;
    CF_CUDA(launch_proximity_select(s.pos_sorted, s.keys[which], s.vals[which], s.cell_start, s.cell_end, false, g, n,
                                    dsq, max_conn, s.prox_slots, s.prox_count, st));
    CF_CUDA(launch_scan_exclusive(s.prox_count, s.prox_count, n + 1, s.scan_tmp, s.scan_tmp_cap, st));
    uint32_t total = 0;
    int word = 0;
    CF_CUDA(cudaMemcpyAsync(&total, s.prox_count + n, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    CF_CUDA(cudaMemcpyAsync(&word, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    CF_CUDA(cudaStreamSynchronize(st));
    if (word) return fail(CF_ERR_DOMAIN, "cf_proximity_edges_noalloc: a position is outside the box or not finite");
    *n_edges = (int)total;
    const int write = (int)(total < (uint32_t)cap ? total : (uint32_t)cap);
    if (write > 0) {
        CF_CUDA(launch_proximity_emit_edges(s.prox_slots, s.prox_count, n, max_conn, d_edges, write, st));
        CF_CUDA(cudaStreamSynchronize(st));
    }
    if (total > (uint32_t)cap) return fail(CF_ERR_CAPACITY, "cf_proximity_edges_noalloc: edge buffer too small");
    return CF_OK;
}
