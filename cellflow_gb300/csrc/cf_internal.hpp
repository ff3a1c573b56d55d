// cf_internal.hpp - shared declarations of the CellFlow GB300 library.
//
// Device data layout (all in HBM, original particle order unless noted):
//   pos4[n]   float4 x, y, z, type (uint32 bits)    16 B/particle
//   vel4[n]   float4 vx, vy, vz, 0                   16 B/particle
//   acc4[n]   float4 ax, ay, az, 0                   16 B/particle
//   counts[n] int32 neighbour counts (read as "previous", rewritten)
// Per-step scratch (cell list, sorted order):
//   keys/vals  uint32 cell id and particle index, two buffers each (radix
//              sort ping-pong); pos_sorted float4[n] snapshot in cell order;
//   cell_start/cell_end uint32[cells]; radix histograms.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <array>
#include <string>
#include <vector>

#include "cellflow.h"

namespace cf {

// Device error word bits (kernels atomicOr them; the host reads at sync).
enum : int {
    kDevErrDomain = 1,  // a position outside [0, extent) or not finite
    kDevErrType = 2,    // a type outside [0, T)
    kDevErrWait = 4,    // a bounded device wait gave up
};

// ---- bounds-checked build (compiled with -DCF_DEBUG_BOUNDS) -------------------
//
// Checked accesses test their index first; in the checked build an index
// outside [0, limit) is recorded (the first one per translation unit, in a
// device variable of that unit) and the access is skipped, so the kernel
// carries on and the host reads the record (cf_debug_bounds).  In the normal
// build the test compiles away.
struct BoundsRecord {
    int flag;  // 1: a violation was recorded
    int line;  // source line of the check
    long long index, limit;
};
#if defined(__CUDACC__)
#ifdef CF_DEBUG_BOUNDS
static __device__ BoundsRecord cf_bounds_rec;
#endif
__device__ __forceinline__ bool bounds_ok(long long idx, long long lim, int line)
{
#ifdef CF_DEBUG_BOUNDS
    if (idx >= 0 && idx < lim) return true;
    if (atomicCAS(&cf_bounds_rec.flag, 0, 1) == 0) {
        cf_bounds_rec.line = line;
        cf_bounds_rec.index = idx;
        cf_bounds_rec.limit = lim;
    }
    return false;
#else
    (void)idx;
    (void)lim;
    (void)line;
    return true;
#endif
}
#define CF_IN_BOUNDS(idx, lim) ::cf::bounds_ok((long long)(idx), (long long)(lim), __LINE__)
// The host reader of a unit's record (read and cleared); defined once per checked unit.
#ifdef CF_DEBUG_BOUNDS
#define CF_BOUNDS_READER(name)                                                               \
    cudaError_t bounds_take_##name(BoundsRecord* out)                                        \
    {                                                                                        \
        cudaError_t e = cudaMemcpyFromSymbol(out, cf_bounds_rec, sizeof(BoundsRecord));      \
        const BoundsRecord zero{};                                                           \
        if (e == cudaSuccess) e = cudaMemcpyToSymbol(cf_bounds_rec, &zero, sizeof(zero));    \
        return e;                                                                            \
    }
#else
#define CF_BOUNDS_READER(name)                        \
    cudaError_t bounds_take_##name(BoundsRecord* out) \
    {                                                 \
        *out = BoundsRecord{};                        \
        return cudaSuccess;                           \
    }
#endif
#endif
cudaError_t bounds_take_celllist(BoundsRecord* out);
cudaError_t bounds_take_step(BoundsRecord* out);
cudaError_t bounds_take_proximity(BoundsRecord* out);

// Tables padded to the maximum type count so any 5-bit type index stays in
// bounds: index = (self & 31) * 32 + (other & 31).
constexpr int kTableStride = CF_MAX_TYPES;
constexpr int kTableSize = CF_MAX_TYPES * CF_MAX_TYPES;

// Per-pair tables for a step, uploaded together.
struct PairTables {
    float force[kTableSize];         // F[self][other]
    float eff[kTableSize];           // effective radius (ParticleSimulation.cu:108-110)
    float threshold[kTableSize];     // smallest float t with sqrtf(t) >= eff
    float threshold_lo[kTableSize];  // contracted d^2 below this interacts for certain
};

// Grid of one cell list.  A batch of independent worlds shares one grid
// shape; a cell id is world * cells_w + (z * m1 + y) * m0 + x.
struct Grid {
    int m[3];         // cells per axis
    float inv[3];     // hash multipliers, float(m / extent)
    int cells;        // total cells: worlds * cells_w
    int key_bits;     // bits of a cell id
    int generic;      // 1: full reference wrap per candidate (some axis < 5 cells)
    int periodic;     // 1: periodic stencil (step), 0: clipped (proximity)
    int worlds;       // independent worlds sharing the grid (1 for a plain world)
    int cells_w;      // cells per world: m0 * m1 * m2
};

// pos4.w of a particle: type in the low 5 bits, world index above.
constexpr int kWorldShift = 5;
constexpr uint32_t kTypeMask = (1u << kWorldShift) - 1u;

// Everything the step kernels read besides the buffers.
struct StepConsts {
    float ext[3];      // W, H, D
    float half[3];     // W*0.5f, ...
    Grid grid;
    int n;
    int num_types;
    int uniform_r;     // all pairs share one effective radius
    float eff_uniform;
    float thr_uniform;
    float inv_eff_uniform;
    float thr_lo_uniform;  // contracted d^2 below this interacts for certain (uniform radius)
    float thr_filter;  // squared-distance bound of the approximate pre-test (>= every exact pass)
    int variant;       // force-kernel staging variant (batch size, occupancy): cf_set_force_variant % 4
    int split;         // warps per item (1, 2, 4): 1 << (cf_set_force_variant / 4)
    float repulsion, attraction, neg_k, balance, force_multiplier, delta_t, friction;
    int max_expected_neighbors;
    const float* world_force;  // per-world force tables, kTableSize floats each (32-stride)
};

// One force-kernel item: up to 32 consecutive sorted particles of one row of
// cells, with the row's cell coordinates inside its world.
struct __align__(16) Item {
    int first;  // first sorted index
    int count;  // particles, 1..32
    int yz;     // y | z << 16
    int world;
};

struct Scratch {
    uint32_t* keys[2] = {nullptr, nullptr};
    uint32_t* vals[2] = {nullptr, nullptr};
    uint32_t* hist = nullptr;       // radix digit histograms / scan partials
    size_t hist_cap = 0;            // entries
    uint32_t* cell_start = nullptr;
    uint32_t* cell_end = nullptr;
    size_t cells_cap = 0;
    float4* pos_sorted = nullptr;
    int n_cap = 0;
    // proximity
    int32_t* prox_slots = nullptr;  // n * CF_MAX_PROX_CONN partner indices
    uint32_t* prox_count = nullptr; // n + 1 (exclusive-scanned in place)
    // triangle mesh
    int32_t* mesh_slots = nullptr;  // n * CF_MESH_MAX_CONN neighbour indices (-1 ends a short list)
    uint32_t* mesh_count = nullptr; // n + 1 triangles per particle, exclusive-scanned in place
    uint32_t* scan_tmp = nullptr;   // block partials of the device-wide scan
    size_t scan_tmp_cap = 0;
    // device staging of index output bound for host memory (edges, triangles)
    int32_t* out_idx = nullptr;
    size_t out_cap = 0;  // int32 entries
    // work counters
    unsigned long long* counters = nullptr;  // [0] C27, [1] I
    uint32_t* cell_pop = nullptr;            // canonical-grid populations
    size_t pop_cap = 0;
    // CSR cell offsets of the step (cells + 1 entries)
    uint32_t* cell_off = nullptr;
    size_t off_cap = 0;
    // force-kernel plan: per-row populations and the row-aligned 32-particle items
    uint32_t* row_count = nullptr;
    size_t rows_cap = 0;
    Item* items = nullptr;       // row-aligned items of the force kernel
    size_t items_cap = 0;
    int* n_items = nullptr;
    // tiled CSR build: arrival slot per particle, per-tile totals
    uint32_t* aux = nullptr;  // n
    uint2* tile_sums = nullptr;
    size_t tiles_cap = 0;
};

// Cells of one tile of the CSR build (whole rows; 16 KB of shared memory).
constexpr int kTileCellsMax = 4096;

// Force-kernel staging variants (batch size and occupancy); a variant index
// of cf_set_force_variant is stage + kForceStages * log2(warps per item).
constexpr int kForceStages = 4;

// Differentiable rollout: checkpoints, one segment of replayed states, the
// adjoint buffers and the record of the last forward (cf_rollout_*).
struct Rollout {
    int n_cap = 0;     // particles the buffers hold
    int ckpt_cap = 0;  // checkpoint states allocated
    int seg_cap = 0;   // segment states per segment buffer (checkpoint_every + 1); two buffers
    float4* ckpt_pos = nullptr;
    float4* ckpt_vel = nullptr;
    int* ckpt_cnt = nullptr;
    float4* seg_pos = nullptr;
    float4* seg_vel = nullptr;
    int* seg_cnt = nullptr;
    float4* fin_pos = nullptr;  // the state after the forward, restored after the backward
    float4* fin_vel = nullptr;
    int* fin_cnt = nullptr;
    // the cell list of every replayed step of a segment (sorted snapshot, sorted
    // keys and indices, CSR offsets), written by the replay, read by the adjoint step
    float4* seg_sorted = nullptr;
    uint32_t* seg_keys = nullptr;
    uint32_t* seg_vals = nullptr;
    uint32_t* seg_off = nullptr;
    int lists_steps = 0;   // steps the lists hold, per segment buffer (two buffers)
    size_t lists_cells = 0;  // cells + 1 per step's offsets
    float4* gx = nullptr;         // dL/dx of the current step boundary
    float4* gv = nullptr;         // dL/dv
    float4* gf_sorted = nullptr;  // dL/df per particle, cell order
    float4* ga_sorted = nullptr;  // (dL/da, density), cell order
    double* gacc = nullptr;       // kTableSize table gradients (32-stride), then CF_GRAD_PARAMS
    // the last forward
    int steps = 0;
    int every = 0;
    int n = 0;
    cf_step_params params{};
    uint64_t table_version = 0;
    float radio[CF_MAX_TYPES] = {};
    // a second stream and fork/join events: while the adjoint steps of segment s
    // run on the world's stream, the replay of segment s - 1 runs on this one
    // (captured into the backward's graph); segment buffers alternate by parity
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // the forward's step loop (checkpoint copies and steps) as one CUDA graph,
    // re-captured when its key changes
    cudaGraphExec_t fwd_graph = nullptr;
    long long fwd_kernels = 0;
    StepConsts fwd_key{};
    int fwd_steps = 0, fwd_every = 0;
    const void* fwd_bufs = nullptr;
    const void* fwd_ckpt = nullptr;
    // the backward as one CUDA graph, re-captured when its key changes
    cudaGraphExec_t bwd_graph = nullptr;
    long long bwd_kernels = 0;  // kernel nodes of bwd_graph
    StepConsts bwd_key{};
    int bwd_steps = 0, bwd_every = 0;
    const void* bwd_bufs = nullptr;
    const void* bwd_lists = nullptr;
    // radial distribution scratch
    float4* rdf_pos = nullptr;
    double* rdf_acc = nullptr;
    unsigned long long* type_count = nullptr;
};
constexpr int kGradAccEntries = kTableSize + 8;

// A cached CUDA graph of a selection pass (0: proximity edges, 1: triangle
// mesh): cell list on its grid, selection kernel, scan, count read-back.
// Per-type colours (r, g, b), passed to the emit kernels by value.
struct ColorTable {
    float c[3 * CF_MAX_TYPES];
};

struct SelGraph {
    cudaGraphExec_t exec = nullptr;
    long long kernels = 0;  // kernel nodes of exec
    Grid g{};
    float dsq = 0.0f;
    int max_conn = -1, n = -1, types = -1;
    // the vertex-emitting selection: its output buffer and colours
    const void* out = nullptr;
    long long out_cap = -1;
    ColorTable colors{};
};

}  // namespace cf

struct cf_world {
    int device = 0;
    int n = 0;
    int num_types = 0;
    float ext[3] = {0, 0, 0};
    // a batch of independent worlds (cf_batch_*): world k owns particles
    // [world_off[k], world_off[k + 1]) and force table world_tables[k]
    int worlds = 1;
    std::vector<int> world_off;
    float* world_tables = nullptr;  // device, worlds * kTableSize floats (32-stride)
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    float4* pos = nullptr;
    float4* vel = nullptr;
    float4* acc = nullptr;
    int* counts = nullptr;
    cf_particle* aos = nullptr;  // staging for AoS transfers (allocated on first use)
    int* err = nullptr;          // device error word
    int* host_words = nullptr;   // pinned host: [0] error word read back, [1] output count read back
    cf::PairTables* tables = nullptr;
    cf::Scratch s;
    // host-side parameter surface
    float raw[cf::kTableSize];
    float table[cf::kTableSize];
    float radio[CF_MAX_TYPES];
    uint64_t table_version = 1;
    // cache of the uploaded pair tables
    uint64_t uploaded_version = 0;
    float uploaded_radius = -1.0f;
    float uploaded_ratio = 0.0f;
    int uploaded_types = -1;
    float uploaded_extent = -1.0f;
    cf::PairTables host_tables;
    // phase profiling (cf_profile_enable): per profiled step a triple of events
    // (start, after the cell list, after the force kernel) from a ring; the
    // times are read when a slot is reused or at cf_profile_read, so profiled
    // steps are not serialised.  Adjoint steps of a profiled backward use the
    // same ring (kind 1: start and end of their kernels).
    bool profiling = false;
    std::vector<std::array<cudaEvent_t, 3>> prof_ring;
    std::vector<unsigned char> prof_kind;  // per ring slot: 0 a step, 1 an adjoint step
    int prof_head = 0, prof_pending = 0;
    double prof_cell_ms = 0.0, prof_force_ms = 0.0, prof_adj_ms = 0.0;
    long long prof_steps = 0, prof_launches = 0, prof_adj_steps = 0;
    // one-step CUDA graphs (index 1: the cell list alone, for profiled steps,
    // whose force kernel is launched between the events), re-captured when the
    // step constants or buffers change
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    long long graph_kernels[2] = {0, 0};  // kernel nodes of graph[k]
    cf::StepConsts graph_key[2];
    const void* graph_bufs[2] = {nullptr, nullptr};
    bool use_graphs = true;
    bool broken = false;  // a particle reallocation failed: no buffers until one succeeds
    int force_variant = 0;  // force-kernel variant, chosen by cf_autotune_step
    // a captured multi-step graph (cf_batch_capture) and the constants it was captured with
    cudaGraphExec_t batch_graph = nullptr;
    int batch_graph_steps = 0;
    long long batch_graph_kernels = 0;  // kernel nodes of the captured graph
    cf::Rollout ro;
    // cf_step_host: upload, step and read-back as one graph, keyed by the step
    // constants, the host buffers and the scratch identity
    cudaGraphExec_t host_graph = nullptr;
    long long host_graph_kernels = 0;
    cf::StepConsts host_key;
    const void* host_in = nullptr;
    void* host_out = nullptr;
    const void* host_bufs = nullptr;
    cf::SelGraph sel_graph[3];  // proximity (counts + scan), triangle mesh, proximity vertices
};

namespace cf {

// Error plumbing (thread-local message, see cf_last_error).
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

// Launch tally: kernels this library has put on a stream since it was loaded.
// Every launch site notes its kernel (nothing is counted while the stream is
// being captured); a graph replay notes the kernel nodes of its graph.
void note_launches(cudaStream_t st, long long k = 1);
long long launch_tally();
// Kernel nodes of a captured graph.
cudaError_t graph_kernel_count(cudaGraph_t graph, long long* kernels);
// Host-side fault injection (cf_inject_cuda_error): the error armed for a
// call site whose text contains the armed substring, else cudaSuccess.  The
// call itself is then not made.
cudaError_t injected_error(const char* site);
#define CF_CUDA(call)                                                   \
    do {                                                                \
        cudaError_t cf_e_ = ::cf::injected_error(#call);                \
        if (cf_e_ == cudaSuccess) cf_e_ = (call);                       \
        if (cf_e_ != cudaSuccess) return ::cf::cuda_fail(cf_e_, #call); \
    } while (0)

// Launchers (return a CUDA error code; called with the world's stream).
cudaError_t launch_cell_hash(const float4* pos, int n, const Grid& g, const float* ext, int num_types,
                             uint32_t* keys, int* err, cudaStream_t st);
cudaError_t launch_radix_sort(Scratch& s, int n, int key_bits, int* which, cudaStream_t st);
cudaError_t launch_cell_bounds(const uint32_t* keys, const uint32_t* vals, int n, const float4* pos, uint32_t* start,
                               uint32_t* end, int cells, float4* pos_sorted, cudaStream_t st);
cudaError_t launch_step_force(const StepConsts& c, const PairTables* tables, const float4* pos_sorted,
                              const uint32_t* keys_sorted, const uint32_t* vals_sorted, const uint32_t* cell_off,
                              const Item* items, const int* n_items, int max_items, float4* pos, float4* vel,
                              float4* acc, int* counts, cudaStream_t st);
// Row-aligned items of at most 32 sorted particles (one cell row each).
cudaError_t launch_force_work(const StepConsts& c, const uint32_t* keys_sorted, const uint32_t* cell_off,
                              const Item* items, const int* n_items, int max_items, unsigned long long* out,
                              cudaStream_t st);
cudaError_t launch_step_plan(const uint32_t* cell_off, int n, const Grid& g, Item* items, int* n_items,
                             cudaStream_t st);
int max_step_items(int n, const Grid& g);
int step_launches(int n);
cudaError_t configure_step_force();
cudaError_t launch_scan_exclusive(const uint32_t* in, uint32_t* out, int n, uint32_t* tmp, size_t tmp_cap,
                                  cudaStream_t st);
size_t scan_tmp_entries(int n);
size_t radix_hist_entries(int n);
int cell_list_launches(int n, int key_bits);
// The step's cell list: CSR offsets (cells + 1), sorted keys / values
// (s.keys[*which], s.vals[*which], stable: cell order, ties in index order),
// the position snapshot s.pos_sorted and, when items is not null, the force
// kernel's row-aligned items.  Rows of at most kTileCellsMax cells take the
// tiled path (5 kernels); longer rows a radix sort.  stable = false (for
// callers whose result does not depend on the order within a cell) leaves the
// particles of a cell in arrival order and saves the stable ranking on the
// tiled path (4 kernels).
cudaError_t launch_cell_list_csr(const float4* pos, int n, const Grid& g, const float* ext, int num_types,
                                 Scratch& s, uint32_t* cell_off, Item* items, int* n_items, int* err, int* which,
                                 cudaStream_t st, bool stable = true);
int cell_list_csr_buffer(int n, const Grid& g);
int cell_list_csr_launches(int n, const Grid& g, bool with_plan);
int cell_list_tiles(const Grid& g);  // 0 when the rows are longer than a tile
// csr: cell_start = CSR offsets and cell_end = offsets + 1 (rows read as
// ranges); else per-cell start/end arrays.
cudaError_t launch_proximity_select(const float4* pos_sorted, const uint32_t* keys_sorted,
                                    const uint32_t* vals_sorted, const uint32_t* cell_start,
                                    const uint32_t* cell_end, bool csr, const Grid& g, int n, float dsq,
                                    int max_conn, int32_t* slots, uint32_t* count, cudaStream_t st);
// cell_start = CSR offsets, cell_end = offsets + 1.
cudaError_t launch_mesh_select(const float4* pos_sorted, const uint32_t* keys_sorted, const uint32_t* vals_sorted,
                               const uint32_t* cell_start, const uint32_t* cell_end, const Grid& g, int n, float dsq,
                               int max_conn, int32_t* slots, uint32_t* count, cudaStream_t st);
cudaError_t launch_mesh_emit(const int32_t* slots, const uint32_t* offsets, int n, const float4* pos,
                             const ColorTable& colors, int n_colors, int32_t* tris, float* vertices, long long cap_tris,
                             cudaStream_t st);
cudaError_t launch_proximity_emit_edges(const int32_t* slots, const uint32_t* offsets, int n, int max_conn,
                                        int32_t* edges, int cap, cudaStream_t st);
// The CSR selection that writes each particle's line vertices itself, at an
// offset reserved by one atomic per particle (vertex order is arbitrary, as the
// reference's atomicAdd append); *total = edges found (zero on entry).
cudaError_t launch_proximity_select_vertices(const float4* pos_sorted, const uint32_t* keys_sorted,
                                             const uint32_t* vals_sorted, const uint32_t* cell_off, const Grid& g,
                                             int n, float dsq, int max_conn, const float4* pos,
                                             const ColorTable& colors, int n_colors, float* vertices,
                                             int cap_vertices, uint32_t* total, cudaStream_t st);
cudaError_t launch_init_particles(float4* pos, float4* vel, float4* acc, int* counts, int n, int num_types,
                                  const float* lo, const float* span, uint64_t seed, cudaStream_t st,
                                  uint32_t world = 0);
cudaError_t launch_move_particles(float4* pos, int n, float dx, float dy, float dz, const float* ext, cudaStream_t st);
cudaError_t launch_aos_to_soa(const cf_particle* aos, float4* pos, float4* vel, float4* acc, int n, cudaStream_t st);
cudaError_t launch_soa_to_aos(const float4* pos, const float4* vel, const float4* acc, cf_particle* aos, int n,
                              cudaStream_t st);
// aos_host: the device view of page-locked host records
cudaError_t launch_aos_to_soa_mapped(const cf_particle* aos_host, float4* pos, float4* vel, float4* acc, int n,
                                     cudaStream_t st);
cudaError_t launch_soa_to_aos_mapped(const float4* pos, const float4* vel, const float4* acc, cf_particle* aos_host,
                                     int n, cudaStream_t st);
cudaError_t launch_work_counters(const float4* pos, const int* counts, int n, const Grid& canon, uint32_t* pop,
                                 unsigned long long* out, cudaStream_t st);

// Adjoint and radial distribution (adjoint.cu).
constexpr int kRdfMaxEntries = 49152;  // T * T * bins held in shared memory
constexpr int kRdfMaxSmem = kRdfMaxEntries * 4;
float rdf_cutoff(int bins, float r_max);
size_t rdf_smem_bytes(int T, int bins);
cudaError_t configure_adjoint();
cudaError_t launch_adjoint_step(const StepConsts& c, const PairTables* tables, const float4* pos_sorted,
                                const uint32_t* keys_sorted, const uint32_t* vals_sorted, const uint32_t* cell_off,
                                const float4* vel, const int* cnt_prev, const int* cnt_new, float4* gx, float4* gv,
                                float4* gf_sorted, float4* ga_sorted, double* gacc, cudaStream_t st);
cudaError_t launch_pack_pos(const float4* src, const float4* typesrc, float4* dst, int n, cudaStream_t st);
cudaError_t launch_rdf(const float* ext, const Grid& g, int n, int T, int bins, float r_max, const float4* pos_sorted,
                       const uint32_t* keys_sorted, const uint32_t* cell_off, double* acc,
                       unsigned long long* type_count, float* hist, cudaStream_t st);
cudaError_t launch_rdf_grad(const float* ext, const Grid& g, int n, int T, int bins, float r_max,
                            const float4* pos, const float4* pos_sorted, const uint32_t* keys_sorted,
                            const uint32_t* vals_sorted, const uint32_t* cell_off, const float* ghist,
                            unsigned long long* type_count, float4* gpos, cudaStream_t st);

// Host helpers (api.cpp).
Grid choose_step_grid(const float* ext, float r_cut, int max_cells);
Grid choose_prox_grid(const float* ext, float distance, int max_cells);
Grid canonical_grid(const float* ext, float r_max);
float sqrt_threshold(float eff);
float cutoff_distance(float threshold);
float certain_bound(float threshold, float max_extent);

}  // namespace cf
