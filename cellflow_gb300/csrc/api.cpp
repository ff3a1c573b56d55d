// api.cpp - the C ABI (include/cellflow.h): world lifetime, parameter
// surface, step driver, proximity graph and introspection.
//
// Host code of the reference this replaces: ParticleSimulation
// (cuda-native/src/ParticleSimulation.cu:426-687).  Built with
// -ffp-contract=off so the pair tables round exactly like the reference's
// per-pair expressions (ParticleSimulation.cu:108-110, 521-531).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "cf_internal.hpp"

namespace cf {
namespace {


thread_local std::string g_error;

constexpr int kMaxCells = 1 << 22;        // cap of the step and proximity grids
constexpr int kProfRing = 1024;           // event triples of profiled steps in flight
constexpr int kMaxCanonicalCells = 1 << 24;  // cap of the work-model grid

uint64_t splitmix64(uint64_t& s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Uniform in [-1, 1), the range of the reference's rand()/RAND_MAX*2-1
// (ParticleSimulation.cu:516, 535), from a seeded generator.
float uniform_pm1(uint64_t& s)
{
    float u = (float)(splitmix64(s) >> 40) * (1.0f / 16777216.0f);
    return u * 2.0f - 1.0f;
}

bool finite_positive(float v) { return std::isfinite(v) && v > 0.0f; }

int check_world(const cf_world* w)
{
    if (!w) return fail(CF_ERR_INVALID, "null world");
    if (w->broken)
        return fail(CF_ERR_INVALID,
                    "the world lost its particle buffers when a reallocation failed; call cf_set_particle_count "
                    "again or destroy it");
    return CF_OK;
}

// Device memory held by the library (every buffer goes through dev_alloc),
// under an optional cap (cf_set_device_memory_limit, 0 = none): a request that
// would exceed it fails like cudaMalloc out of memory.
std::mutex g_mem_mu;
std::unordered_map<void*, size_t> g_mem_sizes;
size_t g_mem_live = 0;
size_t g_mem_limit = 0;
thread_local bool g_mem_capped = false;  // the last allocation failure came from the cap

cudaError_t raw_alloc(void** p, size_t bytes)
{
    *p = nullptr;
    g_mem_capped = false;
    {
        std::lock_guard<std::mutex> lock(g_mem_mu);
        if (g_mem_limit != 0 && g_mem_live + bytes > g_mem_limit) {
            g_mem_capped = true;
            return cudaErrorMemoryAllocation;
        }
    }
    const cudaError_t inj = injected_error("cudaMalloc");
    if (inj != cudaSuccess) return inj;
#ifdef CF_DEBUG_BOUNDS
    // the bounds-checked build pads every buffer, so an index that a check missed
    // a little past the end still lands in this allocation
    const cudaError_t e = cudaMalloc(p, bytes + (64u << 10));
#else
    const cudaError_t e = cudaMalloc(p, bytes);
#endif
    if (e != cudaSuccess) {
        *p = nullptr;
        return e;
    }
    std::lock_guard<std::mutex> lock(g_mem_mu);
    g_mem_sizes[*p] = bytes;
    g_mem_live += bytes;
    return cudaSuccess;
}

template <typename T>
cudaError_t dev_alloc(T** p, size_t count)
{
    if (count == 0) count = 1;
    void* q = nullptr;
    const cudaError_t e = raw_alloc(&q, sizeof(T) * count);
    *p = static_cast<T*>(q);
    return e;
}

void dev_free(void* p)
{
    if (!p) return;
    {
        std::lock_guard<std::mutex> lock(g_mem_mu);
        auto it = g_mem_sizes.find(p);
        if (it != g_mem_sizes.end()) {
            g_mem_live -= it->second;
            g_mem_sizes.erase(it);
        }
    }
    cudaFree(p);
}

// The armed injection: the next `skip` matching sites pass, the one after
// returns `error` (once).
std::mutex g_inj_mu;
std::string g_inj_site;
int g_inj_skip = 0;
cudaError_t g_inj_error = cudaSuccess;
std::atomic<bool> g_inj_armed{false};

void apply_worlds(Grid& g, int worlds);

void drop_graphs(cf_world* w)
{
    if (w->batch_graph) cudaGraphExecDestroy(w->batch_graph);
    w->batch_graph = nullptr;
    w->batch_graph_steps = 0;
    // the rollout's graphs capture the cell-list scratch (offsets, tile
    // totals, items) by address, so any reallocation must drop them too
    if (w->ro.bwd_graph) cudaGraphExecDestroy(w->ro.bwd_graph);
    w->ro.bwd_graph = nullptr;
    if (w->ro.fwd_graph) cudaGraphExecDestroy(w->ro.fwd_graph);
    w->ro.fwd_graph = nullptr;
    for (int k = 0; k < 2; k++) {
        if (w->graph[k]) cudaGraphExecDestroy(w->graph[k]);
        w->graph[k] = nullptr;
        w->graph_bufs[k] = nullptr;
    }
    if (w->host_graph) cudaGraphExecDestroy(w->host_graph);
    w->host_graph = nullptr;
    w->host_bufs = nullptr;
    for (auto& sg : w->sel_graph) {
        if (sg.exec) cudaGraphExecDestroy(sg.exec);
        sg = SelGraph();
    }
}

// (Re)allocate per-particle state and scratch for w->n particles.
int alloc_particles(cf_world* w)
{
    const int n = w->n;
    Scratch& s = w->s;
    CF_CUDA(dev_alloc(&w->pos, n));
    CF_CUDA(dev_alloc(&w->vel, n));
    CF_CUDA(dev_alloc(&w->acc, n));
    CF_CUDA(dev_alloc(&w->counts, n));
    CF_CUDA(cudaMemsetAsync(w->counts, 0, sizeof(int) * (size_t)std::max(n, 1), w->stream));
    for (int b = 0; b < 2; b++) {
        CF_CUDA(dev_alloc(&s.keys[b], n));
        CF_CUDA(dev_alloc(&s.vals[b], n));
    }
    CF_CUDA(dev_alloc(&s.pos_sorted, n));
    CF_CUDA(dev_alloc(&s.aux, n));
    s.hist_cap = radix_hist_entries(n);
    CF_CUDA(dev_alloc(&s.hist, s.hist_cap));
    s.scan_tmp_cap = std::max(scan_tmp_entries((int)s.hist_cap), scan_tmp_entries(n + 1));
    CF_CUDA(dev_alloc(&s.scan_tmp, s.scan_tmp_cap));
    CF_CUDA(dev_alloc(&s.counters, 2));
    s.n_cap = n;
    return CF_OK;
}

void free_rollout(cf_world* w)
{
    Rollout& r = w->ro;
    if (r.bwd_graph) cudaGraphExecDestroy(r.bwd_graph);
    if (r.fwd_graph) cudaGraphExecDestroy(r.fwd_graph);
    if (r.ev_fork) cudaEventDestroy(r.ev_fork);
    if (r.ev_join) cudaEventDestroy(r.ev_join);
    if (r.side) cudaStreamDestroy(r.side);
    for (void* p : {(void*)r.ckpt_pos, (void*)r.ckpt_vel, (void*)r.ckpt_cnt, (void*)r.seg_pos, (void*)r.seg_vel,
                    (void*)r.seg_cnt, (void*)r.fin_pos, (void*)r.fin_vel, (void*)r.fin_cnt, (void*)r.gx,
                    (void*)r.gv, (void*)r.gf_sorted, (void*)r.ga_sorted, (void*)r.gacc, (void*)r.rdf_pos,
                    (void*)r.rdf_acc, (void*)r.type_count, (void*)r.seg_sorted, (void*)r.seg_keys,
                    (void*)r.seg_vals, (void*)r.seg_off})
        dev_free(p);
    r = Rollout();
}

void free_particles(cf_world* w)
{
    drop_graphs(w);
    free_rollout(w);
    Scratch& s = w->s;
    dev_free(w->pos);
    dev_free(w->vel);
    dev_free(w->acc);
    dev_free(w->counts);
    for (int b = 0; b < 2; b++) {
        dev_free(s.keys[b]);
        dev_free(s.vals[b]);
    }
    dev_free(s.pos_sorted);
    dev_free(s.aux);
    dev_free(s.tile_sums);
    dev_free(s.hist);
    dev_free(s.scan_tmp);
    dev_free(s.cell_start);
    dev_free(s.cell_end);
    dev_free(s.prox_slots);
    dev_free(s.prox_count);
    dev_free(s.mesh_slots);
    dev_free(s.mesh_count);
    dev_free(s.out_idx);
    dev_free(s.counters);
    dev_free(s.cell_pop);
    dev_free(s.row_count);
    dev_free(s.items);
    dev_free(s.n_items);
    dev_free(s.cell_off);
    dev_free(w->aos);
    w->pos = w->vel = w->acc = nullptr;
    w->counts = nullptr;
    w->aos = nullptr;
    s = Scratch();
}

int ensure_cells(cf_world* w, int cells)
{
    Scratch& s = w->s;
    if ((size_t)cells <= s.cells_cap) return CF_OK;
    CF_CUDA(cudaStreamSynchronize(w->stream));
    drop_graphs(w);
    dev_free(s.cell_start);
    dev_free(s.cell_end);
    s.cell_start = s.cell_end = nullptr;
    s.cells_cap = 0;
    CF_CUDA(dev_alloc(&s.cell_start, cells));
    CF_CUDA(dev_alloc(&s.cell_end, cells));
    s.cells_cap = (size_t)cells;
    return CF_OK;
}

// CSR offsets (cells + 1 entries) and the scan partials they need.
int ensure_offsets(cf_world* w, int cells)
{
    Scratch& s = w->s;
    const size_t need_tmp = scan_tmp_entries(cells + 1);
    // tiles of the CSR build: at most 257 on grids spread thin, else every tile
    // holds more than kTileCellsMax / 2 cells
    const size_t need_tiles = (size_t)cells / (kTileCellsMax / 2) + 2 + 257;
    if ((size_t)cells + 1 <= s.off_cap && need_tmp <= s.scan_tmp_cap && need_tiles <= s.tiles_cap) return CF_OK;
    CF_CUDA(cudaStreamSynchronize(w->stream));
    drop_graphs(w);
    if (need_tiles > s.tiles_cap) {
        dev_free(s.tile_sums);
        s.tile_sums = nullptr;
        s.tiles_cap = 0;
        CF_CUDA(dev_alloc(&s.tile_sums, need_tiles));
        s.tiles_cap = need_tiles;
    }
    if ((size_t)cells + 1 > s.off_cap) {
        dev_free(s.cell_off);
        s.cell_off = nullptr;
        s.off_cap = 0;
        CF_CUDA(dev_alloc(&s.cell_off, (size_t)cells + 1));
        s.off_cap = (size_t)cells + 1;
    }
    if (need_tmp > s.scan_tmp_cap) {
        dev_free(s.scan_tmp);
        s.scan_tmp = nullptr;
        s.scan_tmp_cap = 0;
        CF_CUDA(dev_alloc(&s.scan_tmp, need_tmp));
        s.scan_tmp_cap = need_tmp;
    }
    return CF_OK;
}

// Buffers of the force kernel's plan for this grid: per-row populations and
// the item list (at most n/32 + rows items).
int ensure_plan(cf_world* w, const Grid& g)
{
    Scratch& s = w->s;
    const size_t rows = (size_t)g.m[1] * g.m[2];
    const size_t items = (size_t)max_step_items(w->n, g);
    if (rows <= s.rows_cap && items <= s.items_cap && s.n_items) return CF_OK;
    CF_CUDA(cudaStreamSynchronize(w->stream));
    drop_graphs(w);
    dev_free(s.row_count);
    dev_free(s.items);
    dev_free(s.n_items);
    s.row_count = nullptr;
    s.items = nullptr;
    s.n_items = nullptr;
    s.rows_cap = s.items_cap = 0;
    CF_CUDA(dev_alloc(&s.row_count, rows));
    CF_CUDA(dev_alloc(&s.items, items));
    CF_CUDA(dev_alloc(&s.n_items, 1));
    s.rows_cap = rows;
    s.items_cap = items;
    return CF_OK;
}

int ensure_aos(cf_world* w)
{
    if (w->aos) return CF_OK;
    CF_CUDA(dev_alloc(&w->aos, w->n));
    return CF_OK;
}

// Two buffers allocated together or not at all (a lazily allocated pair is
// tested by its first member).
template <typename A, typename B>
int alloc_pair(A** a, size_t na, B** b, size_t nb)
{
    A* x = nullptr;
    B* y = nullptr;
    cudaError_t e = dev_alloc(&x, na);
    if (e == cudaSuccess) e = dev_alloc(&y, nb);
    if (e != cudaSuccess) {
        dev_free(x);
        return cuda_fail(e, "dev_alloc(scratch pair)");
    }
    *a = x;
    *b = y;
    return CF_OK;
}

int ensure_prox(cf_world* w)
{
    Scratch& s = w->s;
    if (s.prox_slots) return CF_OK;
    return alloc_pair(&s.prox_slots, (size_t)w->n * CF_MAX_PROX_CONN, &s.prox_count, (size_t)w->n + 1);
}

int ensure_mesh(cf_world* w)
{
    Scratch& s = w->s;
    if (s.mesh_slots) return CF_OK;
    return alloc_pair(&s.mesh_slots, (size_t)w->n * CF_MESH_MAX_CONN, &s.mesh_count, (size_t)w->n + 1);
}

// Staging for index output copied to host memory: grows to the largest
// request and is kept, so repeated frames allocate nothing.
int ensure_out(cf_world* w, size_t entries)
{
    Scratch& s = w->s;
    if (entries <= s.out_cap) return CF_OK;
    CF_CUDA(cudaStreamSynchronize(w->stream));
    dev_free(s.out_idx);
    s.out_idx = nullptr;
    s.out_cap = 0;
    CF_CUDA(dev_alloc(&s.out_idx, entries));
    s.out_cap = entries;
    return CF_OK;
}

// The per-type colours as the emit kernels' by-value table.
ColorTable color_table(const cf_world* w, const cf_color* colors)
{
    ColorTable t{};
    for (int k = 0; k < w->num_types; k++) {
        t.c[3 * k] = colors[k].r;
        t.c[3 * k + 1] = colors[k].g;
        t.c[3 * k + 2] = colors[k].b;
    }
    return t;
}

// Wait for the world's stream and turn the device error word into a status.
int sync_and_check(cf_world* w)
{
    CF_CUDA(cudaMemcpyAsync(&w->host_words[0], w->err, sizeof(int), cudaMemcpyDeviceToHost, w->stream));
    CF_CUDA(cudaStreamSynchronize(w->stream));
    const int word = w->host_words[0];
    if (word) {
        CF_CUDA(cudaMemsetAsync(w->err, 0, sizeof(int), w->stream));
        CF_CUDA(cudaStreamSynchronize(w->stream));
        if (word & kDevErrWait) return fail(CF_ERR_DEVICE, "a bounded device wait gave up");
        if (word & kDevErrType) return fail(CF_ERR_DOMAIN, "a particle type is outside [0, T)");
        return fail(CF_ERR_DOMAIN, "a particle position is outside [0, extent) or not finite");
    }
    return CF_OK;
}

// Pair tables for a step (ParticleSimulation.cu:108-110, 116): effective
// radius per type pair in the reference's float expression, the exact
// sqrt threshold, and the force table; uploaded when anything changed.
int update_pair_tables(cf_world* w, const cf_step_params* p, float* r_cut, int* uniform_r, float* eff_u,
                       float* thr_u, float* thr_max_out)
{
    const int T = w->num_types;
    PairTables& h = w->host_tables;
    const float max_ext = std::max(p->canvas_width, std::max(p->canvas_height, p->canvas_depth));
    bool changed = w->uploaded_version != w->table_version || w->uploaded_radius != p->radius ||
                   w->uploaded_ratio != p->ratio_with_lfo || w->uploaded_types != T ||
                   w->uploaded_extent != max_ext;
    if (changed) {
        std::fill(std::begin(h.force), std::end(h.force), 0.0f);
        std::fill(std::begin(h.eff), std::end(h.eff), 0.0f);
        std::fill(std::begin(h.threshold), std::end(h.threshold), 0.0f);
        std::fill(std::begin(h.threshold_lo), std::end(h.threshold_lo), 0.0f);
        for (int a = 0; a < T; a++) {
            for (int b = 0; b < T; b++) {
                const float ra = p->radius * (1.0f + w->radio[a] * p->ratio_with_lfo);
                const float rb = p->radius * (1.0f + w->radio[b] * p->ratio_with_lfo);
                const float eff = (ra + rb) * 0.5f;
                const int k = a * kTableStride + b;
                h.force[k] = w->table[a * T + b];
                h.eff[k] = eff;
                h.threshold[k] = sqrt_threshold(eff);
                h.threshold_lo[k] = certain_bound(h.threshold[k], max_ext);
            }
        }
        CF_CUDA(cudaMemcpyAsync(w->tables, &h, sizeof(PairTables), cudaMemcpyHostToDevice, w->stream));
        w->uploaded_version = w->table_version;
        w->uploaded_radius = p->radius;
        w->uploaded_ratio = p->ratio_with_lfo;
        w->uploaded_types = T;
        w->uploaded_extent = max_ext;
    }
    float thr_max = 0.0f;
    bool uniform = true;
    const uint32_t* eff_bits = reinterpret_cast<const uint32_t*>(h.eff);
    for (int a = 0; a < T; a++)
        for (int b = 0; b < T; b++) {
            const int k = a * kTableStride + b;
            thr_max = std::max(thr_max, h.threshold[k]);
            uniform = uniform && eff_bits[k] == eff_bits[0];
        }
    *r_cut = cutoff_distance(thr_max);
    *thr_max_out = thr_max;
    *uniform_r = uniform ? 1 : 0;
    *eff_u = h.eff[0];
    *thr_u = h.threshold[0];
    return CF_OK;
}

int check_params(const cf_world* w, const cf_step_params* p)
{
    if (!p) return fail(CF_ERR_INVALID, "null step parameters");
    if (p->num_particle_types != w->num_types)
        return fail(CF_ERR_INVALID, "num_particle_types differs from the world's type count");
    if (!finite_positive(p->canvas_width) || !finite_positive(p->canvas_height) || !finite_positive(p->canvas_depth))
        return fail(CF_ERR_INVALID, "canvas extents must be finite and positive");
    if (!std::isfinite(p->radius)) return fail(CF_ERR_INVALID, "radius must be finite");
    return CF_OK;
}


// Bound below which the force kernel's contracted squared distance proves the
// exact test passes: d2a < bound  implies  fl(d2e + 1e-4) < t, with the same
// displacement slack as filter_bound.  Pairs between this and the filter
// bound take the exact test.
float certain_bound_impl(float thr, float max_extent)
{
    if (std::isinf(thr)) return INFINITY;
    const double b = (double)thr * (1.0 - 0x1p-22) - (double)0.0001f;
    if (!(b > 0.0)) return 0.0f;
    int ex = 0;
    std::frexp(2.0 * (double)max_extent, &ex);
    const double delta = 3.0 * std::ldexp(1.0, ex - 24);
    const double lo = b - 3.47 * delta * std::sqrt(b) - 3.0 * delta * delta - 0x1p-20 * b;
    if (!(lo > 0.0)) return 0.0f;
    return nextafterf((float)lo, 0.0f);
}

// Bound for the force kernel's approximate pre-test: every pair whose exact
// test fl(d^2 + 1e-4) < t passes fl(fma-contracted d^2 of a pre-shifted
// displacement) < bound.  The kernel's displacement (candidate plus rounded
// shift-minus-origin, less the rounded origin-relative home) and the
// reference's (difference, then wrap) each differ from the exact shifted
// difference by a few roundings at the box scale: together at most delta =
// 3 ulp(2 * extent) per axis.  The rest is relative rounding slack.
float filter_bound(float thr_max, float max_extent)
{
    if (std::isinf(thr_max)) return INFINITY;
    const double b = ((double)thr_max * (1.0 + 0x1p-24) - (double)0.0001f) / (1.0 - 0x1p-22);
    if (!(b > 0.0)) return -1.0f;
    int ex = 0;
    std::frexp(2.0 * (double)max_extent, &ex);
    const double delta = 3.0 * std::ldexp(1.0, ex - 24);  // 3 ulp of 2 * extent
    const double bound = (b + 3.47 * delta * std::sqrt(b) + 3.0 * delta * delta) * (1.0 + 0x1p-21);
    // On generic grids the kernel compares fma(dz, dz, fma(dy, dy, dx * dx)) with
    // this: three roundings of at most 2^-24 max(d^2, bound') each, covered by
    // bound' = bound (1 + 2^-19).  Elsewhere the kernel widens it again by the
    // rounding of its expanded form (at the scale of the stencil box).
    return nextafterf((float)(bound * (1.0 + 0x1p-19)), INFINITY);
}

int prepare_step(cf_world* w, const cf_step_params* p, StepConsts* c)
{
    int rc = check_params(w, p);
    if (rc) return rc;
    float r_cut = 0.0f, thr_max = 0.0f;
    std::memset(c, 0, sizeof(*c));
    rc = update_pair_tables(w, p, &r_cut, &c->uniform_r, &c->eff_uniform, &c->thr_uniform, &thr_max);
    if (rc) return rc;
    c->ext[0] = p->canvas_width;
    c->ext[1] = p->canvas_height;
    c->ext[2] = p->canvas_depth;
    for (int a = 0; a < 3; a++) c->half[a] = c->ext[a] * 0.5f;
    c->inv_eff_uniform = 1.0f / c->eff_uniform;
    c->thr_lo_uniform = w->host_tables.threshold_lo[0];
    if (w->force_variant < kForceStages * 3) {
        c->variant = w->force_variant % kForceStages;
        c->split = 1 << (w->force_variant / kForceStages);
    } else {
        // the balanced drain (staging 4): variants 12, 13, 14 for 1, 2, 4 warps per item
        c->variant = kForceStages;
        c->split = 1 << (w->force_variant - kForceStages * 3);
    }
    c->thr_filter = filter_bound(thr_max, std::max(c->ext[0], std::max(c->ext[1], c->ext[2])));
    c->grid = choose_step_grid(c->ext, r_cut, kMaxCells);
    apply_worlds(c->grid, w->worlds);
    // force tables: one per world (a plain world uses the pair tables' own)
    c->world_force = w->worlds > 1 ? w->world_tables : w->tables->force;
    c->n = w->n;
    c->num_types = w->num_types;
    c->repulsion = p->repulsion;
    c->attraction = p->attraction;
    c->neg_k = -p->k;
    c->balance = p->balance;
    c->force_multiplier = p->force_multiplier;
    c->delta_t = p->delta_t;
    c->friction = p->friction;
    c->max_expected_neighbors = p->max_expected_neighbors;
    return CF_OK;
}

// Extend a per-world grid to a batch of worlds sharing its shape.
void apply_worlds(Grid& g, int worlds)
{
    g.worlds = worlds;
    g.cells_w = g.m[0] * g.m[1] * g.m[2];
    g.cells = worlds * g.cells_w;
    g.key_bits = 0;
    while ((1ll << g.key_bits) < (long long)g.cells) g.key_bits++;
}

// One step's launches on the world's stream: cell list, then the fused force,
// density and integrator kernel; with the three profiling events when prof
// (recorded as external event nodes when the stream is being captured).
// The step's two phases.  The cell list leaves the sorted keys and values in
// buffer `which` of the scratch pair, a function of the grid alone
// (cell_list_csr_buffer), which the force kernel reads.
int enqueue_cell_list(cf_world* w, const StepConsts& c, int* which)
{
    Scratch& s = w->s;
    CF_CUDA(launch_cell_list_csr(w->pos, w->n, c.grid, c.ext, w->num_types, s, s.cell_off, s.items, s.n_items, w->err,
                                 which, w->stream));
    return CF_OK;
}

int enqueue_force(cf_world* w, const StepConsts& c, int which)
{
    Scratch& s = w->s;
    CF_CUDA(launch_step_force(c, w->tables, s.pos_sorted, s.keys[which], s.vals[which], s.cell_off, s.items,
                              s.n_items, max_step_items(w->n, c.grid), w->pos, w->vel, w->acc, w->counts,
                              w->stream));
    return CF_OK;
}

int enqueue_step(cf_world* w, const StepConsts& c, int prof)
{
    (void)prof;
    int which = 0;
    int rc = enqueue_cell_list(w, c, &which);
    if (rc) return rc;
    return enqueue_force(w, c, which);
}

// The one-step graph for these constants (prof = 1: the cell list alone),
// captured on first use and again whenever the constants or the scratch
// buffers change.
int step_graph(cf_world* w, const StepConsts& c, int prof, cudaGraphExec_t* out)
{
    const void* bufs = w->s.cell_start;
    if (w->graph[prof] && w->graph_bufs[prof] == bufs && std::memcmp(&w->graph_key[prof], &c, sizeof(c)) == 0) {
        *out = w->graph[prof];
        return CF_OK;
    }
    if (w->graph[prof]) {
        cudaGraphExecDestroy(w->graph[prof]);
        w->graph[prof] = nullptr;
    }
    cudaGraph_t graph = nullptr;
    CF_CUDA(cudaStreamBeginCapture(w->stream, cudaStreamCaptureModeThreadLocal));
    int which = 0;
    int rc = prof ? enqueue_cell_list(w, c, &which) : enqueue_step(w, c, 0);
    cudaError_t e = cudaStreamEndCapture(w->stream, &graph);
    if (rc) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    e = graph_kernel_count(graph, &w->graph_kernels[prof]);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&w->graph[prof], graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    w->graph_key[prof] = c;
    w->graph_bufs[prof] = bufs;
    *out = w->graph[prof];
    return CF_OK;
}

// Adds the phase times of the `count` oldest profiled steps of the ring (waiting
// for each one's last event) to the world's totals.
int harvest_profile(cf_world* w, int count)
{
    const int size = (int)w->prof_ring.size();
    for (int k = 0; k < count && w->prof_pending > 0; k++) {
        const int slot = ((w->prof_head - w->prof_pending) % size + size) % size;
        const auto& ev = w->prof_ring[slot];
        CF_CUDA(cudaEventSynchronize(ev[2]));
        float a = 0.0f, b = 0.0f;
        CF_CUDA(cudaEventElapsedTime(&a, ev[0], ev[1]));
        if (w->prof_kind[slot] == 0) {
            CF_CUDA(cudaEventElapsedTime(&b, ev[1], ev[2]));
            w->prof_cell_ms += a;
            w->prof_force_ms += b;
            w->prof_steps++;
        } else {
            w->prof_adj_ms += a;
            w->prof_adj_steps++;
        }
        w->prof_pending--;
    }
    return CF_OK;
}

int respawn(cf_world* w, uint64_t seed, float spawn_region)
{
    float lo[3], span[3];
    for (int a = 0; a < 3; a++) {
        span[a] = std::min(spawn_region, w->ext[a]);
        lo[a] = (w->ext[a] - span[a]) * 0.5f;
    }
    CF_CUDA(launch_init_particles(w->pos, w->vel, w->acc, w->counts, w->n, w->num_types, lo, span, seed, w->stream));
    return CF_OK;
}

void seed_tables(cf_world* w, uint64_t seed)
{
    uint64_t s = seed ^ 0xC3A5C85C97CB3127ull;
    const int T = w->num_types;
    for (int i = 0; i < T * T; i++) w->raw[i] = uniform_pm1(s);
    for (int i = 0; i < T; i++) w->radio[i] = uniform_pm1(s);
}

void transform_table(cf_world* w, float range, float bias, float offset)
{
    // ParticleSimulation.cu:524-527, tanh on a float resolves to tanhf
    const int T = w->num_types;
    for (int i = 0; i < T * T; i++) {
        const float t = tanhf(w->raw[i] * offset) * range + bias;
        w->table[i] = fmaxf(-1.0f, fminf(1.0f, t));
    }
    w->table_version++;
}

}  // namespace

int fail(int code, const std::string& msg)
{
    g_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what)
{
    g_error = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation && g_mem_capped) {
        g_error += " (the library's device memory limit of " + std::to_string(g_mem_limit) +
                   " bytes would be exceeded; cf_set_device_memory_limit)";
        g_mem_capped = false;
    }
    return e == cudaErrorMemoryAllocation ? CF_ERR_ALLOC : CF_ERR_CUDA;
}

cudaError_t injected_error(const char* site)
{
    if (!g_inj_armed.load(std::memory_order_relaxed)) return cudaSuccess;
    std::lock_guard<std::mutex> lock(g_inj_mu);
    if (!g_inj_armed.load(std::memory_order_relaxed) || std::strstr(site, g_inj_site.c_str()) == nullptr)
        return cudaSuccess;
    if (g_inj_skip > 0) {
        g_inj_skip--;
        return cudaSuccess;
    }
    g_inj_armed.store(false, std::memory_order_relaxed);
    return g_inj_error;
}

namespace {
std::atomic<long long> g_launches{0};
}

void note_launches(cudaStream_t st, long long k)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    // a launch recorded into a graph is counted when the graph is launched
    if (cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) return;
    g_launches.fetch_add(k, std::memory_order_relaxed);
}

long long launch_tally() { return g_launches.load(std::memory_order_relaxed); }

cudaError_t graph_kernel_count(cudaGraph_t graph, long long* kernels)
{
    *kernels = 0;
    size_t nodes = 0;
    cudaError_t e = cudaGraphGetNodes(graph, nullptr, &nodes);
    if (e != cudaSuccess || nodes == 0) return e;
    std::vector<cudaGraphNode_t> list(nodes);
    e = cudaGraphGetNodes(graph, list.data(), &nodes);
    for (size_t i = 0; i < nodes && e == cudaSuccess; i++) {
        cudaGraphNodeType t;
        e = cudaGraphNodeGetType(list[i], &t);
        if (e == cudaSuccess && t == cudaGraphNodeTypeKernel) ++*kernels;
    }
    return e;
}

// Smallest float t >= 0 with sqrtf(t) >= eff.  sqrtf is monotone, so for
// every s: sqrtf(s) < eff  <=>  s < t.
float sqrt_threshold(float eff)
{
    if (!(eff > 0.0f)) return 0.0f;
    if (std::isinf(eff)) return INFINITY;
    float t = eff * eff;
    if (std::isinf(t)) t = FLT_MAX;
    while (t > 0.0f && sqrtf(t) >= eff) t = nextafterf(t, 0.0f);
    while (sqrtf(t) < eff) {
        t = nextafterf(t, INFINITY);
        if (std::isinf(t)) break;
    }
    return t;
}

float certain_bound(float threshold, float max_extent) { return certain_bound_impl(threshold, max_extent); }

// Largest true distance a pair can have and still pass fl(d^2 + 1e-4) < t,
// with slack for the rounding of the displacement, the squares and sums.
float cutoff_distance(float threshold)
{
    if (std::isinf(threshold)) return INFINITY;
    double t = (double)threshold * (1.0 + 0x1p-22) - 0.0001 * (1.0 - 0x1p-22);
    if (!(t > 0.0)) return 0.0f;
    return (float)(std::sqrt(t / (1.0 - 0x1p-20)) * (1.0 + 0x1p-20));
}

namespace {

// Cells per axis for a cutoff: the largest m whose cell side exceeds the
// cutoff by the hash rounding slack (cell coordinates are computed as
// fl(x * fl(m / L)), off by at most m * 2^-23 cells).
int cells_for_cutoff(double extent, double cut)
{
    if (!(cut > 0.0) || !std::isfinite(cut)) return cut > 0.0 ? 1 : 4096;
    double m = std::floor(extent / cut);
    if (m > 4096) m = 4096;
    if (m < 1) m = 1;
    int mi = (int)m;
    while (mi > 1 && extent / mi < cut / (1.0 - 4.0 * mi * 0x1p-23) * (1.0 + 0x1p-20)) mi--;
    return mi;
}

void finish_grid(Grid& g, const float* ext, int max_cells)
{
    // cap the total by coarsening the finest axis
    while ((long long)g.m[0] * g.m[1] * g.m[2] > max_cells) {
        int a = 0;
        for (int b = 1; b < 3; b++)
            if (g.m[b] > g.m[a]) a = b;
        g.m[a] = std::max(1, g.m[a] * 3 / 4);
    }
    if (g.periodic) {
        g.generic = 0;
        for (int a = 0; a < 3; a++)
            if (g.m[a] < 5) g.generic = 1;
        if (g.generic)
            for (int a = 0; a < 3; a++)
                if (g.m[a] < 3) g.m[a] = 1;
    }
    for (int a = 0; a < 3; a++) g.inv[a] = (float)((double)g.m[a] / (double)ext[a]);
    g.cells = g.m[0] * g.m[1] * g.m[2];
    g.worlds = 1;
    g.cells_w = g.cells;
    g.key_bits = 0;
    while ((1ll << g.key_bits) < (long long)g.cells) g.key_bits++;
}

}  // namespace

Grid choose_step_grid(const float* ext, float r_cut, int max_cells)
{
    Grid g;
    std::memset(&g, 0, sizeof(g));
    g.periodic = 1;
    for (int a = 0; a < 3; a++) g.m[a] = cells_for_cutoff(ext[a], r_cut);
    finish_grid(g, ext, max_cells);
    return g;
}

Grid choose_prox_grid(const float* ext, float distance, int max_cells)
{
    Grid g;
    std::memset(&g, 0, sizeof(g));
    g.periodic = 0;
    double dsq = (double)(distance * distance);
    double cut = std::sqrt(dsq * (1.0 + 0x1p-22) / (1.0 - 0x1p-20)) * (1.0 + 0x1p-20);
    for (int a = 0; a < 3; a++) g.m[a] = distance > 0.0f ? cells_for_cutoff(ext[a], cut) : 1;
    finish_grid(g, ext, max_cells);
    return g;
}

// The work model's grid: floor(L / r_max) cells per axis of side L / cells.
Grid canonical_grid(const float* ext, float r_max)
{
    Grid g;
    std::memset(&g, 0, sizeof(g));
    g.periodic = 1;
    for (int a = 0; a < 3; a++) {
        double m = r_max > 0.0f ? std::floor((double)ext[a] / (double)r_max) : 1.0;
        g.m[a] = (int)std::min(std::max(m, 1.0), 4096.0);
    }
    while ((long long)g.m[0] * g.m[1] * g.m[2] > kMaxCanonicalCells) {
        int a = 0;
        for (int b = 1; b < 3; b++)
            if (g.m[b] > g.m[a]) a = b;
        g.m[a] = std::max(1, g.m[a] * 3 / 4);
    }
    for (int a = 0; a < 3; a++) g.inv[a] = (float)((double)g.m[a] / (double)ext[a]);
    g.cells = g.m[0] * g.m[1] * g.m[2];
    g.worlds = 1;
    g.cells_w = g.cells;
    return g;
}

}  // namespace cf

using namespace cf;

extern "C" {

const char* cf_last_error(void) { return g_error.c_str(); }

const char* cf_version(void) { return "cellflow-gb300 0.1 (sm_103a)"; }

long long cf_kernel_launches(void) { return launch_tally(); }

int cf_set_device_memory_limit(size_t bytes)
{
    std::lock_guard<std::mutex> lock(g_mem_mu);
    g_mem_limit = bytes;
    return CF_OK;
}

int cf_device_memory_in_use(size_t* bytes)
{
    if (!bytes) return fail(CF_ERR_INVALID, "null output");
    std::lock_guard<std::mutex> lock(g_mem_mu);
    *bytes = g_mem_live;
    return CF_OK;
}

int cf_inject_cuda_error(const char* site, int cuda_error, int skip)
{
    std::lock_guard<std::mutex> lock(g_inj_mu);
    if (!site) {
        g_inj_armed.store(false);
        return CF_OK;
    }
    if (cuda_error <= 0 || skip < 0) return fail(CF_ERR_INVALID, "cuda_error must be a cudaError_t > 0, skip >= 0");
    g_inj_site = site;
    g_inj_error = static_cast<cudaError_t>(cuda_error);
    g_inj_skip = skip;
    g_inj_armed.store(true);
    return CF_OK;
}

int cf_injection_pending(void) { return g_inj_armed.load() ? 1 : 0; }

void cf_default_params(cf_step_params* p)
{
    if (!p) return;
    // SimulationParams.h:15-29
    p->radius = 42.07f;
    p->delta_t = 0.18f;
    p->friction = 0.51f;
    p->repulsion = 64.83f;
    p->attraction = 3.06f;
    p->k = 29.45f;
    p->balance = 0.79f;
    p->canvas_width = 8000.0f;
    p->canvas_height = 8000.0f;
    p->canvas_depth = 8000.0f;
    p->num_particle_types = 6;
    p->ratio_with_lfo = 0.0f;
    p->force_multiplier = 2.33f;
    p->max_expected_neighbors = 400;
}

int cf_create(int n, int num_types, float w_, float h_, float d_, uint64_t seed, cf_world** out)
{
    if (!out) return fail(CF_ERR_INVALID, "null output handle");
    *out = nullptr;
    if (n < 0) return fail(CF_ERR_INVALID, "particle count must be >= 0");
    if (num_types < 1 || num_types > CF_MAX_TYPES) return fail(CF_ERR_INVALID, "type count must be in [1, 32]");
    if (!finite_positive(w_) || !finite_positive(h_) || !finite_positive(d_))
        return fail(CF_ERR_INVALID, "box extents must be finite and positive");
    cf_world* w = new cf_world();
    w->n = n;
    w->num_types = num_types;
    w->ext[0] = w_;
    w->ext[1] = h_;
    w->ext[2] = d_;
    std::memset(w->raw, 0, sizeof(w->raw));
    std::memset(w->table, 0, sizeof(w->table));
    std::memset(w->radio, 0, sizeof(w->radio));
    auto bail = [&](int rc) {
        cf_destroy(w);
        return rc;
    };
    cudaError_t e = cudaGetDevice(&w->device);
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaGetDevice"));
    e = cudaStreamCreateWithFlags(&w->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaStreamCreateWithFlags"));
    w->stream = w->own_stream;
    e = dev_alloc(&w->err, 1);
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaMalloc(error word)"));
    e = cudaMallocHost(&w->host_words, 4 * sizeof(int));
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaMallocHost(status words)"));
    std::memset(w->host_words, 0, 4 * sizeof(int));
    e = cudaMemsetAsync(w->err, 0, sizeof(int), w->stream);
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaMemsetAsync"));
    e = dev_alloc(&w->tables, 1);
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaMalloc(tables)"));
    e = configure_step_force();
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaFuncSetAttribute(step_force_kernel)"));
    int rc = alloc_particles(w);
    if (rc) return bail(rc);
    // ParticleSimulation.cu:430-434: particles, force table (0.28, -0.20, 1.0), radius table
    seed_tables(w, seed);
    transform_table(w, 0.28f, -0.20f, 1.0f);
    rc = respawn(w, seed, 2000.0f);
    if (rc) return bail(rc);
    rc = sync_and_check(w);
    if (rc) return bail(rc);
    *out = w;
    return CF_OK;
}

int cf_destroy(cf_world* w)
{
    if (!w) return CF_OK;
    if (w->stream) cudaStreamSynchronize(w->stream);
    for (auto& ev : w->prof_ring)
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
    w->prof_ring.clear();
    drop_graphs(w);
    free_particles(w);
    dev_free(w->err);
    if (w->host_words) cudaFreeHost(w->host_words);
    dev_free(w->tables);
    dev_free(w->world_tables);
    if (w->own_stream) cudaStreamDestroy(w->own_stream);
    delete w;
    return CF_OK;
}

int cf_set_stream(cf_world* w, void* stream)
{
    int rc = check_world(w);
    if (rc) return rc;
    CF_CUDA(cudaStreamSynchronize(w->stream));
    w->stream = stream ? (cudaStream_t)stream : w->own_stream;
    return CF_OK;
}

int cf_sync(cf_world* w)
{
    int rc = check_world(w);
    if (rc) return rc;
    return sync_and_check(w);
}

int cf_particle_count(const cf_world* w, int* n)
{
    int rc = check_world(w);
    if (rc) return rc;
    if (!n) return fail(CF_ERR_INVALID, "null output");
    *n = w->n;
    return CF_OK;
}

int cf_num_particle_types(const cf_world* w, int* t)
{
    int rc = check_world(w);
    if (rc) return rc;
    if (!t) return fail(CF_ERR_INVALID, "null output");
    *t = w->num_types;
    return CF_OK;
}

int cf_set_particle_count(cf_world* w, int n, uint64_t seed)
{
    if (!w) return fail(CF_ERR_INVALID, "null world");  // a broken world may be reallocated
    if (n < 0) return fail(CF_ERR_INVALID, "particle count must be >= 0");
    if (n == w->n && !w->broken) return CF_OK;  // ParticleSimulation.cu:565
    CF_CUDA(cudaStreamSynchronize(w->stream));
    free_particles(w);
    w->n = n;
    int rc = alloc_particles(w);
    if (rc) {
        // no half-allocated world: every later call reports this until a reallocation succeeds
        const std::string msg = cf_last_error();
        free_particles(w);
        w->broken = true;
        return fail(rc, msg);
    }
    w->broken = false;
    rc = respawn(w, seed, 2000.0f);
    if (rc) return rc;
    return sync_and_check(w);
}

int cf_set_num_particle_types(cf_world* w, int t, uint64_t seed)
{
    int rc = check_world(w);
    if (rc) return rc;
    if (t < 1 || t > CF_MAX_TYPES) return fail(CF_ERR_INVALID, "type count must be in [1, 32]");
    w->num_types = t;  // ParticleSimulation.cu:575-578
    seed_tables(w, seed);
    transform_table(w, 0.28f, -0.20f, 1.0f);
    rc = respawn(w, seed, 2000.0f);
    if (rc) return rc;
    return sync_and_check(w);
}

int cf_set_canvas(cf_world* w, float width, float height, float depth)
{
    int rc = check_world(w);
    if (rc) return rc;
    if (!finite_positive(width) || !finite_positive(height) || !finite_positive(depth))
        return fail(CF_ERR_INVALID, "box extents must be finite and positive");
    if (width == w->ext[0] && height == w->ext[1] && depth == w->ext[2]) return CF_OK;
    // the cached selection graphs hold the old extents as kernel arguments
    CF_CUDA(cudaStreamSynchronize(w->stream));
    drop_graphs(w);
    w->ext[0] = width;
    w->ext[1] = height;
    w->ext[2] = depth;
    return CF_OK;
}

int cf_move_universe(cf_world* w, float dx, float dy, float dz)
{
    int rc = check_world(w);
    if (rc) return rc;
    if (!std::isfinite(dx) || !std::isfinite(dy) || !std::isfinite(dz))
        return fail(CF_ERR_INVALID, "the shift must be finite");
    CF_CUDA(launch_move_particles(w->pos, w->n, dx, dy, dz, w->ext, w->stream));
    return CF_OK;
}

int cf_initialize_particles(cf_world* w, uint64_t seed, float spawn_region)
{
    int rc = check_world(w);
    if (rc) return rc;
    if (!(spawn_region > 0.0f)) return fail(CF_ERR_INVALID, "spawn region must be positive");
    rc = respawn(w, seed, spawn_region);
    if (rc) return rc;
    return sync_and_check(w);
}

namespace {
void* device_view(const void* p);  // page-locked host memory's device view, or nullptr
}  // namespace

int cf_get_particles(cf_world* w, cf_particle* out, int n)
{
    int rc = check_world(w);
    if (rc) return rc;
    if (n != w->n || (!out && n > 0)) return fail(CF_ERR_INVALID, "output must hold exactly n particles");
    rc = ensure_aos(w);
    if (rc) return rc;
    if (void* dout = n > 0 ? device_view(out) : nullptr) {
        // page-locked: written word by word through its device view, no staging copy
        CF_CUDA(launch_soa_to_aos_mapped(w->pos, w->vel, w->acc, static_cast<cf_particle*>(dout), n, w->stream));
        return sync_and_check(w);
    }
    CF_CUDA(launch_soa_to_aos(w->pos, w->vel, w->acc, w->aos, n, w->stream));
    if (n > 0)
        CF_CUDA(cudaMemcpyAsync(out, w->aos, sizeof(cf_particle) * (size_t)n, cudaMemcpyDeviceToHost, w->stream));
    return sync_and_check(w);
}

int cf_set_particles(cf_world* w, const cf_particle* in, int n)
{
    int rc = check_world(w);
    if (rc) return rc;
    if (n != w->n || (!in && n > 0)) return fail(CF_ERR_INVALID, "input must hold exactly n particles");
    rc = ensure_aos(w);
    if (rc) return rc;
    if (const void* din = n > 0 ? device_view(in) : nullptr) {
        // page-locked: read word by word through its device view, no staging copy
        CF_CUDA(launch_aos_to_soa_mapped(static_cast<const cf_particle*>(din), w->pos, w->vel, w->acc, n, w->stream));
        return CF_OK;
    }
    if (n > 0)
        CF_CUDA(cudaMemcpyAsync(w->aos, in, sizeof(cf_particle) * (size_t)n, cudaMemcpyHostToDevice, w->stream));
    CF_CUDA(launch_aos_to_soa(w->aos, w->pos, w->vel, w->acc, n, w->stream));
    return CF_OK;
}

int cf_get_state(cf_world* w, float* pos4, float* vel4, int* counts)
{
    int rc = check_world(w);
    if (rc) return rc;
    const size_t n = (size_t)w->n;
    if (n > 0) {
        if (pos4) CF_CUDA(cudaMemcpyAsync(pos4, w->pos, 16 * n, cudaMemcpyDeviceToHost, w->stream));
        if (vel4) CF_CUDA(cudaMemcpyAsync(vel4, w->vel, 16 * n, cudaMemcpyDeviceToHost, w->stream));
        if (counts) CF_CUDA(cudaMemcpyAsync(counts, w->counts, 4 * n, cudaMemcpyDeviceToHost, w->stream));
    }
    return sync_and_check(w);
}

int cf_set_state(cf_world* w, const float* pos4, const float* vel4, const int* counts)
{
    int rc = check_world(w);
    if (rc) return rc;
    const size_t n = (size_t)w->n;
    if (n > 0) {
        if (pos4) CF_CUDA(cudaMemcpyAsync(w->pos, pos4, 16 * n, cudaMemcpyHostToDevice, w->stream));
        if (vel4) CF_CUDA(cudaMemcpyAsync(w->vel, vel4, 16 * n, cudaMemcpyHostToDevice, w->stream));
        if (counts) CF_CUDA(cudaMemcpyAsync(w->counts, counts, 4 * n, cudaMemcpyHostToDevice, w->stream));
    }
    CF_CUDA(cudaStreamSynchronize(w->stream));
    return CF_OK;
}

int cf_get_neighbor_counts(cf_world* w, int* out, int n)
{
    int rc = check_world(w);
    if (rc) return rc;
    if (n != w->n || (!out && n > 0)) return fail(CF_ERR_INVALID, "output must hold exactly n counts");
    if (n > 0) CF_CUDA(cudaMemcpyAsync(out, w->counts, 4 * (size_t)n, cudaMemcpyDeviceToHost, w->stream));
    return sync_and_check(w);
}

int cf_device_buffers(cf_world* w, cf_device_view* out)
{
    int rc = check_world(w);
    if (rc) return rc;
    if (!out) return fail(CF_ERR_INVALID, "null output");
    out->pos4 = w->pos;
    out->vel4 = w->vel;
    out->acc4 = w->acc;
    out->counts = w->counts;
    out->n = w->n;
    return CF_OK;
}

int cf_get_raw_force_table(cf_world* w, float* raw, int count)
{
    int rc = check_world(w);
    if (rc) return rc;
    if (!raw || count != w->num_types * w->num_types) return fail(CF_ERR_INVALID, "count must be T*T");
    std::memcpy(raw, w->raw, sizeof(float) * count);
    return CF_OK;
}

int cf_set_raw_force_table(cf_world* w, const float* raw, int count)
{
    int rc = check_world(w);
    if (rc) return rc;
    if (!raw || count != w->num_types * w->num_types) return fail(CF_ERR_INVALID, "count must be T*T");
    std::memcpy(w->raw, raw, sizeof(float) * count);
    return CF_OK;
}

int cf_regenerate_force_table(cf_world* w, uint64_t seed)
{
    int rc = check_world(w);
    if (rc) return rc;
    // ParticleSimulation.cu:513-519: new raw values, then (0.28, -0.20, 1.0)
    uint64_t s = seed ^ 0x2545F4914F6CDD1Dull;
    for (int i = 0; i < w->num_types * w->num_types; i++) w->raw[i] = uniform_pm1(s);
    transform_table(w, 0.28f, -0.20f, 1.0f);
    return CF_OK;
}

int cf_update_force_table(cf_world* w, float range, float bias, float offset)
{
    int rc = check_world(w);
    if (rc) return rc;
    transform_table(w, range, bias, offset);
    return CF_OK;
}

int cf_set_force_table(cf_world* w, const float* table, int count)
{
    int rc = check_world(w);
    if (rc) return rc;
    if (!table || count != w->num_types * w->num_types) return fail(CF_ERR_INVALID, "count must be T*T");
    std::memcpy(w->table, table, sizeof(float) * count);
    w->table_version++;
    return CF_OK;
}

int cf_get_force_table(cf_world* w, float* table, int count)
{
    int rc = check_world(w);
    if (rc) return rc;
    if (!table || count != w->num_types * w->num_types) return fail(CF_ERR_INVALID, "count must be T*T");
    std::memcpy(table, w->table, sizeof(float) * count);
    return CF_OK;
}

int cf_get_radio_by_type(cf_world* w, float* out, int count)
{
    int rc = check_world(w);
    if (rc) return rc;
    if (!out || count != w->num_types) return fail(CF_ERR_INVALID, "count must be T");
    std::memcpy(out, w->radio, sizeof(float) * count);
    return CF_OK;
}

int cf_set_radio_by_type(cf_world* w, const float* values, int count)
{
    int rc = check_world(w);
    if (rc) return rc;
    if (!values || count != w->num_types) return fail(CF_ERR_INVALID, "count must be T");
    std::memcpy(w->radio, values, sizeof(float) * count);
    w->table_version++;
    return CF_OK;
}

int cf_set_radio_by_type_value(cf_world* w, int index, float value)
{
    int rc = check_world(w);
    if (rc) return rc;
    // ParticleSimulation.cu:615-622: out-of-range indices are ignored
    if (index >= 0 && index < w->num_types) {
        w->radio[index] = value;
        w->table_version++;
    }
    return CF_OK;
}

int cf_rotate_radio_by_type(cf_world* w)
{
    int rc = check_world(w);
    if (rc) return rc;
    // ParticleSimulation.cu:594-600
    const int T = w->num_types;
    const float last = w->radio[T - 1];
    for (int i = T - 1; i > 0; i--) w->radio[i] = w->radio[i - 1];
    w->radio[0] = last;
    w->table_version++;
    return CF_OK;
}

float cf_lfo_ratio(float ratio, float lfo_a, float lfo_s, float t_seconds)
{
    // CellFlowWidget.cpp:414-421
    if (lfo_a != 0.0f) {
        const float lfo = (float)(lfo_a * std::sin(2.0f * M_PI * lfo_s * t_seconds));
        return ratio + lfo;
    }
    return ratio;
}

int cf_step(cf_world* w, const cf_step_params* p, int nsteps)
{
    int rc = check_world(w);
    if (rc) return rc;
    if (nsteps < 0) return fail(CF_ERR_INVALID, "nsteps must be >= 0");
    StepConsts c;
    rc = prepare_step(w, p, &c);
    if (rc) return rc;
    rc = ensure_cells(w, c.grid.cells);
    if (rc) return rc;
    rc = ensure_plan(w, c.grid);
    if (rc) return rc;
    rc = ensure_offsets(w, c.grid.cells);
    if (rc) return rc;
    const int prof = w->profiling ? 1 : 0;
    cudaGraphExec_t exec = nullptr;
    if (w->use_graphs && w->stream != nullptr && nsteps > 0) {
        rc = step_graph(w, c, prof, &exec);
        if (rc) return rc;
    }
    const long long launches = cell_list_csr_launches(w->n, c.grid, true) + step_launches(w->n);
    for (int s = 0; s < nsteps; s++) {
        if (!prof) {
            if (exec) {
                CF_CUDA(cudaGraphLaunch(exec, w->stream));
                note_launches(w->stream, w->graph_kernels[0]);
            } else {
                rc = enqueue_step(w, c, 0);
                if (rc) return rc;
            }
            continue;
        }
        // profiled: events from the ring around the cell list (its graph) and the force kernel
        if (w->prof_pending == (int)w->prof_ring.size()) {
            rc = harvest_profile(w, 1);
            if (rc) return rc;
        }
        const auto& ev = w->prof_ring[w->prof_head];
        w->prof_kind[w->prof_head] = 0;
        w->prof_head = (w->prof_head + 1) % (int)w->prof_ring.size();
        w->prof_pending++;
        CF_CUDA(cudaEventRecord(ev[0], w->stream));
        int which = 0;
        if (exec) {
            CF_CUDA(cudaGraphLaunch(exec, w->stream));
            note_launches(w->stream, w->graph_kernels[1]);
            which = cell_list_csr_buffer(w->n, c.grid);
        } else {
            rc = enqueue_cell_list(w, c, &which);
            if (rc) return rc;
        }
        CF_CUDA(cudaEventRecord(ev[1], w->stream));
        rc = enqueue_force(w, c, which);
        if (rc) return rc;
        CF_CUDA(cudaEventRecord(ev[2], w->stream));
        w->prof_launches += launches;
    }
    return CF_OK;
}

namespace {

// Page-locked host memory (cudaHostAlloc or cudaHostRegister): copies from and
// to it can be recorded in a CUDA graph.
// The device view of page-locked host memory, or nullptr (pageable memory,
// device memory, or a pointer the runtime does not know).
void* device_view(const void* p)
{
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

bool page_locked(const void* p)
{
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

// Records upload, step and read-back (and the error word's read-back) on the
// world's stream.  Page-locked records are read and written in place over the
// CPU-GPU link by the conversion kernels (one 32-bit word per thread, so a warp
// moves 128 contiguous bytes; 16-B accesses in tiles of records moved no more
// over the link); pageable ones go through the device staging buffer.
int enqueue_host_step(cf_world* w, const StepConsts& c, const cf_particle* in, cf_particle* out)
{
    const size_t bytes = sizeof(cf_particle) * (size_t)w->n;
    // records in and out by kernels reading and writing the page-locked buffers
    // through their device views (no staging copies); a buffer without one takes
    // the staging path
    if (const void* din = device_view(in)) {
        CF_CUDA(launch_aos_to_soa_mapped(static_cast<const cf_particle*>(din), w->pos, w->vel, w->acc, w->n,
                                         w->stream));
    } else {
        CF_CUDA(cudaMemcpyAsync(w->aos, in, bytes, cudaMemcpyHostToDevice, w->stream));
        CF_CUDA(launch_aos_to_soa(w->aos, w->pos, w->vel, w->acc, w->n, w->stream));
    }
    int rc = enqueue_step(w, c, 0);
    if (rc) return rc;
    if (void* dout = device_view(out)) {
        CF_CUDA(launch_soa_to_aos_mapped(w->pos, w->vel, w->acc, static_cast<cf_particle*>(dout), w->n, w->stream));
    } else {
        CF_CUDA(launch_soa_to_aos(w->pos, w->vel, w->acc, w->aos, w->n, w->stream));
        CF_CUDA(cudaMemcpyAsync(out, w->aos, bytes, cudaMemcpyDeviceToHost, w->stream));
    }
    CF_CUDA(cudaMemcpyAsync(&w->host_words[0], w->err, sizeof(int), cudaMemcpyDeviceToHost, w->stream));
    return CF_OK;
}

}  // namespace

int cf_step_host(cf_world* w, const cf_step_params* p, const cf_particle* in, cf_particle* out, int n)
{
    int rc = check_world(w);
    if (rc) return rc;
    if (n != w->n || ((!in || !out) && n > 0)) return fail(CF_ERR_INVALID, "in and out must hold exactly n particles");
    rc = ensure_aos(w);
    if (rc) return rc;
    const bool graphed = n > 0 && w->use_graphs && w->stream != nullptr && !w->profiling && page_locked(in) &&
                         page_locked(out);
    if (!graphed) {
        rc = cf_set_particles(w, in, n);
        if (!rc) rc = cf_step(w, p, 1);
        if (!rc) rc = cf_get_particles(w, out, n);
        return rc;
    }
    StepConsts c;
    rc = prepare_step(w, p, &c);
    if (!rc) rc = ensure_cells(w, c.grid.cells);
    if (!rc) rc = ensure_plan(w, c.grid);
    if (!rc) rc = ensure_offsets(w, c.grid.cells);
    if (rc) return rc;
    const void* bufs = w->s.cell_start;
    if (!(w->host_graph && w->host_in == in && w->host_out == out && w->host_bufs == bufs &&
          std::memcmp(&w->host_key, &c, sizeof(c)) == 0)) {
        if (w->host_graph) cudaGraphExecDestroy(w->host_graph);
        w->host_graph = nullptr;
        cudaGraph_t graph = nullptr;
        CF_CUDA(cudaStreamBeginCapture(w->stream, cudaStreamCaptureModeThreadLocal));
        rc = enqueue_host_step(w, c, in, out);
        cudaError_t e = cudaStreamEndCapture(w->stream, &graph);
        if (rc) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
        e = graph_kernel_count(graph, &w->host_graph_kernels);
        if (e == cudaSuccess) e = cudaGraphInstantiate(&w->host_graph, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
        w->host_key = c;
        w->host_in = in;
        w->host_out = out;
        w->host_bufs = bufs;
    }
    CF_CUDA(cudaGraphLaunch(w->host_graph, w->stream));
    note_launches(w->stream, w->host_graph_kernels);
    CF_CUDA(cudaStreamSynchronize(w->stream));
    const int word = w->host_words[0];
    if (word) {
        CF_CUDA(cudaMemsetAsync(w->err, 0, sizeof(int), w->stream));
        CF_CUDA(cudaStreamSynchronize(w->stream));
        if (word & kDevErrWait) return fail(CF_ERR_DEVICE, "a bounded device wait gave up");
        if (word & kDevErrType) return fail(CF_ERR_DOMAIN, "a particle type is outside [0, T)");
        return fail(CF_ERR_DOMAIN, "a particle position is outside [0, extent) or not finite");
    }
    return CF_OK;
}

int cf_set_force_variant(cf_world* w, int variant)
{
    int rc = check_world(w);
    if (rc) return rc;
    if (variant < 0 || variant >= CF_FORCE_VARIANTS) return fail(CF_ERR_INVALID, "force variant must be in [0, 15)");
    w->force_variant = variant;
    return CF_OK;
}

int cf_autotune_step(cf_world* w, const cf_step_params* p, int steps, int* chosen_variant)
{
    int rc = check_world(w);
    if (rc) return rc;
    if (steps < 1) steps = 1;
    const size_t n = (size_t)w->n;
    if (n == 0) return CF_OK;
    // the trial steps must leave the world as it was: save the state
    float4 *pos = nullptr, *vel = nullptr, *acc = nullptr;
    int* cnt = nullptr;
    CF_CUDA(dev_alloc(&pos, n));
    CF_CUDA(dev_alloc(&vel, n));
    CF_CUDA(dev_alloc(&acc, n));
    CF_CUDA(dev_alloc(&cnt, n));
    auto save = [&](bool to_backup) -> cudaError_t {
        cudaError_t e = cudaSuccess;
        const cudaMemcpyKind k = cudaMemcpyDeviceToDevice;
        if (to_backup) {
            e = cudaMemcpyAsync(pos, w->pos, 16 * n, k, w->stream);
            if (!e) e = cudaMemcpyAsync(vel, w->vel, 16 * n, k, w->stream);
            if (!e) e = cudaMemcpyAsync(acc, w->acc, 16 * n, k, w->stream);
            if (!e) e = cudaMemcpyAsync(cnt, w->counts, 4 * n, k, w->stream);
        } else {
            e = cudaMemcpyAsync(w->pos, pos, 16 * n, k, w->stream);
            if (!e) e = cudaMemcpyAsync(w->vel, vel, 16 * n, k, w->stream);
            if (!e) e = cudaMemcpyAsync(w->acc, acc, 16 * n, k, w->stream);
            if (!e) e = cudaMemcpyAsync(w->counts, cnt, 4 * n, k, w->stream);
        }
        return e;
    };
    float best_ms = 1e30f;
    int best = w->force_variant;
    const int saved_variant = w->force_variant;
    const bool saved_prof = w->profiling;
    w->profiling = false;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaEventCreate(&e0);
    if (!e) e = cudaEventCreate(&e1);
    if (!e) e = save(true);
    for (int k = 0; k < CF_FORCE_VARIANTS && !e && rc == CF_OK; k++) {
        w->force_variant = k;
        rc = cf_step(w, p, 1);  // capture and warm
        if (rc) break;
        e = cudaEventRecord(e0, w->stream);
        if (!e) rc = cf_step(w, p, steps);
        if (!e && !rc) e = cudaEventRecord(e1, w->stream);
        if (!e && !rc) e = cudaEventSynchronize(e1);
        float ms = 0.0f;
        if (!e && !rc) e = cudaEventElapsedTime(&ms, e0, e1);
        if (!e && !rc && ms < best_ms) {
            best_ms = ms;
            best = k;
        }
        if (!e) e = save(false);
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaStreamSynchronize(w->stream);
    dev_free(pos);
    dev_free(vel);
    dev_free(acc);
    dev_free(cnt);
    w->profiling = saved_prof;
    if (rc) {
        w->force_variant = saved_variant;
        return rc;
    }
    if (e) {
        w->force_variant = saved_variant;
        return cuda_fail(e, "cf_autotune_step");
    }
    w->force_variant = best;
    if (chosen_variant) *chosen_variant = best;
    return sync_and_check(w);
}

int cf_profile_enable(cf_world* w, int on)
{
    int rc = check_world(w);
    if (rc) return rc;
    CF_CUDA(cudaStreamSynchronize(w->stream));
    if (w->prof_ring.empty()) {
        w->prof_ring.resize(kProfRing);
        w->prof_kind.assign(kProfRing, 0);
        for (auto& ev : w->prof_ring)
            for (auto& e : ev) e = nullptr;
        for (auto& ev : w->prof_ring)
            for (auto& e : ev) CF_CUDA(cudaEventCreate(&e));
    }
    w->profiling = on != 0;
    w->prof_head = w->prof_pending = 0;
    w->prof_cell_ms = w->prof_force_ms = w->prof_adj_ms = 0.0;
    w->prof_steps = w->prof_launches = w->prof_adj_steps = 0;
    return CF_OK;
}

int cf_profile_read(cf_world* w, cf_phase_times* out)
{
    int rc = check_world(w);
    if (rc) return rc;
    if (!out) return fail(CF_ERR_INVALID, "null output");
    CF_CUDA(cudaStreamSynchronize(w->stream));
    rc = harvest_profile(w, w->prof_pending);
    if (rc) return rc;
    out->cell_list_ms = w->prof_cell_ms;
    out->force_ms = w->prof_force_ms;
    out->steps = w->prof_steps;
    out->launches = w->prof_launches;
    out->adjoint_ms = w->prof_adj_ms;
    out->adjoint_steps = w->prof_adj_steps;
    w->prof_cell_ms = w->prof_force_ms = w->prof_adj_ms = 0.0;
    w->prof_steps = w->prof_launches = w->prof_adj_steps = 0;
    return CF_OK;
}

int cf_get_grid(cf_world* w, const cf_step_params* p, cf_grid_info* out)
{
    int rc = check_world(w);
    if (rc) return rc;
    if (!out) return fail(CF_ERR_INVALID, "null output");
    StepConsts c;
    rc = prepare_step(w, p, &c);
    if (rc) return rc;
    for (int a = 0; a < 3; a++) {
        out->cells[a] = c.grid.m[a];
        out->inv_cell[a] = c.grid.inv[a];
    }
    float r_max = 0.0f;
    for (int a = 0; a < w->num_types; a++)
        for (int b = 0; b < w->num_types; b++) r_max = std::max(r_max, w->host_tables.eff[a * kTableStride + b]);
    out->r_max = r_max;
    out->generic_wrap = c.grid.generic;
    out->key_bits = c.grid.key_bits;
    return CF_OK;
}

int cf_debug_cell_list(cf_world* w, const cf_step_params* p, uint32_t* cell_of, uint32_t* sorted_idx,
                       uint32_t* cell_start, uint32_t* cell_end, int cells_cap)
{
    int rc = check_world(w);
    if (rc) return rc;
    StepConsts c;
    rc = prepare_step(w, p, &c);
    if (rc) return rc;
    if (cells_cap < c.grid.cells) return fail(CF_ERR_CAPACITY, "cell arrays smaller than the grid");
    rc = ensure_cells(w, c.grid.cells);
    if (rc) return rc;
    rc = ensure_offsets(w, c.grid.cells);
    if (rc) return rc;
    // the step's own cell list: CSR offsets, stable radix order
    int which = 0;
    CF_CUDA(launch_cell_list_csr(w->pos, w->n, c.grid, c.ext, w->num_types, w->s, w->s.cell_off, nullptr, nullptr,
                                 w->err, &which, w->stream));
    // the hash wrote cell ids in original order into keys[0] before sorting;
    // recompute them (the sort may have reused that buffer)
    CF_CUDA(launch_cell_hash(w->pos, w->n, c.grid, c.ext, w->num_types, w->s.keys[which ^ 1], w->err, w->stream));
    const size_t n = (size_t)w->n;
    if (n > 0) {
        if (cell_of) CF_CUDA(cudaMemcpyAsync(cell_of, w->s.keys[which ^ 1], 4 * n, cudaMemcpyDeviceToHost, w->stream));
        if (sorted_idx)
            CF_CUDA(cudaMemcpyAsync(sorted_idx, w->s.vals[which], 4 * n, cudaMemcpyDeviceToHost, w->stream));
    }
    std::vector<uint32_t> off((size_t)c.grid.cells + 1);
    CF_CUDA(cudaMemcpyAsync(off.data(), w->s.cell_off, 4 * off.size(), cudaMemcpyDeviceToHost, w->stream));
    rc = sync_and_check(w);
    if (rc) return rc;
    for (int k = 0; k < c.grid.cells; k++) {
        const bool empty = off[k + 1] == off[k];
        if (cell_start) cell_start[k] = empty ? 0u : off[k];
        if (cell_end) cell_end[k] = empty ? 0u : off[k + 1];
    }
    return CF_OK;
}

int cf_force_work(cf_world* w, const cf_step_params* p, uint64_t* staged, uint64_t* tested)
{
    int rc = check_world(w);
    if (rc) return rc;
    StepConsts c;
    rc = prepare_step(w, p, &c);
    if (!rc) rc = ensure_cells(w, c.grid.cells);
    if (!rc) rc = ensure_plan(w, c.grid);
    if (!rc) rc = ensure_offsets(w, c.grid.cells);
    if (rc) return rc;
    int which = 0;
    rc = enqueue_cell_list(w, c, &which);
    if (rc) return rc;
    Scratch& s = w->s;
    CF_CUDA(launch_force_work(c, s.keys[which], s.cell_off, s.items, s.n_items, max_step_items(w->n, c.grid),
                              s.counters, w->stream));
    unsigned long long host[2] = {0, 0};
    CF_CUDA(cudaMemcpyAsync(host, s.counters, sizeof(host), cudaMemcpyDeviceToHost, w->stream));
    rc = sync_and_check(w);
    if (rc) return rc;
    if (staged) *staged = host[0];
    if (tested) *tested = host[1];
    return CF_OK;
}

int cf_debug_bounds(int* checked, int* found, char* where, int where_cap, long long* index, long long* limit)
{
#ifdef CF_DEBUG_BOUNDS
    if (checked) *checked = 1;
#else
    if (checked) *checked = 0;
#endif
    if (found) *found = 0;
    if (where && where_cap > 0) where[0] = 0;
    const struct {
        const char* file;
        cudaError_t (*take)(BoundsRecord*);
    } units[] = {{"celllist.cu", bounds_take_celllist}, {"step.cu", bounds_take_step},
                 {"proximity.cu", bounds_take_proximity}};
    bool first = true;
    for (const auto& u : units) {
        BoundsRecord r{};
        CF_CUDA(u.take(&r));
        if (!r.flag || !first) continue;
        first = false;
        if (found) *found = 1;
        if (where && where_cap > 0) std::snprintf(where, (size_t)where_cap, "%s:%d", u.file, r.line);
        if (index) *index = r.index;
        if (limit) *limit = r.limit;
    }
    return CF_OK;
}

int cf_debug_force_bad_item(cf_world* w, const cf_step_params* p, int first)
{
#ifndef CF_DEBUG_BOUNDS
    (void)w;
    (void)p;
    (void)first;
    return fail(CF_ERR_INVALID, "cf_debug_force_bad_item needs the bounds-checked library");
#else
    int rc = check_world(w);
    if (rc) return rc;
    StepConsts c;
    rc = prepare_step(w, p, &c);
    if (!rc) rc = ensure_cells(w, c.grid.cells);
    if (!rc) rc = ensure_plan(w, c.grid);
    if (!rc) rc = ensure_offsets(w, c.grid.cells);
    if (rc) return rc;
    int which = 0;
    rc = enqueue_cell_list(w, c, &which);
    if (rc) return rc;
    // the first item's first particle (Item::first, its first field) overwritten
    CF_CUDA(cudaMemcpyAsync(w->s.items, &first, sizeof(int), cudaMemcpyHostToDevice, w->stream));
    CF_CUDA(cudaStreamSynchronize(w->stream));
    rc = enqueue_force(w, c, which);
    if (rc) return rc;
    return sync_and_check(w);
#endif
}

int cf_work_counters(cf_world* w, const cf_step_params* p, uint64_t* c27, uint64_t* interacting)
{
    int rc = check_world(w);
    if (rc) return rc;
    StepConsts c;
    rc = prepare_step(w, p, &c);
    if (rc) return rc;
    float r_max = 0.0f;
    for (int a = 0; a < w->num_types; a++)
        for (int b = 0; b < w->num_types; b++) r_max = std::max(r_max, w->host_tables.eff[a * kTableStride + b]);
    Grid g = canonical_grid(c.ext, r_max);
    apply_worlds(g, w->worlds);
    Scratch& s = w->s;
    if ((size_t)g.cells > s.pop_cap) {
        CF_CUDA(cudaStreamSynchronize(w->stream));
        dev_free(s.cell_pop);
        s.cell_pop = nullptr;
        s.pop_cap = 0;
        CF_CUDA(dev_alloc(&s.cell_pop, g.cells));
        s.pop_cap = (size_t)g.cells;
    }
    CF_CUDA(launch_work_counters(w->pos, w->counts, w->n, g, s.cell_pop, s.counters, w->stream));
    unsigned long long host[2] = {0, 0};
    CF_CUDA(cudaMemcpyAsync(host, s.counters, sizeof(host), cudaMemcpyDeviceToHost, w->stream));
    rc = sync_and_check(w);
    if (rc) return rc;
    if (c27) *c27 = host[0];
    if (interacting) *interacting = host[1];
    return CF_OK;
}

namespace {

// Proximity selection: cell list with the proximity grid, per-particle
// edges, exclusive scan.  Enqueues only: offsets land in prox_count[0..n] and
// the edge total in host_words[1] once the stream has reached this point.
// Runs a selection pass through its cached graph (captured on first use and
// whenever the grid, distance, limit, particle or type count changes; buffer
// reallocations drop it), or directly when graphs are off.
extern "C++" {
template <typename Body>
int run_selection(cf_world* w, int kind, const Grid& g, float dsq, int max_conn, Body body, const void* out = nullptr,
                  long long out_cap = -1, const ColorTable* colors = nullptr)
{
    if (!w->use_graphs || w->stream == nullptr) return body();
    SelGraph& sg = w->sel_graph[kind];
    const ColorTable ct = colors ? *colors : ColorTable{};
    if (!(sg.exec && std::memcmp(&sg.g, &g, sizeof(g)) == 0 && sg.dsq == dsq && sg.max_conn == max_conn &&
          sg.n == w->n && sg.types == w->num_types && sg.out == out && sg.out_cap == out_cap &&
          std::memcmp(&sg.colors, &ct, sizeof(ct)) == 0)) {
        if (sg.exec) cudaGraphExecDestroy(sg.exec);
        sg = SelGraph();
        cudaGraph_t graph = nullptr;
        CF_CUDA(cudaStreamBeginCapture(w->stream, cudaStreamCaptureModeThreadLocal));
        const int rc = body();
        cudaError_t e = cudaStreamEndCapture(w->stream, &graph);
        if (rc) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
        e = graph_kernel_count(graph, &sg.kernels);
        if (e == cudaSuccess) e = cudaGraphInstantiate(&sg.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
        sg.g = g;
        sg.dsq = dsq;
        sg.max_conn = max_conn;
        sg.n = w->n;
        sg.types = w->num_types;
        sg.out = out;
        sg.out_cap = out_cap;
        sg.colors = ct;
    }
    CF_CUDA(cudaGraphLaunch(sg.exec, w->stream));
    note_launches(w->stream, sg.kernels);
    return CF_OK;
}
}  // extern "C++"

int proximity_enqueue(cf_world* w, float distance, int max_conn)
{
    if (!(distance >= 0.0f) || !std::isfinite(distance)) return fail(CF_ERR_INVALID, "distance must be finite, >= 0");
    if (max_conn < 0 || max_conn > CF_MAX_PROX_CONN)
        return fail(CF_ERR_INVALID, "max_conn must be in [0, 16] (the reference overflowed its buffer above 16)");
    int rc = ensure_prox(w);
    if (rc) return rc;
    Grid g = choose_prox_grid(w->ext, distance, kMaxCells);
    rc = ensure_offsets(w, g.cells);
    if (rc) return rc;
    Scratch& s = w->s;
    const float dsq = distance * distance;  // ParticleSimulation.cu:660
    return run_selection(w, 0, g, dsq, max_conn, [&]() -> int {
        // the tiled cell list on the proximity grid, unordered within a cell (the selection
        // keeps the smallest qualifying indices whatever the order): cell c holds
        // cell_off[c] .. cell_off[c + 1]
        int which = 0;
        CF_CUDA(launch_cell_list_csr(w->pos, w->n, g, w->ext, w->num_types, s, s.cell_off, nullptr, nullptr, w->err,
                                     &which, w->stream, false));
        CF_CUDA(cudaMemsetAsync(s.prox_count + w->n, 0, sizeof(uint32_t), w->stream));
        CF_CUDA(launch_proximity_select(s.pos_sorted, s.keys[which], s.vals[which], s.cell_off, s.cell_off + 1, true, g,
                                        w->n, dsq, max_conn, s.prox_slots, s.prox_count, w->stream));
        CF_CUDA(launch_scan_exclusive(s.prox_count, s.prox_count, w->n + 1, s.scan_tmp, s.scan_tmp_cap, w->stream));
        CF_CUDA(cudaMemcpyAsync(&w->host_words[1], s.prox_count + w->n, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                w->stream));
        return CF_OK;
    });
}

// Triangle selection: cell list on the proximity grid of the mesh distance,
// per-particle triangle counts, exclusive scan.  Enqueues only: offsets land
// in mesh_count[0..n] and the triangle total in host_words[1] once the stream
// has reached this point.
int mesh_enqueue(cf_world* w, float distance, int max_conn)
{
    if (!(distance >= 0.0f) || !std::isfinite(distance)) return fail(CF_ERR_INVALID, "distance must be finite, >= 0");
    if (max_conn < 0) return fail(CF_ERR_INVALID, "max_conn must be >= 0");
    if (w->worlds > 1) return fail(CF_ERR_INVALID, "the triangle mesh covers a single world");
    int rc = ensure_mesh(w);
    if (rc) return rc;
    // ParticleSimulation.cu:723-724: 20 % hysteresis on the distance
    const float hysteresis = 1.2f;
    const float dsq = distance * distance * (hysteresis * hysteresis);
    Grid g = choose_prox_grid(w->ext, nextafterf(std::sqrt(dsq), INFINITY), kMaxCells);
    rc = ensure_offsets(w, g.cells);
    if (rc) return rc;
    Scratch& s = w->s;
    return run_selection(w, 1, g, dsq, max_conn, [&]() -> int {
        int which = 0;
        CF_CUDA(launch_cell_list_csr(w->pos, w->n, g, w->ext, w->num_types, s, s.cell_off, nullptr, nullptr, w->err,
                                     &which, w->stream, false));
        CF_CUDA(cudaMemsetAsync(s.mesh_count + w->n, 0, sizeof(uint32_t), w->stream));
        CF_CUDA(launch_mesh_select(s.pos_sorted, s.keys[which], s.vals[which], s.cell_off, s.cell_off + 1, g, w->n,
                                   dsq, std::min(max_conn, CF_MESH_MAX_CONN), s.mesh_slots, s.mesh_count, w->stream));
        CF_CUDA(launch_scan_exclusive(s.mesh_count, s.mesh_count, w->n + 1, s.scan_tmp, s.scan_tmp_cap, w->stream));
        CF_CUDA(cudaMemcpyAsync(&w->host_words[1], s.mesh_count + w->n, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                w->stream));
        return CF_OK;
    });
}

// Copy `entries` int32 of the staging buffer to host memory and wait.
int copy_out(cf_world* w, int32_t* host, size_t entries)
{
    CF_CUDA(cudaMemcpyAsync(host, w->s.out_idx, sizeof(int32_t) * entries, cudaMemcpyDeviceToHost, w->stream));
    return sync_and_check(w);
}

}  // namespace

// Host output needs the total before the copy: one synchronisation for the
// count, then the emit kernel into the kept staging buffer and the copy.
int cf_triangle_mesh(cf_world* w, float distance, int max_conn, int32_t* triangles, int cap, int* n_triangles)
{
    int rc = check_world(w);
    if (rc) return rc;
    if (cap < 0 || (cap > 0 && !triangles)) return fail(CF_ERR_INVALID, "bad triangle buffer");
    rc = mesh_enqueue(w, distance, max_conn);
    if (rc) return rc;
    rc = sync_and_check(w);
    if (rc) return rc;
    const uint32_t total = (uint32_t)w->host_words[1];
    if (n_triangles) *n_triangles = (int)total;
    const int write = (int)std::min<uint32_t>(total, (uint32_t)cap);
    if (write > 0) {
        rc = ensure_out(w, 3 * (size_t)write);
        if (rc) return rc;
        CF_CUDA(launch_mesh_emit(w->s.mesh_slots, w->s.mesh_count, w->n, w->pos, ColorTable{}, 1, w->s.out_idx, nullptr,
                                 write, w->stream));
        rc = copy_out(w, triangles, 3 * (size_t)write);
        if (rc) return rc;
    }
    if (!triangles && cap == 0) return CF_OK;  // a count query
    if (total > (uint32_t)cap) return fail(CF_ERR_CAPACITY, "triangle buffer smaller than the triangle count");
    return CF_OK;
}

// Device output: the emit kernel stops at the caller's capacity by itself, so
// selection, emission and the count read-back share one synchronisation.
int cf_triangle_mesh_device(cf_world* w, float distance, int max_conn, const cf_color* colors, int n_colors,
                            float* vertices, int cap_vertices, int* vertex_count)
{
    int rc = check_world(w);
    if (rc) return rc;
    if (!colors || n_colors < w->num_types) return fail(CF_ERR_INVALID, "need one colour per type");
    if (cap_vertices < 0 || (cap_vertices > 0 && !vertices)) return fail(CF_ERR_INVALID, "bad vertex buffer");
    rc = mesh_enqueue(w, distance, max_conn);
    if (rc) return rc;
    if (cap_vertices >= 3) {
        // ParticleSimulation.cu:356 indexes colours by type % numParticleTypes
        CF_CUDA(launch_mesh_emit(w->s.mesh_slots, w->s.mesh_count, w->n, w->pos, color_table(w, colors),
                                 w->num_types, nullptr, vertices, cap_vertices / 3, w->stream));
    }
    rc = sync_and_check(w);
    if (rc) return rc;
    const uint32_t total = (uint32_t)w->host_words[1];
    if (vertex_count) *vertex_count = (int)(3 * total);
    if (!vertices && cap_vertices == 0) return CF_OK;  // a count query
    if (3 * (size_t)total > (size_t)cap_vertices) return fail(CF_ERR_CAPACITY, "vertex buffer too small");
    return CF_OK;
}

int cf_proximity_edges(cf_world* w, float distance, int max_conn, int32_t* edges, int cap, int* n_edges)
{
    int rc = check_world(w);
    if (rc) return rc;
    if (cap < 0 || (cap > 0 && !edges)) return fail(CF_ERR_INVALID, "bad edge buffer");
    rc = proximity_enqueue(w, distance, max_conn);
    if (rc) return rc;
    // the edges go to the staging buffer right behind the selection, sized for the most
    // a call can find (max_conn per particle, at most the caller's capacity), so the
    // count and the edges arrive with one synchronisation; only the copy follows it
    const int staged = (int)std::min<size_t>((size_t)cap, (size_t)w->n * (size_t)max_conn);
    if (staged > 0) {
        rc = ensure_out(w, 2 * (size_t)staged);
        if (rc) return rc;
        CF_CUDA(launch_proximity_emit_edges(w->s.prox_slots, w->s.prox_count, w->n, max_conn, w->s.out_idx, staged,
                                            w->stream));
    }
    rc = sync_and_check(w);
    if (rc) return rc;
    const uint32_t total = (uint32_t)w->host_words[1];
    if (n_edges) *n_edges = (int)total;
    const int write = (int)std::min<uint32_t>(total, (uint32_t)cap);
    if (write > 0) {
        rc = copy_out(w, edges, 2 * (size_t)write);
        if (rc) return rc;
    }
    if (total > (uint32_t)cap) return fail(CF_ERR_CAPACITY, "edge buffer smaller than the edge count");
    return CF_OK;
}

int cf_proximity_vertices_device(cf_world* w, float distance, int max_conn, const cf_color* colors, int n_colors,
                                 float* vertices, int cap_vertices, int* vertex_count)
{
    int rc = check_world(w);
    if (rc) return rc;
    if (!colors || n_colors < w->num_types) return fail(CF_ERR_INVALID, "need one colour per type");
    if (cap_vertices < 0 || (cap_vertices > 0 && !vertices)) return fail(CF_ERR_INVALID, "bad vertex buffer");
    if (!(distance >= 0.0f) || !std::isfinite(distance)) return fail(CF_ERR_INVALID, "distance must be finite, >= 0");
    if (max_conn < 0 || max_conn > CF_MAX_PROX_CONN)
        return fail(CF_ERR_INVALID, "max_conn must be in [0, 16] (the reference overflowed its buffer above 16)");
    rc = ensure_prox(w);
    if (rc) return rc;
    Grid g = choose_prox_grid(w->ext, distance, kMaxCells);
    rc = ensure_offsets(w, g.cells);
    if (rc) return rc;
    Scratch& s = w->s;
    const float dsq = distance * distance;  // ParticleSimulation.cu:660
    // ParticleSimulation.cu:253 indexes colours by type % numParticleTypes
    const ColorTable ct = color_table(w, colors);
    // one pass: the selection writes each particle's line vertices at places reserved by
    // one atomic per particle (arbitrary order, as the reference's atomicAdd append,
    // ParticleSimulation.cu:250); the edge total is read back
    uint32_t* total = s.prox_count + w->n;
    rc = run_selection(
        w, 2, g, dsq, max_conn,
        [&]() -> int {
            int which = 0;
            CF_CUDA(launch_cell_list_csr(w->pos, w->n, g, w->ext, w->num_types, s, s.cell_off, nullptr, nullptr,
                                         w->err, &which, w->stream, false));
            CF_CUDA(cudaMemsetAsync(total, 0, sizeof(uint32_t), w->stream));
            CF_CUDA(launch_proximity_select_vertices(s.pos_sorted, s.keys[which], s.vals[which], s.cell_off, g, w->n,
                                                     dsq, max_conn, w->pos, ct, w->num_types, vertices, cap_vertices,
                                                     total, w->stream));
            CF_CUDA(cudaMemcpyAsync(&w->host_words[1], total, sizeof(uint32_t), cudaMemcpyDeviceToHost, w->stream));
            return CF_OK;
        },
        vertices, cap_vertices, &ct);
    if (rc) return rc;
    rc = sync_and_check(w);
    if (rc) return rc;
    const uint32_t edges = (uint32_t)w->host_words[1];
    if (vertex_count) *vertex_count = (int)(2 * edges);
    if (2 * (size_t)edges > (size_t)cap_vertices) return fail(CF_ERR_CAPACITY, "vertex buffer too small");
    return CF_OK;
}

}  // extern "C"

// ---- batched ensembles ------------------------------------------------------
//
// A batch is one cf_world whose particles belong to several independent
// worlds: world k owns particles [off[k], off[k+1]), carries its index in the
// bits of pos4.w above the type, and has its own force table.  Cell ids are
// world * cells_per_world + cell, so one cell list, one plan and one force
// launch per step cover every world; no pair ever crosses worlds.

struct cf_batch {
    cf_world* w = nullptr;
};

namespace {

int check_batch(const cf_batch* b)
{
    if (!b || !b->w) return fail(CF_ERR_INVALID, "null batch");
    return CF_OK;
}

}  // namespace

extern "C" {

int cf_batch_create(int worlds, const int* n_per_world, int num_types, float w_, float h_, float d_, uint64_t seed,
                    cf_batch** out)
{
    if (!out) return fail(CF_ERR_INVALID, "null output handle");
    *out = nullptr;
    if (worlds < 1 || worlds > (1 << 20) || !n_per_world) return fail(CF_ERR_INVALID, "worlds must be in [1, 2^20]");
    long long total = 0;
    for (int k = 0; k < worlds; k++) {
        if (n_per_world[k] < 0) return fail(CF_ERR_INVALID, "particle counts must be >= 0");
        total += n_per_world[k];
    }
    if (total > (1ll << 27) - 1) return fail(CF_ERR_INVALID, "a batch holds at most 2^27 - 1 particles");
    cf_world* w = nullptr;
    int rc = cf_create((int)total, num_types, w_, h_, d_, seed, &w);
    if (rc) return rc;
    w->worlds = worlds;
    w->world_off.assign(worlds + 1, 0);
    for (int k = 0; k < worlds; k++) w->world_off[k + 1] = w->world_off[k] + n_per_world[k];
    cudaError_t e = dev_alloc(&w->world_tables, (size_t)worlds * kTableSize);
    if (e != cudaSuccess) {
        cf_destroy(w);
        return cuda_fail(e, "cudaMalloc(world tables)");
    }
    // world k: particles spawned from seed + k, raw table from seed + k, the
    // default transform (ParticleSimulation.cu:513-519)
    std::vector<float> tables((size_t)worlds * kTableSize, 0.0f);
    float lo[3], span[3];
    for (int a = 0; a < 3; a++) {
        span[a] = std::min(2000.0f, w->ext[a]);
        lo[a] = (w->ext[a] - span[a]) * 0.5f;
    }
    for (int k = 0; k < worlds && e == cudaSuccess; k++) {
        const int off = w->world_off[k], n = n_per_world[k];
        e = launch_init_particles(w->pos + off, w->vel + off, w->acc + off, w->counts + off, n, num_types, lo, span,
                                  seed + (uint64_t)k, w->stream, (uint32_t)k);
        uint64_t s = (seed + (uint64_t)k) ^ 0x2545F4914F6CDD1Dull;
        for (int a = 0; a < num_types; a++)
            for (int b2 = 0; b2 < num_types; b2++) {
                const float raw = uniform_pm1(s);
                const float t = tanhf(raw * 1.0f) * 0.28f + -0.20f;
                tables[(size_t)k * kTableSize + a * kTableStride + b2] = fmaxf(-1.0f, fminf(1.0f, t));
            }
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(w->world_tables, tables.data(), sizeof(float) * tables.size(), cudaMemcpyHostToDevice,
                            w->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(w->stream);
    if (e != cudaSuccess) {
        cf_destroy(w);
        return cuda_fail(e, "cf_batch_create");
    }
    cf_batch* b = new cf_batch();
    b->w = w;
    *out = b;
    return CF_OK;
}

int cf_batch_destroy(cf_batch* b)
{
    if (!b) return CF_OK;
    cf_destroy(b->w);
    delete b;
    return CF_OK;
}

int cf_batch_world(cf_batch* b, cf_world** out)
{
    int rc = check_batch(b);
    if (rc) return rc;
    if (!out) return fail(CF_ERR_INVALID, "null output");
    *out = b->w;
    return CF_OK;
}

int cf_batch_info(const cf_batch* b, int* worlds, int* total, int* offsets)
{
    int rc = check_batch(b);
    if (rc) return rc;
    if (worlds) *worlds = b->w->worlds;
    if (total) *total = b->w->n;
    if (offsets) std::memcpy(offsets, b->w->world_off.data(), sizeof(int) * (b->w->worlds + 1));
    return CF_OK;
}

int cf_batch_set_state(cf_batch* b, const float* pos4, const float* vel4, const int* counts)
{
    int rc = check_batch(b);
    if (rc) return rc;
    cf_world* w = b->w;
    std::vector<float> tagged;
    if (pos4) {
        // add each particle's world index above its type bits
        tagged.assign(pos4, pos4 + 4 * (size_t)w->n);
        for (int k = 0; k < w->worlds; k++)
            for (int i = w->world_off[k]; i < w->world_off[k + 1]; i++) {
                uint32_t bits;
                std::memcpy(&bits, &tagged[4 * (size_t)i + 3], 4);
                bits = (bits & kTypeMask) | ((uint32_t)k << kWorldShift);
                std::memcpy(&tagged[4 * (size_t)i + 3], &bits, 4);
            }
    }
    return cf_set_state(w, pos4 ? tagged.data() : nullptr, vel4, counts);
}

int cf_batch_get_state(cf_batch* b, float* pos4, float* vel4, int* counts)
{
    int rc = check_batch(b);
    if (rc) return rc;
    rc = cf_get_state(b->w, pos4, vel4, counts);
    if (rc || !pos4) return rc;
    for (size_t i = 0; i < (size_t)b->w->n; i++) {
        uint32_t bits;
        std::memcpy(&bits, &pos4[4 * i + 3], 4);
        bits &= kTypeMask;
        std::memcpy(&pos4[4 * i + 3], &bits, 4);
    }
    return CF_OK;
}

int cf_batch_set_force_tables(cf_batch* b, const float* tables, int count)
{
    int rc = check_batch(b);
    if (rc) return rc;
    cf_world* w = b->w;
    const int T = w->num_types;
    if (!tables || count != w->worlds * T * T) return fail(CF_ERR_INVALID, "count must be worlds * T * T");
    std::vector<float> padded((size_t)w->worlds * kTableSize, 0.0f);
    for (int k = 0; k < w->worlds; k++)
        for (int a = 0; a < T; a++)
            for (int c = 0; c < T; c++)
                padded[(size_t)k * kTableSize + a * kTableStride + c] = tables[((size_t)k * T + a) * T + c];
    CF_CUDA(cudaMemcpyAsync(w->world_tables, padded.data(), sizeof(float) * padded.size(), cudaMemcpyHostToDevice,
                            w->stream));
    CF_CUDA(cudaStreamSynchronize(w->stream));
    return CF_OK;
}

int cf_batch_step(cf_batch* b, const cf_step_params* p, int nsteps)
{
    int rc = check_batch(b);
    if (rc) return rc;
    return cf_step(b->w, p, nsteps);
}

int cf_batch_capture(cf_batch* b, const cf_step_params* p, int nsteps)
{
    int rc = check_batch(b);
    if (rc) return rc;
    cf_world* w = b->w;
    if (nsteps < 1) return fail(CF_ERR_INVALID, "nsteps must be >= 1");
    if (!w->stream) return fail(CF_ERR_INVALID, "capture needs a non-default stream");
    StepConsts c;
    rc = prepare_step(w, p, &c);
    if (rc) return rc;
    rc = ensure_cells(w, c.grid.cells);
    if (!rc) rc = ensure_plan(w, c.grid);
    if (!rc) rc = ensure_offsets(w, c.grid.cells);
    if (rc) return rc;
    CF_CUDA(cudaStreamSynchronize(w->stream));
    if (w->batch_graph) cudaGraphExecDestroy(w->batch_graph);
    w->batch_graph = nullptr;
    w->batch_graph_steps = 0;
    cudaGraph_t graph = nullptr;
    CF_CUDA(cudaStreamBeginCapture(w->stream, cudaStreamCaptureModeThreadLocal));
    for (int s = 0; s < nsteps && rc == CF_OK; s++) rc = enqueue_step(w, c, 0);
    cudaError_t e = cudaStreamEndCapture(w->stream, &graph);
    if (rc) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    long long kernels = 0;
    e = graph_kernel_count(graph, &kernels);
    if (e != cudaSuccess) {
        cudaGraphDestroy(graph);
        return cuda_fail(e, "cudaGraphGetNodes");
    }
    e = cudaGraphInstantiate(&w->batch_graph, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    w->batch_graph_steps = nsteps;
    w->batch_graph_kernels = kernels;
    return CF_OK;
}

int cf_batch_graph_info(const cf_batch* b, int* steps, long long* kernels)
{
    int rc = check_batch(b);
    if (rc) return rc;
    if (steps) *steps = b->w->batch_graph_steps;
    if (kernels) *kernels = b->w->batch_graph_kernels;
    return CF_OK;
}

int cf_batch_replay(cf_batch* b)
{
    int rc = check_batch(b);
    if (rc) return rc;
    if (!b->w->batch_graph) return fail(CF_ERR_INVALID, "no captured graph (cf_batch_capture)");
    CF_CUDA(cudaGraphLaunch(b->w->batch_graph, b->w->stream));
    note_launches(b->w->stream, b->w->batch_graph_kernels);
    return CF_OK;
}

int cf_batch_autotune(cf_batch* b, const cf_step_params* p, int steps, int* chosen_variant)
{
    int rc = check_batch(b);
    if (rc) return rc;
    return cf_autotune_step(b->w, p, steps, chosen_variant);
}

int cf_batch_sync(cf_batch* b)
{
    int rc = check_batch(b);
    if (rc) return rc;
    return cf_sync(b->w);
}

int cf_batch_set_stream(cf_batch* b, void* stream)
{
    int rc = check_batch(b);
    if (rc) return rc;
    return cf_set_stream(b->w, stream);
}

}  // extern "C"

// ---- differentiable rollout ---------------------------------------------------

namespace cf {
namespace {

int ensure_rollout(cf_world* w, int ckpts, int seg_states)
{
    Rollout& r = w->ro;
    const int n = w->n;
    if (r.n_cap == n && r.gx && ckpts <= r.ckpt_cap && seg_states <= r.seg_cap) return CF_OK;
    CF_CUDA(cudaStreamSynchronize(w->stream));
    const Rollout keep = r;  // the record of the last forward survives a reallocation
    free_rollout(w);
    r.steps = 0;
    const size_t nn = (size_t)std::max(n, 1);
    const size_t ck = (size_t)std::max(ckpts, keep.n_cap == n ? keep.ckpt_cap : 0);
    const size_t sg = (size_t)std::max(seg_states, keep.n_cap == n ? keep.seg_cap : 0);
    CF_CUDA(dev_alloc(&r.ckpt_pos, nn * ck));
    CF_CUDA(dev_alloc(&r.ckpt_vel, nn * ck));
    CF_CUDA(dev_alloc(&r.ckpt_cnt, nn * ck));
    CF_CUDA(dev_alloc(&r.seg_pos, nn * sg * 2));
    CF_CUDA(dev_alloc(&r.seg_vel, nn * sg * 2));
    CF_CUDA(dev_alloc(&r.seg_cnt, nn * sg * 2));
    CF_CUDA(dev_alloc(&r.fin_pos, nn));
    CF_CUDA(dev_alloc(&r.fin_vel, nn));
    CF_CUDA(dev_alloc(&r.fin_cnt, nn));
    CF_CUDA(dev_alloc(&r.gx, nn));
    CF_CUDA(dev_alloc(&r.gv, nn));
    CF_CUDA(dev_alloc(&r.gf_sorted, nn));
    CF_CUDA(dev_alloc(&r.ga_sorted, nn));
    CF_CUDA(dev_alloc(&r.gacc, (size_t)kGradAccEntries));
    r.n_cap = n;
    r.ckpt_cap = (int)ck;
    r.seg_cap = (int)sg;
    return CF_OK;
}

// Per-step cell lists of one checkpoint segment (steps = checkpoint interval).
int ensure_rollout_lists(cf_world* w, int steps, int cells)
{
    Rollout& r = w->ro;
    const size_t offs = (size_t)cells + 1;
    if (r.seg_off && steps <= r.lists_steps && offs <= r.lists_cells) return CF_OK;
    CF_CUDA(cudaStreamSynchronize(w->stream));
    // the backward's graph reads these lists by address: drop it with them
    if (r.bwd_graph) cudaGraphExecDestroy(r.bwd_graph);
    r.bwd_graph = nullptr;
    for (void* p : {(void*)r.seg_sorted, (void*)r.seg_keys, (void*)r.seg_vals, (void*)r.seg_off}) dev_free(p);
    r.seg_sorted = nullptr;
    r.seg_keys = r.seg_vals = r.seg_off = nullptr;
    r.lists_steps = 0;
    r.lists_cells = 0;
    const size_t nn = (size_t)std::max(w->n, 1) * (size_t)steps * 2;
    CF_CUDA(dev_alloc(&r.seg_sorted, nn));
    CF_CUDA(dev_alloc(&r.seg_keys, nn));
    CF_CUDA(dev_alloc(&r.seg_vals, nn));
    CF_CUDA(dev_alloc(&r.seg_off, offs * (size_t)steps * 2));
    r.lists_steps = steps;
    r.lists_cells = offs;
    return CF_OK;
}

// Radial distribution scratch (freed with the rest of the rollout buffers
// whenever the particle count changes).
int ensure_rdf(cf_world* w)
{
    Rollout& r = w->ro;
    if (r.rdf_pos) return CF_OK;
    if (!r.rdf_acc) {
        const int rc = alloc_pair(&r.rdf_acc, (size_t)kRdfMaxEntries, &r.type_count, (size_t)CF_MAX_TYPES);
        if (rc) return rc;
    }
    CF_CUDA(dev_alloc(&r.rdf_pos, (size_t)std::max(w->n, 1)));  // last: it marks the set complete
    return CF_OK;
}

// Copy a state (positions, velocities, counts) between device buffers.
int copy_state(cf_world* w, float4* dp, float4* dv, int* dc, const float4* sp, const float4* sv, const int* sc)
{
    const size_t n = (size_t)w->n;
    CF_CUDA(cudaMemcpyAsync(dp, sp, sizeof(float4) * n, cudaMemcpyDeviceToDevice, w->stream));
    CF_CUDA(cudaMemcpyAsync(dv, sv, sizeof(float4) * n, cudaMemcpyDeviceToDevice, w->stream));
    CF_CUDA(cudaMemcpyAsync(dc, sc, sizeof(int) * n, cudaMemcpyDeviceToDevice, w->stream));
    return CF_OK;
}

// The whole backward on the world's stream: save the final state, then per
// segment (last first) replay the forward from its checkpoint keeping every
// state, and run the adjoint steps of the segment in reverse; restore the
// final state.  gx / gv hold dL/dx_K and dL/dv_K on entry, dL/dx_0 and
// dL/dv_0 on exit; gacc collects the parameter gradients.
// Segment buffer `buf` (0 or 1) of the replayed states and cell lists.
struct SegBuf {
    float4 *pos, *vel, *sorted;
    int* cnt;
    uint32_t *keys, *vals, *off;
};

SegBuf seg_buf(const Rollout& r, size_t n, int buf)
{
    const size_t states = (size_t)r.seg_cap * n * (size_t)buf;
    const size_t lists = (size_t)r.lists_steps * n * (size_t)buf;
    SegBuf b;
    b.pos = r.seg_pos + states;
    b.vel = r.seg_vel + states;
    b.cnt = r.seg_cnt + states;
    b.sorted = r.seg_sorted ? r.seg_sorted + lists : nullptr;
    b.keys = r.seg_keys ? r.seg_keys + lists : nullptr;
    b.vals = r.seg_vals ? r.seg_vals + lists : nullptr;
    b.off = r.seg_off ? r.seg_off + r.lists_cells * (size_t)r.lists_steps * (size_t)buf : nullptr;
    return b;
}

// Replay of segment `seg` from its checkpoint on the world's stream, keeping
// every state in buffer `buf` and, with lists, every step's cell list.
int replay_segment(cf_world* w, const StepConsts& c, int seg, const SegBuf& b, bool lists)
{
    Rollout& r = w->ro;
    const size_t n = (size_t)w->n;
    const int len = std::min(r.every, r.steps - seg * r.every);
    Scratch& s = w->s;
    int rc = copy_state(w, w->pos, w->vel, w->counts, r.ckpt_pos + n * seg, r.ckpt_vel + n * seg,
                        r.ckpt_cnt + n * seg);
    if (rc) return rc;
    for (int t = 0; t < len; t++) {
        rc = copy_state(w, b.pos + n * t, b.vel + n * t, b.cnt + n * t, w->pos, w->vel, w->counts);
        if (rc) return rc;
        if (lists) {
            // the replayed step builds its cell list straight into step t's arrays
            // (the tiled build leaves it in keys[1] / vals[1]), kept for the adjoint step
            float4* const ps = s.pos_sorted;
            uint32_t* const k1 = s.keys[1];
            uint32_t* const v1 = s.vals[1];
            uint32_t* const off = s.cell_off;
            s.pos_sorted = b.sorted + n * t;
            s.keys[1] = b.keys + n * t;
            s.vals[1] = b.vals + n * t;
            s.cell_off = b.off + r.lists_cells * t;
            rc = enqueue_step(w, c, 0);
            s.pos_sorted = ps;
            s.keys[1] = k1;
            s.vals[1] = v1;
            s.cell_off = off;
        } else {
            rc = enqueue_step(w, c, 0);
        }
        if (rc) return rc;
    }
    CF_CUDA(cudaMemcpyAsync(b.cnt + n * len, w->counts, sizeof(int) * n, cudaMemcpyDeviceToDevice, w->stream));
    return CF_OK;
}

// The adjoint steps of segment `seg` in reverse, from buffer `buf`.
int adjoint_segment(cf_world* w, const StepConsts& c, int seg, const SegBuf& b, bool lists)
{
    Rollout& r = w->ro;
    const size_t n = (size_t)w->n;
    const int len = std::min(r.every, r.steps - seg * r.every);
    Scratch& s = w->s;
    for (int t = len - 1; t >= 0; t--) {
        const float4* ps = s.pos_sorted;
        const uint32_t *ks = nullptr, *vs = nullptr, *off = s.cell_off;
        if (lists) {
            ps = b.sorted + n * t;
            ks = b.keys + n * t;
            vs = b.vals + n * t;
            off = b.off + r.lists_cells * t;
        } else {
            int which = 0;
            CF_CUDA(launch_cell_list_csr(b.pos + n * t, w->n, c.grid, c.ext, w->num_types, s, s.cell_off, nullptr,
                                         nullptr, w->err, &which, w->stream));
            ks = s.keys[which];
            vs = s.vals[which];
        }
        const std::array<cudaEvent_t, 3>* ev = nullptr;
        if (w->profiling) {
            // profiled backward (no graph, no overlap): events around the adjoint kernels
            if (w->prof_pending == (int)w->prof_ring.size()) {
                const int e = harvest_profile(w, 1);
                if (e) return e;
            }
            ev = &w->prof_ring[w->prof_head];
            w->prof_kind[w->prof_head] = 1;
            w->prof_head = (w->prof_head + 1) % (int)w->prof_ring.size();
            w->prof_pending++;
            CF_CUDA(cudaEventRecord((*ev)[0], w->stream));
        }
        CF_CUDA(launch_adjoint_step(c, w->tables, ps, ks, vs, off, b.vel + n * t, b.cnt + n * t, b.cnt + n * (t + 1),
                                    r.gx, r.gv, r.gf_sorted, r.ga_sorted, r.gacc, w->stream));
        if (ev) {
            CF_CUDA(cudaEventRecord((*ev)[1], w->stream));
            CF_CUDA(cudaEventRecord((*ev)[2], w->stream));
        }
    }
    return CF_OK;
}

// The whole backward: save the final state, then per segment (last first)
// replay the forward from its checkpoint keeping every state, and run the
// adjoint steps of the segment in reverse; restore the final state.  gx / gv
// hold dL/dx_K and dL/dv_K on entry, dL/dx_0 and dL/dv_0 on exit.  With
// `overlap` (while capturing the backward's graph, per-step cell lists kept),
// the replay of segment s - 1 runs on the side stream while the adjoint steps
// of segment s run on the world's stream: the replay touches the world state,
// the cell-list scratch and segment buffer (s - 1) & 1 only, the adjoint steps
// buffer s & 1 and the gradients only; the replay forks after the adjoint
// steps of segment s + 1 (which read the same buffer) and joins before those
// of segment s - 1.
int enqueue_rollout_backward(cf_world* w, const StepConsts& c, bool overlap)
{
    Rollout& r = w->ro;
    int rc = copy_state(w, r.fin_pos, r.fin_vel, r.fin_cnt, w->pos, w->vel, w->counts);
    if (rc) return rc;
    CF_CUDA(cudaMemsetAsync(r.gacc, 0, sizeof(double) * kGradAccEntries, w->stream));
    const int segs = (r.steps + r.every - 1) / r.every;
    // keep the replay's cell lists when the tiled build is used (it always leaves the
    // sorted keys and indices in buffer 1) and the lists are allocated for this grid
    const bool lists = cell_list_tiles(c.grid) > 0 && r.seg_off && r.lists_steps >= std::min(r.every, r.steps) &&
                       r.lists_cells >= (size_t)c.grid.cells + 1;
    const size_t n = (size_t)w->n;
    if (!(overlap && lists && segs > 1 && r.side)) {
        const SegBuf b = seg_buf(r, n, 0);
        for (int seg = segs - 1; seg >= 0; seg--) {
            rc = replay_segment(w, c, seg, b, lists);
            if (!rc) rc = adjoint_segment(w, c, seg, b, lists);
            if (rc) return rc;
        }
        return copy_state(w, w->pos, w->vel, w->counts, r.fin_pos, r.fin_vel, r.fin_cnt);
    }
    const cudaStream_t own = w->stream;
    rc = replay_segment(w, c, segs - 1, seg_buf(r, n, (segs - 1) & 1), lists);
    if (rc) return rc;
    for (int seg = segs - 1; seg >= 0; seg--) {
        if (seg > 0) {
            CF_CUDA(cudaEventRecord(r.ev_fork, own));
            CF_CUDA(cudaStreamWaitEvent(r.side, r.ev_fork, 0));
            w->stream = r.side;
            rc = replay_segment(w, c, seg - 1, seg_buf(r, n, (seg - 1) & 1), lists);
            w->stream = own;
            if (rc) return rc;
            CF_CUDA(cudaEventRecord(r.ev_join, r.side));
        }
        rc = adjoint_segment(w, c, seg, seg_buf(r, n, seg & 1), lists);
        if (rc) return rc;
        if (seg > 0) CF_CUDA(cudaStreamWaitEvent(own, r.ev_join, 0));
    }
    return copy_state(w, w->pos, w->vel, w->counts, r.fin_pos, r.fin_vel, r.fin_cnt);
}

}  // namespace
}  // namespace cf

extern "C" {

int cf_rollout_forward(cf_world* w, const cf_step_params* p, const float* d_pos4_in, const float* d_vel4_in,
                       int nsteps, int checkpoint_every, float* d_pos4_out, float* d_vel4_out)
{
    int rc = check_world(w);
    if (rc) return rc;
    if (w->worlds > 1) return fail(CF_ERR_INVALID, "a rollout runs on a single world");
    if (nsteps < 1) return fail(CF_ERR_INVALID, "nsteps must be >= 1");
    if (checkpoint_every < 1) return fail(CF_ERR_INVALID, "checkpoint_every must be >= 1");
    StepConsts c;
    rc = prepare_step(w, p, &c);
    if (!rc) rc = ensure_cells(w, c.grid.cells);
    if (!rc) rc = ensure_plan(w, c.grid);
    if (!rc) rc = ensure_offsets(w, c.grid.cells);
    if (rc) return rc;
    const int ckpts = (nsteps + checkpoint_every - 1) / checkpoint_every;
    rc = ensure_rollout(w, ckpts, std::min(checkpoint_every, nsteps) + 1);
    if (rc) return rc;
    Rollout& r = w->ro;
    r.steps = 0;
    const size_t n = (size_t)w->n;
    if (d_pos4_in) CF_CUDA(launch_pack_pos(reinterpret_cast<const float4*>(d_pos4_in), w->pos, w->pos, w->n, w->stream));
    if (d_vel4_in)
        CF_CUDA(cudaMemcpyAsync(w->vel, d_vel4_in, sizeof(float4) * n, cudaMemcpyDeviceToDevice, w->stream));
    // the step loop with its checkpoint copies
    auto loop = [&]() -> int {
        for (int s = 0; s < nsteps; s++) {
            if (s % checkpoint_every == 0) {
                const int k = s / checkpoint_every;
                const int e = copy_state(w, r.ckpt_pos + n * k, r.ckpt_vel + n * k, r.ckpt_cnt + n * k, w->pos,
                                         w->vel, w->counts);
                if (e) return e;
            }
            const int e = enqueue_step(w, c, 0);
            if (e) return e;
        }
        return CF_OK;
    };
    if (w->use_graphs && w->stream != nullptr) {
        // one graph for the whole loop, re-captured when its shape or buffers change
        const void* bufs = w->s.cell_start;
        if (!(r.fwd_graph && r.fwd_steps == nsteps && r.fwd_every == checkpoint_every && r.fwd_bufs == bufs &&
              r.fwd_ckpt == r.ckpt_pos && std::memcmp(&r.fwd_key, &c, sizeof(c)) == 0)) {
            if (r.fwd_graph) cudaGraphExecDestroy(r.fwd_graph);
            r.fwd_graph = nullptr;
            cudaGraph_t graph = nullptr;
            CF_CUDA(cudaStreamBeginCapture(w->stream, cudaStreamCaptureModeThreadLocal));
            rc = loop();
            cudaError_t e = cudaStreamEndCapture(w->stream, &graph);
            if (rc) {
                if (graph) cudaGraphDestroy(graph);
                return rc;
            }
            if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
            e = graph_kernel_count(graph, &r.fwd_kernels);
            if (e == cudaSuccess) e = cudaGraphInstantiate(&r.fwd_graph, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
            r.fwd_key = c;
            r.fwd_steps = nsteps;
            r.fwd_every = checkpoint_every;
            r.fwd_bufs = bufs;
            r.fwd_ckpt = r.ckpt_pos;
        }
        CF_CUDA(cudaGraphLaunch(r.fwd_graph, w->stream));
        note_launches(w->stream, r.fwd_kernels);
    } else if ((rc = loop())) {
        return rc;
    }
    if (d_pos4_out)
        CF_CUDA(cudaMemcpyAsync(d_pos4_out, w->pos, sizeof(float4) * n, cudaMemcpyDeviceToDevice, w->stream));
    if (d_vel4_out)
        CF_CUDA(cudaMemcpyAsync(d_vel4_out, w->vel, sizeof(float4) * n, cudaMemcpyDeviceToDevice, w->stream));
    r.steps = nsteps;
    r.every = checkpoint_every;
    r.n = w->n;
    r.params = *p;
    r.table_version = w->table_version;
    std::memcpy(r.radio, w->radio, sizeof(r.radio));
    return CF_OK;
}

int cf_rollout_backward(cf_world* w, const float* d_gpos4, const float* d_gvel4, float* d_gpos4_out,
                        float* d_gvel4_out, float* grad_force, int grad_force_count, float* grad_params)
{
    int rc = check_world(w);
    if (rc) return rc;
    Rollout& r = w->ro;
    if (r.steps < 1) return fail(CF_ERR_INVALID, "no rollout to differentiate (cf_rollout_forward)");
    if (r.n != w->n || r.table_version != w->table_version || std::memcmp(r.radio, w->radio, sizeof(r.radio)) != 0)
        return fail(CF_ERR_INVALID, "the particle count, force table or radii changed since cf_rollout_forward");
    const int T = w->num_types;
    if (grad_force && grad_force_count != T * T) return fail(CF_ERR_INVALID, "grad_force_count must be T * T");
    StepConsts c;
    rc = prepare_step(w, &r.params, &c);
    if (!rc) rc = ensure_cells(w, c.grid.cells);
    if (!rc) rc = ensure_plan(w, c.grid);
    if (!rc) rc = ensure_offsets(w, c.grid.cells);
    if (!rc) rc = ensure_rollout_lists(w, std::min(r.every, r.steps), c.grid.cells);
    if (rc) return rc;
    const size_t n = (size_t)w->n;
    if (d_gpos4)
        CF_CUDA(cudaMemcpyAsync(r.gx, d_gpos4, sizeof(float4) * n, cudaMemcpyDeviceToDevice, w->stream));
    else
        CF_CUDA(cudaMemsetAsync(r.gx, 0, sizeof(float4) * n, w->stream));
    if (d_gvel4)
        CF_CUDA(cudaMemcpyAsync(r.gv, d_gvel4, sizeof(float4) * n, cudaMemcpyDeviceToDevice, w->stream));
    else
        CF_CUDA(cudaMemsetAsync(r.gv, 0, sizeof(float4) * n, w->stream));
    if (w->use_graphs && w->stream != nullptr && !w->profiling) {
        const void* bufs = w->s.cell_start;
        const bool same = r.bwd_graph && r.bwd_steps == r.steps && r.bwd_every == r.every && r.bwd_bufs == bufs &&
                          r.bwd_lists == r.seg_off && std::memcmp(&r.bwd_key, &c, sizeof(c)) == 0;
        if (!same) {
            if (r.bwd_graph) cudaGraphExecDestroy(r.bwd_graph);
            r.bwd_graph = nullptr;
            cudaGraph_t graph = nullptr;
            if (!r.side) {
                CF_CUDA(cudaStreamCreateWithFlags(&r.side, cudaStreamNonBlocking));
                CF_CUDA(cudaEventCreateWithFlags(&r.ev_fork, cudaEventDisableTiming));
                CF_CUDA(cudaEventCreateWithFlags(&r.ev_join, cudaEventDisableTiming));
            }
            CF_CUDA(cudaStreamBeginCapture(w->stream, cudaStreamCaptureModeThreadLocal));
            rc = enqueue_rollout_backward(w, c, true);
            cudaError_t e = cudaStreamEndCapture(w->stream, &graph);
            if (rc) {
                if (graph) cudaGraphDestroy(graph);
                return rc;
            }
            if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
            e = graph_kernel_count(graph, &r.bwd_kernels);
            if (e == cudaSuccess) e = cudaGraphInstantiate(&r.bwd_graph, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
            r.bwd_key = c;
            r.bwd_steps = r.steps;
            r.bwd_every = r.every;
            r.bwd_bufs = bufs;
            r.bwd_lists = r.seg_off;
        }
        CF_CUDA(cudaGraphLaunch(r.bwd_graph, w->stream));
        note_launches(w->stream, r.bwd_kernels);
    } else {
        rc = enqueue_rollout_backward(w, c, false);
        if (rc) return rc;
    }
    if (d_gpos4_out)
        CF_CUDA(cudaMemcpyAsync(d_gpos4_out, r.gx, sizeof(float4) * n, cudaMemcpyDeviceToDevice, w->stream));
    if (d_gvel4_out)
        CF_CUDA(cudaMemcpyAsync(d_gvel4_out, r.gv, sizeof(float4) * n, cudaMemcpyDeviceToDevice, w->stream));
    if (grad_force || grad_params) {
        std::vector<double> acc(kGradAccEntries);
        CF_CUDA(cudaMemcpyAsync(acc.data(), r.gacc, sizeof(double) * kGradAccEntries, cudaMemcpyDeviceToHost,
                                w->stream));
        rc = sync_and_check(w);
        if (rc) return rc;
        if (grad_force)
            for (int a = 0; a < T; a++)
                for (int b = 0; b < T; b++) grad_force[a * T + b] = (float)acc[a * kTableStride + b];
        if (grad_params)
            for (int g = 0; g < CF_GRAD_PARAMS; g++) grad_params[g] = (float)acc[kTableSize + g];
        return CF_OK;
    }
    return CF_OK;
}

int cf_rdf(cf_world* w, const float* d_pos4, int bins, float r_max, float* d_hist)
{
    int rc = check_world(w);
    if (rc) return rc;
    if (w->worlds > 1) return fail(CF_ERR_INVALID, "the radial distribution covers a single world");
    const int T = w->num_types;
    if (bins < 1 || !d_hist || (long long)T * T * bins > kRdfMaxEntries)
        return fail(CF_ERR_INVALID, "bins must be >= 1 with T * T * bins <= 49152, d_hist not NULL");
    if (!(r_max > 0.0f) || !std::isfinite(r_max)) return fail(CF_ERR_INVALID, "r_max must be finite and positive");
    rc = ensure_rdf(w);
    if (rc) return rc;
    Grid g = choose_step_grid(w->ext, rdf_cutoff(bins, r_max), kMaxCells);
    apply_worlds(g, 1);
    rc = ensure_cells(w, g.cells);
    if (!rc) rc = ensure_offsets(w, g.cells);
    if (rc) return rc;
    CF_CUDA(configure_adjoint());
    Rollout& r = w->ro;
    const float4* pos = w->pos;
    if (d_pos4) {
        CF_CUDA(launch_pack_pos(reinterpret_cast<const float4*>(d_pos4), w->pos, r.rdf_pos, w->n, w->stream));
        pos = r.rdf_pos;
    }
    Scratch& s = w->s;
    int which = 0;
    CF_CUDA(launch_cell_list_csr(pos, w->n, g, w->ext, T, s, s.cell_off, nullptr, nullptr, w->err, &which, w->stream));
    CF_CUDA(launch_rdf(w->ext, g, w->n, T, bins, r_max, s.pos_sorted, s.keys[which], s.cell_off, r.rdf_acc,
                       r.type_count, d_hist, w->stream));
    return CF_OK;
}

int cf_rdf_backward(cf_world* w, const float* d_pos4, int bins, float r_max, const float* d_ghist, float* d_gpos4)
{
    int rc = check_world(w);
    if (rc) return rc;
    if (w->worlds > 1) return fail(CF_ERR_INVALID, "the radial distribution covers a single world");
    const int T = w->num_types;
    if (bins < 1 || !d_ghist || !d_gpos4 || (long long)T * T * bins > kRdfMaxEntries)
        return fail(CF_ERR_INVALID, "bins must be >= 1 with T * T * bins <= 49152, buffers not NULL");
    if (!(r_max > 0.0f) || !std::isfinite(r_max)) return fail(CF_ERR_INVALID, "r_max must be finite and positive");
    rc = ensure_rdf(w);
    if (rc) return rc;
    Grid g = choose_step_grid(w->ext, rdf_cutoff(bins, r_max), kMaxCells);
    apply_worlds(g, 1);
    rc = ensure_cells(w, g.cells);
    if (!rc) rc = ensure_offsets(w, g.cells);
    if (rc) return rc;
    CF_CUDA(configure_adjoint());
    Rollout& r = w->ro;
    const float4* pos = w->pos;
    if (d_pos4) {
        CF_CUDA(launch_pack_pos(reinterpret_cast<const float4*>(d_pos4), w->pos, r.rdf_pos, w->n, w->stream));
        pos = r.rdf_pos;
    }
    Scratch& s = w->s;
    int which = 0;
    CF_CUDA(launch_cell_list_csr(pos, w->n, g, w->ext, T, s, s.cell_off, nullptr, nullptr, w->err, &which, w->stream));
    CF_CUDA(launch_rdf_grad(w->ext, g, w->n, T, bins, r_max, pos, s.pos_sorted, s.keys[which], s.vals[which],
                            s.cell_off, d_ghist, r.type_count, reinterpret_cast<float4*>(d_gpos4), w->stream));
    return CF_OK;
}

}  // extern "C"
