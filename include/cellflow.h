/*
 * cellflow.h - C ABI of the GB300 CellFlow simulation step.
 *
 * This ABI replaces the C++ class `ParticleSimulation`
 * (cuda-native/include/ParticleSimulation.cuh:10-103) and the physics subset of
 * `SimulationParams` (cuda-native/include/SimulationParams.h:14-37).  Every entry
 * point below names the reference member it stands in for.
 *
 * Conventions
 *   - Every function returns an int status: CF_OK (0) or a negative CF_ERR_*
 *     code.  cf_last_error() returns a message for the last failure on the
 *     calling thread.  The reference printed and called exit(1) instead
 *     (cuda-native/src/ParticleSimulation.cu:10-18).
 *   - One cf_world owns its device buffers and one CUDA stream.  Calls that
 *     launch work are asynchronous on that stream; cf_sync() waits and reports
 *     device-side errors (a particle that left the domain, a bounded wait that
 *     gave up).  Calls that return data to host memory synchronise first.  A
 *     handle is not re-entrant: use it from one thread at a time.
 *   - Host pointers are plain host memory (pinned or pageable).  Functions with
 *     a `_device` suffix take device pointers on the world's device.
 *   - Positions live in the periodic box [0,W)x[0,H)x[0,D).  The step keeps the
 *     reference's Jacobi-consistent meaning: every particle sees the positions
 *     of the start of the step (the reference kernel raced here, reading slots
 *     other threads were rewriting; ParticleSimulation.cu:89 vs :164).
 */
#ifndef CELLFLOW_H
#define CELLFLOW_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CF_OK 0
#define CF_ERR_INVALID (-1)  /* bad argument or size                        */
#define CF_ERR_CUDA (-2)     /* a CUDA runtime call failed                    */
#define CF_ERR_ALLOC (-3)    /* device or host allocation failed              */
#define CF_ERR_DOMAIN (-4)   /* a position is outside [0,W) or not finite     */
#define CF_ERR_DEVICE (-5)   /* a kernel raised its error word                */
#define CF_ERR_CAPACITY (-6) /* an output buffer is too small                 */

#define CF_MAX_TYPES 32     /* the reference capped at 10 (SimulationParams.h:64) */
#define CF_MAX_PROX_CONN 16 /* the reference overflowed nearby[32] above 16 (ParticleSimulation.cu:210,215) */

/* Particle record, byte-compatible with the reference `Particle`
 * (SimulationParams.h:6-12): 44 bytes, pos, vel, acc, type, pad. */
typedef struct cf_particle {
    float pos[3];
    float vel[3];
    float acc[3];
    uint32_t ptype;
    float pad;
} cf_particle;

/* RGB colour per type, the reference `ParticleColor` (SimulationParams.h:60-62). */
typedef struct cf_color {
    float r, g, b;
} cf_color;

/* Physics parameters of one step: the fields of `SimulationParams`
 * (SimulationParams.h:15-29) that the step kernel reads
 * (ParticleSimulation.cu:97-161), in the same order and meaning. */
typedef struct cf_step_params {
    float radius;               /* interaction radius                         */
    float delta_t;              /* time step                                  */
    float friction;             /* velocity multiplier per step               */
    float repulsion;            /* repulsion amplitude                        */
    float attraction;           /* attraction slope                           */
    float k;                    /* repulsion decay                            */
    float balance;              /* density balance                            */
    float canvas_width;         /* W: box extent in x                         */
    float canvas_height;        /* H: box extent in y                         */
    float canvas_depth;         /* D: box extent in z                         */
    int num_particle_types;     /* T                                          */
    float ratio_with_lfo;       /* per-type radius modulation ratio           */
    float force_multiplier;     /* global force scale                         */
    int max_expected_neighbors; /* density normaliser                         */
} cf_step_params;

typedef struct cf_world cf_world;

/* Grid chosen for a step (introspection for tests and tools). */
typedef struct cf_grid_info {
    int cells[3];      /* cells per axis                                      */
    float inv_cell[3]; /* cells per unit length, the hash multiplier          */
    float r_max;       /* largest effective radius over type pairs            */
    int generic_wrap;  /* 1: per-candidate reference wrap; 0: per-cell shift  */
    int key_bits;      /* bits of the linear cell id                          */
} cf_grid_info;

/* Device buffers of a world (all in original particle order). */
typedef struct cf_device_view {
    void* pos4;   /* float4[n]: x, y, z, type (uint32 bits in .w)             */
    void* vel4;   /* float4[n]: vx, vy, vz, 0                                 */
    void* acc4;   /* float4[n]: ax, ay, az, 0 (the last step's scaled force)  */
    void* counts; /* int32[n]: neighbour counts of the last step              */
    int n;
} cf_device_view;

/* ---- library ----------------------------------------------------------- */

const char* cf_last_error(void);
const char* cf_version(void);
/* Kernels this library has put on CUDA streams since it was loaded, all worlds
 * and threads together: every direct launch, and every kernel node of each
 * CUDA graph it launches (a step, a batch replay, a selection pass, a rollout
 * backward).  The difference around a region is that region's launch count. */
long long cf_kernel_launches(void);

/* ---- host-side fault injection and limits (no counterpart in the reference,
 * whose CUDA_CHECK printed and exited, ParticleSimulation.cu:10-18) -------- */

/* Cap on the device memory the library itself holds (every buffer of every
 * world and batch), in bytes; 0 removes the cap.  An allocation that would
 * exceed it fails as cudaMalloc out of memory would: CF_ERR_ALLOC, with the
 * cap named in cf_last_error().  Lowering it frees nothing already held. */
int cf_set_device_memory_limit(size_t bytes);
/* Device memory the library holds now, in bytes. */
int cf_device_memory_in_use(size_t* bytes);
/* Arms a one-shot injected CUDA error: the CUDA call sites whose text
 * contains `site` (e.g. "cudaMalloc", "cudaStreamSynchronize",
 * "launch_step_force") pass `skip` times, then the next one returns
 * `cuda_error` (a cudaError_t value) without making the call, and the
 * library reports it as it would a real failure (CF_ERR_CUDA, or CF_ERR_ALLOC
 * for cudaErrorMemoryAllocation).  NULL disarms.  Process-wide. */
int cf_inject_cuda_error(const char* site, int cuda_error, int skip);
/* 1 while an injected error is armed and has not fired, else 0. */
int cf_injection_pending(void);
/* SimulationParams defaults (SimulationParams.h:15-29). */
void cf_default_params(cf_step_params* p);

/* ---- lifetime ---------------------------------------------------------- */

/* ParticleSimulation(int) / (int, float, float) (ParticleSimulation.cuh:12-13,
 * ParticleSimulation.cu:427-445).  Allocates n particles of num_types types in
 * a W x H x D box, fills a seeded force table and radius table and spawns the
 * particles with cf_initialize_particles(seed, min(2000, box)). */
int cf_create(int n, int num_types, float w, float h, float d, uint64_t seed, cf_world** out);
/* ~ParticleSimulation (ParticleSimulation.cu:447-449). */
int cf_destroy(cf_world* w);
/* Run the world's work on a caller-owned cudaStream_t (NULL restores the
 * world's own stream).  The caller keeps the stream alive. */
int cf_set_stream(cf_world* w, void* cuda_stream);
int cf_sync(cf_world* w);
int cf_particle_count(const cf_world* w, int* n);
int cf_num_particle_types(const cf_world* w, int* t);

/* setParticleCount (ParticleSimulation.cu:564-572): reallocates and respawns.
 * If the reallocation fails (CF_ERR_ALLOC), the world holds no particle buffers
 * and every other call on it returns CF_ERR_INVALID until a later
 * cf_set_particle_count succeeds (or cf_destroy). */
int cf_set_particle_count(cf_world* w, int n, uint64_t seed);
/* setNumParticleTypes (ParticleSimulation.cu:574-579): new type count, new
 * seeded raw table and radius table, respawn. */
int cf_set_num_particle_types(cf_world* w, int t, uint64_t seed);
/* initializeParticles (ParticleSimulation.cu:484-505, kernel :29-66): uniform
 * positions in a centred spawn cube of side min(spawn, extent), zero velocity
 * and acceleration, uniform types.  Seeded counter-based generator instead of
 * the reference's time-seeded cuRAND state; the type is clamped to T-1 (the
 * reference could produce T when its uniform draw was exactly 1.0). */
int cf_initialize_particles(cf_world* w, uint64_t seed, float spawn_region);
/* updateCanvasDimensions / initializeParticles(W, H) (ParticleSimulation.cu:497-503,
 * :486-489): the box that cf_initialize_particles spawns in and
 * cf_move_universe wraps into; the step itself wraps with the extents in its
 * cf_step_params, as the reference's kernel does (:159-161). */
int cf_set_canvas(cf_world* w, float width, float height, float depth);
/* moveUniverse (ParticleSimulation.cuh:50, ParticleSimulation.cu:585-592,
 * kernel :169-185): every position becomes fmodf((p + d) + W, W) per axis.
 * The reference wrapped with a default-constructed SimulationParams' 8000-unit
 * canvas whatever the world's box; here the world's own box is used.  A shift
 * below -W leaves negative coordinates, as there; the next step reports them
 * (CF_ERR_DOMAIN).  Asynchronous on the world's stream. */
int cf_move_universe(cf_world* w, float dx, float dy, float dz);

/* ---- particle state ---------------------------------------------------- */

/* getParticleData (ParticleSimulation.cu:558-562): AoS 44-byte records;
 * synchronises.  A page-locked `out` is written directly by the conversion
 * kernel through its device view (no staging copy). */
int cf_get_particles(cf_world* w, cf_particle* out, int n);
/* Upload AoS records (the reference had no setter; its init kernel wrote
 * them).  Positions must lie in [0,W)x[0,H)x[0,D), types in [0,T).  A
 * page-locked `in` is read directly by the conversion kernel, later on the
 * world's stream: keep it unchanged until the stream has passed that point
 * (cf_sync), as with any asynchronous copy from page-locked memory. */
int cf_set_particles(cf_world* w, const cf_particle* in, int n);
/* Structure-of-arrays state: pos4/vel4 are float[4n] (type bits in pos4.w),
 * counts int[n] (the neighbour counts the next step reads as "previous"). */
int cf_get_state(cf_world* w, float* pos4, float* vel4, int* counts);
int cf_set_state(cf_world* w, const float* pos4, const float* vel4, const int* counts);
/* The neighbour counts written by the last step (neighborCountsOut,
 * ParticleSimulation.cu:165). */
int cf_get_neighbor_counts(cf_world* w, int* out, int n);
int cf_device_buffers(cf_world* w, cf_device_view* out);

/* ---- parameter surface ------------------------------------------------- */

/* getRawForceTableValues (ParticleSimulation.cuh:47): T*T raw values. */
int cf_get_raw_force_table(cf_world* w, float* raw, int count);
int cf_set_raw_force_table(cf_world* w, const float* raw, int count);
/* regenerateForceTable / initializeForceTable (ParticleSimulation.cu:513-519,
 * 581-583): raw values uniform in [-1,1] from a seeded generator, then
 * updateForceTable(0.28, -0.20, 1.0). */
int cf_regenerate_force_table(cf_world* w, uint64_t seed);
/* updateForceTable (ParticleSimulation.cu:521-531):
 * F = clamp(tanhf(raw*offset)*range + bias, -1, 1), row-major [self*T+other]. */
int cf_update_force_table(cf_world* w, float range, float bias, float offset);
/* Set the final device table directly (T*T values, used unclamped). */
int cf_set_force_table(cf_world* w, const float* table, int count);
int cf_get_force_table(cf_world* w, float* table, int count);
/* radioByType (ParticleSimulation.cu:533-539, 594-622). */
int cf_get_radio_by_type(cf_world* w, float* out, int count);
int cf_set_radio_by_type(cf_world* w, const float* values, int count);
int cf_set_radio_by_type_value(cf_world* w, int index, float value);
int cf_rotate_radio_by_type(cf_world* w);
/* The caller-side LFO of CellFlowWidget::paintGL (CellFlowWidget.cpp:414-421):
 * returns ratio + lfo_a*sin(2*pi*lfo_s*t), or ratio when lfo_a == 0. */
float cf_lfo_ratio(float ratio, float lfo_a, float lfo_s, float t_seconds);

/* ---- the step ----------------------------------------------------------- */

/* simulate (ParticleSimulation.cu:541-556), run nsteps times.  Each step
 * builds the cell list, computes forces, neighbour counts and the
 * density-adaptive scale, integrates and wraps.  Asynchronous. */
int cf_step(cf_world* w, const cf_step_params* p, int nsteps);
/* One step with host buffers, for a caller that keeps the particles in host
 * memory: uploads the 44-B records from `in`, steps once (as cf_step), and
 * writes the records to `out`; synchronises and reports device errors.
 * Equivalent to cf_set_particles + cf_step + cf_get_particles.  When `in` and
 * `out` are page-locked (cudaHostAlloc / cudaHostRegister) the conversion
 * kernels read and write them directly and the step runs as one cached CUDA
 * graph; otherwise as the three calls.  `in`
 * and `out` may be the same buffer.  No counterpart in the reference (its
 * state stays on the device and only getParticleData copies it back). */
int cf_step_host(cf_world* w, const cf_step_params* p, const cf_particle* in, cf_particle* out, int n);

/* Force-kernel variants: v % 4 picks the staging: 0 = 256 candidates staged
 * per warp batch, register budget for 8 blocks per SM; 1 = 256 staged, 6
 * blocks per SM; 2 = as 1 with lanes paired in the drain (the lane with the
 * fewest hits of a batch takes part of the busiest lane's, and so on down the
 * sorted hit counts); 3 = 384 staged, 6 blocks per SM.  v / 4 picks the warps
 * per 32-particle item: 1, 2 or 4 (each warp takes an equal share of the
 * item's candidates; more warps for worlds too small to fill the GPU).
 * Variants 12, 13 and 14 use the balanced drain (256 staged, 6 blocks per
 * SM) with 1, 2 or 4 warps per item: a batch's hits, home by home, are split
 * into 32 equal ranges, one per lane, and each home adds the partial sums of
 * its pieces in lane order.
 * Results are bit-identical across stagings 0, 1 and 3; with lane pairing,
 * the balanced drain, and 2 or 4 warps, partial sums are added in a fixed
 * order, which differs from the single-lane order by rounding only. */
#define CF_FORCE_VARIANTS 15
/* Autotuner of the step (no counterpart in the reference): runs `steps`
 * trial steps with each force-kernel variant, restores the particle state,
 * keeps the fastest variant for later steps and returns it in
 * *chosen_variant. */
int cf_autotune_step(cf_world* w, const cf_step_params* p, int steps, int* chosen_variant);
/* Select a force-kernel variant directly. */
int cf_set_force_variant(cf_world* w, int variant);
/* The grid cf_step would use for these parameters. */
int cf_get_grid(cf_world* w, const cf_step_params* p, cf_grid_info* out);
/* Build the cell list of the current positions with the step's grid and
 * return it: cell id per particle, particle indices in stable cell order,
 * and per-cell [start,end) into that order (cells with no particle: 0,0).
 * Sizes: n, n, cells, cells where cells = product of cf_grid_info.cells. */
int cf_debug_cell_list(cf_world* w, const cf_step_params* p, uint32_t* cell_of, uint32_t* sorted_idx,
                       uint32_t* cell_start, uint32_t* cell_end, int cells_cap);
/* Work counters of the current positions with the canonical grid of the
 * work model (cells per axis floor(L/r_max)): directed candidate pairs in
 * the 27-cell stencil (C27) and directed interacting pairs (I). */
int cf_work_counters(cf_world* w, const cf_step_params* p, uint64_t* c27, uint64_t* interacting);
/* The force kernel's filter work for the current state (no counterpart in the
 * reference): the candidates its items stage (the union of each item's homes'
 * 27-cell stencils, summed over items) and the candidate tests of the items'
 * particles (staged x particles per item).  tested / n against the work model's
 * C27 / n is the filter's excess over the canonical stencil.  Builds the step's
 * cell list; the particle state is unchanged. */
int cf_force_work(cf_world* w, const cf_step_params* p, uint64_t* staged, uint64_t* tested);

/* Bounds-checked library (libcellflow_bounds.so, built with -DCF_DEBUG_BOUNDS;
 * no counterpart in the reference, whose kernels had no index checks).  The
 * cell-list, force and proximity kernels test their derived indices before
 * each access; an index outside its buffer is recorded (the first per source
 * file) and the access skipped, instead of faulting.  cf_debug_bounds reports
 * whether this library is the checked one, and the first recorded violation
 * ("file.cu:line", the index and its limit), then clears the records.  In the
 * normal library checked = 0 and nothing is ever found. */
int cf_debug_bounds(int* checked, int* found, char* where, int where_cap, long long* index, long long* limit);
/* Checked library only (else CF_ERR_INVALID): builds the step's cell list,
 * overwrites the first force-kernel item's first particle with `first`, and
 * runs the force kernel: a first outside [0, n) must be recorded by
 * cf_debug_bounds and that item skipped.  The other items are stepped. */
int cf_debug_force_bad_item(cf_world* w, const cf_step_params* p, int first);

/* ---- proximity graph ---------------------------------------------------- */

/* generateProximityGraph (ParticleSimulation.cu:625-687, kernel :188-277) with
 * the GL buffer replaced by plain output.  For each particle i: the first
 * 2*max_conn particles j>i of the same type with non-periodic squared distance
 * below distance^2, in index order; of those the max_conn nearest (ties keep
 * index order).  Edges are written as (i, j) pairs, ordered by i, then by
 * distance.  max_conn must be in [0, CF_MAX_PROX_CONN].  Writes up to cap
 * edges to `edges` (int32[2*cap], host); *n_edges receives the full count
 * (CF_ERR_CAPACITY when it exceeds cap). */
int cf_proximity_edges(cf_world* w, float distance, int max_conn, int32_t* edges, int cap, int* n_edges);
/* Same edge set, written as the reference's line vertices: per edge two
 * vertices of 6 floats (x, y, z, r, g, b), colour of particle i's type
 * (colors[type % T]).  `vertices` is a DEVICE buffer of cap_vertices*6
 * floats standing in for the GL VBO; *vertex_count = 2 * edges.  The edges'
 * order in the buffer is arbitrary, as with the reference's atomicAdd append
 * (ParticleSimulation.cu:250): each particle's edges are placed by one atomic
 * in the selection pass itself. */
int cf_proximity_vertices_device(cf_world* w, float distance, int max_conn, const cf_color* colors, int n_colors,
                                 float* vertices, int cap_vertices, int* vertex_count);

/* Triangle mesh, generateTriangleMesh (ParticleSimulation.cu:689-747, kernel
 * :280-424): for each particle i, the first min(max_conn, 32) other particles
 * of its type in index order with non-periodic squared distance below
 * distance^2 * 1.2^2 (the reference's hysteresis, :723-724); every pair (a, b)
 * of them with both indices above i is a triangle (i, a, b), at most 64 per
 * particle.  Output in i order, then pair order (the reference appended
 * through an atomicAdd, so its order varied; the set is the same).
 * cf_triangle_mesh writes 3 indices per triangle to host memory
 * (CF_ERR_CAPACITY when the count exceeds cap, *n_triangles always set;
 * triangles NULL with cap 0 only counts, as does a NULL vertex buffer with
 * cap_vertices 0 below). */
#define CF_MESH_MAX_CONN 32
int cf_triangle_mesh(cf_world* w, float distance, int max_conn, int32_t* triangles, int cap, int* n_triangles);
/* The same triangles as the reference's vertices: 3 per triangle, 9 floats
 * each (x, y, z, flat normal, colour of i's type: colors[type % T]) into a
 * DEVICE buffer of cap_vertices*9 floats standing in for the GL VBO;
 * *vertex_count = 3 * triangles. */
int cf_triangle_mesh_device(cf_world* w, float distance, int max_conn, const cf_color* colors, int n_colors,
                            float* vertices, int cap_vertices, int* vertex_count);

/* Proximity edges without allocating: the same edges, in the same order, as
 * cf_proximity_edges, for callers that may not allocate device memory while
 * they run -- a renderer's frame loop building the graph every frame (an
 * allocation can stall the device inside the frame), or a host application
 * whose device memory is owned by its own pool.  No counterpart in the
 * reference (its wrapper allocated and freed buffers on every call).
 *   d_pos4   DEVICE float4[n]: x, y, z, type bits (cf_device_view.pos4 layout),
 *            positions inside [0,width)x[0,height)x[0,depth)
 *   d_edges  DEVICE int32[2*cap] receiving (i, j) pairs; *n_edges (host) the
 *            full count (CF_ERR_CAPACITY when it exceeds cap)
 *   stream   cudaStream_t the work runs on (NULL: the legacy default stream);
 *            the call waits for it before returning
 * Limits: n <= 65536 (CF_ERR_INVALID above); the proximity grid is coarsened
 * to at most 65536 cells.  All scratch lives in one fixed device array of
 * about 6.9 MB that every device holds from the library's first use there
 * until the process exits.  The first call on a device looks up that array's
 * address, so make it before any stream capture.  Calls share the array and
 * it keeps the previous call's contents (the call clears what must start at
 * zero): calls whose work overlaps on the GPU -- other streams, other threads
 * on the same device -- race and must be serialised by the caller.
 * It calls no cudaMalloc, cudaFree or other allocating routine. */
int cf_proximity_edges_noalloc(const void* d_pos4, int n, float width, float height, float depth, float distance,
                               int max_conn, int32_t* d_edges, int cap, int* n_edges, void* stream);

/* ---- batched ensembles (no counterpart in the reference) ------------------ */

/* Many independent worlds of uneven size, each with its own force table,
 * sharing the step parameters and box; one cell list, one plan and one force
 * launch per step cover all of them.  World k owns particles
 * [offsets[k], offsets[k+1]) of the concatenated state.  A batch of one world
 * steps exactly like cf_step; every world of a batch steps exactly like the
 * same world run alone (bit for bit). */
typedef struct cf_batch cf_batch;

/* Worlds spawned as cf_initialize_particles(seed + k, 2000) and given the
 * default force table of a raw table drawn from seed + k. */
int cf_batch_create(int worlds, const int* n_per_world, int num_types, float w, float h, float d, uint64_t seed,
                    cf_batch** out);
int cf_batch_destroy(cf_batch* b);
/* worlds, total particles, offsets[worlds + 1] (any may be NULL). */
int cf_batch_info(const cf_batch* b, int* worlds, int* total, int* offsets);
/* The batch as one cf_world (profiling, work counters, device buffers); its
 * pos4.w carries the world index above the type bits. */
int cf_batch_world(cf_batch* b, cf_world** out);
/* Concatenated SoA state; pos4.w = type (the world index is implied by the
 * offsets). */
int cf_batch_set_state(cf_batch* b, const float* pos4, const float* vel4, const int* counts);
int cf_batch_get_state(cf_batch* b, float* pos4, float* vel4, int* counts);
/* worlds * T * T values, world-major, each row-major [self*T + other]. */
int cf_batch_set_force_tables(cf_batch* b, const float* tables, int count);
int cf_batch_step(cf_batch* b, const cf_step_params* p, int nsteps);
/* Capture nsteps steps into one CUDA graph; cf_batch_replay launches it. */
int cf_batch_capture(cf_batch* b, const cf_step_params* p, int nsteps);
int cf_batch_replay(cf_batch* b);
/* Steps and kernel nodes of the captured graph (0 and 0 before any capture). */
int cf_batch_graph_info(const cf_batch* b, int* steps, long long* kernels);
int cf_batch_autotune(cf_batch* b, const cf_step_params* p, int steps, int* chosen_variant);
int cf_batch_sync(cf_batch* b);
int cf_batch_set_stream(cf_batch* b, void* cuda_stream);

/* ---- differentiable rollout (no counterpart in the reference) ---------------
 *
 * The gradient of a loss of the state after K steps with respect to the
 * initial positions and velocities, the force table (as cf_set_force_table
 * sets it) and six step parameters.  Neighbour counts are held constant (their
 * derivative is zero almost everywhere), the periodic wrap counts as the
 * identity, and the neighbour sets are recomputed in the backward pass from
 * states replayed out of checkpoints taken every `checkpoint_every` steps, so
 * device memory stays O(n (K / checkpoint_every + checkpoint_every)).
 * Device pointers hold n float4 values (x, y, z, unused), on the world's
 * device, ordered like the world's particles; types never change and come
 * from the world. */
#define CF_GRAD_REPULSION 0
#define CF_GRAD_ATTRACTION 1
#define CF_GRAD_K 2
#define CF_GRAD_FORCE_MULTIPLIER 3
#define CF_GRAD_BALANCE 4
#define CF_GRAD_FRICTION 5
#define CF_GRAD_PARAMS 6

/* Run nsteps steps from (d_pos4_in, d_vel4_in) — either may be NULL to start
 * from the world's current positions or velocities — with the world's
 * neighbour counts as the previous counts of the first step, keeping
 * checkpoints.  The world ends in the state after nsteps steps, also copied
 * to d_pos4_out / d_vel4_out when they are not NULL. */
int cf_rollout_forward(cf_world* w, const cf_step_params* p, const float* d_pos4_in, const float* d_vel4_in,
                       int nsteps, int checkpoint_every, float* d_pos4_out, float* d_vel4_out);
/* Adjoint of the last cf_rollout_forward: from dL/dx_K and dL/dv_K (either may
 * be NULL for zero) to dL/dx_0 and dL/dv_0 (device, either may be NULL),
 * dL/dF (host, T*T row-major, or NULL) and dL/dparams (host, CF_GRAD_PARAMS
 * values in CF_GRAD_* order, or NULL).  Fails with CF_ERR_INVALID when the
 * force table, the radii or the particle count changed since the forward.
 * The world's state is left as the forward left it. */
int cf_rollout_backward(cf_world* w, const float* d_gpos4, const float* d_gvel4, float* d_gpos4_out,
                        float* d_gvel4_out, float* grad_force, int grad_force_count, float* grad_params);
/* Soft type-resolved radial distribution of the positions d_pos4 (NULL: the
 * world's current ones): bins of width D = r_max / bins, cubic B-spline
 * weights of support 2 bins each side of the centre (k + 1/2) D, each entry
 * normalised by N_a (N_b / V) 4 pi c_k^2 D.  d_hist receives T * T * bins
 * floats [a][b][k] (device).  T * T * bins <= 49152. */
int cf_rdf(cf_world* w, const float* d_pos4, int bins, float r_max, float* d_hist);
/* dL/dpos (device, n float4) of L(hist) given d_ghist = dL/dhist (device). */
int cf_rdf_backward(cf_world* w, const float* d_pos4, int bins, float r_max, const float* d_ghist, float* d_gpos4);

/* ---- presets ----------------------------------------------------------------
 *
 * The reference's preset files (CellFlowWidget::loadPreset / savePreset,
 * cuda-native/src/CellFlowWidget.cpp:1070-1259): one JSON object with the
 * reference's keys.  Keys this library does not interpret (rendering,
 * camera, effect) are kept as JSON text and written back unchanged. */
#define CF_PRESET_PARTICLE_COUNT (1u << 0)   /* PARTICLE_COUNT                         */
#define CF_PRESET_NUM_TYPES (1u << 1)        /* numParticleTypes                       */
#define CF_PRESET_RADIUS (1u << 2)           /* radius                                 */
#define CF_PRESET_DELTA_T (1u << 3)          /* delta_t                                */
#define CF_PRESET_FRICTION (1u << 4)         /* friction                               */
#define CF_PRESET_REPULSION (1u << 5)        /* repulsion                              */
#define CF_PRESET_ATTRACTION (1u << 6)       /* attraction                             */
#define CF_PRESET_K (1u << 7)                /* k                                      */
#define CF_PRESET_BALANCE (1u << 8)          /* balance                                */
#define CF_PRESET_FORCE_MULTIPLIER (1u << 9) /* forceMultiplier                        */
#define CF_PRESET_CANVAS (1u << 10)          /* canvasWidth / canvasHeight / canvasDepth */
#define CF_PRESET_FORCE_TRANSFORM (1u << 11) /* forceRange / forceBias / forceOffset   */
#define CF_PRESET_LFO (1u << 12)             /* ratio / lfoA / lfoS                    */
#define CF_PRESET_SPAWN_REGION (1u << 13)    /* spawnRegionSize                        */
#define CF_PRESET_RADIO (1u << 14)           /* radioByType                            */
#define CF_PRESET_RAW_TABLE (1u << 15)       /* rawForceTable                          */
#define CF_PRESET_COLORS (1u << 16)          /* particleColors                         */

typedef struct cf_preset {
    unsigned present;         /* CF_PRESET_* bits of the keys found                 */
    int particle_count;       /* PARTICLE_COUNT                                      */
    cf_step_params params;    /* SimulationParams defaults where a key is absent;
                               * num_particle_types = numParticleTypes               */
    float force_range, force_bias, force_offset; /* defaults 0.28, -0.20, 1.0      */
    float ratio, lfo_a, lfo_s;                   /* defaults 0, 0, 0.1             */
    float spawn_region;       /* spawnRegionSize                                     */
    int n_radio;              /* radioByType                                         */
    float radio[CF_MAX_TYPES];
    int n_raw;                /* rawForceTable, row-major [self*T + other]           */
    float raw[CF_MAX_TYPES * CF_MAX_TYPES];
    int n_colors;             /* particleColors                                      */
    cf_color colors[CF_MAX_TYPES];
    char extra[8192];         /* uninterpreted keys, as JSON members                 */
} cf_preset;

/* Parse preset JSON text (UTF-8, len bytes).  Numbers as QJsonValue::toDouble
 * reads them, narrowed to float as the reference's float fields hold them;
 * malformed JSON returns CF_ERR_INVALID with the offset in cf_last_error(). */
int cf_preset_parse(const char* json, size_t len, cf_preset* out);
/* loadPreset (CellFlowWidget.cpp:1070-1180) on a world: the particle count
 * and the type count (each respawns from seed), the radius values for
 * i < min(len, T), the raw table for i < min(len, T*T), then
 * cf_update_force_table(force_range, force_bias, force_offset).  The step
 * parameters present in the preset are written into *params (others kept),
 * params->num_particle_types = T. */
int cf_preset_apply(cf_world* w, const cf_preset* p, uint64_t seed, cf_step_params* params);
/* savePreset (CellFlowWidget.cpp:1182-1259): JSON text with the reference's
 * keys, the count, types, radius values and raw table from the world and the
 * rest from *p.  buf NULL: only the length (without the terminating NUL) in
 * *len; otherwise cap must exceed it. */
int cf_preset_write(cf_world* w, const cf_preset* p, char* buf, size_t cap, size_t* len);

/* ---- measurement ---------------------------------------------------------- */

/* Device time of the step's phases, accumulated over the steps run since
 * profiling was enabled or last read, from CUDA events recorded on the
 * world's stream around each phase; and of the adjoint steps of
 * cf_rollout_backward (their per-particle and pair kernels), which run one
 * after another, outside any graph, while profiling is on. */
typedef struct cf_phase_times {
    double cell_list_ms;     /* hash + radix sort + start/end + sorted snapshot */
    double force_ms;         /* force + density + integrator kernel           */
    long long steps;         /* steps covered                                  */
    long long launches;      /* kernel launches of the library in those steps  */
    double adjoint_ms;       /* adj_prep + adj_pair kernels of backward steps  */
    long long adjoint_steps; /* backward steps covered                         */
} cf_phase_times;

/* No counterpart in the reference (it had only a frame counter,
 * CellFlowWidget.cpp:705-713).  Enabling adds events around each phase (no
 * synchronisation: the times are read when cf_profile_read is called). */
int cf_profile_enable(cf_world* w, int on);
int cf_profile_read(cf_world* w, cf_phase_times* out);
/* Measured FP32 FMA throughput of the current device in TFLOP/s (an FMA
 * counts 2 flops): dependent FMA chains on every SM, timed with events. */
int cf_measure_fp32_peak(double* tflops);

#ifdef __cplusplus
}
#endif

#endif /* CELLFLOW_H */
