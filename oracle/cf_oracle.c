/*
 * cf_oracle.c - CPU restatement of the CellFlow step, for checking only.
 *
 * TEST INFRASTRUCTURE.  Only the tests, the smoke check and the CPU-baseline
 * leg of the benchmark load this file's library, and only as the checker or
 * as the timed CPU baseline.  The product path never calls it.
 *
 * Arithmetic rules
 *   Built with -ffp-contract=off: every float operation is rounded on its
 *   own, in the order the reference source writes it.  This pins the
 *   reference's rounding, which nvcc would otherwise contract into FMAs.
 *   Library functions: sqrtf, expf, fmodf, floorf, tanhf from the C library.
 *
 * Semantics
 *   The reference step kernel updates particles in place while other threads
 *   read them (ParticleSimulation.cu:89 reads particles[j], :164 writes
 *   particles[idx]).  The oracle gives every particle the start-of-step
 *   state of all others (Jacobi), the only scheduling-independent reading.
 *
 * Parity anchors (reference file:line, paths inside aaronsb/CellFlow)
 *   cfo_step_f32        cuda-native/src/ParticleSimulation.cu:78-165
 *   cfo_step_f64        same maths in double, for error reports
 *   cfo_force_table     cuda-native/src/ParticleSimulation.cu:521-531
 *   cfo_rotate          cuda-native/src/ParticleSimulation.cu:594-605
 *   cfo_proximity_edges cuda-native/src/ParticleSimulation.cu:198-276
 *   cfo_triangle_mesh   cuda-native/src/ParticleSimulation.cu:290-423, 723-724
 *   cfo_lfo             cuda-native/src/CellFlowWidget.cpp:414-421
 *   cfo_cell_list       no reference counterpart (the reference is O(N^2));
 *                       defines the stable cell order the GPU list must match.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* Same field order as cf_step_params and the physics part of the reference
 * SimulationParams (cuda-native/include/SimulationParams.h:15-29). */
typedef struct cfo_params {
    float radius, delta_t, friction, repulsion, attraction, k, balance;
    float w, h, d;
    int num_types;
    float ratio_with_lfo;
    float force_multiplier;
    int max_expected_neighbors;
} cfo_params;

/* Effective radius of a pair (ParticleSimulation.cu:108-110). */
static float eff_radius(const cfo_params* p, const float* rb, uint32_t a, uint32_t b)
{
    float ra = p->radius * (1.0f + rb[a] * p->ratio_with_lfo);
    float rbb = p->radius * (1.0f + rb[b] * p->ratio_with_lfo);
    return (ra + rbb) * 0.5f;
}

/* Minimum-image step of one displacement (ParticleSimulation.cu:97-102):
 * two sequential tests, half extent computed as extent * 0.5f. */
static float min_image(float dx, float extent)
{
    if (dx > extent * 0.5f) dx -= extent;
    if (dx < -extent * 0.5f) dx += extent;
    return dx;
}

/*
 * One FP32 step for particles i = i_begin, i_begin + i_stride, ... < i_end.
 * pos/vel: float[3n], type: uint32[n], cnt_in: int[n] (previous counts),
 * F: float[T*T] row-major [self*T + other], rb: float[T].
 * Outputs are written only for the selected i, at index i.
 * ParticleSimulation.cu:78-165.
 */
void cfo_step_f32(int n, const float* pos, const float* vel, const uint32_t* type, const int* cnt_in, const float* F,
                  const float* rb, const cfo_params* p, int i_begin, int i_end, int i_stride, float* pos_out,
                  float* vel_out, float* acc_out, int* cnt_out)
{
    if (i_stride < 1) i_stride = 1;
    int rows = (i_end - i_begin + i_stride - 1) / i_stride;
#pragma omp parallel for schedule(dynamic, 8)
    for (int r = 0; r < rows; r++) {
        int i = i_begin + r * i_stride;
        float px = pos[3 * i], py = pos[3 * i + 1], pz = pos[3 * i + 2];
        uint32_t tp = type[i];
        float fx = 0.0f, fy = 0.0f, fz = 0.0f;
        int count = 0;
        for (int j = 0; j < n; j++) {
            if (j == i) continue;
            float dx = min_image(pos[3 * j] - px, p->w);
            float dy = min_image(pos[3 * j + 1] - py, p->h);
            float dz = min_image(pos[3 * j + 2] - pz, p->d);
            float dist_sq = dx * dx + dy * dy + dz * dz;
            float dist = sqrtf(dist_sq + 0.0001f);
            uint32_t to = type[j];
            float eff = eff_radius(p, rb, tp, to);
            if (dist < eff) {
                count++;
                float fv = F[tp * (uint32_t)p->num_types + to];
                float r_ = dist / eff;
                float rep = p->repulsion * expf(-p->k * r_ * r_);
                float att = p->attraction * r_;
                float net = rep - att;
                net *= fv;
                fx += (dx / dist) * net;
                fy += (dy / dist) * net;
                fz += (dz / dist) * net;
            }
        }
        /* density-adaptive scale, ParticleSimulation.cu:136-143 */
        float avg = (float)(count + cnt_in[i]) * 0.5f;
        float density = fminf(avg / (float)p->max_expected_neighbors, 1.0f);
        float adapt = 1.0f - (1.0f - p->balance) * density;
        float scale = p->force_multiplier * adapt;
        fx *= scale;
        fy *= scale;
        fz *= scale;
        /* friction integrator and wrap, ParticleSimulation.cu:146-161 */
        float vx = vel[3 * i] * p->friction + fx * p->delta_t;
        float vy = vel[3 * i + 1] * p->friction + fy * p->delta_t;
        float vz = vel[3 * i + 2] * p->friction + fz * p->delta_t;
        float nx = px + vx * p->delta_t;
        float ny = py + vy * p->delta_t;
        float nz = pz + vz * p->delta_t;
        pos_out[3 * i] = fmodf(nx + p->w, p->w);
        pos_out[3 * i + 1] = fmodf(ny + p->h, p->h);
        pos_out[3 * i + 2] = fmodf(nz + p->d, p->d);
        vel_out[3 * i] = vx;
        vel_out[3 * i + 1] = vy;
        vel_out[3 * i + 2] = vz;
        acc_out[3 * i] = fx;
        acc_out[3 * i + 1] = fy;
        acc_out[3 * i + 2] = fz;
        cnt_out[i] = count;
    }
}

/*
 * The same step in double precision from the same FP32 inputs, for error
 * reports.  Also returns, per particle,
 *     mag[i] = |scale| * sum_j |F_j| * (rep * exp(-k r_j^2) + att * r_j),
 * the size of the quantities whose rounded combination is the force: each
 * term is a difference (repulsion minus attraction, which cancels near their
 * crossing) and the terms are summed, so any evaluation order or few-ulp
 * function error moves the result by a small multiple of this, not of the
 * (possibly cancelled) result.  Rows selected as in cfo_step_f32.
 * ParticleSimulation.cu:78-165.
 */
void cfo_step_f64(int n, const float* pos, const float* vel, const uint32_t* type, const int* cnt_in, const float* F,
                  const float* rb, const cfo_params* p, int i_begin, int i_end, int i_stride, double* pos_out,
                  double* vel_out, double* acc_out, int* cnt_out, double* mag)
{
    if (i_stride < 1) i_stride = 1;
    int rows = (i_end - i_begin + i_stride - 1) / i_stride;
#pragma omp parallel for schedule(dynamic, 8)
    for (int r = 0; r < rows; r++) {
        int i = i_begin + r * i_stride;
        double px = pos[3 * i], py = pos[3 * i + 1], pz = pos[3 * i + 2];
        double W = p->w, H = p->h, D = p->d;
        uint32_t tp = type[i];
        double fx = 0, fy = 0, fz = 0, sum_abs = 0;
        int count = 0;
        for (int j = 0; j < n; j++) {
            if (j == i) continue;
            double dx = pos[3 * j] - px, dy = pos[3 * j + 1] - py, dz = pos[3 * j + 2] - pz;
            if (dx > W * 0.5) dx -= W;
            if (dx < -W * 0.5) dx += W;
            if (dy > H * 0.5) dy -= H;
            if (dy < -H * 0.5) dy += H;
            if (dz > D * 0.5) dz -= D;
            if (dz < -D * 0.5) dz += D;
            double dist = sqrt(dx * dx + dy * dy + dz * dz + 0.0001);
            uint32_t to = type[j];
            double ra = (double)p->radius * (1.0 + (double)rb[tp] * p->ratio_with_lfo);
            double ro = (double)p->radius * (1.0 + (double)rb[to] * p->ratio_with_lfo);
            double eff = (ra + ro) * 0.5;
            if (dist < eff) {
                count++;
                double r_ = dist / eff;
                double rep = (double)p->repulsion * exp(-(double)p->k * r_ * r_);
                double att = (double)p->attraction * r_;
                double fv = (double)F[tp * (uint32_t)p->num_types + to];
                double net = (rep - att) * fv;
                fx += dx / dist * net;
                fy += dy / dist * net;
                fz += dz / dist * net;
                sum_abs += (fabs(rep) + fabs(att)) * fabs(fv);
            }
        }
        double avg = (count + cnt_in[i]) * 0.5;
        double density = avg / (double)p->max_expected_neighbors;
        if (density > 1.0) density = 1.0;
        double scale = (double)p->force_multiplier * (1.0 - (1.0 - (double)p->balance) * density);
        fx *= scale;
        fy *= scale;
        fz *= scale;
        double vx = vel[3 * i] * (double)p->friction + fx * p->delta_t;
        double vy = vel[3 * i + 1] * (double)p->friction + fy * p->delta_t;
        double vz = vel[3 * i + 2] * (double)p->friction + fz * p->delta_t;
        double nx = fmod(px + vx * p->delta_t + W, W);
        double ny = fmod(py + vy * p->delta_t + H, H);
        double nz = fmod(pz + vz * p->delta_t + D, D);
        pos_out[3 * i] = nx;
        pos_out[3 * i + 1] = ny;
        pos_out[3 * i + 2] = nz;
        vel_out[3 * i] = vx;
        vel_out[3 * i + 1] = vy;
        vel_out[3 * i + 2] = vz;
        acc_out[3 * i] = fx;
        acc_out[3 * i + 1] = fy;
        acc_out[3 * i + 2] = fz;
        cnt_out[i] = count;
        mag[i] = fabs(scale) * sum_abs;
    }
}

/*
 * Force table transform (ParticleSimulation.cu:521-531).  The reference is
 * compiled by nvcc, whose headers resolve tanh(float) to the float overload,
 * so the transform runs in float: tanhf, then * range + bias, then clamp.
 */
void cfo_force_table(const float* raw, int count, float range, float bias, float offset, float* out)
{
    for (int i = 0; i < count; i++) {
        float t = tanhf(raw[i] * offset) * range + bias;
        out[i] = fmaxf(-1.0f, fminf(1.0f, t));
    }
}

/* rotateRadioByType (ParticleSimulation.cu:594-600): every value moves to
 * the next type, the last wraps to type 0. */
void cfo_rotate(float* values, int count)
{
    if (count < 1) return;
    float last = values[count - 1];
    for (int i = count - 1; i > 0; i--) values[i] = values[i - 1];
    values[0] = last;
}

/* Caller LFO (CellFlowWidget.cpp:414-421): the product is formed in double
 * (M_PI is a double) and rounded to float once, then added in float. */
float cfo_lfo(float ratio, float lfo_a, float lfo_s, float t)
{
    if (lfo_a != 0.0f) {
        float lfo = (float)(lfo_a * sin(2.0 * M_PI * (double)lfo_s * (double)t));
        return ratio + lfo;
    }
    return ratio;
}

/*
 * Proximity edges (ParticleSimulation.cu:198-276).  For each i: scan j > i
 * in index order while fewer than 2*max_conn candidates are held; keep j of
 * the same type with non-periodic squared distance below distance^2; sort the
 * candidates by squared distance with a stable insertion sort; emit the first
 * max_conn as edges (i, j).  Edges are written in i order.  Returns the edge
 * count (edges beyond cap are counted, not written).
 */
long cfo_proximity_edges(int n, const float* pos, const uint32_t* type, float distance, int max_conn_in,
                         int32_t* edges, long cap)
{
    float dsq = distance * distance;
    int max_conn = max_conn_in < 32 ? max_conn_in : 32;
    if (max_conn < 0) max_conn = 0;
    /* per-particle results first (rows are independent), then compaction in i order */
    int* kept = (int*)malloc(sizeof(int) * ((size_t)n * (max_conn > 0 ? max_conn : 1) + 1));
    int* kept_n = (int*)calloc((size_t)n + 1, sizeof(int));
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < n; i++) {
        float cd[64];
        int cj[64];
        int held = 0;
        for (int j = i + 1; j < n && held < max_conn * 2; j++) {
            if (type[i] != type[j]) continue;
            float dx = pos[3 * j] - pos[3 * i];
            float dy = pos[3 * j + 1] - pos[3 * i + 1];
            float dz = pos[3 * j + 2] - pos[3 * i + 2];
            float d2 = dx * dx + dy * dy + dz * dz;
            if (d2 < dsq) {
                cd[held] = d2;
                cj[held] = j;
                held++;
            }
        }
        for (int a = 1; a < held; a++) {
            float kd = cd[a];
            int kj = cj[a];
            int b = a - 1;
            while (b >= 0 && cd[b] > kd) {
                cd[b + 1] = cd[b];
                cj[b + 1] = cj[b];
                b--;
            }
            cd[b + 1] = kd;
            cj[b + 1] = kj;
        }
        int emit = held < max_conn ? held : max_conn;
        for (int e = 0; e < emit; e++) kept[(size_t)i * max_conn + e] = cj[e];
        kept_n[i] = emit;
    }
    long total = 0;
    for (int i = 0; i < n; i++) {
        for (int e = 0; e < kept_n[i]; e++) {
            if (total < cap) {
                edges[2 * total] = i;
                edges[2 * total + 1] = kept[(size_t)i * max_conn + e];
            }
            total++;
        }
    }
    free(kept);
    free(kept_n);
    return total;
}

/* Cell coordinate along one axis: floor(x * inv_cell), clamped to the grid. */
static int cell_coord(float x, float inv_cell, int m)
{
    float u = x * inv_cell;
    int c = (int)floorf(u);
    if (c < 0) c = 0;
    if (c > m - 1) c = m - 1;
    return c;
}

/*
 * Uniform-grid cell list with the stable order the GPU list must reproduce:
 * cell id (z*My + y)*Mx + x per particle, particle indices sorted by cell id
 * with ties in index order (a stable sort), and per-cell [start, end) into
 * that order (0, 0 for an empty cell).  m[3] cells per axis, inv_cell[3]
 * the hash multipliers (cells per unit length, as float).
 */
void cfo_cell_list(int n, const float* pos, const int* m, const float* inv_cell, uint32_t* cell_of,
                   uint32_t* sorted_idx, uint32_t* start, uint32_t* end)
{
    long cells = (long)m[0] * m[1] * m[2];
    uint32_t* fill = (uint32_t*)calloc((size_t)cells + 1, sizeof(uint32_t));
    for (int i = 0; i < n; i++) {
        int cx = cell_coord(pos[3 * i], inv_cell[0], m[0]);
        int cy = cell_coord(pos[3 * i + 1], inv_cell[1], m[1]);
        int cz = cell_coord(pos[3 * i + 2], inv_cell[2], m[2]);
        cell_of[i] = (uint32_t)(((long)cz * m[1] + cy) * m[0] + cx);
        fill[cell_of[i] + 1]++;
    }
    for (long c = 0; c < cells; c++) fill[c + 1] += fill[c];
    memset(start, 0, (size_t)cells * sizeof(uint32_t));
    memset(end, 0, (size_t)cells * sizeof(uint32_t));
    for (long c = 0; c < cells; c++) {
        if (fill[c + 1] > fill[c]) {
            start[c] = fill[c];
            end[c] = fill[c + 1];
        }
    }
    for (int i = 0; i < n; i++) sorted_idx[fill[cell_of[i]]++] = (uint32_t)i;
    free(fill);
}

/*
 * Work counters of the frozen work model: with the canonical grid m[3]
 * (floor(L / r_max) cells per axis) and hash multipliers inv_cell[3],
 * returns C27 = sum over particles of the particles in the distinct cells
 * of the 27-cell periodic stencil around its cell, excluding itself.
 */
double cfo_c27(int n, const float* pos, const int* m, const float* inv_cell)
{
    long cells = (long)m[0] * m[1] * m[2];
    uint32_t* pop = (uint32_t*)calloc((size_t)cells, sizeof(uint32_t));
    uint32_t* cell = (uint32_t*)malloc((size_t)n * sizeof(uint32_t));
    for (int i = 0; i < n; i++) {
        int cx = cell_coord(pos[3 * i], inv_cell[0], m[0]);
        int cy = cell_coord(pos[3 * i + 1], inv_cell[1], m[1]);
        int cz = cell_coord(pos[3 * i + 2], inv_cell[2], m[2]);
        cell[i] = (uint32_t)(((long)cz * m[1] + cy) * m[0] + cx);
        pop[cell[i]]++;
    }
    double total = 0.0;
    for (int i = 0; i < n; i++) {
        long c = cell[i];
        int cx = (int)(c % m[0]), cy = (int)((c / m[0]) % m[1]), cz = (int)(c / ((long)m[0] * m[1]));
        int ox[3], oy[3], oz[3], nx = 0, ny = 0, nz = 0;
        for (int o = -1; o <= 1; o++) {
            int v = ((cx + o) % m[0] + m[0]) % m[0];
            int dup = 0;
            for (int q = 0; q < nx; q++) dup |= ox[q] == v;
            if (!dup) ox[nx++] = v;
            v = ((cy + o) % m[1] + m[1]) % m[1];
            dup = 0;
            for (int q = 0; q < ny; q++) dup |= oy[q] == v;
            if (!dup) oy[ny++] = v;
            v = ((cz + o) % m[2] + m[2]) % m[2];
            dup = 0;
            for (int q = 0; q < nz; q++) dup |= oz[q] == v;
            if (!dup) oz[nz++] = v;
        }
        for (int a = 0; a < nz; a++)
            for (int b = 0; b < ny; b++)
                for (int e = 0; e < nx; e++) total += pop[((long)oz[a] * m[1] + oy[b]) * m[0] + ox[e]];
        total -= 1.0;
    }
    free(pop);
    free(cell);
    return total;
}

/*
 * Triangle mesh (ParticleSimulation.cu:290-423, host wrapper :723-724).  For
 * each i: scan j != i in index order while fewer than min(max_conn, 32) are
 * held, keeping j of the same type with non-periodic squared distance below
 * distance^2 * 1.2^2; every pair (a, b), a < b, of the held list whose
 * indices both exceed i is a triangle (i, a, b), at most 64 per i, in that
 * order.  Each triangle: 3 vertices of 9 floats (x, y, z, flat normal,
 * colour of i's type % T).  tris gets 3 indices per triangle, verts 27 floats
 * (either may be NULL).  Triangles beyond cap are counted, not written.
 * Returns the triangle count.
 */
long cfo_triangle_mesh(int n, const float* pos, const uint32_t* type, float distance, int max_conn_in,
                       const float* colors, int num_types, int32_t* tris, float* verts, long cap)
{
    const float hysteresis = 1.2f;
    const float dsq = distance * distance * (hysteresis * hysteresis);
    int max_conn = max_conn_in < 32 ? max_conn_in : 32;
    long total = 0;
    for (int i = 0; i < n; i++) {
        int near[32];
        int held = 0;
        for (int j = 0; j < n && held < max_conn; j++) {
            if (j == i || type[i] != type[j]) continue;
            float dx = pos[3 * j] - pos[3 * i];
            float dy = pos[3 * j + 1] - pos[3 * i + 1];
            float dz = pos[3 * j + 2] - pos[3 * i + 2];
            float d2 = dx * dx + dy * dy + dz * dz;
            if (d2 < dsq) near[held++] = j;
        }
        int made = 0;
        const float* c = colors + 3 * (type[i] % (uint32_t)num_types);
        for (int a = 0; a < held && made < 64; a++) {
            for (int b = a + 1; b < held && made < 64; b++) {
                int n1 = near[a], n2 = near[b];
                if (!(i < n1 && i < n2)) continue;
                if (total < cap) {
                    if (tris) {
                        tris[3 * total] = i;
                        tris[3 * total + 1] = n1;
                        tris[3 * total + 2] = n2;
                    }
                    if (verts) {
                        const float* v1 = pos + 3 * i;
                        const float* v2 = pos + 3 * n1;
                        const float* v3 = pos + 3 * n2;
                        float e1x = v2[0] - v1[0], e1y = v2[1] - v1[1], e1z = v2[2] - v1[2];
                        float e2x = v3[0] - v1[0], e2y = v3[1] - v1[1], e2z = v3[2] - v1[2];
                        float nx = e1y * e2z - e1z * e2y;
                        float ny = e1z * e2x - e1x * e2z;
                        float nz = e1x * e2y - e1y * e2x;
                        float len = sqrtf(nx * nx + ny * ny + nz * nz);
                        if (len > 0.0001f) {
                            nx /= len;
                            ny /= len;
                            nz /= len;
                        }
                        const float* vs[3] = {v1, v2, v3};
                        for (int k = 0; k < 3; k++) {
                            float* o = verts + 27 * total + 9 * k;
                            o[0] = vs[k][0];
                            o[1] = vs[k][1];
                            o[2] = vs[k][2];
                            o[3] = nx;
                            o[4] = ny;
                            o[5] = nz;
                            o[6] = c[0];
                            o[7] = c[1];
                            o[8] = c[2];
                        }
                    }
                }
                total++;
                made++;
            }
        }
    }
    return total;
}
