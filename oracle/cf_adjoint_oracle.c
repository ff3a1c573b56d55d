/*
 * cf_adjoint_oracle.c - FP64 restatement of a differentiable CellFlow rollout,
 * for checking only.
 *
 * TEST INFRASTRUCTURE.  Only the tests and the CPU-baseline leg of the
 * benchmark load this file's library, as the checker; the product path never
 * calls it.
 *
 * Forward (cuda-native/src/ParticleSimulation.cu:78-165, in double):
 *   d_ij  = min-image(x_j - x_i)                                   :97-102
 *   dist  = sqrt(|d|^2 + 1e-4),  r = dist / eff_ij                 :105,113
 *   j is a neighbour of i when dist < eff_ij                        :111
 *   f_i   = sum_j F[t_i][t_j] (R exp(-k r^2) - A r) d / dist        :114-124
 *   scale = M (1 - (1 - b) min((c_new + c_prev) / 2 / Ne, 1))       :136-143
 *   v'    = phi v + dt scale f,   x' = fmod(x + dt v' + L, L)       :146-161
 * The effective radii eff_ij are given as the float values the step uses,
 * so the neighbour sets agree with the FP32 step away from the cutoff.
 *
 * Adjoint (no counterpart in the reference).  Neighbour counts are held
 * constant (their derivative is zero almost everywhere) and the wrap is the
 * identity almost everywhere.  With P(d) = d n(dist) / dist, n = R e - A r:
 *   dP/dd = (n / dist) I + h d d^T,  h = (n' dist - n) / dist^3,
 *   n'    = (R e (-2 k r) - A) / eff,
 * and the adjoint of one step, from (gx', gv') of its outputs:
 *   gw = gv' + dt gx',  gv = phi gw,  ga = dt gw,  gf_i = scale_i ga_i,
 *   gx_i = gx'_i + sum_{j in N(i)} dP/dd(d_ij) (F[t_j][t_i] gf_j - F[t_i][t_j] gf_i),
 *   gF[t_i][t_j] += (gf_i . d / dist) n,  gR += q F e,  gA -= q F r,  gk -= q F R e r^2,
 *   gM += adapt_i (f_i . ga_i),  gb += M density_i (f_i . ga_i),  gphi += v . gw.
 *
 * Soft radial distribution (the rollout loss; no counterpart in the
 * reference): bins of width D = r_max / bins, centres c_k = (k + 1/2) D, a
 * cubic B-spline kernel B((r - c_k) / D) (support |t| < 2), so every ordered
 * pair with r < r_max + 1.5 D contributes:
 *   h[a][b][k] = sum_{i in a, j in b, j != i} B((r_ij - c_k) / D)
 *                / (N_a (N_b / V) 4 pi c_k^2 D).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define CFO_MAX_T 32

typedef struct cfo_phys64 {
    double repulsion, attraction, k, force_multiplier, balance, friction, delta_t;
    int max_expected_neighbors;
} cfo_phys64;

/* Indices of the parameter gradient vector. */
enum { G_REP = 0, G_ATT, G_K, G_MULT, G_BAL, G_FRIC, G_COUNT };

static double min_image64(double dx, double L)
{
    if (dx > L * 0.5) dx -= L;
    if (dx < -L * 0.5) dx += L;
    return dx;
}

/* A uniform cell list over a periodic box, rebuilt per position set. */
typedef struct cell_list {
    int m[3];
    int brute;  /* fewer than 3 cells on some axis: test every pair */
    int* start; /* cells + 1 */
    int* order;
} cell_list;

static void cl_build(cell_list* cl, int n, const double* pos, const double* ext, double rcut)
{
    cl->brute = 0;
    for (int a = 0; a < 3; a++) {
        cl->m[a] = (int)floor(ext[a] / rcut);
        if (cl->m[a] < 3) cl->brute = 1;
        if (cl->m[a] > 256) cl->m[a] = 256;
    }
    if (cl->brute) {
        cl->start = NULL;
        cl->order = NULL;
        return;
    }
    const int cells = cl->m[0] * cl->m[1] * cl->m[2];
    cl->start = (int*)calloc((size_t)cells + 1, sizeof(int));
    cl->order = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    int* cell_of = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    for (int i = 0; i < n; i++) {
        int c[3];
        for (int a = 0; a < 3; a++) {
            int v = (int)floor(pos[3 * i + a] / ext[a] * cl->m[a]);
            if (v < 0) v = 0;
            if (v >= cl->m[a]) v = cl->m[a] - 1;
            c[a] = v;
        }
        cell_of[i] = (c[2] * cl->m[1] + c[1]) * cl->m[0] + c[0];
        cl->start[cell_of[i] + 1]++;
    }
    for (int c = 0; c < cells; c++) cl->start[c + 1] += cl->start[c];
    int* fill = (int*)malloc(sizeof(int) * (size_t)cells);
    memcpy(fill, cl->start, sizeof(int) * (size_t)cells);
    for (int i = 0; i < n; i++) cl->order[fill[cell_of[i]]++] = i;
    free(fill);
    free(cell_of);
}

static void cl_free(cell_list* cl)
{
    free(cl->start);
    free(cl->order);
}

/* Runs the trailing statement block for every candidate j of particle i
 * (j != i is excluded by the caller). */
#define CL_FOR_EACH(cl, n, pos, ext, i, j, ...)                                                    \
    do {                                                                                           \
        if ((cl)->brute) {                                                                         \
            for (int j = 0; j < (n); j++) { __VA_ARGS__ }                                          \
        } else {                                                                                   \
            int ci_[3];                                                                            \
            for (int a_ = 0; a_ < 3; a_++) {                                                       \
                int v_ = (int)floor((pos)[3 * (i) + a_] / (ext)[a_] * (cl)->m[a_]);                \
                ci_[a_] = v_ < 0 ? 0 : (v_ >= (cl)->m[a_] ? (cl)->m[a_] - 1 : v_);                 \
            }                                                                                      \
            for (int oz_ = -1; oz_ <= 1; oz_++)                                                    \
                for (int oy_ = -1; oy_ <= 1; oy_++)                                                \
                    for (int ox_ = -1; ox_ <= 1; ox_++) {                                          \
                        int x_ = (ci_[0] + ox_ + (cl)->m[0]) % (cl)->m[0];                         \
                        int y_ = (ci_[1] + oy_ + (cl)->m[1]) % (cl)->m[1];                         \
                        int z_ = (ci_[2] + oz_ + (cl)->m[2]) % (cl)->m[2];                         \
                        int c_ = (z_ * (cl)->m[1] + y_) * (cl)->m[0] + x_;                         \
                        for (int q_ = (cl)->start[c_]; q_ < (cl)->start[c_ + 1]; q_++) {           \
                            int j = (cl)->order[q_];                                               \
                            __VA_ARGS__                                                            \
                        }                                                                          \
                    }                                                                              \
        }                                                                                          \
    } while (0)

static double max_eff(const float* eff, int T)
{
    double m = 0.0;
    for (int a = 0; a < T; a++)
        for (int b = 0; b < T; b++)
            if (eff[a * T + b] > m) m = eff[a * T + b];
    return m;
}

/*
 * One forward step in double.  pos/vel: n*3, cnt_prev/cnt_new: n, F: T*T,
 * eff: T*T.  Writes pos_out/vel_out/cnt_new and, when f_out is not NULL, the
 * unscaled force.  min_margin: smallest |dist - eff| / eff over candidate pairs.
 */
static void step64(int n, const double* pos, const double* vel, const uint32_t* type, const int* cnt_prev,
                   const double* F, const float* eff, int T, const cfo_phys64* ph, const double* ext,
                   double* pos_out, double* vel_out, int* cnt_new, double* f_out, double* min_margin)
{
    cell_list cl;
    cl_build(&cl, n, pos, ext, max_eff(eff, T) * 1.0001 + 1e-9);
    double mm = INFINITY;
#pragma omp parallel for schedule(dynamic, 64) reduction(min : mm)
    for (int i = 0; i < n; i++) {
        const uint32_t ti = type[i];
        double f[3] = {0, 0, 0};
        int count = 0;
        CL_FOR_EACH(&cl, n, pos, ext, i, j, {
            if (j != i) {
                double d[3];
                for (int a = 0; a < 3; a++) d[a] = min_image64(pos[3 * j + a] - pos[3 * i + a], ext[a]);
                const double dist = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2] + 1e-4);
                const uint32_t tj = type[j];
                const double e = eff[ti * T + tj];
                const double margin = fabs(dist - e) / e;
                if (margin < mm) mm = margin;
                if (dist < e) {
                    count++;
                    const double r = dist / e;
                    const double net = (ph->repulsion * exp(-ph->k * r * r) - ph->attraction * r) * F[ti * T + tj];
                    for (int a = 0; a < 3; a++) f[a] += d[a] / dist * net;
                }
            }
        });
        const double avg = (count + cnt_prev[i]) * 0.5;
        double density = avg / ph->max_expected_neighbors;
        if (density > 1.0) density = 1.0;
        const double scale = ph->force_multiplier * (1.0 - (1.0 - ph->balance) * density);
        for (int a = 0; a < 3; a++) {
            const double v = vel[3 * i + a] * ph->friction + f[a] * scale * ph->delta_t;
            vel_out[3 * i + a] = v;
            pos_out[3 * i + a] = fmod(pos[3 * i + a] + v * ph->delta_t + ext[a], ext[a]);
            if (f_out) f_out[3 * i + a] = f[a];
        }
        cnt_new[i] = count;
    }
    cl_free(&cl);
    if (min_margin && mm < *min_margin) *min_margin = mm;
}

/*
 * Rollout of `steps` steps in double.  pos/vel (n*3) and cnt (n) are updated
 * in place.  min_margin (may be NULL) receives the smallest relative distance
 * of any candidate pair to its cutoff over the rollout; fingerprint (may be
 * NULL) a hash of every step's neighbour counts, equal for two rollouts whose
 * neighbour counts agree at every step.
 */
void cfo_rollout_f64(int n, double* pos, double* vel, const uint32_t* type, int* cnt, const double* F,
                     const float* eff, int T, const cfo_phys64* ph, const double* ext, int steps, double* min_margin,
                     uint64_t* fingerprint)
{
    uint64_t fp = 0x9E3779B97F4A7C15ull;
    double* p2 = (double*)malloc(sizeof(double) * 3 * (size_t)(n > 0 ? n : 1));
    double* v2 = (double*)malloc(sizeof(double) * 3 * (size_t)(n > 0 ? n : 1));
    int* c2 = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    double mm = INFINITY;
    for (int s = 0; s < steps; s++) {
        step64(n, pos, vel, type, cnt, F, eff, T, ph, ext, p2, v2, c2, NULL, &mm);
        memcpy(pos, p2, sizeof(double) * 3 * (size_t)n);
        memcpy(vel, v2, sizeof(double) * 3 * (size_t)n);
        memcpy(cnt, c2, sizeof(int) * (size_t)n);
        for (int i = 0; i < n; i++) fp = (fp ^ (uint64_t)(uint32_t)cnt[i]) * 0x100000001B3ull;
    }
    if (min_margin) *min_margin = mm;
    if (fingerprint) *fingerprint = fp;
    free(p2);
    free(v2);
    free(c2);
}

/*
 * Gradient of L(x_K, v_K) through `steps` steps, given gpos_K = dL/dx_K and
 * gvel_K = dL/dv_K.  Outputs dL/dx_0, dL/dv_0, dL/dF (T*T) and the parameter
 * gradient gph[G_COUNT] (repulsion, attraction, k, force_multiplier, balance,
 * friction).  The initial state is not modified.
 */
static void adjoint_on_states(int n, const double* P, const double* V, const int* Cn, const double* Fs,
                              const uint32_t* type, const double* F, const float* eff, int T, const cfo_phys64* ph,
                              const double* ext, int steps, const double* gpos_K, const double* gvel_K, double* gpos0,
                              double* gvel0, double* gF, double* gph);

void cfo_rollout_grad_f64(int n, const double* pos0, const double* vel0, const uint32_t* type, const int* cnt0,
                          const double* F, const float* eff, int T, const cfo_phys64* ph, const double* ext,
                          int steps, const double* gpos_K, const double* gvel_K, double* gpos0, double* gvel0,
                          double* gF, double* gph)
{
    const size_t n3 = 3 * (size_t)n;
    double* P = (double*)malloc(sizeof(double) * n3 * (size_t)(steps + 1) + 8);
    double* V = (double*)malloc(sizeof(double) * n3 * (size_t)(steps + 1) + 8);
    int* Cn = (int*)malloc(sizeof(int) * (size_t)n * (size_t)(steps + 1) + 8);
    double* Fs = (double*)malloc(sizeof(double) * n3 * (size_t)(steps > 0 ? steps : 1) + 8);
    memcpy(P, pos0, sizeof(double) * n3);
    memcpy(V, vel0, sizeof(double) * n3);
    memcpy(Cn, cnt0, sizeof(int) * (size_t)n);
    for (int s = 0; s < steps; s++)
        step64(n, P + n3 * s, V + n3 * s, type, Cn + (size_t)n * s, F, eff, T, ph, ext, P + n3 * (s + 1),
               V + n3 * (s + 1), Cn + (size_t)n * (s + 1), Fs + n3 * s, NULL);
    adjoint_on_states(n, P, V, Cn, Fs, type, F, eff, T, ph, ext, steps, gpos_K, gvel_K, gpos0, gvel0, gF, gph);
    free(P);
    free(V);
    free(Cn);
    free(Fs);
}

/*
 * The same adjoint along a given trajectory: positions P and velocities V,
 * (steps + 1) * n * 3 each, and neighbour counts Cn, (steps + 1) * n, of the
 * states before every step and after the last (for instance an FP32 rollout).
 * The counts are taken as given; the neighbour sets and forces are
 * recomputed in double from the given positions.
 */
void cfo_rollout_grad_traj_f64(int n, const double* P, const double* V, const int* Cn, const uint32_t* type,
                               const double* F, const float* eff, int T, const cfo_phys64* ph, const double* ext,
                               int steps, const double* gpos_K, const double* gvel_K, double* gpos0, double* gvel0,
                               double* gF, double* gph)
{
    const size_t n3 = 3 * (size_t)n;
    double* Fs = (double*)malloc(sizeof(double) * n3 * (size_t)(steps > 0 ? steps : 1) + 8);
    double* tp = (double*)malloc(sizeof(double) * n3 + 8);
    double* tv = (double*)malloc(sizeof(double) * n3 + 8);
    int* tc = (int*)malloc(sizeof(int) * (size_t)n + 8);
    for (int s = 0; s < steps; s++)
        step64(n, P + n3 * s, V + n3 * s, type, Cn + (size_t)n * s, F, eff, T, ph, ext, tp, tv, tc, Fs + n3 * s,
               NULL);
    adjoint_on_states(n, P, V, Cn, Fs, type, F, eff, T, ph, ext, steps, gpos_K, gvel_K, gpos0, gvel0, gF, gph);
    free(Fs);
    free(tp);
    free(tv);
    free(tc);
}

static void adjoint_on_states(int n, const double* P, const double* V, const int* Cn, const double* Fs,
                              const uint32_t* type, const double* F, const float* eff, int T, const cfo_phys64* ph,
                              const double* ext, int steps, const double* gpos_K, const double* gvel_K, double* gpos0,
                              double* gvel0, double* gF, double* gph)
{
    const size_t n3 = 3 * (size_t)n;
    double* gx = (double*)malloc(sizeof(double) * n3 + 8);
    double* gv = (double*)malloc(sizeof(double) * n3 + 8);
    double* gx2 = (double*)malloc(sizeof(double) * n3 + 8);
    double* gf = (double*)malloc(sizeof(double) * n3 + 8);
    memcpy(gx, gpos_K, sizeof(double) * n3);
    memcpy(gv, gvel_K, sizeof(double) * n3);
    memset(gF, 0, sizeof(double) * (size_t)T * T);
    for (int g = 0; g < G_COUNT; g++) gph[g] = 0.0;
    const double dt = ph->delta_t, M = ph->force_multiplier;

    for (int s = steps - 1; s >= 0; s--) {
        const double* x = P + n3 * s;
        const double* v = V + n3 * s;
        const int* cp = Cn + (size_t)n * s;
        const int* cn = Cn + (size_t)n * (s + 1);
        const double* f = Fs + n3 * s;
        double g_fric = 0, g_mult = 0, g_bal = 0;
        /* per particle: gf, gv, friction / multiplier / balance gradients */
        for (int i = 0; i < n; i++) {
            double density = (cn[i] + cp[i]) * 0.5 / ph->max_expected_neighbors;
            if (density > 1.0) density = 1.0;
            const double adapt = 1.0 - (1.0 - ph->balance) * density;
            const double scale = M * adapt;
            double fga = 0.0;
            for (int a = 0; a < 3; a++) {
                const double gw = gv[3 * i + a] + dt * gx[3 * i + a];
                const double ga = dt * gw;
                g_fric += v[3 * i + a] * gw;
                gv[3 * i + a] = ph->friction * gw;
                gf[3 * i + a] = scale * ga;
                fga += f[3 * i + a] * ga;
            }
            g_mult += adapt * fga;
            g_bal += M * density * fga;
        }
        gph[G_FRIC] += g_fric;
        gph[G_MULT] += g_mult;
        gph[G_BAL] += g_bal;

        /* pair terms */
        cell_list cl;
        cl_build(&cl, n, x, ext, max_eff(eff, T) * 1.0001 + 1e-9);
        double g_rep = 0, g_att = 0, g_k = 0;
        double* gFloc = (double*)calloc((size_t)T * T, sizeof(double));
#pragma omp parallel
        {
            double* gFt = (double*)calloc((size_t)T * T, sizeof(double));
            double tr = 0, ta = 0, tk = 0;
#pragma omp for schedule(dynamic, 64)
            for (int i = 0; i < n; i++) {
                const uint32_t ti = type[i];
                double acc[3] = {0, 0, 0};
                CL_FOR_EACH(&cl, n, x, ext, i, j, {
                    if (j != i) {
                        double d[3];
                        for (int a = 0; a < 3; a++) d[a] = min_image64(x[3 * j + a] - x[3 * i + a], ext[a]);
                        const double dist = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2] + 1e-4);
                        const uint32_t tj = type[j];
                        const double e = eff[ti * T + tj];
                        if (dist < e) {
                            const double r = dist / e;
                            const double ex = exp(-ph->k * r * r);
                            const double nraw = ph->repulsion * ex - ph->attraction * r;
                            const double dn = (ph->repulsion * ex * (-2.0 * ph->k * r) - ph->attraction) / e;
                            const double phi = nraw / dist;
                            const double h = (dn * dist - nraw) / (dist * dist * dist);
                            const double Fij = F[ti * T + tj], Fji = F[tj * T + ti];
                            double w[3], dw = 0.0, q = 0.0;
                            for (int a = 0; a < 3; a++) {
                                w[a] = Fji * gf[3 * j + a] - Fij * gf[3 * i + a];
                                dw += d[a] * w[a];
                                q += gf[3 * i + a] * d[a];
                            }
                            q /= dist;
                            for (int a = 0; a < 3; a++) acc[a] += phi * w[a] + h * dw * d[a];
                            gFt[ti * T + tj] += q * nraw;
                            tr += q * Fij * ex;
                            ta -= q * Fij * r;
                            tk -= q * Fij * ph->repulsion * ex * r * r;
                        }
                    }
                });
                for (int a = 0; a < 3; a++) gx2[3 * i + a] = gx[3 * i + a] + acc[a];
            }
#pragma omp critical
            {
                for (int q = 0; q < T * T; q++) gFloc[q] += gFt[q];
                g_rep += tr;
                g_att += ta;
                g_k += tk;
            }
            free(gFt);
        }
        for (int q = 0; q < T * T; q++) gF[q] += gFloc[q];
        free(gFloc);
        gph[G_REP] += g_rep;
        gph[G_ATT] += g_att;
        gph[G_K] += g_k;
        cl_free(&cl);
        memcpy(gx, gx2, sizeof(double) * n3);
    }
    memcpy(gpos0, gx, sizeof(double) * n3);
    memcpy(gvel0, gv, sizeof(double) * n3);
    free(gx);
    free(gv);
    free(gx2);
    free(gf);
}

/* Cubic B-spline of support |t| < 2 and its derivative. */
static double bspline3(double t)
{
    const double a = fabs(t);
    if (a < 1.0) return 2.0 / 3.0 - a * a + 0.5 * a * a * a;
    if (a < 2.0) {
        const double u = 2.0 - a;
        return u * u * u / 6.0;
    }
    return 0.0;
}

static double bspline3_d(double t)
{
    const double a = fabs(t);
    double g;
    if (a < 1.0)
        g = -2.0 * a + 1.5 * a * a;
    else if (a < 2.0) {
        const double u = 2.0 - a;
        g = -0.5 * u * u;
    } else
        g = 0.0;
    return t < 0.0 ? -g : g;
}

/* Normalisation denominators den[a][b][k] (0 where a type is absent). */
static void rdf_den(int n, const uint32_t* type, int T, const double* ext, int bins, double r_max, double* den)
{
    long na[CFO_MAX_T] = {0};
    for (int i = 0; i < n; i++) na[type[i]]++;
    const double V = ext[0] * ext[1] * ext[2], D = r_max / bins;
    for (int a = 0; a < T; a++)
        for (int b = 0; b < T; b++)
            for (int k = 0; k < bins; k++) {
                const double c = (k + 0.5) * D;
                den[((size_t)a * T + b) * bins + k] = (double)na[a] * ((double)na[b] / V) * 4.0 * M_PI * c * c * D;
            }
}

/* Soft type-resolved radial distribution h[T][T][bins]. */
void cfo_rdf_f64(int n, const double* pos, const uint32_t* type, int T, const double* ext, int bins, double r_max,
                 double* hist)
{
    const double D = r_max / bins, rc = r_max + 1.5 * D;
    const size_t H = (size_t)T * T * bins;
    memset(hist, 0, sizeof(double) * H);
    cell_list cl;
    cl_build(&cl, n, pos, ext, rc * 1.0001);
#pragma omp parallel
    {
        double* ht = (double*)calloc(H, sizeof(double));
#pragma omp for schedule(dynamic, 64)
        for (int i = 0; i < n; i++) {
            CL_FOR_EACH(&cl, n, pos, ext, i, j, {
                if (j != i) {
                    double d2 = 0.0;
                    for (int a = 0; a < 3; a++) {
                        const double d = min_image64(pos[3 * j + a] - pos[3 * i + a], ext[a]);
                        d2 += d * d;
                    }
                    const double r = sqrt(d2);
                    if (r < rc) {
                        const double t0 = r / D - 0.5;
                        int k0 = (int)ceil(t0 - 2.0), k1 = (int)floor(t0 + 2.0);
                        if (k0 < 0) k0 = 0;
                        if (k1 > bins - 1) k1 = bins - 1;
                        double* row = ht + ((size_t)type[i] * T + type[j]) * bins;
                        for (int k = k0; k <= k1; k++) row[k] += bspline3(t0 - k);
                    }
                }
            });
        }
#pragma omp critical
        for (size_t q = 0; q < H; q++) hist[q] += ht[q];
        free(ht);
    }
    cl_free(&cl);
    double* den = (double*)malloc(sizeof(double) * H);
    rdf_den(n, type, T, ext, bins, r_max, den);
    for (size_t q = 0; q < H; q++) hist[q] = den[q] > 0.0 ? hist[q] / den[q] : 0.0;
    free(den);
}

/* dL/dpos (n*3) of L(h) given ghist = dL/dh. */
void cfo_rdf_grad_f64(int n, const double* pos, const uint32_t* type, int T, const double* ext, int bins,
                      double r_max, const double* ghist, double* gpos)
{
    const double D = r_max / bins, rc = r_max + 1.5 * D;
    const size_t H = (size_t)T * T * bins;
    double* g = (double*)malloc(sizeof(double) * H);
    rdf_den(n, type, T, ext, bins, r_max, g);
    for (size_t q = 0; q < H; q++) g[q] = g[q] > 0.0 ? ghist[q] / g[q] : 0.0;
    cell_list cl;
    cl_build(&cl, n, pos, ext, rc * 1.0001);
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < n; i++) {
        double acc[3] = {0, 0, 0};
        CL_FOR_EACH(&cl, n, pos, ext, i, j, {
            if (j != i) {
                double d[3], d2 = 0.0;
                for (int a = 0; a < 3; a++) {
                    d[a] = min_image64(pos[3 * j + a] - pos[3 * i + a], ext[a]);
                    d2 += d[a] * d[a];
                }
                const double r = sqrt(d2);
                if (r < rc && r > 0.0) {
                    const double t0 = r / D - 0.5;
                    int k0 = (int)ceil(t0 - 2.0), k1 = (int)floor(t0 + 2.0);
                    if (k0 < 0) k0 = 0;
                    if (k1 > bins - 1) k1 = bins - 1;
                    const double* gij = g + ((size_t)type[i] * T + type[j]) * bins;
                    const double* gji = g + ((size_t)type[j] * T + type[i]) * bins;
                    double G = 0.0;
                    for (int k = k0; k <= k1; k++) G += (gij[k] + gji[k]) * bspline3_d(t0 - k);
                    G /= D;
                    for (int a = 0; a < 3; a++) acc[a] -= G * d[a] / r;
                }
            }
        });
        for (int a = 0; a < 3; a++) gpos[3 * i + a] = acc[a];
    }
    cl_free(&cl);
    free(g);
}
