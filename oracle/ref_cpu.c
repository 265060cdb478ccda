/*
 * ref_cpu.c -- ORACLE (test infrastructure, never product code).
 *
 * FP64 CPU restatement of the reference's voxel SPH step,
 * VoxelSPHStrategy.compute_next_state of iwoplaza/cuda-sph, used only by the
 * parity tests, the smoke check and the CPU baseline of bench.py.  Each
 * function cites the reference lines it follows.  Pinned against golden
 * vectors produced by executing the reference's own Python step code
 * (tests/golden/make_golden.py).
 *
 * Semantics kept from the reference, quirks included:
 *  - voxel coordinate = int32(pos / voxel_size) (voxel_kernels.py:10-12);
 *    here clamped to the voxel table, which changes nothing for positions
 *    inside [0, space) and keeps out-of-domain particles in the table;
 *  - table dims ceil(space/voxel) (voxel_sph_strategy.py:70-73); walk dims
 *    either the same (SPHGB_WALK_CEIL) or int(space/voxel)
 *    (SPHGB_WALK_TRUNCATED, voxel_sph_strategy.py:110-116);
 *  - voxel order (voxel, particle id) (voxel_sph_strategy.py:84-89);
 *  - walk dx outer, dy, dz inner; members in ascending particle id; a
 *    neighbour is sqrt(d2) <= INF_R; self counts; stop at MAX_NEIGHBOURS
 *    (voxel_kernels.py:30-85); never-written voxel slots are empty;
 *  - density excludes self (voxel_kernels.py:127-132); pressure has no MASS
 *    factor (:159-171); viscosity clamps min(1, .) per component (:211);
 *  - F = ext - P + V, v += F / rho * dt, x += v * dt (base_kernels.py:30-53);
 *  - box: clamp to 1e-3 / size - 1e-3 and v = -v * DAMP (base_kernels.py:75-98);
 *  - pipe: base_kernels.py:56-72, 101-127 with util_kernels.py:39-204; the
 *    respawn uniforms come from Philox4x32-10 instead of numba's xoroshiro128p.
 *
 * Build: see oracle/build_oracle.py (gcc -O2 -fopenmp -ffp-contract=off).
 */
#define SPHGB_NO_FUNCTIONS
#include "../include/sphgb.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define PI 3.141592653589793

typedef struct {
    int dims[3];    /* table dims (ceil) */
    int wdims[3];   /* walk dims */
    int64_t n_voxels;
    double h, h2, w_const, grad_w_const, lap_w_const;
} Derived;

/* config.py:24-29 */
static void derive(const SphgbSceneParams* sp, Derived* d) {
    for (int a = 0; a < 3; ++a) {
        double q = sp->space_size[a] / sp->voxel_size[a];
        d->dims[a] = (int)ceil(q);                         /* voxel_sph_strategy.py:70-73 */
        d->wdims[a] = sp->walk_dims == SPHGB_WALK_TRUNCATED ? (int)q : d->dims[a];
        if (d->dims[a] < 1) d->dims[a] = 1;
    }
    d->n_voxels = (int64_t)d->dims[0] * d->dims[1] * d->dims[2];
    d->h = sp->inf_r;
    d->h2 = sp->inf_r * sp->inf_r;
    double h6 = pow(sp->inf_r, 6.0), h9 = pow(sp->inf_r, 9.0);
    d->w_const = 315.0 / (64.0 * PI * h9);
    d->grad_w_const = -45.0 / (PI * h6);
    d->lap_w_const = 45.0 / (PI * h6);
}

int ref_derived(const SphgbSceneParams* sp, int32_t* dims6, double* consts5) {
    Derived d;
    derive(sp, &d);
    for (int a = 0; a < 3; ++a) { dims6[a] = d.dims[a]; dims6[3 + a] = d.wdims[a]; }
    consts5[0] = d.h; consts5[1] = d.h2; consts5[2] = d.w_const;
    consts5[3] = d.grad_w_const; consts5[4] = d.lap_w_const;
    return 0;
}

/* voxel_kernels.py:10-12 (int32 truncation), clamped to [0, dim) */
static int voxel_coord(double x, double vs, int dim) {
    double q = x / vs;
    if (!(q >= 0.0)) return 0;                 /* negative or NaN */
    if (q >= (double)dim) return dim - 1;
    int v = (int)q;
    return v < dim ? v : dim - 1;
}

/* voxel_kernels.py:89-105 with compute_1d_idx :16-17 (ceil dims) */
int ref_assign_voxels(const SphgbSceneParams* sp, int64_t n, const double* pos, int32_t* voxel) {
    Derived d;
    derive(sp, &d);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        int vx = voxel_coord(pos[3 * i + 0], sp->voxel_size[0], d.dims[0]);
        int vy = voxel_coord(pos[3 * i + 1], sp->voxel_size[1], d.dims[1]);
        int vz = voxel_coord(pos[3 * i + 2], sp->voxel_size[2], d.dims[2]);
        voxel[i] = vx + vy * d.dims[0] + vz * d.dims[0] * d.dims[1];
    }
    return 0;
}

/* voxel_sph_strategy.py:84-107: order by (voxel id, particle id) and the
 * voxel table.  start[v] = first sorted slot, count[v] = members (the
 * reference's voxel_begin[v] is start[v] when count[v] > 0, else -1). */
int ref_organize(const SphgbSceneParams* sp, int64_t n, const int32_t* voxel,
                 int32_t* sorted_pid, int32_t* start, int32_t* count) {
    Derived d;
    derive(sp, &d);
    memset(count, 0, sizeof(int32_t) * (size_t)d.n_voxels);
    for (int64_t i = 0; i < n; ++i) count[voxel[i]]++;
    int64_t acc = 0;
    for (int64_t v = 0; v < d.n_voxels; ++v) { start[v] = (int32_t)acc; acc += count[v]; }
    int32_t* fill = (int32_t*)calloc((size_t)d.n_voxels, sizeof(int32_t));
    if (!fill) return -3;
    for (int64_t i = 0; i < n; ++i) {       /* ascending particle id: stable */
        int32_t v = voxel[i];
        sorted_pid[start[v] + fill[v]++] = (int32_t)i;
    }
    free(fill);
    return 0;
}

/* voxel_kernels.py:20-26: sqrt((dx)**2 + (dy)**2 + (dz)**2) <= INF_R */
static inline double dist2(const double* a, const double* b) {
    double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    double s = dx * dx;
    s = s + dy * dy;
    s = s + dz * dz;
    return s;
}

/* get_neighbours, voxel_kernels.py:30-85.  Writes up to cap entries (cap <= 0:
 * unlimited, list may be NULL) and returns the count.  *uncapped receives the
 * full count when non-NULL (walk continued past the cap). */
static int walk(const SphgbSceneParams* sp, const Derived* d, int64_t i, const double* pos,
                const int32_t* sorted_pid, const int32_t* start, const int32_t* count,
                int cap, int32_t* list, int* uncapped) {
    const double* pi = pos + 3 * i;
    int v[3];
    for (int a = 0; a < 3; ++a) v[a] = voxel_coord(pi[a], sp->voxel_size[a], d->dims[a]);
    int n_capped = 0, n_all = 0, capped_done = 0;
    for (int dx = -1; dx <= 1; ++dx)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dz = -1; dz <= 1; ++dz) {
                int nv[3] = {v[0] + dx, v[1] + dy, v[2] + dz};
                int in = 1;
                for (int a = 0; a < 3; ++a)
                    if (nv[a] < 0 || nv[a] >= d->wdims[a]) { in = 0; break; }
                if (!in) continue;
                int64_t id = nv[0] + (int64_t)nv[1] * d->wdims[0] +
                             (int64_t)nv[2] * d->wdims[0] * d->wdims[1];
                int32_t c = count[id];
                int32_t s0 = start[id];
                for (int32_t m = 0; m < c; ++m) {
                    int32_t j = sorted_pid[s0 + m];
                    if (sqrt(dist2(pi, pos + 3 * (int64_t)j)) <= d->h) {
                        n_all++;
                        if (!capped_done) {
                            if (list) list[n_capped] = j;
                            n_capped++;
                            if (cap > 0 && n_capped >= cap) {
                                capped_done = 1;
                                if (!uncapped) return n_capped;
                            }
                        }
                    }
                }
            }
    if (uncapped) *uncapped = n_all;
    return n_capped;
}

int ref_neighbours(const SphgbSceneParams* sp, int64_t n, const double* pos,
                   const int32_t* sorted_pid, const int32_t* start, const int32_t* count,
                   int32_t* list, int list_stride, int32_t* n_capped, int32_t* n_uncapped) {
    Derived d;
    derive(sp, &d);
    int cap = sp->max_neighbours;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < n; ++i) {
        int un = 0;
        int32_t* li = list ? list + (int64_t)i * list_stride : NULL;
        if (li) for (int t = 0; t < list_stride; ++t) li[t] = -1;
        int c = walk(sp, &d, i, pos, sorted_pid, start, count, cap, li,
                     n_uncapped ? &un : NULL);
        if (n_capped) n_capped[i] = c;
        if (n_uncapped) n_uncapped[i] = un;
    }
    return 0;
}

static int list_cap(const SphgbSceneParams* sp) {
    return sp->max_neighbours > 0 ? sp->max_neighbours : 0;
}

/* density_kernel, voxel_kernels.py:109-132 with compute_w, base_kernels.py:6-9 */
int ref_density(const SphgbSceneParams* sp, int64_t n, const double* pos,
                const int32_t* sorted_pid, const int32_t* start, const int32_t* count,
                double* rho) {
    Derived d;
    derive(sp, &d);
    int cap = list_cap(sp);
    int stride = cap > 0 ? cap : (int)(n < 1 ? 1 : n);
    int err = 0;
#pragma omp parallel
    {
        int32_t* nb = (int32_t*)malloc(sizeof(int32_t) * (size_t)stride);
        if (!nb) {
#pragma omp atomic write
            err = -3;
        }
#pragma omp for schedule(dynamic, 256)
        for (int64_t i = 0; i < n; ++i) {
            if (!nb) continue;
            int c = walk(sp, &d, i, pos, sorted_pid, start, count, cap, nb, NULL);
            double acc = 0.0;
            for (int t = 0; t < c; ++t) {
                int32_t j = nb[t];
                if (j == i) continue;
                double q = d.h2 - dist2(pos + 3 * i, pos + 3 * (int64_t)j);
                acc += d.w_const * (q * q * q);
            }
            rho[i] = acc * sp->mass;
        }
        free(nb);
    }
    return err;
}

/* pressure_kernel :136-171 and viscosity_kernel :175-211 (voxel_kernels.py),
 * compute_grad_w / compute_lap_w (base_kernels.py:12-27).  *_scale receive
 * the sums of |term| per component (rounding-error scale for tolerances). */
int ref_forces(const SphgbSceneParams* sp, int64_t n, const double* pos, const double* vel,
               const double* rho, const int32_t* sorted_pid, const int32_t* start,
               const int32_t* count, double* pressure, double* viscosity,
               double* p_scale, double* v_scale) {
    Derived d;
    derive(sp, &d);
    int cap = list_cap(sp);
    int stride = cap > 0 ? cap : (int)(n < 1 ? 1 : n);
    int err = 0;
#pragma omp parallel
    {
        int32_t* nb = (int32_t*)malloc(sizeof(int32_t) * (size_t)stride);
        if (!nb) {
#pragma omp atomic write
            err = -3;
        }
#pragma omp for schedule(dynamic, 256)
        for (int64_t i = 0; i < n; ++i) {
            if (!nb) continue;
            int c = walk(sp, &d, i, pos, sorted_pid, start, count, cap, nb, NULL);
            double pt[3] = {0, 0, 0}, vt[3] = {0, 0, 0}, ps[3] = {0, 0, 0}, vs[3] = {0, 0, 0};
            const double* pi = pos + 3 * i;
            for (int t = 0; t < c; ++t) {
                int64_t j = nb[t];
                if (j == i) continue;
                const double* pj = pos + 3 * j;
                double p_i = sp->k * (rho[i] - sp->rho_0);
                double p_j = sp->k * (rho[j] - sp->rho_0);
                double factor = p_i / (rho[i] * rho[i]) + p_j / (rho[j] * rho[j]);
                double dist = sqrt(dist2(pi, pj));
                double hd = d.h - dist;
                double gfac = d.grad_w_const * (hd * hd);
                double lap = d.lap_w_const * (d.h - dist);
                for (int a = 0; a < 3; ++a) {
                    double g = gfac * (pi[a] - pj[a]) / dist;
                    double term = factor * g;
                    pt[a] += term;
                    ps[a] += fabs(term);
                    double vj = (vel[3 * j + a] - vel[3 * i + a]) / rho[j] * lap;
                    double vterm = vj * sp->mass * sp->visc / rho[i];
                    vt[a] += vterm;
                    vs[a] += fabs(vterm);
                }
            }
            for (int a = 0; a < 3; ++a) {
                pressure[3 * i + a] = pt[a];
                viscosity[3 * i + a] = vt[a] < 1.0 ? vt[a] : 1.0;   /* min(1, .) */
                if (p_scale) p_scale[3 * i + a] = ps[a];
                if (v_scale) v_scale[3 * i + a] = vs[a];
            }
        }
        free(nb);
    }
    return err;
}

/* ---- Philox4x32-10 (Salmon et al., SC 2011) ---------------------------- */
static void philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
        uint32_t n1 = (uint32_t)p1;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
        uint32_t n3 = (uint32_t)p0;
        c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
        if (r != 9) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    }
}

double ref_philox_uniform(uint64_t seed, int32_t pid, int32_t step, int32_t draw) {
    uint32_t c[4] = {(uint32_t)draw, (uint32_t)step, (uint32_t)pid, 0u};
    philox(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    uint64_t bits = ((uint64_t)c[0] << 21) | (c[1] >> 11);
    return (double)bits * (1.0 / 9007199254740992.0);
}

/* ---- pipe geometry, util_kernels.py ------------------------------------ */
#define P(r, c) pipe[(r) * 5 + (c)]

/* :38-43 */
double ref_x_at_segment_beginning(const double* pipe, int seg) {
    double xb = P(0, 0);
    for (int i = 0; i < seg; ++i) xb += P(i, 4);
    return xb;
}

/* :56-69 */
double ref_radius_in_position(const double* p, const double* pipe, int seg) {
    double r0 = P(seg, 3), r1 = P(seg + 1, 3);
    if (r0 == r1) return r0;
    if (r0 < r1) {
        double delta = p[0] - ref_x_at_segment_beginning(pipe, seg);
        double tl = P(seg, 4) * r0 / (r1 - r0);
        return r0 * (1.0 + delta / tl);
    }
    double delta = ref_x_at_segment_beginning(pipe, seg) + P(seg, 4) - p[0];
    double tl = P(seg, 4) * r1 / (r0 - r1);
    return r1 * (1.0 + delta / tl);
}

/* :72-77 */
int ref_find_segment(const double* p, const double* pipe, int rows) {
    for (int j = 0; j < rows - 1; ++j)
        if (P(j, 0) <= p[0] && p[0] < P(j + 1, 0)) return j;
    return -1;
}

/* :46-53 */
int ref_is_out_of_pipe(const double* p, const double* pipe, int seg) {
    double yn = p[1] - P(seg, 1), zn = p[2] - P(seg, 2);
    double hh = sqrt(yn * yn + zn * zn);
    return hh > ref_radius_in_position(p, pipe, seg);
}

static double vlen(const double* v) {            /* :97-102 */
    double l = 0.0;
    for (int i = 0; i < 3; ++i) l += v[i] * v[i];
    return sqrt(l);
}

static double vcos(const double* a, const double* b, double la, double lb) {   /* :80-85 */
    double s = 0.0;
    for (int i = 0; i < 3; ++i) s = s + a[i] * b[i];
    return s / (la * lb);
}

/* :182-204 with :88-179 */
void ref_solve_collision(double* p, double* v, const double* pipe, int seg) {
    double r0 = P(seg, 3), r1 = P(seg + 1, 3);
    /* calc_edge_vector :152-171 */
    double yn = p[1] - P(seg, 1), zn = p[2] - P(seg, 2);
    double hh = sqrt(yn * yn + zn * zn);
    double first[3], second[3], edge[3];
    first[0] = P(seg, 0);
    second[0] = P(seg + 1, 0);
    for (int a = 1; a < 3; ++a) {
        first[a] = (p[a] - P(seg, a)) / hh * r0;
        second[a] = (p[a] - P(seg, a)) / hh * r1;
    }
    for (int a = 0; a < 3; ++a) edge[a] = second[a] - first[a];
    for (int a = 1; a < 3; ++a) first[a] = first[a] + P(seg, a);
    /* calc_collision_point :174-179 with calc_dt :113-121 */
    double sl = vlen(v), el = vlen(edge);
    double cos_a = vcos(v, edge, sl, el);
    double pv[3], cr[3];
    for (int a = 0; a < 3; ++a) pv[a] = first[a] - p[a];        /* :124-135 */
    cr[0] = edge[1] * pv[2] - edge[2] * pv[1];                 /* :138-142 */
    cr[1] = edge[2] * pv[0] - edge[0] * pv[2];
    cr[2] = edge[0] * pv[1] - edge[1] * pv[0];
    double dd = vlen(cr) / vlen(edge);
    double sin_a = sqrt(1.0 - cos_a * cos_a);
    double d_to = dd / (sin_a + 0.001);
    double dt = -d_to / sl;
    double cp[3];
    for (int a = 0; a < 3; ++a) cp[a] = p[a] + v[a] * dt;
    if (r0 == r1) {
        v[1] = -v[1];
        v[2] = -v[2];
    } else {                                                  /* :88-94 */
        double ll = vlen(edge), pl = vlen(v);
        double c = vcos(edge, v, ll, pl);
        double sv[3];
        for (int a = 0; a < 3; ++a) sv[a] = 2.0 * edge[a] / ll * c * pl;
        for (int a = 0; a < 3; ++a) v[a] = sv[a] - v[a];
    }
    double way = 0.0;                                          /* :105-110 */
    for (int a = 0; a < 3; ++a) way += (p[a] - cp[a]) * (p[a] - cp[a]);
    way = sqrt(way);
    double svl = vlen(v);
    for (int a = 0; a < 3; ++a) p[a] = cp[a] + v[a] * way / svl;
}

/* collision_kernel, base_kernels.py:56-72, with put_particle_at_pipe_begin
 * :101-113 and rand_position_inside_pipe :116-127 */
void ref_collide_pipe_one(double* p, double* v, const double* pipe, int rows,
                          uint64_t seed, int32_t pid, int32_t step) {
    int seg = ref_find_segment(p, pipe, rows);
    if (seg == -1) {
        if (p[0] < 0) {
            p[0] = -p[0];
            v[0] = -v[0];
            if (ref_is_out_of_pipe(p, pipe, 0)) ref_solve_collision(p, v, pipe, 0);
        } else {
            p[0] = 0.0;
            int s = ref_find_segment(p, pipe, rows);
            double R = ref_radius_in_position(p, pipe, s);
            double r = R * sqrt(ref_philox_uniform(seed, pid, step, 0));
            double th = ref_philox_uniform(seed, pid, step, 1) * 2.0 * PI;
            p[1] = pipe[1] + r * cos(th);     /* row 0: [x0, y0, z0, r, len] */
            p[2] = pipe[2] + r * sin(th);
        }
    } else if (ref_is_out_of_pipe(p, pipe, seg)) {
        ref_solve_collision(p, v, pipe, seg);
    }
}
#undef P

/* integrating_kernel (base_kernels.py:30-53) then the wall response
 * (collision_kernel_box :75-98 or collision_kernel :56-72), in place. */
int ref_integrate(const SphgbSceneParams* sp, int64_t n, double* pos, double* vel,
                  const double* rho, const double* pressure, const double* viscosity,
                  double* force_out, const double* pipe, int32_t step) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        for (int a = 0; a < 3; ++a) {
            double f = sp->external_force[a] + -pressure[3 * i + a] + viscosity[3 * i + a];
            if (force_out) force_out[3 * i + a] = f;
            vel[3 * i + a] += f / rho[i] * sp->dt;
            pos[3 * i + a] += vel[3 * i + a] * sp->dt;
        }
        if (sp->mode == SPHGB_MODE_PIPE) {
            ref_collide_pipe_one(pos + 3 * i, vel + 3 * i, pipe, sp->pipe_rows, sp->seed,
                                 (int32_t)i, step);
        } else {
            for (int a = 0; a < 3; ++a) {
                int bounced = 0;
                if (pos[3 * i + a] < 0) { pos[3 * i + a] = 1e-3; bounced = 1; }
                if (pos[3 * i + a] > sp->space_size[a]) {
                    pos[3 * i + a] = sp->space_size[a] - 1e-3;
                    bounced = 1;
                }
                if (bounced) { vel[3 * i + a] *= -1; vel[3 * i + a] *= sp->damp; }
            }
        }
    }
    return 0;
}

/* The whole step, compute_next_state (abstract_sph_strategy.py:31-46): pos and
 * vel are updated in place; rho, pressure, viscosity, force (each optional
 * except rho) receive the step's intermediates. */
int ref_step(const SphgbSceneParams* sp, int64_t n, double* pos, double* vel, double* rho,
             double* pressure, double* viscosity, double* force, const double* pipe,
             int32_t step) {
    Derived d;
    derive(sp, &d);
    int rc = 0;
    int32_t* voxel = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    int32_t* spid = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    int32_t* start = (int32_t*)malloc(sizeof(int32_t) * (size_t)d.n_voxels);
    int32_t* count = (int32_t*)malloc(sizeof(int32_t) * (size_t)d.n_voxels);
    double* pt = pressure ? pressure : (double*)malloc(sizeof(double) * 3 * (size_t)(n > 0 ? n : 1));
    double* vt = viscosity ? viscosity : (double*)malloc(sizeof(double) * 3 * (size_t)(n > 0 ? n : 1));
    if (!voxel || !spid || !start || !count || !pt || !vt) { rc = -3; goto done; }
    ref_assign_voxels(sp, n, pos, voxel);
    if ((rc = ref_organize(sp, n, voxel, spid, start, count))) goto done;
    if ((rc = ref_density(sp, n, pos, spid, start, count, rho))) goto done;
    if ((rc = ref_forces(sp, n, pos, vel, rho, spid, start, count, pt, vt, NULL, NULL))) goto done;
    rc = ref_integrate(sp, n, pos, vel, rho, pt, vt, force, pipe, step);
done:
    free(voxel); free(spid); free(start); free(count);
    if (!pressure) free(pt);
    if (!viscosity) free(vt);
    return rc;
}

int ref_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void ref_set_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ---- start states (config.py:79-121; base_kernels.py:102-112, 130-143) --
 * Same draws and operation order as the library's generator: Philox uniforms
 * keyed (seed, particle id) with counter word 1 = 0xFFFFFFFF. */
static double gen_u(uint64_t seed, int64_t i, int draw) {
    return ref_philox_uniform(seed, (int32_t)(uint32_t)i, -1, draw);
}

/* Box-Muller (Box and Muller, 1958) */
static double gen_normal(uint64_t seed, int64_t i, int d) {
    double u1 = 1.0 - gen_u(seed, i, d);
    double u2 = gen_u(seed, i, d + 1);
    double r = sqrt(-2.0 * log(u1));
    return r * cos(u2 * 2.0 * PI);
}

int ref_generate(const SphgbGenerator* g, const double* pipe, int rows, int64_t n, double* pos,
                 double* vel) {
    if (g->kind == SPHGB_GEN_LATTICE &&
        (int64_t)g->lattice[0] * g->lattice[1] * g->lattice[2] != n)
        return -1;
    if (g->kind == SPHGB_GEN_PIPE_FILL && (!pipe || rows < 2)) return -1;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        double p[3], v[3];
        int normal_v = 0;
        if (g->kind == SPHGB_GEN_LATTICE) {
            int64_t ny = g->lattice[1], nz = g->lattice[2];
            int64_t idx[3] = {i / (ny * nz), (i / nz) % ny, i % nz};
            for (int a = 0; a < 3; ++a) {
                double base = g->origin[a] + ((double)idx[a] + 0.5) * g->spacing;
                p[a] = base + g->jitter * (2.0 * gen_u(g->seed, i, a) - 1.0);
                v[a] = g->velocity[a];
            }
            normal_v = g->velocity_sigma != 0.0;
        } else if (g->kind == SPHGB_GEN_BOX_WALL) {
            for (int a = 0; a < 3; ++a) {
                p[a] = gen_u(g->seed, i, a) * g->extent[a];
                v[a] = g->velocity[a] + (gen_u(g->seed, i, 3 + a) - 0.5) * g->velocity_spread;
            }
        } else {
            p[0] = g->x_range[0] + gen_u(g->seed, i, 0) * (g->x_range[1] - g->x_range[0]);
            p[1] = p[2] = 0.0;
            int seg = ref_find_segment(p, pipe, rows);
            if (seg < 0) seg = 0;
            double R = ref_radius_in_position(p, pipe, seg);
            double r = sqrt(gen_u(g->seed, i, 1)) * R * g->fill;
            double th = gen_u(g->seed, i, 2) * 2.0 * PI;
            p[1] = pipe[1] + r * cos(th);     /* row 0: [x0, y0, z0, r, len] */
            p[2] = pipe[2] + r * sin(th);
            for (int a = 0; a < 3; ++a) v[a] = g->velocity[a];
            normal_v = g->velocity_sigma != 0.0;
        }
        if (normal_v)
            for (int a = 0; a < 3; ++a) v[a] += g->velocity_sigma * gen_normal(g->seed, i, 3 + 2 * a);
        for (int a = 0; a < 3; ++a) {
            pos[3 * i + a] = p[a];
            vel[3 * i + a] = v[a];
        }
    }
    return 0;
}

/* ---- point-field vertex stage (vis/assets/point_field.vert:14-23) ------ */
static void mat_mul(const float* a, const float* b, float* out) {   /* column-major */
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) {
            float s = a[r] * b[c * 4];
            for (int k = 1; k < 4; ++k) s = s + a[k * 4 + r] * b[c * 4 + k];
            out[c * 4 + r] = s;
        }
}

void ref_point_field(const float* pos, int stride, const float* rho, int64_t n, const float* proj,
                     const float* model, const float* view, float* clip, float* colour,
                     float* size) {
    float pv[16], m[16];
    mat_mul(proj, view, pv);
    mat_mul(pv, model, m);
    const float b0 = 0.3f * 0.7f, b1 = 0.4f * 0.7f, b2 = 0.7f;
    for (int64_t i = 0; i < n; ++i) {
        const float x[4] = {pos[i * stride], pos[i * stride + 1], pos[i * stride + 2], 1.0f};
        for (int r = 0; r < 4; ++r) {
            float s = m[r] * x[0];
            for (int k = 1; k < 4; ++k) s = s + m[k * 4 + r] * x[k];
            clip[4 * i + r] = s;
        }
        float t = fminf(rho[i] / 10.0f, 1.0f);
        float omt = 1.0f - t;
        colour[4 * i + 0] = 0.1f * omt + b0 * t;
        colour[4 * i + 1] = 0.7f * omt + b1 * t;
        colour[4 * i + 2] = 0.5f * omt + b2 * t;
        colour[4 * i + 3] = 0.5f;
        float big = 40.0f + omt * 20.0f;
        size[i] = fminf(fmaxf(1.0f, big / clip[4 * i + 2]), 13.0f);
    }
}
