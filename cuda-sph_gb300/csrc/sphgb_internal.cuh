// sphgb_internal.cuh -- device-side building blocks shared by the kernels.
//
// Numerical contract (matches an FP64 evaluation of the reference on FP32
// inputs; reference = iwoplaza/cuda-sph, sim/src/sph/kernels/*.py):
//  * voxel coordinate: floor(x / voxel) computed exactly for FP32 x, voxel
//    (rounded quotient corrected by an exact fma residual).  For FP32 inputs
//    this equals the reference's int32(x / voxel) in FP64
//    (voxel_kernels.py:10-12) for 0 <= x; coordinates are clamped to the table.
//  * neighbour test sqrt(dx^2 + dy^2 + dz^2) <= INF_R (voxel_kernels.py:20-26):
//    evaluated in FP32 with a relative guard band of 2^-18 around h^2; inside
//    the band it is re-evaluated in FP64 exactly as the reference writes it
//    (no contraction, same operation order), so the decision is identical to
//    the FP64 one.  The FP32 error of d^2 is below 2^-21 relative.
//  * the physics sums (density, pressure, viscosity) are FP32 with Kahan
//    compensation; FP64 is used only in the guard band, the pipe-flow position
//    accumulator with its wall response, and the conservation reductions.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

struct SphgbGenerator;   // include/sphgb.h

namespace sphgb {

constexpr int kBlock = 256;

// One scene as the kernels see it (built on the host from SphgbSceneParams).
struct SceneDev {
    int32_t p_begin, p_count;   // slots [p_begin, p_begin + p_count) in sorted state
    int32_t v_begin, v_count;   // voxel table range: v_count voxels of the grid plus one
                                // overflow bucket (index v_begin + v_count) that holds
                                // particles with non-finite positions and is never walked
    int32_t dims[3];            // table dims, ceil(space / voxel)
    int32_t wdims[3];           // walk dims (== dims, or truncated)
    float vs[3];                // voxel size
    float h, h2, h2_lo, h2_hi;  // INF_R, INF_R^2 and the FP32 guard band
    float cull2;                // squared distance beyond which a voxel is skipped
    float w_const, grad_w_const, lap_w_const;  // W_CONST h^6, GRAD_W_CONST h^2, LAP_W_CONST h
    float mass, rho0, k, visc, damp, dt;
    float ext[3];
    float space[3];
    float wall_lo, wall_hi[3];  // 1e-3 and space - 1e-3 (base_kernels.py:75-98)
    double h_d;                 // (double)h for the guard-band path
    double dt_d;
    int32_t cap;                // MAX_NEIGHBOURS, or a huge value when uncapped
    int32_t mode;               // 0 box, 1 pipe
    int32_t walk_trunc;         // 1 when wdims != dims (no voxel culling then)
    int32_t pipe_off, pipe_rows;
    int32_t tiled;              // 1: voxel table in 4x4x4 tiles (see voxel_index), 0: row-major
    int32_t nt0, nt1;           // tiles along x and y when tiled
    int32_t pad;
    uint64_t seed;
    // the two divisors of a table index -> coordinates decode (nt0, nt1 when
    // tiled, else dims[0], dims[1]) as multiply-shift reciprocals (see Udiv)
    uint32_t div_m[2];
    int32_t div_s[2];
};

// floor(n / d) for 0 <= n < 2^31 and a divisor 1 <= d < 2^31 given as
// m = ceil(2^p / d), p = 31 + ceil(log2 d): with e = m - 2^p/d in [0, 1),
// n m / 2^p = n/d + n e / 2^p and n e / 2^p < 2^31 / 2^p = 2^-ceil(log2 d)
// <= 1/d, which never carries n/d past the next integer (Granlund and
// Montgomery, PLDI 1994, division by invariant integers).  m < 2^32.
struct Udiv {
    uint32_t m;
    int32_t p;
    __host__ __device__ __forceinline__ int div(int n) const {
        return (int)(((unsigned long long)(unsigned)n * m) >> p);
    }
};

inline Udiv make_udiv(uint32_t d) {
    int L = 0;
    while ((1ull << L) < d) ++L;
    const int p = 31 + L;
    const unsigned long long m = ((1ull << p) + d - 1) / d;
    return Udiv{(uint32_t)m, p};
}

// Table index of voxel (x, y, z) of a scene.  Row-major, x fastest (the
// reference's compute_1d_idx, voxel_kernels.py:14-17, with the stride dims
// d0, d1), or, for the fused step, in 4x4x4 tiles: tile (x/4, y/4, z/4) in
// row-major tile order, 64 voxels per tile, x fastest inside.  Tiles keep
// spatial neighbours close in the sorted state, which the passes that gather
// neighbour data read through L1.
__host__ __device__ __forceinline__ int voxel_index(int x, int y, int z, int tiled, int d0, int d1,
                                                    int nt0, int nt1) {
    if (tiled)
        return ((((z >> 2) * nt1 + (y >> 2)) * nt0 + (x >> 2)) << 6) | ((z & 3) << 4) |
               ((y & 3) << 2) | (x & 3);
    return x + y * d0 + z * d0 * d1;
}

// ---- scene lookup ---------------------------------------------------------
// pbegin has n_scenes + 1 entries (prefix of particle counts).
__device__ __forceinline__ int scene_of(int s, const int32_t* __restrict__ pbegin, int n_scenes) {
    int lo = 0, hi = n_scenes - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (__ldg(pbegin + mid) <= s) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// ---- per-scene step limits --------------------------------------------------
// With step limits bound (sphgb_ctx_set_step_limits), a scene whose step
// counter has reached its limit is frozen: a step leaves its state unchanged.
__device__ __forceinline__ bool scene_frozen(const int32_t* __restrict__ limit,
                                             const int32_t* __restrict__ step, int si) {
    return limit && __ldg(step + si) >= __ldg(limit + si);
}

// ---- exact voxel coordinate ----------------------------------------------
__device__ __forceinline__ int voxel_coord(float x, float vs, int dim) {
    if (!(x >= 0.0f)) return 0;                  // negative or NaN: first voxel
    float q = floorf(__fdiv_rn(x, vs));
    // the rounded quotient is floor(x/vs) or one more; the sign of the exact
    // residual x - q*vs (one rounding, sign preserved) decides
    if (__fmaf_rn(-q, vs, x) < 0.0f) q -= 1.0f;
    if (q >= (float)dim) return dim - 1;
    return (int)q;
}

// ---- neighbour predicate --------------------------------------------------
static __device__ __noinline__ bool within_exact(float xi, float yi, float zi, float xj, float yj,
                                          float zj, double h) {
    double dx = __dsub_rn((double)xi, (double)xj);
    double dy = __dsub_rn((double)yi, (double)yj);
    double dz = __dsub_rn((double)zi, (double)zj);
    double s = __dmul_rn(dx, dx);
    s = __dadd_rn(s, __dmul_rn(dy, dy));
    s = __dadd_rn(s, __dmul_rn(dz, dz));
    return __dsqrt_rn(s) <= h;
}

// d2 of the pair in FP32; returns the reference's decision.
__device__ __forceinline__ bool within(const float4& pi, const float4& pj, float h2_lo, float h2_hi,
                                       double h_d, float& dx, float& dy, float& dz, float& d2) {
    dx = __fsub_rn(pi.x, pj.x);
    dy = __fsub_rn(pi.y, pj.y);
    dz = __fsub_rn(pi.z, pj.z);
    d2 = __fmul_rn(dx, dx);
    d2 = __fmaf_rn(dy, dy, d2);
    d2 = __fmaf_rn(dz, dz, d2);
    if (d2 < h2_lo) return true;
    if (d2 > h2_hi) return false;
    return within_exact(pi.x, pi.y, pi.z, pj.x, pj.y, pj.z, h_d);
}

__device__ __forceinline__ bool finite3(const float4& p) {
    return isfinite(p.x) && isfinite(p.y) && isfinite(p.z);
}

// ---- Kahan summation ------------------------------------------------------
// s - c is the running sum; c the rounding error still to be taken off.
struct Kahan {
    float s = 0.0f, c = 0.0f;
    __device__ __forceinline__ void add(float x) {
        float y = __fsub_rn(x, c);
        float t = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(t, s), y);
        s = t;
    }
    // the sum of b's terms added after this one's: b.s, then b's pending -c
    __device__ __forceinline__ void merge(const Kahan& b) {
        add(b.s);
        add(-b.c);
    }
};

// The density sum of a particle runs in two compensated parts that are then
// merged: its accepted list entries (walk order, the particle itself counted
// in the position) below kSumSplit, and the rest.  The warp-cooperative pass
// gives the two parts to two lanes; the thread-per-particle pass uses the
// same split, so both give the same bits.
constexpr int kSumSplit = 16;

// ---- the 27-voxel walk ----------------------------------------------------
// Scene geometry the walk needs, loaded once per thread into registers.
struct WalkGeom {
    float vs0, vs1, vs2;
    int d0, d1, d2;        // table dims
    int w0, w1, w2;        // walk dims
    int v_begin;
    float h2_lo, h2_hi, cull2;
    double h_d;
    int cap;
    bool cull;
    int tiled, nt0, nt1;
};

__device__ __forceinline__ WalkGeom load_geom(const SceneDev& sc) {
    WalkGeom g;
    g.vs0 = sc.vs[0]; g.vs1 = sc.vs[1]; g.vs2 = sc.vs[2];
    g.d0 = sc.dims[0]; g.d1 = sc.dims[1]; g.d2 = sc.dims[2];
    g.w0 = sc.wdims[0]; g.w1 = sc.wdims[1]; g.w2 = sc.wdims[2];
    g.v_begin = sc.v_begin;
    g.h2_lo = sc.h2_lo; g.h2_hi = sc.h2_hi; g.cull2 = sc.cull2;
    g.h_d = sc.h_d;
    g.cap = sc.cap;
    g.cull = !sc.walk_trunc;
    g.tiled = sc.tiled;
    g.nt0 = sc.nt0;
    g.nt1 = sc.nt1;
    return g;
}

// Visits neighbours of a particle in the reference's order (voxel_kernels.py:
// 46-61 dx outer, dy, dz inner; members in ascending particle id, which is
// slot order inside a voxel) and stops after `cap` accepted neighbours
// (self included, :77-84).  visit(j, dx, dy, dz, d2) is called per accepted
// neighbour slot j.  Returns the number accepted.  A particle with a
// non-finite coordinate has no neighbours (every distance test fails).
// kLayout: the scene's voxel table is row-major (0), tiled (1), or either,
// read from g.tiled (2).
template <int kLayout = 2, class Visit>
__device__ __forceinline__ int walk(const float4 pi, const WalkGeom& g,
                                    const int32_t* __restrict__ vstart,
                                    const int32_t* __restrict__ vcount,
                                    const float4* __restrict__ pos, int cap, Visit&& visit) {
    if (!finite3(pi)) return 0;
    const int cx = voxel_coord(pi.x, g.vs0, g.d0);
    const int cy = voxel_coord(pi.y, g.vs1, g.d1);
    const int cz = voxel_coord(pi.z, g.vs2, g.d2);
    // squared distances to the lower/upper faces of the own voxel, used to skip
    // voxels that lie entirely beyond h (only when walk dims == table dims)
    const float fx = pi.x - (float)cx * g.vs0;
    const float fy = pi.y - (float)cy * g.vs1;
    const float fz = pi.z - (float)cz * g.vs2;
    const float gx0 = fx * fx, gx2 = (g.vs0 - fx) * (g.vs0 - fx);
    const float gy0 = fy * fy, gy2 = (g.vs1 - fy) * (g.vs1 - fy);
    const float gz0 = fz * fz, gz2 = (g.vs2 - fz) * (g.vs2 - fz);
    int n = 0;
#pragma unroll 1
    for (int ddx = 0; ddx < 3; ++ddx) {
        const int nx = cx + ddx - 1;
        if (nx < 0 || nx >= g.w0) continue;
        const float gx = ddx == 0 ? gx0 : (ddx == 2 ? gx2 : 0.0f);
#pragma unroll 1
        for (int ddy = 0; ddy < 3; ++ddy) {
            const int ny = cy + ddy - 1;
            if (ny < 0 || ny >= g.w1) continue;
            const float gxy = gx + (ddy == 0 ? gy0 : (ddy == 2 ? gy2 : 0.0f));
#pragma unroll 1
            for (int ddz = 0; ddz < 3; ++ddz) {
                const int nz = cz + ddz - 1;
                if (nz < 0 || nz >= g.w2) continue;
                if (g.cull && gxy + (ddz == 0 ? gz0 : (ddz == 2 ? gz2 : 0.0f)) > g.cull2) continue;
                const int tiled = kLayout == 2 ? g.tiled : kLayout;
                const int vid = g.v_begin + voxel_index(nx, ny, nz, tiled, g.w0, g.w1, g.nt0, g.nt1);
                const int c = __ldg(vcount + vid);
                if (c == 0) continue;
                const int s0 = __ldg(vstart + vid);
#pragma unroll 2
                for (int m = 0; m < c; ++m) {
                    const int j = s0 + m;
                    const float4 pj = __ldg(pos + j);
                    float dx, dy, dz, d2;
                    if (within(pi, pj, g.h2_lo, g.h2_hi, g.h_d, dx, dy, dz, d2)) {
                        visit(j, dx, dy, dz, d2);
                        if (++n >= cap) return n;
                    }
                }
            }
        }
    }
    return n;
}

// ---- Philox4x32-10 (Salmon, Moraes, Dror, Shaw; SC 2011) -----------------
__device__ __forceinline__ double philox_uniform(uint64_t seed, uint32_t pid, uint32_t step,
                                                 uint32_t draw) {
    uint32_t c0 = draw, c1 = step, c2 = pid, c3 = 0u;
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        if (r != 9) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    }
    uint64_t bits = ((uint64_t)c0 << 21) | (c1 >> 11);
    return (double)bits * (1.0 / 9007199254740992.0);
}

// ---- pipe geometry in FP64 (util_kernels.py) -------------------------------
// pipe rows: [x0, y0, z0, r_start, length] (Pipe.to_numpy, data_classes.py:34-44)
struct PipeView {
    const double* p;
    int rows;
    __device__ __forceinline__ double at(int r, int c) const { return p[r * 5 + c]; }
};

// util_kernels.py:38-43
__device__ inline double pipe_x_begin(const PipeView& P, int seg) {
    double xb = P.at(0, 0);
    for (int i = 0; i < seg; ++i) xb = __dadd_rn(xb, P.at(i, 4));
    return xb;
}

// util_kernels.py:56-69
__device__ inline double pipe_radius(const double* p, const PipeView& P, int seg) {
    double r0 = P.at(seg, 3), r1 = P.at(seg + 1, 3), L = P.at(seg, 4);
    if (r0 == r1) return r0;
    if (r0 < r1) {
        double delta = __dsub_rn(p[0], pipe_x_begin(P, seg));
        double tl = __ddiv_rn(__dmul_rn(L, r0), __dsub_rn(r1, r0));
        return __dmul_rn(r0, __dadd_rn(1.0, __ddiv_rn(delta, tl)));
    }
    double delta = __dsub_rn(__dadd_rn(pipe_x_begin(P, seg), L), p[0]);
    double tl = __ddiv_rn(__dmul_rn(L, r1), __dsub_rn(r0, r1));
    return __dmul_rn(r1, __dadd_rn(1.0, __ddiv_rn(delta, tl)));
}

// util_kernels.py:72-77
__device__ inline int pipe_find_segment(const double* p, const PipeView& P) {
    for (int j = 0; j < P.rows - 1; ++j)
        if (P.at(j, 0) <= p[0] && p[0] < P.at(j + 1, 0)) return j;
    return -1;
}

__device__ __forceinline__ double len3(const double* v) {
    double l = __dmul_rn(v[0], v[0]);
    l = __dadd_rn(l, __dmul_rn(v[1], v[1]));
    l = __dadd_rn(l, __dmul_rn(v[2], v[2]));
    return __dsqrt_rn(l);
}

__device__ __forceinline__ double dot3(const double* a, const double* b) {
    double s = __dmul_rn(a[0], b[0]);
    s = __dadd_rn(s, __dmul_rn(a[1], b[1]));
    s = __dadd_rn(s, __dmul_rn(a[2], b[2]));
    return s;
}

// util_kernels.py:46-53
__device__ inline bool pipe_is_out(const double* p, const PipeView& P, int seg, double* radius) {
    double yn = __dsub_rn(p[1], P.at(seg, 1)), zn = __dsub_rn(p[2], P.at(seg, 2));
    double hh = __dsqrt_rn(__dadd_rn(__dmul_rn(yn, yn), __dmul_rn(zn, zn)));
    double r = pipe_radius(p, P, seg);
    if (radius) *radius = r;
    return hh > r;
}

// solve_collision, util_kernels.py:182-204 with the helpers of :80-179
__device__ inline void pipe_solve_collision(double* p, double* v, const PipeView& P, int seg) {
    const double r0 = P.at(seg, 3), r1 = P.at(seg + 1, 3);
    // calc_edge_vector :152-171
    double yn = __dsub_rn(p[1], P.at(seg, 1)), zn = __dsub_rn(p[2], P.at(seg, 2));
    double hh = __dsqrt_rn(__dadd_rn(__dmul_rn(yn, yn), __dmul_rn(zn, zn)));
    double first[3], second[3], edge[3];
    first[0] = P.at(seg, 0);
    second[0] = P.at(seg + 1, 0);
    for (int a = 1; a < 3; ++a) {
        double q = __ddiv_rn(__dsub_rn(p[a], P.at(seg, a)), hh);
        first[a] = __dmul_rn(q, r0);
        second[a] = __dmul_rn(q, r1);
    }
    for (int a = 0; a < 3; ++a) edge[a] = __dsub_rn(second[a], first[a]);
    for (int a = 1; a < 3; ++a) first[a] = __dadd_rn(first[a], P.at(seg, a));
    // calc_collision_point :174-179, calc_dt :113-121, calc_distance_to_pipe :124-135
    const double sl = len3(v), el = len3(edge);
    const double cos_a = __ddiv_rn(dot3(v, edge), __dmul_rn(sl, el));
    double pv[3], cr[3];
    for (int a = 0; a < 3; ++a) pv[a] = __dsub_rn(first[a], p[a]);
    cr[0] = __dsub_rn(__dmul_rn(edge[1], pv[2]), __dmul_rn(edge[2], pv[1]));
    cr[1] = __dsub_rn(__dmul_rn(edge[2], pv[0]), __dmul_rn(edge[0], pv[2]));
    cr[2] = __dsub_rn(__dmul_rn(edge[0], pv[1]), __dmul_rn(edge[1], pv[0]));
    const double dd = __ddiv_rn(len3(cr), len3(edge));
    const double sin_a = __dsqrt_rn(__dsub_rn(1.0, __dmul_rn(cos_a, cos_a)));
    const double d_to = __ddiv_rn(dd, __dadd_rn(sin_a, 0.001));
    const double dtc = __ddiv_rn(-d_to, sl);
    double cp[3];
    for (int a = 0; a < 3; ++a) cp[a] = __dadd_rn(p[a], __dmul_rn(v[a], dtc));
    if (r0 == r1) {
        v[1] = -v[1];
        v[2] = -v[2];
    } else {  // calc_summary_vector :88-94
        const double ll = len3(edge), pl = len3(v);
        const double c = __ddiv_rn(dot3(edge, v), __dmul_rn(ll, pl));
        double sv[3];
        for (int a = 0; a < 3; ++a)
            sv[a] = __dmul_rn(__dmul_rn(__ddiv_rn(__dmul_rn(2.0, edge[a]), ll), c), pl);
        for (int a = 0; a < 3; ++a) v[a] = __dsub_rn(sv[a], v[a]);
    }
    double w[3];
    for (int a = 0; a < 3; ++a) w[a] = __dsub_rn(p[a], cp[a]);
    const double way = len3(w);
    const double svl = len3(v);
    for (int a = 0; a < 3; ++a) p[a] = __dadd_rn(cp[a], __ddiv_rn(__dmul_rn(v[a], way), svl));
}

// collision_kernel (base_kernels.py:56-72) with put_particle_at_pipe_begin
// (:101-113) and rand_position_inside_pipe (:116-127); respawn uniforms from
// Philox keyed by (seed, particle id) with counter (draw, step).
__device__ inline void pipe_collide(double* p, double* v, const PipeView& P, uint64_t seed,
                                    uint32_t pid, uint32_t step) {
    int seg = pipe_find_segment(p, P);
    if (seg == -1) {
        if (p[0] < 0.0) {
            p[0] = -p[0];
            v[0] = -v[0];
            if (pipe_is_out(p, P, 0, nullptr)) pipe_solve_collision(p, v, P, 0);
        } else {
            p[0] = 0.0;
            int s = pipe_find_segment(p, P);
            if (s < 0) s = 0;  // a pipe starting after x = 0 (reference reads row -1)
            double R = pipe_radius(p, P, s);
            double r = __dmul_rn(R, __dsqrt_rn(philox_uniform(seed, pid, step, 0)));
            double th = __dmul_rn(__dmul_rn(philox_uniform(seed, pid, step, 1), 2.0),
                                  3.141592653589793);
            double sn, cs;
            sincos(th, &sn, &cs);
            p[1] = __dadd_rn(P.at(0, 1), __dmul_rn(r, cs));
            p[2] = __dadd_rn(P.at(0, 2), __dmul_rn(r, sn));
        }
    } else if (pipe_is_out(p, P, seg, nullptr)) {
        pipe_solve_collision(p, v, P, seg);
    }
}

// ---- 256-bit global accesses ----------------------------------------------
// One thread moves 32 bytes with one instruction (sm_100 and later; the
// address must be 32-byte aligned).  In a gather, where the lanes of a warp
// touch unrelated lines, an L1 pass costs per line touched, so one 32-byte
// load of a force record costs half of two 16-byte loads.
__device__ __forceinline__ void ldg256(const float4* p, float4& a, float4& b) {
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}
__device__ __forceinline__ void ldg256(const int32_t* p, int (&v)[8]) {
    asm("ld.global.nc.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
          "=r"(v[7])
        : "l"(p));
}
__device__ __forceinline__ void stg256(float4* p, const float4& a, const float4& b) {
    asm volatile("st.global.v8.f32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};"
                 :: "l"(p), "f"(a.x), "f"(a.y), "f"(a.z), "f"(a.w), "f"(b.x), "f"(b.y),
                    "f"(b.z), "f"(b.w)
                 : "memory");
}

// ---- neighbour list --------------------------------------------------------
// Neighbours (other than self) of every particle in walk order, recorded by
// the density pass and read by the force pass.  One row per particle:
// idx[s * kListCap + k]; rows are 128-byte aligned (idx from cudaMalloc), so
// the force pass reads a row eight entries per load.
constexpr int kListCap = 32;
struct NbrList {
    int32_t* idx = nullptr;     // kListCap * n entries
    int32_t* count = nullptr;   // n entries; -1 = more than kListCap neighbours
};

// Force pass over a range of particles in original order (scene offset +
// particle id): particle i is at slot slot_of[i], and its next position and
// velocity are also written as FP64 rows i of pos / vel (the host-buffer
// entry point downloads each range while the next one is computed).
// Velocities that the density pass gathers itself (pipelined host entry):
// the uploaded FP64 rows in original order, converted as k_load_aos converts
// them, into the slot-order state and the second half of the force records.
// vel64 null: off.
struct VelRows {
    const double* vel64 = nullptr;   // (n, 3) FP64, scene offset + particle id
    const int32_t* pid = nullptr;    // particle id per slot
    float4* vel_out = nullptr;       // slot order
};

struct PidRange {
    const int32_t* slot_of = nullptr;
    int i0 = 0, i1 = 0;
    // list mode (slots set): the pass runs slots[0..n_slots) in that order
    // instead, each writing the rows of its particle id, density included
    const int32_t* slots = nullptr;
    int n_slots = 0;
    double* pos = nullptr;      // (n, 3) FP64
    double* vel = nullptr;      // (n, 3) FP64
    double* rho = nullptr;      // (n,) FP64, list mode
};

// Particles a lean force pass defers to a second launch (see kForceLean in
// walk.cu): entries idx[base + k] for k < *count, each a slot, or a row of
// the PidRange in range mode.  Unset (count null): one pass does every
// particle.
struct RareList {
    int32_t* idx = nullptr;
    int32_t* count = nullptr;   // zeroed before the pass
    int base = 0;
};

// ---- launchers (host) -----------------------------------------------------
// Streaming multiprocessors of the current device, queried once per device
// ordinal (cudaDevAttrMultiProcessorCount) and cached; persistent and
// one-block-per-SM grids are sized from it.
int device_sm_count();

struct Launch {
    const SceneDev* scenes;     // device array
    const int32_t* pbegin;      // device, n_scenes + 1
    int n_scenes;
    int n;                      // particles (all scenes)
    int v_total;                // voxels (all scenes)
    const double* pipe;         // device pipe table (may be null)
    bool pipe_scenes;           // some scene is in pipe mode
    int sort_block = kBlock;    // threads per block of the per-particle sort kernels
    int big_voxel = 64;         // voxels above this many members are sorted per block
    int layout = 0;             // voxel tables: 0 all row-major, 1 all tiled, 2 mixed
    cudaStream_t stream;
    // per-scene step limits and counters (device, n_scenes each); limits null:
    // no scene is frozen.  A frozen scene's particles keep their slots in the
    // sort, get no density task and are copied through by the force pass.
    const int32_t* step_limit = nullptr;
    const int32_t* scene_step = nullptr;
};

// cell[s] = voxel id, or ~id (negative) for a particle in its scene's overflow
// bucket; slot[s] = its arrival slot in the voxel.  Particles i0..i1 (i1 < 0:
// all): the histogram may be filled in several launches over parts of the state
// (the arrival order inside a voxel is dropped by the rank-gather).
cudaError_t launch_hash_count(const Launch& L, const float4* pos, int32_t* cell, int32_t* slot,
                              int32_t* vcount, int i0 = 0, int i1 = -1);
cudaError_t launch_scan(const Launch& L, const int32_t* vcount, int32_t* vstart,
                        int32_t* tile_sums, int n_tiles);
int scan_tiles(int v_total);
cudaError_t launch_scatter(const Launch& L, const int32_t* cell, const int32_t* slot,
                           const int32_t* pid, const int32_t* vstart, const int32_t* vcount,
                           int32_t* tmp_pid, int32_t* big_list, int32_t* big_count);
// voxels with more than Launch::big_voxel members (default kBigVoxel) get their
// member ids sorted by one block each (the rank-gather then binary-searches
// them instead of counting); the threshold is never below kMinBigVoxel
constexpr int kBigVoxel = 64;
constexpr int kMinBigVoxel = 16;
cudaError_t launch_sort_big(const Launch& L, const int32_t* big_list, const int32_t* big_count,
                            const int32_t* vstart, const int32_t* vcount, int32_t* tmp_pid);
// Density tasks: one (voxel, first slot) entry per run of up to kTaskRun
// sorted slots of a voxel; a warp of the density pass takes one task at a time.
constexpr int kTaskRun = 16;
// tasks (optional): one (voxel, first slot) entry per run of up to kTaskRun
// sorted slots of a voxel, appended at task_count.  tmp_pid must be 16-byte aligned
// with 4 entries of room past n (the rank count reads it in aligned quads).
cudaError_t launch_rank_gather(const Launch& L, const int32_t* cell, const int32_t* slot,
                               const int32_t* pid, const int32_t* tmp_pid, const int32_t* vstart,
                               const int32_t* vcount, const float4* pos, const float4* vel,
                               const double* pos64, float4* pos_out, float4* vel_out,
                               int32_t* pid_out, double* pos64_out, int2* tasks = nullptr,
                               int32_t* task_count = nullptr);
// fin (optional, with vel): the force inputs of each particle, two float4
// per particle: (x, y, z, p/rho^2) and (vx, vy, vz, 1/rho)
cudaError_t launch_density(const Launch& L, const float4* pos, const float4* vel,
                           const int32_t* vstart, const int32_t* vcount, float* rho,
                           float4* fin, NbrList nbr);
// the step's density pass: one warp per task (<= kTaskRun particles of one voxel);
// task_next: a zeroed counter from which the warps take the tasks
// task_offset (optional, device): the tasks start at tasks[*task_offset] (one
// bucket of a bucketed list)
cudaError_t launch_density_wc(const Launch& L, const float4* pos, const float4* vel,
                              const int32_t* vstart, const int32_t* vcount, float* rho,
                              float4* fin, NbrList nbr, const int2* tasks,
                              const int32_t* task_count, int32_t* task_next,
                              const int32_t* task_offset = nullptr, VelRows vrows = VelRows{});
// k_gather_vel over the slots of a bucket of density tasks
cudaError_t launch_gather_vel_tasks(const Launch& L, const int32_t* pid, const int2* tasks,
                                    const int32_t* task_count, const int32_t* task_offset,
                                    const int32_t* vstart, const int32_t* vcount,
                                    const double* vel64, const float* rho, float4* vel_out,
                                    float4* fin);
cudaError_t launch_gather_vel(const Launch& L, const int32_t* pid, const float4* vel_in,
                              const float* rho, float4* vel_out, float4* fin);
cudaError_t launch_forces(const Launch& L, const float4* pos, const float4* vel,
                          const float* rho, const float4* fin, const int32_t* vstart,
                          const int32_t* vcount, float4* pressure, float4* viscosity);
cudaError_t launch_integrate(const Launch& L, const float4* pos, const float4* vel,
                             const float* rho, const float4* fin, const int32_t* pid,
                             const double* pos64, const int32_t* vstart, const int32_t* vcount,
                             const int32_t* scene_step, NbrList nbr, float4* pos_out,
                             float4* vel_out, int32_t* pid_out, double* pos64_out,
                             float4* force_out, RareList rare = RareList{});
cudaError_t launch_integrate_range(const Launch& L, const float4* pos, const float4* vel,
                                   const float* rho, const float4* fin, const int32_t* pid,
                                   const double* pos64, const int32_t* vstart,
                                   const int32_t* vcount, const int32_t* scene_step, NbrList nbr,
                                   float4* pos_out, float4* vel_out, int32_t* pid_out,
                                   double* pos64_out, PidRange range,
                                   RareList rare = RareList{});
cudaError_t launch_neighbours(const Launch& L, const float4* pos, const int32_t* vstart,
                              const int32_t* vcount, int32_t* list, int stride,
                              int32_t* n_capped, int32_t* n_uncapped);
// the force inputs from a given density (stage entry points)
cudaError_t launch_force_inputs(const Launch& L, const float4* pos, const float4* vel,
                                const float* rho, float4* fin);

// generate.cu: start states and the point-field vertex stage
cudaError_t launch_generate(const SphgbGenerator& g, const double* pipe, int pipe_rows, int64_t n,
                            double* pos, double* vel, cudaStream_t st);
cudaError_t launch_point_field(const float* pos, int stride, const float* rho, int64_t n,
                               const float* proj16, const float* model16, const float* view16,
                               float* clip, float* colour, float* size, cudaStream_t st);

}  // namespace sphgb
