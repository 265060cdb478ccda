// walk.cu -- neighbour walk kernels: density (warp-cooperative for the step,
// thread per particle for the stage entry points), forces, fused force +
// integrate + wall response, and the neighbour list/count kernel used for
// parity.
//
// Particles are in voxel-sorted order, so the threads or warps of a block walk
// overlapping voxel neighbourhoods and their candidate loads are served from
// L1.  The walk order and the 32-neighbour cap are the reference's
// (get_neighbours, sim/src/sph/kernels/voxel_kernels.py:30-85).
#include "sphgb_internal.cuh"

namespace sphgb {

namespace {

inline int blocks_for(int n) { return (n + kBlock - 1) / kBlock; }

// density_kernel, voxel_kernels.py:109-132: rho_i = MASS * sum_{j != i} W_ij,
// W = W_CONST (h^2 - r^2)^3 (base_kernels.py:6-9), written here as
// W_CONST h^6 (1 - r^2/h^2)^3 so the FP32 sum stays in range for any h.
// Also writes the particle's force inputs (see write_force_inputs) with the
// per-particle factors of the force pass, p_i / rho_i^2 and 1 / rho_i, p = K (rho
// - RHO_0) (voxel_kernels.py:162-164, :205-208),
// and, when nbr is given, the particle's neighbours other than itself in walk
// order (the set every later kernel of the step uses), one row per particle,
// nbr.idx[s * kListCap + k]; nbr.count[s] = their number, or -1 when more
// than kListCap (the force pass then walks again).
// Force inputs of particle s: fin[2s] = (x, y, z, p/rho^2), fin[2s + 1] =
// (vx, vy, vz, 1/rho), one 32-byte record that the force pass reads per
// neighbour instead of three separate arrays.  With vel null only the first
// half is written; k_gather_vel writes the second once the velocities are in.
// first half of a force record: position and p / rho^2
__device__ __forceinline__ float4 force_record_a(const float4& pi, const SceneDev& sc, float r) {
    const float p = sc.k * (r - sc.rho0);
    return make_float4(pi.x, pi.y, pi.z, p / (r * r));
}

__device__ __forceinline__ void write_force_inputs(int s, const float4& pi, const SceneDev& sc,
                                                   const float4* __restrict__ vel, float r,
                                                   float4* __restrict__ fin) {
    const float4 a = force_record_a(pi, sc, r);
    if (vel) {
        const float4 v = __ldg(vel + s);
        stg256(fin + 2 * s, a, make_float4(v.x, v.y, v.z, 1.0f / r));
    } else {
        fin[2 * s] = a;
    }
}

// One particle's density by a thread-private walk: the walk records neighbour
// slots in row[k * stride] (k < kListCap), the sum runs afterwards in walk
// order in the two parts of kSumSplit; with more neighbours than that the
// walk is repeated, summing in one part.  fin (with vel) is optional.
// kLayout: see walk().
template <int kLayout>
__device__ __forceinline__ void density_one(int s, const float4& pi, const SceneDev& sc,
                                            const float4* __restrict__ pos,
                                            const float4* __restrict__ vel,
                                            const int32_t* __restrict__ vstart,
                                            const int32_t* __restrict__ vcount, int n,
                                            float* __restrict__ rho, float4* __restrict__ fin,
                                            const NbrList& nbr, int32_t* row, int stride) {
    const WalkGeom g = load_geom(sc);
    int others = 0, lo = 0;   // lo: neighbours in the first part of the sum
    bool self_seen = false;
    walk<kLayout>(pi, g, vstart, vcount, pos, g.cap, [&](int j, float, float, float, float) {
        if (j != s) {
            if (others + (self_seen ? 1 : 0) < kSumSplit) ++lo;
            if (others < kListCap) row[others * stride] = j;
            ++others;
        } else {
            self_seen = true;
        }
    });
    const float inv_h2 = 1.0f / sc.h2;
    Kahan acc;
    if (others <= kListCap) {
        Kahan acc2;
#pragma unroll 4
        for (int k = 0; k < others; ++k) {
            const float4 pj = __ldg(pos + row[k * stride]);
            const float dx = __fsub_rn(pi.x, pj.x);
            const float dy = __fsub_rn(pi.y, pj.y);
            const float dz = __fsub_rn(pi.z, pj.z);
            float d2 = __fmul_rn(dx, dx);
            d2 = __fmaf_rn(dy, dy, d2);
            d2 = __fmaf_rn(dz, dz, d2);
            const float u = __fmaf_rn(-d2, inv_h2, 1.0f);
            if (k < lo) acc.add(u * u * u); else acc2.add(u * u * u);
        }
        acc.merge(acc2);
        if (nbr.idx)
            for (int k = 0; k < others; ++k) nbr.idx[(size_t)s * kListCap + k] = row[k * stride];
    } else {
        // more neighbours than the list holds (no cap or a cap above it):
        // walk again, summing on the way
        walk<kLayout>(pi, g, vstart, vcount, pos, g.cap, [&](int j, float, float, float, float d2) {
            if (j != s) {
                const float u = __fmaf_rn(-d2, inv_h2, 1.0f);
                acc.add(u * u * u);
            }
        });
    }
    const float r = (acc.s * sc.w_const) * sc.mass;
    rho[s] = r;
    if (fin) write_force_inputs(s, pi, sc, vel, r, fin);
    if (nbr.count) nbr.count[s] = others <= kListCap ? others : -1;
}

// thread per particle (used by the stage entry points and as the reference
// path of the warp-cooperative kernel below)
template <int kLayout>
__global__ void __launch_bounds__(kBlock)
k_density(const SceneDev* __restrict__ scenes, const int32_t* __restrict__ pbegin, int n_scenes,
          int n, const float4* __restrict__ pos, const float4* __restrict__ vel,
          const int32_t* __restrict__ vstart, const int32_t* __restrict__ vcount,
          float* __restrict__ rho, float4* __restrict__ fin, NbrList nbr,
          const int32_t* __restrict__ step_limit, const int32_t* __restrict__ scene_step) {
    __shared__ int32_t s_list[kListCap][kBlock];
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int si = scene_of(s, pbegin, n_scenes);
    if (scene_frozen(step_limit, scene_step, si)) return;   // state and density stay
    const SceneDev& sc = scenes[si];
    density_one<kLayout>(s, __ldg(pos + s), sc, pos, vel, vstart, vcount, n, rho, fin, nbr,
                         &s_list[0][threadIdx.x], kBlock);
}

// squared distance with the walk's arithmetic (within() in sphgb_internal.cuh)
__device__ __forceinline__ float dist2(const float4& a, const float4& b) {
    const float dx = __fsub_rn(a.x, b.x);
    const float dy = __fsub_rn(a.y, b.y);
    const float dz = __fsub_rn(a.z, b.z);
    float d2 = __fmul_rn(dx, dx);
    d2 = __fmaf_rn(dy, dy, d2);
    return __fmaf_rn(dz, dz, d2);
}

// Warp-cooperative density pass of the step.  One warp per task: up to
// kTaskRun particles of one voxel (tasks listed by the rank-gather).  The 27
// walk voxels of that voxel are laid end to end in walk order; each batch of
// 96 candidates is loaded coalesced, three per lane (a candidate's slot found
// from voxel-boundary bit masks built with one warp OR-reduction per 32
// candidates), and every home particle is
// tested against the whole batch at once: a ballot gives its accepted
// candidates in walk order and popc ranks them against the cap, so the
// accepted set is exactly the reference's first MAX_NEIGHBOURS (self
// included).  Each accepted entry keeps its slot and its squared distance.
// Then the density terms are computed from those distances with one lane per
// list entry and summed in walk order with one lane per home particle, the
// arithmetic of density_one: the results are bit-identical to the
// thread-per-particle kernel.
constexpr int kWcWarps = 8;
// list entry of the particle itself once entries hold density terms: a NaN
// bit pattern, which no term (a cube of a finite number) takes
constexpr int kSelfTerm = 0x7fc0dead;
constexpr int kWcList = kListCap;       // accepted neighbours per particle, self included
constexpr int kWcPerLane = 3;           // candidates per lane in one batch
constexpr int kWcBatch = 32 * kWcPerLane;
constexpr int kWcCullMin = 4 * kWcBatch;  // walks longer than this skip unreachable batches

// Bit k (k = 9 (dx + 1) + 3 (dy + 1) + dz + 1, the walk order) is set when walk
// voxel k of voxel (vx, vy, vz) may hold a particle within h of p: the same
// box-distance test as walk() in sphgb_internal.cuh, against the widened
// bound cull2.
__device__ __forceinline__ unsigned reach_mask(const float4& p, int vx, int vy, int vz,
                                               const SceneDev& sc) {
    const float fx = p.x - (float)vx * sc.vs[0];
    const float fy = p.y - (float)vy * sc.vs[1];
    const float fz = p.z - (float)vz * sc.vs[2];
    const float gx[3] = {fx * fx, 0.0f, (sc.vs[0] - fx) * (sc.vs[0] - fx)};
    const float gy[3] = {fy * fy, 0.0f, (sc.vs[1] - fy) * (sc.vs[1] - fy)};
    const float gz[3] = {fz * fz, 0.0f, (sc.vs[2] - fz) * (sc.vs[2] - fz)};
    unsigned m = 0;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            const float gxy = gx[a] + gy[b];
#pragma unroll
            for (int c = 0; c < 3; ++c)
                if (!(gxy + gz[c] > sc.cull2)) m |= 1u << (9 * a + 3 * b + c);
        }
    return m;
}

// Per warp.  An accepted entry is its slot and its squared distance (int
// bits), the distance the candidate loop decided on, so the density term
// needs no second gather of the neighbour's position; the candidate loop
// writes both with one 8-byte store.  Phase (a) replaces the distance with
// the term (kSelfTerm for the particle itself).
static_assert(kTaskRun <= 16 && kTaskRun <= kSumSplit, "phase (b) gives each home two lanes");
struct WcShared {
    float4 home[kTaskRun];
    int2 e[kTaskRun][kWcList + 1];   // (slot, squared distance or term)
    int32_t off[27];    // first slot - first walk index of each non-empty walk voxel, by rank
};

// The candidate loop of k_density_wc for one task: batches of kWcBatch
// candidates in walk order, each tested against every home particle still
// below the cap.  Accepted entries go to S.e[i] in walk order
// and the counts to cnt (lane i: home particle i).  Lane k < 27 holds walk voxel k's first
// walk index Pk and member count ck.  kCull: a home particle skips the batches
// that lie wholly in walk voxels outside its reach mask.
template <bool kCull>
__device__ __forceinline__ void wc_candidates(WcShared& S, int& cnt, bool home, int cap, int M,
                                              int Pk, int ck, bool nzk, unsigned reach,
                                              const float4* __restrict__ pos, float h2_lo,
                                              float h2_hi, double h_d) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const unsigned le = (2u << lane) - 1u;      // bits 0..lane
    const float inf = __int_as_float(0x7f800000);
    for (int b0 = 0; b0 < M; b0 += kWcBatch) {
        // home particles still below the cap
        unsigned todo = __ballot_sync(full, home && cnt < cap);
        if (!todo) break;
        if (kCull) {
            // walk voxels overlapping this batch, and the homes that reach one
            const unsigned span =
                __ballot_sync(full, nzk && Pk < b0 + kWcBatch && Pk + ck > b0);
            todo &= __ballot_sync(full, (reach & span) != 0u);
            if (!todo) continue;
        }
        // Batch candidates q = b0 + 32 u + lane.  Bw[u] bit l: a non-empty
        // walk voxel starts at q = b0 + 32 u + l (l >= 1 when u = 0); the
        // rank of the voxel holding q is the number of non-empty voxels
        // starting at or before b0, minus one, plus the set bits up to q.
        const int pk = Pk - b0;
        unsigned Bw[kWcPerLane];
#pragma unroll
        for (int u = 0; u < kWcPerLane; ++u)
            Bw[u] = __reduce_or_sync(
                full, (nzk && pk >= 1 && (pk >> 5) == u) ? (1u << (pk & 31)) : 0u);
        int rank = __popc(__ballot_sync(full, nzk && pk <= 0)) - 1;
        // past the end of the walk: +inf coordinates, never within h
        float4 pj[kWcPerLane];
        int sj[kWcPerLane];
#pragma unroll
        for (int u = 0; u < kWcPerLane; ++u) {
            const int q = b0 + 32 * u + lane;
            pj[u] = make_float4(inf, inf, inf, 0.f);
            sj[u] = -1;
            if (q < M) {
                sj[u] = q + S.off[rank + __popc(Bw[u] & le)];
                pj[u] = __ldg(pos + sj[u]);
            }
            rank += __popc(Bw[u]);
        }
        // Fast pass: FP32 decisions only.  A pair in the FP32 guard band
        // around h^2 is rare; if any occurs, the whole batch is redone from
        // the counts it started with, deciding those pairs in FP64.  Every
        // list entry below the final counts is rewritten by the redo.
        const int cnt0 = cnt;
        bool band_seen = false;
        for (unsigned t = todo; t; t &= t - 1) {
            const int i = __ffs(t) - 1;
            int r = __shfl_sync(full, cnt, i);
            const float4 ph = S.home[i];
#pragma unroll
            for (int u = 0; u < kWcPerLane; ++u) {
                const float d2 = dist2(ph, pj[u]);
                const bool acc = d2 < h2_lo;
                band_seen |= !acc && d2 <= h2_hi;
                const unsigned m = __ballot_sync(full, acc);
                const int ru = r + __popc(m & lt);
                if (acc && ru < cap) S.e[i][ru] = make_int2(sj[u], __float_as_int(d2));
                r += __popc(m);
            }
            if (lane == i) cnt = r;
        }
        if (__any_sync(full, band_seen)) {
            cnt = cnt0;
            for (unsigned t = todo; t; t &= t - 1) {
                const int i = __ffs(t) - 1;
                int r = __shfl_sync(full, cnt, i);
                const float4 ph = S.home[i];
#pragma unroll
                for (int u = 0; u < kWcPerLane; ++u) {
                    const float d2 = dist2(ph, pj[u]);
                    bool acc = d2 < h2_lo;
                    if (!acc && d2 <= h2_hi)
                        acc = within_exact(ph.x, ph.y, ph.z, pj[u].x, pj[u].y, pj[u].z, h_d);
                    const unsigned m = __ballot_sync(full, acc);
                    const int ru = r + __popc(m & lt);
                    if (acc && ru < cap) S.e[i][ru] = make_int2(sj[u], __float_as_int(d2));
                    r += __popc(m);
                }
                if (lane == i) cnt = r;
            }
        }
    }
}

// slot s's velocity from the FP64 rows (VelRows)
__device__ __forceinline__ float4 vel_row(const VelRows& vr, int s,
                                          const int32_t* __restrict__ pbegin, int n_scenes) {
    const double* r =
        vr.vel64 + 3 * (size_t)(__ldg(pbegin + scene_of(s, pbegin, n_scenes)) + __ldg(vr.pid + s));
    return make_float4((float)__ldg(r), (float)__ldg(r + 1), (float)__ldg(r + 2), 0.0f);
}

// kLayout: 0 every scene's voxel table row-major, 1 every one tiled, 2 per scene.
// kGather: the task's velocities too, from FP64 rows (vrows).
template <int kLayout, bool kGather>
__global__ void __launch_bounds__(kWcWarps * 32, 4)
k_density_wc(const SceneDev* __restrict__ scenes, const int32_t* __restrict__ pbegin,
             int n_scenes, int n, const float4* __restrict__ pos,
             const float4* __restrict__ vel, const int32_t* __restrict__ vstart,
             const int32_t* __restrict__ vcount, float* __restrict__ rho,
             float4* __restrict__ fin, NbrList nbr,
             const int2* __restrict__ tasks, const int32_t* __restrict__ task_count,
             int32_t* __restrict__ task_next, const int32_t* __restrict__ task_offset,
             VelRows vrows) {
    __shared__ WcShared sh[kWcWarps];
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    WcShared& S = sh[threadIdx.x >> 5];
    const unsigned lt = (1u << lane) - 1u;
    const int n_tasks = *task_count;
    if (task_offset) tasks += *task_offset;   // one bucket of a bucketed task list
    // Each warp takes its next task from a counter when it is done with the
    // last one: the cost of a task varies with its voxel's neighbourhood, and
    // a fixed share per warp left warps idle at the end of the pass (15 % of
    // its time on the 4M box).
    auto next_task = [&]() {
        int t = 0;
        if (lane == 0) t = atomicAdd(task_next, 1);
        return __shfl_sync(full, t, 0);
    };
    for (int t = next_task(); t < n_tasks; t = next_task()) {
        const int2 task = tasks[t];
        const int vid = task.x, d0 = task.y;
        const SceneDev& sc = scenes[scene_of(d0, pbegin, n_scenes)];
        const int vst = __ldg(vstart + vid), vc = __ldg(vcount + vid);
        const int c_t = min(kTaskRun, vst + vc - d0);
        const int s = d0 + lane;
        const bool home = lane < c_t;
        const float4 pi = home ? __ldg(pos + s) : make_float4(0.f, 0.f, 0.f, 0.f);
        const int local = vid - sc.v_begin;
        const int cap = sc.cap;
        if (local == sc.v_count || cap > kListCap) {
            // overflow bucket (non-finite positions) or a cap beyond the shared
            // list: thread-private walk per particle
            if (home) {   // S.e[lane] serves as its row buffer
                density_one<kLayout>(s, pi, sc, pos, vel, vstart, vcount, n, rho, fin, nbr,
                                     &S.e[lane][0].x, 1);
                if (kGather) {
                    const float4 v = vel_row(vrows, s, pbegin, n_scenes);
                    vrows.vel_out[s] = v;
                    fin[2 * s + 1] = make_float4(v.x, v.y, v.z, 1.0f / rho[s]);
                }
            }
            __syncwarp();
            continue;
        }
        if (home) S.home[lane] = pi;
        // the 27 walk voxels (voxel_kernels.py:46-61 order), from the table coords
        const int tiled = kLayout == 2 ? sc.tiled : kLayout;
        // index -> coordinates with the scene's multiply-shift reciprocals
        const Udiv q0{sc.div_m[0], sc.div_s[0]}, q1{sc.div_m[1], sc.div_s[1]};
        int vx, vy, vz;
        if (tiled) {
            const int tl = local >> 6, in = local & 63;
            const int r0 = q0.div(tl), r1 = q1.div(r0);
            vx = ((tl - r0 * sc.nt0) << 2) | (in & 3);
            vy = ((r0 - r1 * sc.nt1) << 2) | ((in >> 2) & 3);
            vz = (r1 << 2) | (in >> 4);
        } else {
            const int r0 = q0.div(local), r1 = q1.div(r0);
            vx = local - r0 * sc.dims[0];
            vy = r0 - r1 * sc.dims[1];
            vz = r1;
        }
        int ck = 0, stk = 0;
        if (lane < 27) {
            const int w0 = sc.wdims[0], w1 = sc.wdims[1], w2 = sc.wdims[2];
            const int nx = vx + lane / 9 - 1, ny = vy + (lane / 3) % 3 - 1, nz = vz + lane % 3 - 1;
            if (nx >= 0 && nx < w0 && ny >= 0 && ny < w1 && nz >= 0 && nz < w2) {
                const int id = sc.v_begin + voxel_index(nx, ny, nz, tiled, w0, w1, sc.nt0, sc.nt1);
                ck = __ldg(vcount + id);
                stk = __ldg(vstart + id);
            }
        }
        int incl = ck;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(full, incl, o);
            if (lane >= o) incl += v;
        }
        const int M = __shfl_sync(full, incl, 26);   // candidates in the whole walk
        // Candidate q (walk order) lies in the non-empty walk voxel with the
        // largest first index P_k <= q; its slot is q + (start_k - P_k).  Lane
        // k keeps P_k; S.off holds start_k - P_k by rank among the non-empty
        // walk voxels.
        const int Pk = incl - ck;
        const bool nzk = lane < 27 && ck > 0;
        const unsigned NZ = __ballot_sync(full, nzk);
        if (nzk) S.off[__popc(NZ & lt)] = stk - Pk;
        __syncwarp();
        const float h2_lo = sc.h2_lo, h2_hi = sc.h2_hi;
        const double h_d = sc.h_d;
        // Dense neighbourhoods: each home particle's 27-bit mask of the walk
        // voxels within h of it (box distance, the walk's culling test), so
        // that a batch lying in voxels it cannot reach is skipped for it.
        // Those voxels hold no accepted candidate: the result is unchanged.
        const bool cull = !sc.walk_trunc && M > kWcCullMin;
        int cnt = 0;    // lane i: accepted candidates of home particle i so far
        if (cull)
            wc_candidates<true>(S, cnt, home, cap, M, Pk, ck, nzk, reach_mask(pi, vx, vy, vz, sc),
                                pos, h2_lo, h2_hi, h_d);
        else
            wc_candidates<false>(S, cnt, home, cap, M, Pk, ck, nzk, 0u, pos, h2_lo, h2_hi, h_d);
        __syncwarp();
        // (a) one lane per list entry: the density term of every accepted pair,
        // from the squared distance its test used, replaces the distance (self
        // gets kSelfTerm), and each particle's list row (neighbours other than
        // itself, walk order) is written coalesced.  Two particles at a time.
        const float inv_h2 = 1.0f / sc.h2;
        for (int i0 = 0; i0 < c_t; i0 += 2) {
            int2 en[2];
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int i = i0 + e;   // i0 even and < c_t <= kTaskRun: i < kTaskRun
                const int na_i = i < c_t ? min(__shfl_sync(full, cnt, i), cap) : 0;
                en[e] = lane < na_i ? S.e[i][lane] : make_int2(-1, 0);
            }
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int i = i0 + e;
                if (i >= c_t) break;
                const int si = d0 + i;
                const int j = en[e].x;
                const bool in = j >= 0;
                const unsigned self = __ballot_sync(full, in && j == si);
                if (in) {
                    int term = kSelfTerm;
                    if (j != si) {
                        const float u = __fmaf_rn(-__int_as_float(en[e].y), inv_h2, 1.0f);
                        term = __float_as_int(u * u * u);
                        if (nbr.idx)
                            nbr.idx[(size_t)si * kListCap + lane - __popc(self & lt)] = j;
                    }
                    S.e[i][lane].y = term;
                }
            }
        }
        __syncwarp();
        // (b) two lanes per particle: lane i sums the entries of home i below
        // kSumSplit, lane 16 + i the rest, each compensated in walk order,
        // then lane i merges them: the arithmetic of density_one
        {
            const int ih = lane & 15;
            const bool upper = lane >= 16;
            const int na = min(__shfl_sync(full, cnt, ih), cap);
            Kahan acc;
            int others = 0;
            if (ih < c_t) {
                const int k1 = upper ? na : min(na, kSumSplit);
                for (int k = upper ? kSumSplit : 0; k < k1; ++k) {
                    const int term = S.e[ih][k].y;
                    if (term == kSelfTerm) continue;
                    acc.add(__int_as_float(term));
                    ++others;
                }
            }
            Kahan rest;
            rest.s = __shfl_down_sync(full, acc.s, 16);
            rest.c = __shfl_down_sync(full, acc.c, 16);
            others += __shfl_down_sync(full, others, 16);
            acc.merge(rest);
            if (home) {
                const float r = (acc.s * sc.w_const) * sc.mass;
                rho[s] = r;
                if (kGather) {
                    const float4 v = vel_row(vrows, s, pbegin, n_scenes);
                    vrows.vel_out[s] = v;
                    stg256(fin + 2 * s, force_record_a(pi, sc, r),
                           make_float4(v.x, v.y, v.z, 1.0f / r));
                } else if (fin) {
                    write_force_inputs(s, pi, sc, vel, r, fin);
                }
                if (nbr.count) nbr.count[s] = others;
            }
        }
        __syncwarp();
    }
}

// Velocities of a state loaded in original particle order (scene offset + id)
// into sorted slot order, with the second half of the force inputs: used when
// the velocities arrive after the rank-gather (the host-buffer entry point
// uploads them while the sort and the density pass run).
__global__ void __launch_bounds__(kBlock)
k_gather_vel(const int32_t* __restrict__ pbegin, int n_scenes, int n,
             const int32_t* __restrict__ pid, const float4* __restrict__ vel_in,
             const float* __restrict__ rho, float4* __restrict__ vel_out,
             float4* __restrict__ fin) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= n) return;
    const float4 v = __ldg(vel_in + __ldg(pbegin + scene_of(d, pbegin, n_scenes)) + __ldg(pid + d));
    vel_out[d] = v;
    fin[2 * d + 1] = make_float4(v.x, v.y, v.z, 1.0f / __ldg(rho + d));
}

// The same for the slots of a bucket of density tasks (pipelined host
// entry): one thread per slot of the bucket's tasks (a task's run of at most
// kTaskRun slots of one voxel), kTaskRun threads per task.  The velocities
// come straight from the uploaded FP64 rows (original order), converted as
// k_load_aos converts them: the float4 state buffer is the force pass's
// output, which earlier force buckets are already writing (in slot order)
// while later buckets gather.
__global__ void __launch_bounds__(kBlock)
k_gather_vel_tasks(const int32_t* __restrict__ pbegin, int n_scenes, const int32_t* __restrict__ pid,
                   const int32_t* __restrict__ vstart, const int32_t* __restrict__ vcount,
                   const int2* __restrict__ tasks, const int32_t* __restrict__ task_count,
                   const int32_t* __restrict__ task_offset, const double* __restrict__ vel64,
                   const float* __restrict__ rho, float4* __restrict__ vel_out,
                   float4* __restrict__ fin) {
    const int64_t n_threads = (int64_t)*task_count * kTaskRun;
    const int2* tk = tasks + *task_offset;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n_threads;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int2 task = tk[q / kTaskRun];
        const int d = task.y + (int)(q % kTaskRun);
        if (d >= __ldg(vstart + task.x) + __ldg(vcount + task.x)) continue;
        const double* r =
            vel64 + 3 * (size_t)(__ldg(pbegin + scene_of(d, pbegin, n_scenes)) + __ldg(pid + d));
        const float4 v = make_float4((float)__ldg(r), (float)__ldg(r + 1), (float)__ldg(r + 2), 0.0f);
        vel_out[d] = v;
        fin[2 * d + 1] = make_float4(v.x, v.y, v.z, 1.0f / __ldg(rho + d));
    }
}

__global__ void __launch_bounds__(kBlock)
k_force_inputs(const SceneDev* __restrict__ scenes, const int32_t* __restrict__ pbegin,
               int n_scenes, int n, const float4* __restrict__ pos,
               const float4* __restrict__ vel, const float* __restrict__ rho,
               float4* __restrict__ fin) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const SceneDev& sc = scenes[scene_of(s, pbegin, n_scenes)];
    write_force_inputs(s, __ldg(pos + s), sc, vel, rho[s], fin);
}

// Pressure and viscosity sums.  Compensated (Kahan) by default; kPlain sums
// plainly, the reference's order, which is used when a factor is non-finite:
// Kahan's compensation turns an infinite partial sum into NaN (inf - inf),
// while the reference's plain sum stays infinite.
template <bool kPlain>
struct Acc {
    float s = 0.0f, c = 0.0f;
    __device__ __forceinline__ void add(float x) {
        if (kPlain) {
            s = __fadd_rn(s, x);
        } else {
            const float y = __fsub_rn(x, c);
            const float t = __fadd_rn(s, y);
            c = __fsub_rn(__fsub_rn(t, s), y);
            s = t;
        }
    }
};

// Two of those sums in one register pair, with sm_100's packed FP32 adds:
// each element is rounded exactly as the scalar add rounds it, so the x and
// y components give the scalar Acc's bits with half the add instructions.
template <bool kPlain>
struct Acc2 {
    float2 s = make_float2(0.0f, 0.0f), c = make_float2(0.0f, 0.0f);
    __device__ __forceinline__ void add(float2 x) {
        if (kPlain) {
            s = __fadd2_rn(s, x);
        } else {
            const float2 y = __fadd2_rn(x, make_float2(-c.x, -c.y));
            const float2 t = __fadd2_rn(s, y);
            c = __fadd2_rn(__fadd2_rn(t, make_float2(-s.x, -s.y)), make_float2(-y.x, -y.y));
            s = t;
        }
    }
};

template <bool kPlain>
struct ForceSums {
    Acc2<kPlain> pxy, vxy;     // x and y components, packed
    Acc<kPlain> pz, vz;
    int terms = 0;      // neighbours other than self
    bool bad = false;   // a neighbour factor was non-finite
};

// pressure_kernel (voxel_kernels.py:136-171) and viscosity_kernel (:175-211)
// for one particle, same neighbour set as the density pass.
//   P_i = sum_j (p_i/rho_i^2 + p_j/rho_j^2) grad W_ij,
//         grad W = GRAD_W_CONST (h - r)^2 (x_i - x_j) / r   (base_kernels.py:12-21)
//   V_i = min(1, sum_j MASS VISC (v_j - v_i) / rho_j lap W_ij / rho_i),
//         lap W = LAP_W_CONST (h - r)                        (base_kernels.py:24-27)
// with (h - r) written as h (1 - r/h).
template <bool kPlain>
__device__ __forceinline__ void add_pair(ForceSums<kPlain>& f, const float4& vi, float a_i,
                                         float inv_h, float gw, float lw, const float2& aj,
                                         const float4& vj, float2 dxy, float dz, float d2) {
    ++f.terms;
    if (!kPlain) f.bad |= !(fabsf(aj.x * aj.y) < INFINITY);
    const float r = sqrtf(d2);
    const float inv_r = 1.0f / r;
    const float t = __fmaf_rn(-r, inv_h, 1.0f);
    const float g = ((a_i + aj.x) * gw) * (t * t) * inv_r;
    f.pxy.add(__fmul2_rn(make_float2(g, g), dxy));
    f.pz.add(g * dz);
    const float l = (lw * t) * aj.y;
    const float2 dv = __fadd2_rn(make_float2(vj.x, vj.y), make_float2(-vi.x, -vi.y));
    f.vxy.add(__fmul2_rn(make_float2(l, l), dv));
    f.vz.add(l * (vj.z - vi.z));
}

template <bool kPlain>
__device__ __forceinline__ void force_sums(int s, const float4& pi, const float4& vi,
                                           float a_i, const SceneDev& sc, const WalkGeom& geom,
                                           const float4* __restrict__ pos,
                                           const float4* __restrict__ fin,
                                           const int32_t* __restrict__ vstart,
                                           const int32_t* __restrict__ vcount,
                                           ForceSums<kPlain>& f) {
    const float inv_h = 1.0f / sc.h;
    const float gw = sc.grad_w_const, lw = sc.lap_w_const;
    walk(pi, geom, vstart, vcount, pos, geom.cap, [&](int j, float dx, float dy, float dz, float d2) {
        if (j == s) return;
        float4 a, b;
        ldg256(fin + 2 * j, a, b);
        add_pair(f, vi, a_i, inv_h, gw, lw, make_float2(a.w, b.w), b, make_float2(dx, dy), dz, d2);
    });
}

// the same sums over the neighbour list recorded by the density pass (same
// neighbours, same order, same pair distances as the walk)
template <bool kPlain>
__device__ __forceinline__ void force_sums_list(const float4& pi, const float4& vi, float a_i,
                                                const SceneDev& sc,
                                                const float4* __restrict__ fin,
                                                const int32_t* __restrict__ list, int n, int cnt,
                                                ForceSums<kPlain>& f) {
    const float inv_h = 1.0f / sc.h;
    const float gw = sc.grad_w_const, lw = sc.lap_w_const;
    // Eight list entries per load, one 32-byte load per neighbour record:
    // this pass is a gather bound by L1 passes per line touched, and by load
    // latency.  Records are loaded two at a time ahead of their arithmetic (the
    // second, past the end of the list, reloads the first).
    for (int k0 = 0; k0 < cnt; k0 += 8) {
        int js[8];
        ldg256(list + k0, js);
#pragma unroll
        for (int u0 = 0; u0 < 8; u0 += 2) {
            if (k0 + u0 >= cnt) break;
            float4 pq[2], vq[2];                // position, p/rho^2; velocity, 1/rho
            ldg256(fin + 2 * js[u0], pq[0], vq[0]);
            ldg256(fin + 2 * (k0 + u0 + 1 < cnt ? js[u0 + 1] : js[u0]), pq[1], vq[1]);
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                if (k0 + u0 + e >= cnt) break;
                const float4& pj = pq[e];
                const float4& vj = vq[e];
                const float2 dxy = __fadd2_rn(make_float2(pi.x, pi.y), make_float2(-pj.x, -pj.y));
                const float dz = __fsub_rn(pi.z, pj.z);
                float d2 = __fmul_rn(dxy.x, dxy.x);
                d2 = __fmaf_rn(dxy.y, dxy.y, d2);
                d2 = __fmaf_rn(dz, dz, d2);
                add_pair(f, vi, a_i, inv_h, gw, lw, make_float2(pj.w, vj.w), vj, dxy, dz, d2);
            }
        }
    }
}

struct Forces {
    float p[3], v[3];   // pressure term, viscosity sum (before the 1/rho_i scale)
    int terms;
};

// Kahan sums, redone plainly when a factor of particle i or of a neighbour
// is non-finite (a particle of density 0).  With a neighbour list (cnt >= 0)
// the neighbours come from it, else from a fresh walk.
__device__ __forceinline__ Forces forces_of(int s, const float4& pi, const float4& vi,
                                            const float2& ai, const SceneDev& sc,
                                            const float4* __restrict__ pos,
                                            const float4* __restrict__ fin,
                                            const int32_t* __restrict__ vstart,
                                            const int32_t* __restrict__ vcount,
                                            const int32_t* __restrict__ list, int n, int cnt) {
    Forces out;
    bool plain = !(fabsf(ai.x * ai.y) < INFINITY);
    if (!plain) {
        ForceSums<false> f;
        if (cnt >= 0) force_sums_list<false>(pi, vi, ai.x, sc, fin, list, n, cnt, f);
        else force_sums<false>(s, pi, vi, ai.x, sc, load_geom(sc), pos, fin, vstart, vcount, f);
        out = Forces{{f.pxy.s.x, f.pxy.s.y, f.pz.s}, {f.vxy.s.x, f.vxy.s.y, f.vz.s}, f.terms};
        plain = f.bad;
    }
    if (plain) {
        ForceSums<true> f;
        if (cnt >= 0) force_sums_list<true>(pi, vi, ai.x, sc, fin, list, n, cnt, f);
        else force_sums<true>(s, pi, vi, ai.x, sc, load_geom(sc), pos, fin, vstart, vcount, f);
        out = Forces{{f.pxy.s.x, f.pxy.s.y, f.pz.s}, {f.vxy.s.x, f.vxy.s.y, f.vz.s}, f.terms};
    }
    return out;
}

__device__ __forceinline__ float clamp1(float x) { return x < 1.0f ? x : 1.0f; }  // min(1, x)

// viscosity term of one component: the reference multiplies every neighbour
// term by MASS * VISC / rho_i (voxel_kernels.py:207-208), so with no
// neighbour terms the sum is 0 even when rho_i is 0
__device__ __forceinline__ float visc_term(const Forces& f, int a, float vscale) {
    return clamp1(f.terms ? f.v[a] * vscale : 0.0f);
}

__global__ void __launch_bounds__(kBlock)
k_forces(const SceneDev* __restrict__ scenes, const int32_t* __restrict__ pbegin, int n_scenes,
         int n, const float4* __restrict__ pos, const float4* __restrict__ vel,
         const float4* __restrict__ fin, const int32_t* __restrict__ vstart,
         const int32_t* __restrict__ vcount, float4* __restrict__ pressure,
         float4* __restrict__ viscosity) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const SceneDev& sc = scenes[scene_of(s, pbegin, n_scenes)];
    const float4 pi = __ldg(pos + s);
    const float4 vi = __ldg(vel + s);
    float4 fa, fb;
    ldg256(fin + 2 * s, fa, fb);
    const float2 ai = make_float2(fa.w, fb.w);
    const Forces f = forces_of(s, pi, vi, ai, sc, pos, fin, vstart, vcount, nullptr, n, -1);
    const float vscale = sc.mass * sc.visc * ai.y;
    pressure[s] = make_float4(f.p[0], f.p[1], f.p[2], 0.0f);
    viscosity[s] = make_float4(visc_term(f, 0, vscale), visc_term(f, 1, vscale),
                               visc_term(f, 2, vscale), 0.0f);
}

// Modes of the force pass.  kForceAll: every particle, every path.  The
// list path alone (the neighbour list, finite factors, Kahan sums) needs far
// fewer registers than the walk fallback and the plain re-sum, whose spills
// slowed it; so a pass with a neighbour list runs as kForceLean, which
// appends each particle needing a rare path to a RareList and writes nothing
// for it, followed by kForceRare, a small grid-stride launch over those
// particles with every path.  The per-particle arithmetic is the same in all
// three: the results are identical.
constexpr int kForceAll = 0, kForceLean = 1, kForceRare = 2;
// kForceRare grid: one block per SM (device_sm_count())

// Which particles a force launch runs: every slot (kBySlot); the particles of
// rows range.i0..i1 in original order, which also write the FP64 rows of the
// next position and velocity (kByRow); or the slots range.slots[0..n_slots)
// (kByList), which also write the FP64 rows of the next position, velocity
// and density, each at its particle's id.
constexpr int kBySlot = 0, kByRow = 1, kByList = 2;

// forces + integrating_kernel (base_kernels.py:30-53) + wall response
// (collision_kernel_box :75-98 or collision_kernel :56-72).  Writes the next
// state into the *_out buffers at the same slot.  kPipe = false is the
// instantiation for contexts without pipe scenes (no FP64 code).  kIdx: see
// kBySlot; the per-particle arithmetic is the same in all three.  kMode: see
// kForceAll.
template <bool kPipe, int kIdx, int kMode>
__global__ void __launch_bounds__(kBlock, 4)
k_integrate(const SceneDev* __restrict__ scenes, const int32_t* __restrict__ pbegin, int n_scenes,
            int n, const double* __restrict__ pipe, const float4* __restrict__ pos,
            const float4* __restrict__ vel, const float* __restrict__ rho,
            const float4* __restrict__ fin, const int32_t* __restrict__ pid,
            const double* __restrict__ pos64, const int32_t* __restrict__ vstart,
            const int32_t* __restrict__ vcount, const int32_t* __restrict__ scene_step,
            NbrList nbr, float4* __restrict__ pos_out, float4* __restrict__ vel_out,
            int32_t* __restrict__ pid_out, double* __restrict__ pos64_out,
            float4* __restrict__ force_out, PidRange range, RareList rare,
            const int32_t* __restrict__ step_limit) {
    // kForceRare and kByList: a grid-stride loop over the deferred particles
    // or the listed slots; otherwise one particle per thread (the body runs once)
    const int m_rare = kMode == kForceRare ? *rare.count : 0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x;; k += gridDim.x * blockDim.x) {
        // deferred particles are listed by row (kByRow) or by slot; rows_out:
        // the FP64 rows are written too
        constexpr bool by_row = kIdx == kByRow;
        constexpr bool rows_out = kIdx != kBySlot;
        int s, row = 0;
        if (kMode == kForceRare) {
            if (k >= m_rare) return;
            row = rare.idx[rare.base + k];
            s = by_row ? __ldg(range.slot_of + row) : row;
        } else if (kIdx == kByList) {
            if (k >= range.n_slots) return;
            s = __ldg(range.slots + k);
        } else if (by_row) {
            row = range.i0 + k;
            if (row >= range.i1) return;
            s = __ldg(range.slot_of + row);
        } else {
            s = k;
            if (s >= n) return;
        }
        const int si = scene_of(s, pbegin, n_scenes);
        if (kIdx == kByList) row = __ldg(pbegin + si) + __ldg(pid + s);
        const SceneDev& sc = scenes[si];
        if (kMode != kForceRare && scene_frozen(step_limit, scene_step, si)) {
            // frozen scene: the state is copied through unchanged (the sort
            // kept its slots; its force records were not written this step)
            const float4 p4 = __ldg(pos + s), v4 = __ldg(vel + s);
            pos_out[s] = p4;
            vel_out[s] = v4;
            pid_out[s] = __ldg(pid + s);
            double x64[3] = {p4.x, p4.y, p4.z};
            if (kPipe && pos64_out) {
                for (int a = 0; a < 3; ++a) {
                    pos64_out[3 * s + a] = pos64[3 * s + a];
                    if (sc.mode == 1) x64[a] = pos64[3 * s + a];
                }
            }
            if (rows_out) {
                for (int a = 0; a < 3; ++a) range.pos[3 * (size_t)row + a] = x64[a];
                range.vel[3 * (size_t)row + 0] = v4.x;
                range.vel[3 * (size_t)row + 1] = v4.y;
                range.vel[3 * (size_t)row + 2] = v4.z;
                if (kIdx == kByList) range.rho[row] = (double)__ldg(rho + s);
            }
            if (force_out) force_out[s] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (kMode == kForceRare || kIdx == kByList) continue;
            return;   // one particle per thread outside kForceRare and kByList
        }
        // the particle's own force record holds its position and velocity too
        // (written from this state by the density pass, k_gather_vel or
        // k_force_inputs), so one 32-byte load serves for both
        float4 fa, fb;
        ldg256(fin + 2 * s, fa, fb);
        const float4 pi = make_float4(fa.x, fa.y, fa.z, 0.0f);
        const float4 vi = make_float4(fb.x, fb.y, fb.z, 0.0f);
        const float2 ai = make_float2(fa.w, fb.w);
        const float rho_i = __ldg(rho + s);
        const int cnt = nbr.count ? __ldg(nbr.count + s) : -1;
        const int32_t* list = nbr.idx ? nbr.idx + (size_t)s * kListCap : nullptr;
        Forces f;
        if (kMode == kForceLean) {
            ForceSums<false> fs;
            bool ok = cnt >= 0 && fabsf(ai.x * ai.y) < INFINITY;
            if (ok) {
                force_sums_list<false>(pi, vi, ai.x, sc, fin, list, n, cnt, fs);
                ok = !fs.bad;
            }
            if (!ok) {
                rare.idx[rare.base + atomicAdd(rare.count, 1)] = by_row ? row : s;
                if (kIdx == kByList) continue;
                return;
            }
            f = Forces{{fs.pxy.s.x, fs.pxy.s.y, fs.pz.s}, {fs.vxy.s.x, fs.vxy.s.y, fs.vz.s}, fs.terms};
        } else {
            f = forces_of(s, pi, vi, ai, sc, pos, fin, vstart, vcount, list, n, cnt);
        }
        const float vscale = sc.mass * sc.visc * ai.y;
        // result_force = ext + -P + V (base_kernels.py:46-52)
        float F[3];
    #pragma unroll
        for (int a = 0; a < 3; ++a) F[a] = (sc.ext[a] + -f.p[a]) + visc_term(f, a, vscale);
        float v[3] = {vi.x, vi.y, vi.z};
    #pragma unroll
        for (int a = 0; a < 3; ++a) v[a] = v[a] + (F[a] / rho_i) * sc.dt;
        const int p_id = __ldg(pid + s);
        if (!kPipe || sc.mode == 0) {
            float x[3] = {pi.x, pi.y, pi.z};
    #pragma unroll
            for (int a = 0; a < 3; ++a) {
                x[a] = x[a] + v[a] * sc.dt;
                bool bounced = false;
                if (x[a] < 0.0f) { x[a] = sc.wall_lo; bounced = true; }
                if (x[a] > sc.space[a]) { x[a] = sc.wall_hi[a]; bounced = true; }
                if (bounced) v[a] = -v[a] * sc.damp;
            }
            pos_out[s] = make_float4(x[0], x[1], x[2], 0.0f);
            if (kPipe && pos64_out) {
                pos64_out[3 * s + 0] = x[0];
                pos64_out[3 * s + 1] = x[1];
                pos64_out[3 * s + 2] = x[2];
            }
            if (rows_out) {
                range.pos[3 * (size_t)row + 0] = x[0];
                range.pos[3 * (size_t)row + 1] = x[1];
                range.pos[3 * (size_t)row + 2] = x[2];
            }
        } else if (kPipe) {
            // pipe flow: FP64 position accumulator and FP64 wall response
            double x[3], vd[3];
    #pragma unroll
            for (int a = 0; a < 3; ++a) {
                vd[a] = (double)v[a];
                x[a] = __dadd_rn(pos64[3 * s + a], __dmul_rn(vd[a], sc.dt_d));
            }
            PipeView P{pipe + 5 * sc.pipe_off, sc.pipe_rows};
            pipe_collide(x, vd, P, sc.seed, (uint32_t)p_id, (uint32_t)__ldg(scene_step + si));
    #pragma unroll
            for (int a = 0; a < 3; ++a) {
                v[a] = (float)vd[a];
                pos64_out[3 * s + a] = x[a];
                if (rows_out) range.pos[3 * (size_t)row + a] = x[a];
            }
            pos_out[s] = make_float4((float)x[0], (float)x[1], (float)x[2], 0.0f);
        }
        vel_out[s] = make_float4(v[0], v[1], v[2], 0.0f);
        if (rows_out) {
            range.vel[3 * (size_t)row + 0] = v[0];
            range.vel[3 * (size_t)row + 1] = v[1];
            range.vel[3 * (size_t)row + 2] = v[2];
            if (kIdx == kByList) range.rho[row] = (double)rho_i;
        }
        pid_out[s] = p_id;
        if (force_out) force_out[s] = make_float4(F[0], F[1], F[2], 0.0f);
        if (kMode != kForceRare && kIdx != kByList) return;
    }
}

__global__ void __launch_bounds__(kBlock)
k_neighbours(const SceneDev* __restrict__ scenes, const int32_t* __restrict__ pbegin,
             int n_scenes, int n, const float4* __restrict__ pos,
             const int32_t* __restrict__ vstart, const int32_t* __restrict__ vcount,
             int32_t* __restrict__ list, int stride, int32_t* __restrict__ n_capped,
             int32_t* __restrict__ n_uncapped) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const WalkGeom g = load_geom(scenes[scene_of(s, pbegin, n_scenes)]);
    const float4 pi = __ldg(pos + s);
    int k = 0;
    int32_t* li = list ? list + (size_t)s * stride : nullptr;
    const int c = walk(pi, g, vstart, vcount, pos, g.cap, [&](int j, float, float, float, float) {
        if (li && k < stride) li[k] = j;
        ++k;
    });
    if (li) for (int t = c; t < stride; ++t) li[t] = -1;
    if (n_capped) n_capped[s] = c;
    if (n_uncapped)
        n_uncapped[s] = walk(pi, g, vstart, vcount, pos, 0x7fffffff,
                             [&](int, float, float, float, float) {});
}

}  // namespace

cudaError_t launch_density(const Launch& L, const float4* pos, const float4* vel,
                           const int32_t* vstart, const int32_t* vcount, float* rho,
                           float4* fin, NbrList nbr) {
    if (L.n == 0) return cudaSuccess;
    auto kernel = L.layout == 1 ? k_density<1> : L.layout == 2 ? k_density<2> : k_density<0>;
    kernel<<<blocks_for(L.n), kBlock, 0, L.stream>>>(L.scenes, L.pbegin, L.n_scenes, L.n, pos, vel,
                                                     vstart, vcount, rho, fin, nbr, L.step_limit,
                                                     L.scene_step);
    return cudaGetLastError();
}

cudaError_t launch_density_wc(const Launch& L, const float4* pos, const float4* vel,
                              const int32_t* vstart, const int32_t* vcount, float* rho,
                              float4* fin, NbrList nbr, const int2* tasks,
                              const int32_t* task_count, int32_t* task_next,
                              const int32_t* task_offset, VelRows vrows) {
    if (L.n == 0) return cudaSuccess;
    // persistent grid: up to 4 blocks of 8 warps per SM, warps take tasks in turn
    int blocks = (L.n + 32 * kWcWarps - 1) / (32 * kWcWarps);
    const int top = device_sm_count() * 4;
    if (blocks > top) blocks = top;
    // the velocity gather is its own instantiation: the step's kernel stays as it is
    auto kernel = vrows.vel64
                      ? (L.layout == 1   ? k_density_wc<1, true>
                         : L.layout == 2 ? k_density_wc<2, true>
                                         : k_density_wc<0, true>)
                      : (L.layout == 1   ? k_density_wc<1, false>
                         : L.layout == 2 ? k_density_wc<2, false>
                                         : k_density_wc<0, false>);
    kernel<<<blocks, kWcWarps * 32, 0, L.stream>>>(L.scenes, L.pbegin, L.n_scenes, L.n, pos, vel,
                                                   vstart, vcount, rho, fin, nbr, tasks, task_count,
                                                   task_next, task_offset, vrows);
    return cudaGetLastError();
}

cudaError_t launch_gather_vel(const Launch& L, const int32_t* pid, const float4* vel_in,
                              const float* rho, float4* vel_out, float4* fin) {
    if (L.n == 0) return cudaSuccess;
    k_gather_vel<<<blocks_for(L.n), kBlock, 0, L.stream>>>(L.pbegin, L.n_scenes, L.n, pid, vel_in,
                                                            rho, vel_out, fin);
    return cudaGetLastError();
}

cudaError_t launch_gather_vel_tasks(const Launch& L, const int32_t* pid, const int2* tasks,
                                    const int32_t* task_count, const int32_t* task_offset,
                                    const int32_t* vstart, const int32_t* vcount,
                                    const double* vel64, const float* rho, float4* vel_out,
                                    float4* fin) {
    if (L.n == 0) return cudaSuccess;
    k_gather_vel_tasks<<<device_sm_count() * 4, kBlock, 0, L.stream>>>(
        L.pbegin, L.n_scenes, pid, vstart, vcount, tasks, task_count, task_offset, vel64, rho,
        vel_out, fin);
    return cudaGetLastError();
}

cudaError_t launch_force_inputs(const Launch& L, const float4* pos, const float4* vel,
                                const float* rho, float4* fin) {
    if (L.n == 0) return cudaSuccess;
    k_force_inputs<<<blocks_for(L.n), kBlock, 0, L.stream>>>(L.scenes, L.pbegin, L.n_scenes, L.n,
                                                              pos, vel, rho, fin);
    return cudaGetLastError();
}

cudaError_t launch_forces(const Launch& L, const float4* pos, const float4* vel,
                          const float* rho, const float4* fin, const int32_t* vstart,
                          const int32_t* vcount, float4* pressure, float4* viscosity) {
    (void)rho;
    if (L.n == 0) return cudaSuccess;
    k_forces<<<blocks_for(L.n), kBlock, 0, L.stream>>>(L.scenes, L.pbegin, L.n_scenes, L.n, pos,
                                                        vel, fin, vstart, vcount, pressure,
                                                        viscosity);
    return cudaGetLastError();
}

namespace {
// the force pass of one launch shape: with a neighbour list and a RareList
// (contexts without pipe scenes), the lean pass then the deferred particles;
// otherwise every particle in one pass
template <int kIdx>
cudaError_t launch_force_pass(const Launch& L, int m, const float4* pos, const float4* vel,
                              const float* rho, const float4* fin, const int32_t* pid,
                              const double* pos64, const int32_t* vstart, const int32_t* vcount,
                              const int32_t* scene_step, NbrList nbr, float4* pos_out,
                              float4* vel_out, int32_t* pid_out, double* pos64_out,
                              float4* force_out, PidRange range, RareList rare) {
    // a slot list runs on a grid of at most 4 blocks per SM, each thread
    // taking list entries in turn: a bucket's list is a few waves long, and
    // no partial last wave is left
    const int grid = kIdx == kByList ? std::min(blocks_for(m), device_sm_count() * 4)
                                     : blocks_for(m);
    if (L.pipe_scenes) {
        k_integrate<true, kIdx, kForceAll><<<grid, kBlock, 0, L.stream>>>(
            L.scenes, L.pbegin, L.n_scenes, L.n, L.pipe, pos, vel, rho, fin, pid, pos64, vstart,
            vcount, scene_step, nbr, pos_out, vel_out, pid_out, pos64_out, force_out, range,
            RareList{}, L.step_limit);
    } else if (nbr.count && rare.count) {
        k_integrate<false, kIdx, kForceLean><<<grid, kBlock, 0, L.stream>>>(
            L.scenes, L.pbegin, L.n_scenes, L.n, L.pipe, pos, vel, rho, fin, pid, pos64, vstart,
            vcount, scene_step, nbr, pos_out, vel_out, pid_out, pos64_out, force_out, range, rare,
            L.step_limit);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        k_integrate<false, kIdx, kForceRare><<<device_sm_count(), kBlock, 0, L.stream>>>(
            L.scenes, L.pbegin, L.n_scenes, L.n, L.pipe, pos, vel, rho, fin, pid, pos64, vstart,
            vcount, scene_step, nbr, pos_out, vel_out, pid_out, pos64_out, force_out, range, rare,
            L.step_limit);
    } else {
        k_integrate<false, kIdx, kForceAll><<<grid, kBlock, 0, L.stream>>>(
            L.scenes, L.pbegin, L.n_scenes, L.n, L.pipe, pos, vel, rho, fin, pid, pos64, vstart,
            vcount, scene_step, nbr, pos_out, vel_out, pid_out, pos64_out, force_out, range,
            RareList{}, L.step_limit);
    }
    return cudaGetLastError();
}
}  // namespace

cudaError_t launch_integrate(const Launch& L, const float4* pos, const float4* vel,
                             const float* rho, const float4* fin, const int32_t* pid,
                             const double* pos64, const int32_t* vstart, const int32_t* vcount,
                             const int32_t* scene_step, NbrList nbr, float4* pos_out,
                             float4* vel_out, int32_t* pid_out, double* pos64_out,
                             float4* force_out, RareList rare) {
    if (L.n == 0) return cudaSuccess;
    return launch_force_pass<kBySlot>(L, L.n, pos, vel, rho, fin, pid, pos64, vstart, vcount,
                                    scene_step, nbr, pos_out, vel_out, pid_out, pos64_out,
                                    force_out, PidRange{}, rare);
}

cudaError_t launch_integrate_range(const Launch& L, const float4* pos, const float4* vel,
                                   const float* rho, const float4* fin, const int32_t* pid,
                                   const double* pos64, const int32_t* vstart,
                                   const int32_t* vcount, const int32_t* scene_step, NbrList nbr,
                                   float4* pos_out, float4* vel_out, int32_t* pid_out,
                                   double* pos64_out, PidRange range, RareList rare) {
    const int m = range.slots ? range.n_slots : range.i1 - range.i0;
    if (m <= 0) return cudaSuccess;
    if (m > L.n || !range.pos || !range.vel ||
        (range.slots ? !range.rho : (range.i0 < 0 || range.i1 > L.n || !range.slot_of)))
        return cudaErrorInvalidValue;
    if (range.slots)
        return launch_force_pass<kByList>(L, m, pos, vel, rho, fin, pid, pos64, vstart, vcount,
                                          scene_step, nbr, pos_out, vel_out, pid_out, pos64_out,
                                          nullptr, range, rare);
    return launch_force_pass<kByRow>(L, m, pos, vel, rho, fin, pid, pos64, vstart, vcount,
                                     scene_step, nbr, pos_out, vel_out, pid_out, pos64_out,
                                     nullptr, range, rare);
}

cudaError_t launch_neighbours(const Launch& L, const float4* pos, const int32_t* vstart,
                              const int32_t* vcount, int32_t* list, int stride,
                              int32_t* n_capped, int32_t* n_uncapped) {
    if (L.n == 0) return cudaSuccess;
    k_neighbours<<<blocks_for(L.n), kBlock, 0, L.stream>>>(L.scenes, L.pbegin, L.n_scenes, L.n,
                                                            pos, vstart, vcount, list, stride,
                                                            n_capped, n_uncapped);
    return cudaGetLastError();
}

}  // namespace sphgb
