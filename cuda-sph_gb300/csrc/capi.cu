// capi.cu -- the extern "C" boundary of libsphgb.so (declared in include/sphgb.h).
//
// A context (SphgbCtx) holds the scene descriptors, the pipe table and every
// scratch buffer of the step; the caller owns the particle state and binds it.
// The step enqueues, per time step:
//   memset(voxel_count) -> hash+histogram -> scan -> scatter -> rank-gather
//   -> density -> force+integrate+wall -> step counter
// which is VoxelSPHStrategy.compute_next_state (sim/src/sph/strategies/
// abstract_sph_strategy.py:31-46, voxel_sph_strategy.py:20-116) without any
// host round trip.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "sphgb_internal.cuh"

#include "../../include/sphgb.h"

using namespace sphgb;

int sphgb::device_sm_count() {
    constexpr int kCached = 64;
    static std::atomic<int> cache[kCached] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    if (dev >= 0 && dev < kCached) {
        const int v = cache[dev].load(std::memory_order_relaxed);
        if (v > 0) return v;
    }
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) {
        cudaGetLastError();
        return 1;
    }
    if (dev >= 0 && dev < kCached) cache[dev].store(v, std::memory_order_relaxed);
    return v;
}

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    return fail(SPHGB_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define SPHGB_CUDA(call)                                    \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

constexpr int kConsChunk = 1024;
constexpr int kConsThreads = 256;
constexpr int kConsFields = 8;

struct ConsChunk {
    int32_t scene, begin, end, pad;
};

}  // namespace

// host-buffer entry point: particle-order ranges of the force pass, and its events
// (start, positions in, velocities in, density done, slot map ready, downloads
// queued, then one per range)
constexpr int64_t kMaxParticles = SPHGB_MAX_PARTICLES;
constexpr double kTileMaxOccupancy = 8.0;   // particles per voxel, table mean
constexpr int kHostRanges = 8;
// the pipelined host order: ranges of the force pass and buckets of the
// density pass (host_step_pipelined)
constexpr int kPipeRanges = 16;
constexpr int kHostFirstRangeEvent = 6;
// the host entry uploads the positions in kHostPosChunks parts; each is
// converted and hashed while the next one is in flight
constexpr int kHostPosChunks = 4;
constexpr int kHostFirstChunkEvent = kHostFirstRangeEvent + kHostRanges;
constexpr int kHostOrganizedEvent = kHostFirstChunkEvent + kHostPosChunks;
constexpr int kHostEvents = kHostOrganizedEvent + 1;
// device counters in big_count: big voxels, density tasks, tasks taken, then the
// deferred particles of the whole force pass and of each host-entry range
constexpr int kCounters = 4 + (kHostRanges > kPipeRanges ? kHostRanges : kPipeRanges);

struct SphgbCtx {
    int device = 0;
    int n_scenes = 0;
    int n = 0;
    // Two voxel-table layouts of the same scenes: the fused step's (4x4x4
    // tiles) and the reference's row-major one, which every stage entry point
    // and sphgb_ctx_sizes use.
    int v_total = 0;           // step layout
    int v_total_ref = 0;       // reference layout
    int layout = 0;            // step layout: 0 all row-major, 1 all tiled, 2 mixed
    bool any_pipe = false;
    std::vector<SceneDev> h_scenes;
    std::vector<int32_t> h_pbegin;
    SceneDev* d_scenes = nullptr;       // step layout
    SceneDev* d_scenes_ref = nullptr;   // reference layout
    int32_t* d_pbegin = nullptr;
    double* d_pipe = nullptr;
    int n_pipe_rows = 0;
    // scratch
    int32_t* cell = nullptr;
    int32_t* slot_of = nullptr;        // original index -> sorted slot (AoS export)
    int32_t* slot = nullptr;
    int32_t* tmp_pid = nullptr;
    int32_t* vstart = nullptr;
    int32_t* vcount = nullptr;
    int32_t* tile_sums = nullptr;
    float4* posB = nullptr;
    float4* velB = nullptr;
    int32_t* pidB = nullptr;
    double* pos64B = nullptr;
    float4* fin = nullptr;             // force inputs, 2 per particle (see launch_density)
    NbrList nbr;                     // neighbour list of the step (density -> force pass)
    int32_t* big_list = nullptr;     // voxels with more than kBigVoxel members
    int32_t* big_count = nullptr;     // counters: [0] big voxels, [1] density tasks, [2] tasks taken,
                                      // [3 + r] deferred particles of force pass r (kCounters)
    int32_t* rare = nullptr;          // deferred particles of the force pass (RareList)
    int2* tasks = nullptr;             // (voxel, first slot) per run of <= kTaskRun slots
    // the neighbour rows in nbr, pidB and posB are those of the latest step
    // (cleared by anything else that sorts into the B buffers)
    bool nbr_valid = false;
    // checked mode (sphgb_ctx_set_checks): a validation kernel after every
    // step ORs SPHGB_CHECK_* bits into d_check[0] (see k_check_step)
    bool checks = false;
    uint32_t* d_check = nullptr;
    // bound (caller-owned) state
    float4* posA = nullptr;
    float4* velA = nullptr;
    float* rho = nullptr;
    int32_t* pidA = nullptr;
    double* pos64A = nullptr;
    int32_t* scene_step = nullptr;
    bool bound = false;
    // optional per-scene step limits (caller-owned device array, see
    // sphgb_ctx_set_step_limits); null: no scene is frozen
    const int32_t* step_limit = nullptr;
    // optional separate output of the step (the input state is then left untouched)
    float4* out_pos = nullptr;
    float4* out_vel = nullptr;
    int32_t* out_pid = nullptr;
    double* out_pos64 = nullptr;
    // state owned by the context for the host-buffer entry point when nothing is bound
    void* owned = nullptr;
    // staging for the host-buffer entry point
    double* stage = nullptr;
    // conservation
    int n_chunks = 0;
    ConsChunk* d_chunks = nullptr;
    double* d_partials = nullptr;
    // buffer capacities (elements), so reconfiguration reuses what is big enough
    struct {
        size_t scenes = 0, scenes_ref = 0, pbegin = 0, pipe = 0, cell = 0, slot_of = 0, slot = 0, tmp_pid = 0,
               vstart = 0,
               vcount = 0, tile_sums = 0, posB = 0, velB = 0, pidB = 0, fin = 0, big_list = 0,
               big_count = 0, rare = 0, tasks = 0, nbr_idx = 0, nbr_count = 0, pos64B = 0, chunks = 0,
               partials = 0;
    } cap;
    // tuning (sphgb_ctx_set_tuning)
    int sort_block = 256;
    int density_variant = SPHGB_DENSITY_WARP;
    int big_voxel = kBigVoxel;
    // streams and graphs
    cudaStream_t cap_stream = nullptr;
    cudaStream_t host_stream = nullptr;
    // second stream and events of the host-buffer entry point: the velocity
    // upload and the density download overlap the step's kernels
    cudaStream_t host_stream2 = nullptr;
    cudaEvent_t host_ev[kHostEvents] = {};
    // force-pass order of the host-buffer entry point (sphgb_ctx_set_host_order)
    int host_order = SPHGB_HOST_ORDER_AUTO;
    int host_calls = 0;         // calls since the order was last set
    double host_ms[4] = {};     // timed call per order (index = order)
    // pipelined order (host_step_pipelined), allocated on its first call:
    // density tasks bucketed by the original-index range of their first
    // particle and the slots of each bucket's tasks, the latest bucket each
    // voxel's tasks fall in, the counters, offsets and dependencies (on the
    // device and page-locked), two more streams and their events
    int2* tasks_b = nullptr;
    int32_t* slots_b = nullptr;
    int32_t* vbucket = nullptr;
    int32_t* pipe_i = nullptr;
    int32_t* h_pipe = nullptr;
    size_t cap_tasks_b = 0, cap_vbucket = 0;
    cudaStream_t host_stream3 = nullptr, host_stream4 = nullptr;
    cudaEvent_t pipe_ev[3 + 2 * kPipeRanges] = {};
    std::map<int, cudaGraphExec_t> graphs;

    Launch launch(cudaStream_t st, bool ref_layout = false) const {
        Launch L;
        L.scenes = ref_layout ? d_scenes_ref : d_scenes;
        L.pbegin = d_pbegin;
        L.n_scenes = n_scenes;
        L.n = n;
        L.v_total = ref_layout ? v_total_ref : v_total;
        L.layout = ref_layout ? 0 : layout;
        L.pipe = d_pipe;
        L.pipe_scenes = any_pipe;
        L.sort_block = sort_block;
        L.big_voxel = big_voxel;
        L.stream = st;
        // the stage entry points step no scene counter: limits apply to the
        // context's own step only
        L.step_limit = ref_layout ? nullptr : step_limit;
        L.scene_step = scene_step;
        return L;
    }
};

namespace {

template <class T>
int dalloc(T** p, size_t count) {
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), count * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return fail(SPHGB_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    return SPHGB_OK;
}

void free_ctx(SphgbCtx* c) {
    if (!c) return;
    for (auto& kv : c->graphs) cudaGraphExecDestroy(kv.second);
    void* ptrs[] = {c->d_scenes, c->d_scenes_ref, c->d_pbegin, c->d_pipe, c->cell, c->slot_of, c->slot, c->tmp_pid,
                    c->vstart, c->vcount, c->tile_sums, c->posB, c->velB, c->pidB,
                    c->pos64B, c->fin, c->owned, c->stage, c->d_chunks, c->d_partials,
                    c->big_list, c->big_count, c->rare, c->nbr.idx, c->nbr.count, c->tasks,
                    c->d_check};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (c->cap_stream) cudaStreamDestroy(c->cap_stream);
    if (c->host_stream) cudaStreamDestroy(c->host_stream);
    if (c->host_stream2) cudaStreamDestroy(c->host_stream2);
    if (c->host_stream3) cudaStreamDestroy(c->host_stream3);
    if (c->host_stream4) cudaStreamDestroy(c->host_stream4);
    for (cudaEvent_t e : c->pipe_ev)
        if (e) cudaEventDestroy(e);
    if (c->tasks_b) cudaFree(c->tasks_b);
    if (c->slots_b) cudaFree(c->slots_b);
    if (c->vbucket) cudaFree(c->vbucket);
    if (c->pipe_i) cudaFree(c->pipe_i);
    if (c->h_pipe) cudaFreeHost(c->h_pipe);
    for (cudaEvent_t e : c->host_ev)
        if (e) cudaEventDestroy(e);
    delete c;
}

float round_down_f(double x) {
    float f = (float)x;
    if ((double)f > x) f = std::nextafter(f, -std::numeric_limits<float>::infinity());
    return f;
}

float round_up_f(double x) {
    float f = (float)x;
    if ((double)f < x) f = std::nextafter(f, std::numeric_limits<float>::infinity());
    return f;
}

int build_scene(const SphgbSceneParams& p, int n_pipe_rows_total, SceneDev& d,
                bool tiled = false) {
    std::memset(&d, 0, sizeof(d));
    if (p.particle_count < 0) return fail(SPHGB_ERR_INVALID, "particle_count < 0");
    if (!(p.inf_r > 0.0) || !std::isfinite(p.inf_r)) return fail(SPHGB_ERR_INVALID, "inf_r must be > 0");
    if (!(p.dt > 0.0)) return fail(SPHGB_ERR_INVALID, "dt must be > 0");
    if (p.mode != SPHGB_MODE_BOX && p.mode != SPHGB_MODE_PIPE)
        return fail(SPHGB_ERR_INVALID, "mode must be SPHGB_MODE_BOX or SPHGB_MODE_PIPE");
    if (p.walk_dims != SPHGB_WALK_CEIL && p.walk_dims != SPHGB_WALK_TRUNCATED)
        return fail(SPHGB_ERR_INVALID, "walk_dims must be SPHGB_WALK_CEIL or SPHGB_WALK_TRUNCATED");
    int64_t nv = 1;
    for (int a = 0; a < 3; ++a) {
        const double vs = (double)(float)p.voxel_size[a];
        const double sp = (double)(float)p.space_size[a];
        if (!(vs > 0.0) || !(sp > 0.0) || !std::isfinite(vs) || !std::isfinite(sp))
            return fail(SPHGB_ERR_INVALID, "space_size and voxel_size must be finite and > 0");
        const double q = sp / vs;
        if (q > 1.0e7) return fail(SPHGB_ERR_RANGE, "space_size / voxel_size too large");
        d.dims[a] = (int)std::ceil(q);                         // voxel_sph_strategy.py:70-73
        if (d.dims[a] < 1) d.dims[a] = 1;
        d.wdims[a] = p.walk_dims == SPHGB_WALK_TRUNCATED ? (int)q : d.dims[a];  // :110-116
        d.vs[a] = (float)p.voxel_size[a];
        d.space[a] = (float)p.space_size[a];
        d.ext[a] = (float)p.external_force[a];
        d.wall_hi[a] = (float)(p.space_size[a] - 1e-3);
        nv *= d.dims[a];
        if (nv > (int64_t)0x7fffffff) return fail(SPHGB_ERR_RANGE, "voxel table over 2^31 entries");
    }
    d.walk_trunc = (d.wdims[0] != d.dims[0] || d.wdims[1] != d.dims[1] || d.wdims[2] != d.dims[2]);
    if (tiled && !d.walk_trunc && (double)p.particle_count <= kTileMaxOccupancy * (double)nv) {
        // 4x4x4 tiles (voxel_index) for sparse scenes, where they shorten the
        // gathers of the force pass.  Dense scenes stay row-major: their
        // voxels fill L1 anyway, and the histogram counters of a cluster
        // would share cache lines, serialising the hash's atomics.  A
        // truncated walk keeps the reference's row-major ids, which it
        // addresses with its own strides.
        d.tiled = 1;
        d.nt0 = (d.dims[0] + 3) / 4;
        d.nt1 = (d.dims[1] + 3) / 4;
        nv = (int64_t)d.nt0 * d.nt1 * ((d.dims[2] + 3) / 4) * 64;
        if (nv > (int64_t)0x7fffffff) return fail(SPHGB_ERR_RANGE, "voxel table over 2^31 entries");
    }
    d.v_count = (int32_t)nv;
    for (int a = 0; a < 2; ++a) {
        const Udiv u = make_udiv((uint32_t)(d.tiled ? (a ? d.nt1 : d.nt0) : d.dims[a]));
        d.div_m[a] = u.m;
        d.div_s[a] = u.p;
    }
    const float h = (float)p.inf_r;
    const double hd = (double)h;
    d.h = h;
    d.h_d = hd;
    const double h2 = hd * hd;  // exact
    d.h2 = (float)h2;
    d.h2_lo = round_down_f(h2 * (1.0 - std::ldexp(1.0, -18)));
    d.h2_hi = round_up_f(h2 * (1.0 + std::ldexp(1.0, -18)));
    d.cull2 = round_up_f((double)d.h2_hi * (1.0 + std::ldexp(1.0, -8)));
    const double pi = 3.141592653589793;
    // normalised kernel constants (config.py:27-29 times the power of h the
    // kernels factor out): W_CONST h^6, GRAD_W_CONST h^2, LAP_W_CONST h
    d.w_const = (float)(315.0 / (64.0 * pi * hd * hd * hd));
    d.grad_w_const = (float)(-45.0 / (pi * hd * hd * hd * hd));
    d.lap_w_const = (float)(45.0 / (pi * hd * hd * hd * hd * hd));
    d.mass = (float)p.mass;
    d.rho0 = (float)p.rho_0;
    d.k = (float)p.k;
    d.visc = (float)p.visc;
    d.damp = (float)p.damp;
    d.dt = (float)p.dt;
    d.dt_d = p.dt;
    d.wall_lo = (float)1e-3;
    d.cap = p.max_neighbours > 0 ? p.max_neighbours : 0x7fffffff;
    d.mode = p.mode;
    d.seed = p.seed;
    if (p.mode == SPHGB_MODE_PIPE) {
        if (p.pipe_rows < 2) return fail(SPHGB_ERR_INVALID, "pipe mode needs >= 2 pipe rows");
        if (p.pipe_row_offset < 0 || p.pipe_row_offset + p.pipe_rows > n_pipe_rows_total)
            return fail(SPHGB_ERR_INVALID, "pipe rows outside the pipe table");
        d.pipe_off = (int32_t)p.pipe_row_offset;
        d.pipe_rows = p.pipe_rows;
    }
    return SPHGB_OK;
}

// rows i0..n-1 of an FP64 AoS state into the float4 state (and the pipe
// accumulator); vel or pos may be null
__global__ void k_load_aos(const SceneDev* __restrict__ scenes, const int32_t* __restrict__ pbegin,
                           int n_scenes, int i0, int n, const double* __restrict__ pos,
                           const double* __restrict__ vel, float4* __restrict__ pos_out,
                           float4* __restrict__ vel_out, int32_t* __restrict__ pid_out,
                           double* __restrict__ pos64_out) {
    const int i = i0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (vel)
        vel_out[i] = make_float4((float)vel[3 * i], (float)vel[3 * i + 1], (float)vel[3 * i + 2], 0.0f);
    if (!pos) return;   // velocities only
    const int si = scene_of(i, pbegin, n_scenes);
    const double x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
    pos_out[i] = make_float4((float)x, (float)y, (float)z, 0.0f);
    pid_out[i] = i - __ldg(pbegin + si);
    if (pos64_out) {
        // the FP64 accumulator takes the input as given (an exported pipe state
        // reloads bit-exactly); FP32-representable input makes it equal pos
        pos64_out[3 * i] = x;
        pos64_out[3 * i + 1] = y;
        pos64_out[3 * i + 2] = z;
    }
    (void)scenes;
}

// slot_of[original index] = sorted slot (the inverse of the particle ids)
__global__ void k_slot_of(const int32_t* __restrict__ pbegin, int n_scenes, int n,
                          const int32_t* __restrict__ pid, int32_t* __restrict__ slot_of) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    slot_of[__ldg(pbegin + scene_of(s, pbegin, n_scenes)) + pid[s]] = s;
}

// state in original particle order as FP64 AoS: one thread per output row,
// so the writes are coalesced (they may go to mapped host memory)
__global__ void k_store_aos(const SceneDev* __restrict__ scenes, const int32_t* __restrict__ pbegin,
                            int n_scenes, int n, const float4* __restrict__ pos,
                            const float4* __restrict__ vel, const float* __restrict__ rho,
                            const int32_t* __restrict__ slot_of, const double* __restrict__ pos64,
                            double* __restrict__ pos_out, double* __restrict__ vel_out,
                            double* __restrict__ rho_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int si = scene_of(i, pbegin, n_scenes);
    const int s = __ldg(slot_of + i);
    if (pos_out) {
        if (pos64 && scenes[si].mode == 1) {
            pos_out[3 * i] = pos64[3 * s];
            pos_out[3 * i + 1] = pos64[3 * s + 1];
            pos_out[3 * i + 2] = pos64[3 * s + 2];
        } else {
            const float4 p = pos[s];
            pos_out[3 * i] = p.x;
            pos_out[3 * i + 1] = p.y;
            pos_out[3 * i + 2] = p.z;
        }
    }
    if (vel_out) {
        const float4 v = vel[s];
        vel_out[3 * i] = v.x;
        vel_out[3 * i + 1] = v.y;
        vel_out[3 * i + 2] = v.z;
    }
    if (rho_out) rho_out[i] = rho ? (double)rho[s] : 0.0;
}

__global__ void k_step_counter(int32_t* scene_step, int n_scenes, const int32_t* step_limit) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_scenes && !(step_limit && scene_step[i] >= step_limit[i])) scene_step[i] += 1;
}

// values per sorted slot -> original particle order (scene offset + pid)
__global__ void k_by_pid(const int32_t* __restrict__ pbegin, int n_scenes, int n,
                         const int32_t* __restrict__ pid, const int32_t* __restrict__ a,
                         const int32_t* __restrict__ b, int32_t* __restrict__ a_out,
                         int32_t* __restrict__ b_out) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int i = __ldg(pbegin + scene_of(s, pbegin, n_scenes)) + pid[s];
    if (a_out) a_out[i] = a[s];
    if (b_out) b_out[i] = b[s];
}

// The step's neighbour rows (slots of the sorted state) -> rows in original
// particle order holding scene-local particle ids, -1 padded.
__global__ void k_export_neighbours(const int32_t* __restrict__ pbegin, int n_scenes, int n,
                                    const int32_t* __restrict__ pid, NbrList nbr,
                                    int32_t* __restrict__ list_out, int32_t* __restrict__ count_out) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int i = __ldg(pbegin + scene_of(s, pbegin, n_scenes)) + pid[s];
    const int c = nbr.count[s];
    if (count_out) count_out[i] = c;
    if (!list_out) return;
    const int32_t* row = nbr.idx + (size_t)s * kListCap;
    int32_t* out = list_out + (size_t)i * kListCap;
    for (int k = 0; k < kListCap; ++k) out[k] = k < c ? pid[row[k]] : -1;
}

// Checked mode: one thread per sorted slot of the step's input validates what
// the step read and wrote, ORs SPHGB_CHECK_* bits into word[0], keeps the
// smallest original index of a flagged particle in word[1] and counts the
// flagged particles in word[2].  It only compares indices against their
// ranges before it uses them, so bad data raises bits, never a fault.  These
// are the places where the reference has undefined behaviour: voxel ids of
// particles outside the box (voxel_kernels.py:10-17, :89-105), never-written
// walk voxels and reads past voxel_begin (:44, :64-65, :70), and non-finite
// coordinates, which its sort and walk do not expect.
__global__ void k_check_step(const SceneDev* __restrict__ scenes, const int32_t* __restrict__ pbegin,
                             int n_scenes, int n, const float4* __restrict__ pos,
                             const float4* __restrict__ vel, const int32_t* __restrict__ pid,
                             const int32_t* __restrict__ vstart, const int32_t* __restrict__ vcount,
                             NbrList nbr, const float* __restrict__ rho,
                             const float4* __restrict__ pos_out, const float4* __restrict__ vel_out,
                             uint32_t* __restrict__ word, const int32_t* __restrict__ step_limit,
                             const int32_t* __restrict__ scene_step) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int si = scene_of(s, pbegin, n_scenes);
    const SceneDev& sc = scenes[si];
    // a frozen scene keeps its slots (not voxel-sorted) and has no list rows
    const bool frozen = scene_frozen(step_limit, scene_step, si);
    const float4 p = pos[s];
    uint32_t bits = 0;
    if (!finite3(p) || !finite3(vel[s])) bits |= SPHGB_CHECK_NONFINITE_INPUT;
    const float xs[3] = {p.x, p.y, p.z};
    for (int a = 0; a < 3; ++a)
        if (isfinite(xs[a]) && !(xs[a] >= 0.0f && xs[a] < sc.space[a])) bits |= SPHGB_CHECK_OUT_OF_DOMAIN;
    // the slot lies inside its own voxel's range, ids ascending within it
    int vid;
    if (finite3(p)) {
        const int vx = voxel_coord(p.x, sc.vs[0], sc.dims[0]);
        const int vy = voxel_coord(p.y, sc.vs[1], sc.dims[1]);
        const int vz = voxel_coord(p.z, sc.vs[2], sc.dims[2]);
        vid = sc.v_begin + voxel_index(vx, vy, vz, sc.tiled, sc.dims[0], sc.dims[1], sc.nt0, sc.nt1);
    } else {
        vid = sc.v_begin + sc.v_count;
    }
    const int st = vstart[vid], c = vcount[vid];
    const int p_lo = sc.p_begin, p_hi = sc.p_begin + sc.p_count;
    if (frozen) {
        // slots kept from an earlier step: nothing to check against the table
    } else if (c <= 0 || st < p_lo || st + c > p_hi || s < st || s >= st + c) {
        bits |= SPHGB_CHECK_VOXEL_TABLE;
    } else if (vid != sc.v_begin + sc.v_count && s > st && !(pid[s - 1] < pid[s])) {
        bits |= SPHGB_CHECK_VOXEL_TABLE;
    }
    const int myid = pid[s];
    if (myid < 0 || myid >= sc.p_count) bits |= SPHGB_CHECK_VOXEL_TABLE;
    // neighbour row: other particles of the same scene within h (guard band).
    // A row holds at most cap others: cap - 1 when the particle itself is
    // among the first cap accepted, cap when more than cap - 1 neighbours come
    // before it in walk order.
    if (nbr.count && !frozen) {
        const int cnt = nbr.count[s];
        if (cnt < -1 || cnt > kListCap || (sc.cap <= kListCap && cnt > sc.cap)) {
            bits |= SPHGB_CHECK_NEIGHBOUR_LIST;
        } else {
            const int32_t* row = nbr.idx + (size_t)s * kListCap;
            for (int k = 0; k < cnt; ++k) {
                const int j = row[k];
                if (j < p_lo || j >= p_hi || j == s) {
                    bits |= SPHGB_CHECK_NEIGHBOUR_LIST;
                    break;
                }
                const float4 q = pos[j];
                const float dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
                if (!(dx * dx + dy * dy + dz * dz <= sc.h2_hi * 1.0001f)) {
                    bits |= SPHGB_CHECK_NEIGHBOUR_LIST;
                    break;
                }
            }
        }
    }
    if (!isfinite(rho[s]) || !finite3(pos_out[s]) || !finite3(vel_out[s]))
        bits |= SPHGB_CHECK_NONFINITE_OUTPUT;
    if (bits) {
        atomicOr(word, bits);
        const int i = __ldg(pbegin + si) + (myid >= 0 && myid < sc.p_count ? myid : 0);
        atomicMin(word + 1, (uint32_t)i);
        atomicAdd(word + 2, 1u);
    }
}

// FP64 conservation sums, one block per chunk of one scene, fixed order.
__global__ void __launch_bounds__(kConsThreads)
k_cons_partial(const SceneDev* __restrict__ scenes, const ConsChunk* __restrict__ chunks,
               const float4* __restrict__ pos, const float4* __restrict__ vel,
               const double* __restrict__ pos64, double* __restrict__ partials) {
    const ConsChunk ch = chunks[blockIdx.x];
    const SceneDev& sc = scenes[ch.scene];
    const double m = (double)sc.mass;
    const double g0 = sc.ext[0], g1 = sc.ext[1], g2 = sc.ext[2];
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (int s = ch.begin + threadIdx.x; s < ch.end; s += kConsThreads) {
        const float4 v = vel[s];
        double x, y, z;
        if (pos64 && sc.mode == 1) {
            x = pos64[3 * s]; y = pos64[3 * s + 1]; z = pos64[3 * s + 2];
        } else {
            const float4 p = pos[s];
            x = p.x; y = p.y; z = p.z;
        }
        const double vx = v.x, vy = v.y, vz = v.z;
        acc[0] += m;
        acc[1] += m * vx;
        acc[2] += m * vy;
        acc[3] += m * vz;
        acc[4] += 0.5 * m * (vx * vx + vy * vy + vz * vz);
        acc[5] += -m * (g0 * x + g1 * y + g2 * z);
    }
    __shared__ double red[kConsThreads / 32][6];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int f = 0; f < 6; ++f) {
        double v = acc[f];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[wid][f] = v;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        double v = 0.0;
        for (int w = 0; w < kConsThreads / 32; ++w) v += red[w][threadIdx.x];
        partials[(size_t)blockIdx.x * 6 + threadIdx.x] = v;
    }
}

// One warp per scene over the scene's own chunks (contiguous, in scene
// order): lane-strided partial sums, then a fixed shuffle tree.  The order
// depends only on the scene's chunk count, so a scene gives the same sums
// alone or batched.
__global__ void k_cons_final(const ConsChunk* __restrict__ chunks, int n_chunks,
                             const double* __restrict__ partials, const SceneDev* __restrict__ scenes,
                             int n_scenes, double* __restrict__ out) {
    const int si = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (si >= n_scenes) return;
    // first chunk of the scene: lower bound of si in the chunks' scene ids
    int lo = 0, hi = n_chunks;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (chunks[mid].scene < si) lo = mid + 1; else hi = mid;
    }
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (int c = lo + lane; c < n_chunks && chunks[c].scene == si; c += 32)
        for (int f = 0; f < 6; ++f) acc[f] += partials[(size_t)c * 6 + f];
#pragma unroll
    for (int f = 0; f < 6; ++f)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc[f] += __shfl_down_sync(0xffffffffu, acc[f], o);
    if (lane != 0) return;
    double* o = out + (size_t)si * kConsFields;
    o[0] = acc[0];
    o[1] = acc[1];
    o[2] = acc[2];
    o[3] = acc[3];
    o[4] = acc[4];
    o[5] = acc[5];
    o[6] = acc[4] + acc[5];
    o[7] = (double)scenes[si].p_count;
}

// ---- pipe geometry wrappers (known-answer tests) ---------------------------
__global__ void k_pipe_find(const double* pos, int n, const double* pipe, int rows, int32_t* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    PipeView P{pipe, rows};
    out[i] = pipe_find_segment(pos + 3 * i, P);
}

__global__ void k_pipe_is_out(const double* pos, const int32_t* seg, int n, const double* pipe,
                              int rows, int32_t* out, double* radius) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    PipeView P{pipe, rows};
    double r = 0.0;
    out[i] = pipe_is_out(pos + 3 * i, P, seg[i], &r) ? 1 : 0;
    if (radius) radius[i] = r;
}

__global__ void k_pipe_xbegin(const int32_t* seg, int n, const double* pipe, int rows, double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    PipeView P{pipe, rows};
    out[i] = pipe_x_begin(P, seg[i]);
}

__global__ void k_pipe_solve(double* pos, double* vel, int n, const double* pipe, int rows,
                             int32_t* seg_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    PipeView P{pipe, rows};
    double p[3] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
    double v[3] = {vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]};
    const int s = pipe_find_segment(p, P);
    if (seg_out) seg_out[i] = s;
    if (s >= 0 && pipe_is_out(p, P, s, nullptr)) pipe_solve_collision(p, v, P, s);
    for (int a = 0; a < 3; ++a) { pos[3 * i + a] = p[a]; vel[3 * i + a] = v[a]; }
}

__global__ void k_philox(uint64_t seed, const int32_t* pid, int n, int step, int draw, double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = philox_uniform(seed, (uint32_t)pid[i], (uint32_t)step, (uint32_t)draw);
}

inline int blocks(int n, int b = kBlock) { return (n + b - 1) / b; }


cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// hash + scan + scatter + big-voxel sort + rank-gather: state (any order) ->
// voxel-sorted copy and voxel table
int enqueue_organize(SphgbCtx* c, const Launch& L, const float4* pos, const float4* vel,
                     const int32_t* pid, const double* pos64, float4* pos_o, float4* vel_o,
                     int32_t* pid_o, double* pos64_o, int32_t* vstart, int32_t* vcount,
                     cudaEvent_t* ev = nullptr, bool with_tasks = false, bool hashed = false) {
    cudaStream_t st = L.stream;
    if (!hashed) {   // else the caller cleared vcount and the counters and hashed every particle
        if (L.v_total > 0) SPHGB_CUDA(cudaMemsetAsync(vcount, 0, sizeof(int32_t) * L.v_total, st));
        SPHGB_CUDA(cudaMemsetAsync(c->big_count, 0, kCounters * sizeof(int32_t), st));
        SPHGB_CUDA(launch_hash_count(L, pos, c->cell, c->slot, vcount));
    }
    if (ev) SPHGB_CUDA(cudaEventRecord(ev[0], st));
    SPHGB_CUDA(launch_scan(L, vcount, vstart, c->tile_sums, scan_tiles(L.v_total)));
    if (ev) SPHGB_CUDA(cudaEventRecord(ev[1], st));
    SPHGB_CUDA(launch_scatter(L, c->cell, c->slot, pid, vstart, vcount, c->tmp_pid, c->big_list,
                              c->big_count));
    SPHGB_CUDA(launch_sort_big(L, c->big_list, c->big_count, vstart, vcount, c->tmp_pid));
    if (ev) SPHGB_CUDA(cudaEventRecord(ev[2], st));
    SPHGB_CUDA(launch_rank_gather(L, c->cell, c->slot, pid, c->tmp_pid, vstart, vcount, pos, vel, pos64,
                                  pos_o, vel_o, pid_o, pos64_o, with_tasks ? c->tasks : nullptr,
                                  with_tasks ? c->big_count + 1 : nullptr));
    if (ev) SPHGB_CUDA(cudaEventRecord(ev[3], st));
    return SPHGB_OK;
}

// force + integrate + wall pass of the step (after the density pass), over
// all slots, or over a range of particles in original order when range is
// given (see PidRange)
int enqueue_forces(SphgbCtx* c, const Launch& L, const PidRange* range, int range_index) {
    const bool sep = c->out_pos != nullptr;
    double* p64B = c->any_pipe ? c->pos64B : nullptr;
    float4* pos_o = sep ? c->out_pos : c->posA;
    float4* vel_o = sep ? c->out_vel : c->velA;
    int32_t* pid_o = sep ? c->out_pid : c->pidA;
    double* p64_o = c->any_pipe ? (sep ? c->out_pos64 : c->pos64A) : nullptr;
    // deferred particles: pass r of the host entry counts in big_count[4 + r]
    // and lists rows of its range from range->i0; the whole pass in [3] from 0
    RareList rare;
    rare.idx = c->rare;
    rare.count = c->big_count + 3 + (range ? 1 + range_index : 0);
    rare.base = !range ? 0 : range->slots ? (int)(range->slots - c->slots_b) : range->i0;
    if (range)
        SPHGB_CUDA(launch_integrate_range(L, c->posB, c->velB, c->rho, c->fin, c->pidB, p64B,
                                          c->vstart, c->vcount, c->scene_step, c->nbr, pos_o,
                                          vel_o, pid_o, p64_o, *range, rare));
    else
        SPHGB_CUDA(launch_integrate(L, c->posB, c->velB, c->rho, c->fin, c->pidB, p64B, c->vstart,
                                    c->vcount, c->scene_step, c->nbr, pos_o, vel_o, pid_o, p64_o,
                                    nullptr, rare));
    return SPHGB_OK;
}

// checked mode: validate the step just enqueued (inputs in the B buffers,
// outputs where enqueue_forces wrote them)
int enqueue_checks(SphgbCtx* c, cudaStream_t st) {
    if (!c->checks || c->n == 0) return SPHGB_OK;
    const bool sep = c->out_pos != nullptr;
    k_check_step<<<blocks(c->n), kBlock, 0, st>>>(c->d_scenes, c->d_pbegin, c->n_scenes, c->n,
                                                  c->posB, c->velB, c->pidB, c->vstart, c->vcount,
                                                  c->nbr, c->rho, sep ? c->out_pos : c->posA,
                                                  sep ? c->out_vel : c->velA, c->d_check,
                                                  c->step_limit, c->scene_step);
    SPHGB_CUDA(cudaGetLastError());
    return SPHGB_OK;
}

// enqueue one full step on stream st; ev (optional, 8 events): ev[0] at the
// start and ev[k] after stage k (see SPHGB_PROFILE_STAGES).  vel_ready
// (optional): the state in A is in original particle order and its
// velocities are still being written on another stream; the sort and the
// density pass go ahead without them and k_gather_vel, after waiting for
// this event, brings them into slot order for the force pass.  density_done
// (optional): recorded after the density pass.
// with_forces = false stops after the density pass (and the velocity gather):
// the caller then runs enqueue_forces itself and the step counter.  hashed:
// the caller has cleared the histogram and the counters and hashed every
// particle (in parts, as they arrived).  organized (optional): recorded once
// the state is voxel-sorted.
int enqueue_step(SphgbCtx* c, cudaStream_t st, cudaEvent_t* ev = nullptr,
                 cudaEvent_t vel_ready = nullptr, cudaEvent_t density_done = nullptr,
                 bool with_forces = true, bool hashed = false, cudaEvent_t organized = nullptr) {
    const Launch L = c->launch(st);
    double* p64A = c->any_pipe ? c->pos64A : nullptr;
    double* p64B = c->any_pipe ? c->pos64B : nullptr;
    if (ev) SPHGB_CUDA(cudaEventRecord(ev[0], st));
    const float4* vel_in = vel_ready ? nullptr : c->velA;   // null: gathered after density
    const float4* vel_s = vel_ready ? nullptr : c->velB;
    int rc = enqueue_organize(c, L, c->posA, vel_in, c->pidA, p64A, c->posB, c->velB, c->pidB,
                              p64B, c->vstart, c->vcount, ev ? ev + 1 : nullptr, true, hashed);
    if (rc) return rc;
    if (organized) SPHGB_CUDA(cudaEventRecord(organized, st));
    if (c->density_variant == SPHGB_DENSITY_WARP)
        SPHGB_CUDA(launch_density_wc(L, c->posB, vel_s, c->vstart, c->vcount, c->rho, c->fin,
                                     c->nbr, c->tasks, c->big_count + 1, c->big_count + 2));
    else
        SPHGB_CUDA(launch_density(L, c->posB, vel_s, c->vstart, c->vcount, c->rho, c->fin,
                                  c->nbr));
    if (ev) SPHGB_CUDA(cudaEventRecord(ev[5], st));
    if (density_done) SPHGB_CUDA(cudaEventRecord(density_done, st));
    if (vel_ready) {
        SPHGB_CUDA(cudaStreamWaitEvent(st, vel_ready, 0));
        SPHGB_CUDA(launch_gather_vel(L, c->pidB, c->velA, c->rho, c->velB, c->fin));
    }
    c->nbr_valid = true;
    if (!with_forces) return SPHGB_OK;
    rc = enqueue_forces(c, L, nullptr, 0);
    if (rc) return rc;
    rc = enqueue_checks(c, st);
    if (rc) return rc;
    if (ev) SPHGB_CUDA(cudaEventRecord(ev[6], st));
    k_step_counter<<<blocks(c->n_scenes, 128), 128, 0, st>>>(c->scene_step, c->n_scenes,
                                                              c->step_limit);
    SPHGB_CUDA(cudaGetLastError());
    if (ev) SPHGB_CUDA(cudaEventRecord(ev[7], st));
    return SPHGB_OK;
}

// (Re)build the scene tables of a context and make every buffer large enough
// for them; buffers keep their capacity and are only replaced when too small.
template <class T>
int ensure(T** p, size_t& cap, size_t need) {
    if (need == 0) need = 1;
    if (*p && cap >= need) return SPHGB_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    cap = 0;
    const size_t want = need + need / 4;   // grow with headroom
    int rc = dalloc(p, want);
    if (rc == SPHGB_OK) cap = want;
    return rc;
}

int configure(SphgbCtx* c, const SphgbSceneParams* scenes, int n_scenes,
              const double* pipe_rows_table, int n_pipe_rows_total) {
    if (!scenes || n_scenes <= 0) return fail(SPHGB_ERR_INVALID, "need at least one scene");
    if (n_pipe_rows_total < 0 || (n_pipe_rows_total > 0 && !pipe_rows_table))
        return fail(SPHGB_ERR_INVALID, "bad pipe table");
    std::vector<SceneDev> hs((size_t)n_scenes), hr((size_t)n_scenes);
    std::vector<int32_t> hp((size_t)n_scenes + 1);
    int64_t n_tot = 0, v_tot = 0, v_tot_ref = 0;
    bool any_pipe = false;
    for (int i = 0; i < n_scenes; ++i) {
        int rc = build_scene(scenes[i], n_pipe_rows_total, hs[i], true);
        if (!rc) rc = build_scene(scenes[i], n_pipe_rows_total, hr[i], false);
        if (rc) return fail(rc, "scene " + std::to_string(i) + ": " + g_last_error);
        SceneDev& d = hs[i];
        d.p_begin = hr[i].p_begin = (int32_t)n_tot;
        d.p_count = hr[i].p_count = (int32_t)scenes[i].particle_count;
        d.v_begin = (int32_t)v_tot;
        hr[i].v_begin = (int32_t)v_tot_ref;
        hp[i] = (int32_t)n_tot;
        n_tot += scenes[i].particle_count;
        v_tot += d.v_count + 1;   // + the scene's overflow bucket
        v_tot_ref += hr[i].v_count + 1;
        // kernels index per-particle rows (3 doubles, 2 float4) in 32-bit arithmetic
        if (n_tot > kMaxParticles)
            return fail(SPHGB_ERR_RANGE, "more than 2^29 particles in one context");
        if (v_tot > (int64_t)0x7fffffff - 1 || v_tot_ref > (int64_t)0x7fffffff - 1)
            return fail(SPHGB_ERR_RANGE, "voxel tables over 2^31 entries in one context");
        if (d.mode == SPHGB_MODE_PIPE) any_pipe = true;
    }
    hp[n_scenes] = (int32_t)n_tot;
    std::vector<ConsChunk> chunks;
    for (int i = 0; i < n_scenes; ++i) {
        const SceneDev& d = hs[i];
        for (int b = 0; b < d.p_count; b += kConsChunk)
            chunks.push_back({i, d.p_begin + b, d.p_begin + std::min(d.p_count, b + kConsChunk), 0});
    }
    const size_t N = (size_t)n_tot, V = (size_t)std::max(v_tot, v_tot_ref);
    const int n_tiles = scan_tiles((int)V);
    auto& k = c->cap;
    int rc = SPHGB_OK;
    rc = rc ? rc : ensure(&c->d_scenes, k.scenes, (size_t)n_scenes);
    rc = rc ? rc : ensure(&c->d_scenes_ref, k.scenes_ref, (size_t)n_scenes);
    rc = rc ? rc : ensure(&c->d_pbegin, k.pbegin, (size_t)n_scenes + 1);
    rc = rc ? rc : ensure(&c->d_pipe, k.pipe, (size_t)n_pipe_rows_total * 5);
    rc = rc ? rc : ensure(&c->cell, k.cell, N);
    rc = rc ? rc : ensure(&c->slot_of, k.slot_of, N);
    rc = rc ? rc : ensure(&c->slot, k.slot, N);
    rc = rc ? rc : ensure(&c->tmp_pid, k.tmp_pid, N + 4);   // + 4: see k_rank_gather
    rc = rc ? rc : ensure(&c->vstart, k.vstart, V);
    rc = rc ? rc : ensure(&c->vcount, k.vcount, V);
    rc = rc ? rc : ensure(&c->tile_sums, k.tile_sums, (size_t)n_tiles);
    rc = rc ? rc : ensure(&c->posB, k.posB, N);
    rc = rc ? rc : ensure(&c->velB, k.velB, N);
    rc = rc ? rc : ensure(&c->pidB, k.pidB, N);
    rc = rc ? rc : ensure(&c->fin, k.fin, 2 * N);
    rc = rc ? rc : ensure(&c->big_list, k.big_list, N / kMinBigVoxel + 1);
    rc = rc ? rc : ensure(&c->big_count, k.big_count, kCounters);
    rc = rc ? rc : ensure(&c->rare, k.rare, N);
    rc = rc ? rc : ensure(&c->tasks, k.tasks, N);
    rc = rc ? rc : ensure(&c->nbr.idx, k.nbr_idx, (size_t)kListCap * N);
    rc = rc ? rc : ensure(&c->nbr.count, k.nbr_count, N);
    if (any_pipe) rc = rc ? rc : ensure(&c->pos64B, k.pos64B, 3 * N);
    rc = rc ? rc : ensure(&c->d_chunks, k.chunks, chunks.size());
    rc = rc ? rc : ensure(&c->d_partials, k.partials, chunks.size() * 6);
    if (rc) return rc;
    SPHGB_CUDA(cudaMemcpy(c->d_scenes, hs.data(), sizeof(SceneDev) * n_scenes,
                          cudaMemcpyHostToDevice));
    SPHGB_CUDA(cudaMemcpy(c->d_scenes_ref, hr.data(), sizeof(SceneDev) * n_scenes,
                          cudaMemcpyHostToDevice));
    SPHGB_CUDA(cudaMemcpy(c->d_pbegin, hp.data(), sizeof(int32_t) * (n_scenes + 1),
                          cudaMemcpyHostToDevice));
    if (n_pipe_rows_total > 0)
        SPHGB_CUDA(cudaMemcpy(c->d_pipe, pipe_rows_table, sizeof(double) * 5 * n_pipe_rows_total,
                              cudaMemcpyHostToDevice));
    if (!chunks.empty())
        SPHGB_CUDA(cudaMemcpy(c->d_chunks, chunks.data(), sizeof(ConsChunk) * chunks.size(),
                              cudaMemcpyHostToDevice));
    c->h_scenes.swap(hs);
    c->h_pbegin.swap(hp);
    c->n_scenes = n_scenes;
    c->n = (int)n_tot;
    c->v_total = (int)v_tot;
    c->v_total_ref = (int)v_tot_ref;
    int n_tiled = 0;
    for (const SceneDev& d : c->h_scenes) n_tiled += d.tiled;
    c->layout = n_tiled == 0 ? 0 : (n_tiled == n_scenes ? 1 : 2);
    c->n_pipe_rows = n_pipe_rows_total;
    c->n_chunks = (int)chunks.size();
    c->any_pipe = any_pipe;
    // the caller binds (new) state and outputs for the new layout
    c->bound = false;
    c->nbr_valid = false;
    c->step_limit = nullptr;   // one entry per scene of the old layout
    // the host-entry orders are timed again on the new scenes
    c->host_calls = 0;
    c->host_ms[1] = c->host_ms[2] = c->host_ms[3] = 0.0;
    c->posA = c->velA = nullptr;
    c->rho = nullptr;
    c->pidA = nullptr;
    c->pos64A = nullptr;
    c->scene_step = nullptr;
    c->out_pos = c->out_vel = nullptr;
    c->out_pid = nullptr;
    c->out_pos64 = nullptr;
    if (c->owned) {
        cudaFree(c->owned);
        c->owned = nullptr;
    }
    if (c->stage) {
        cudaFree(c->stage);
        c->stage = nullptr;
    }
    for (auto& kv : c->graphs) cudaGraphExecDestroy(kv.second);
    c->graphs.clear();
    return SPHGB_OK;
}

}  // namespace

extern "C" {

int sphgb_abi_version(void) { return SPHGB_ABI_VERSION; }

int sphgb_scene_params_size(void) { return (int)sizeof(SphgbSceneParams); }

const char* sphgb_last_error(void) { return g_last_error.c_str(); }

int sphgb_ctx_create(const SphgbSceneParams* scenes, int n_scenes, const double* pipe_rows_table,
                     int n_pipe_rows_total, SphgbCtx** out_ctx) {
    if (!out_ctx) return fail(SPHGB_ERR_INVALID, "out_ctx is null");
    *out_ctx = nullptr;
    // argument checks before any CUDA call
    if (!scenes || n_scenes <= 0) return fail(SPHGB_ERR_INVALID, "need at least one scene");
    if (n_pipe_rows_total < 0 || (n_pipe_rows_total > 0 && !pipe_rows_table))
        return fail(SPHGB_ERR_INVALID, "bad pipe table");
    for (int i = 0; i < n_scenes; ++i) {
        SceneDev probe;
        int rc = build_scene(scenes[i], n_pipe_rows_total, probe);
        if (rc) return fail(rc, "scene " + std::to_string(i) + ": " + g_last_error);
    }
    SphgbCtx* c = new (std::nothrow) SphgbCtx();
    if (!c) return fail(SPHGB_ERR_NOMEM, "host allocation failed");
    cudaGetDevice(&c->device);
    cudaError_t e = cudaStreamCreateWithFlags(&c->cap_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->host_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->host_stream2, cudaStreamNonBlocking);
    for (cudaEvent_t& ev : c->host_ev)
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        free_ctx(c);
        return cuda_fail(e, "sphgb_ctx_create");
    }
    int rc = configure(c, scenes, n_scenes, pipe_rows_table, n_pipe_rows_total);
    if (rc) {
        std::string m = g_last_error;
        free_ctx(c);
        return fail(rc, m);
    }
    *out_ctx = c;
    return SPHGB_OK;
}

int sphgb_ctx_reconfigure(SphgbCtx* ctx, const SphgbSceneParams* scenes, int n_scenes,
                          const double* pipe_rows_table, int n_pipe_rows_total) {
    if (!ctx) return fail(SPHGB_ERR_INVALID, "ctx is null");
    SPHGB_CUDA(cudaDeviceSynchronize());   // nothing in flight may use the old tables
    return configure(ctx, scenes, n_scenes, pipe_rows_table, n_pipe_rows_total);
}

int sphgb_ctx_set_tuning(SphgbCtx* ctx, int sort_block, int density_variant, int big_voxel) {
    if (!ctx) return fail(SPHGB_ERR_INVALID, "ctx is null");
    if (sort_block != 128 && sort_block != 256 && sort_block != 512)
        return fail(SPHGB_ERR_INVALID, "sort_block must be 128, 256 or 512");
    if (density_variant != SPHGB_DENSITY_WARP && density_variant != SPHGB_DENSITY_THREAD)
        return fail(SPHGB_ERR_INVALID, "density_variant must be SPHGB_DENSITY_WARP or _THREAD");
    if (big_voxel < kMinBigVoxel || big_voxel > 4096)
        return fail(SPHGB_ERR_INVALID, "big_voxel must be in [16, 4096]");
    ctx->sort_block = sort_block;
    ctx->density_variant = density_variant;
    ctx->big_voxel = big_voxel;
    for (auto& kv : ctx->graphs) cudaGraphExecDestroy(kv.second);
    ctx->graphs.clear();
    return SPHGB_OK;
}

int sphgb_ctx_destroy(SphgbCtx* ctx) {
    if (!ctx) return SPHGB_OK;
    cudaDeviceSynchronize();
    free_ctx(ctx);
    return SPHGB_OK;
}

int sphgb_ctx_sizes(const SphgbCtx* ctx, int64_t* n_particles, int64_t* n_voxels) {
    if (!ctx) return fail(SPHGB_ERR_INVALID, "ctx is null");
    if (n_particles) *n_particles = ctx->n;
    if (n_voxels) *n_voxels = ctx->v_total_ref;
    return SPHGB_OK;
}

int sphgb_ctx_bind_state(SphgbCtx* ctx, float* d_pos, float* d_vel, float* d_rho, int32_t* d_pid,
                         double* d_pos64, int32_t* d_scene_step) {
    if (!ctx) return fail(SPHGB_ERR_INVALID, "ctx is null");
    if (ctx->n > 0 && (!d_pos || !d_vel || !d_rho || !d_pid))
        return fail(SPHGB_ERR_INVALID, "state pointers must not be null");
    if (!d_scene_step) return fail(SPHGB_ERR_INVALID, "scene_step must not be null");
    if (ctx->any_pipe && ctx->n > 0 && !d_pos64)
        return fail(SPHGB_ERR_INVALID, "pipe scenes need the FP64 position buffer");
    if (((uintptr_t)d_pos | (uintptr_t)d_vel) & 15u)
        return fail(SPHGB_ERR_INVALID, "position/velocity buffers must be 16-byte aligned");
    ctx->posA = reinterpret_cast<float4*>(d_pos);
    ctx->velA = reinterpret_cast<float4*>(d_vel);
    ctx->rho = d_rho;
    ctx->pidA = d_pid;
    ctx->pos64A = ctx->any_pipe ? d_pos64 : nullptr;
    ctx->scene_step = d_scene_step;
    ctx->bound = true;
    for (auto& kv : ctx->graphs) cudaGraphExecDestroy(kv.second);
    ctx->graphs.clear();
    return SPHGB_OK;
}

int sphgb_ctx_bind_output(SphgbCtx* ctx, float* d_pos_out, float* d_vel_out, int32_t* d_pid_out,
                          double* d_pos64_out) {
    if (!ctx) return fail(SPHGB_ERR_INVALID, "ctx is null");
    const bool any = d_pos_out || d_vel_out || d_pid_out || d_pos64_out;
    if (any && ctx->n > 0 && (!d_pos_out || !d_vel_out || !d_pid_out ||
                              (ctx->any_pipe && !d_pos64_out)))
        return fail(SPHGB_ERR_INVALID, "bind all output buffers or none");
    if (((uintptr_t)d_pos_out | (uintptr_t)d_vel_out) & 15u)
        return fail(SPHGB_ERR_INVALID, "position/velocity buffers must be 16-byte aligned");
    ctx->out_pos = reinterpret_cast<float4*>(d_pos_out);
    ctx->out_vel = reinterpret_cast<float4*>(d_vel_out);
    ctx->out_pid = d_pid_out;
    ctx->out_pos64 = d_pos64_out;
    for (auto& kv : ctx->graphs) cudaGraphExecDestroy(kv.second);
    ctx->graphs.clear();
    return SPHGB_OK;
}

int sphgb_ctx_load_aos_f64(SphgbCtx* ctx, const double* d_pos_aos, const double* d_vel_aos,
                           void* stream) {
    if (!ctx) return fail(SPHGB_ERR_INVALID, "ctx is null");
    if (!ctx->bound) return fail(SPHGB_ERR_STATE, "no state bound");
    if (ctx->n == 0) return SPHGB_OK;
    if (!d_pos_aos || !d_vel_aos) return fail(SPHGB_ERR_INVALID, "null input");
    cudaStream_t st = as_stream(stream);
    k_load_aos<<<blocks(ctx->n), kBlock, 0, st>>>(ctx->d_scenes, ctx->d_pbegin, ctx->n_scenes,
                                                 0, ctx->n, d_pos_aos, d_vel_aos, ctx->posA,
                                                 ctx->velA, ctx->pidA, ctx->pos64A);
    SPHGB_CUDA(cudaGetLastError());
    return SPHGB_OK;
}

int sphgb_ctx_store_aos_f64(SphgbCtx* ctx, double* d_pos_aos, double* d_vel_aos, double* d_rho,
                            void* stream) {
    if (!ctx) return fail(SPHGB_ERR_INVALID, "ctx is null");
    if (!ctx->bound) return fail(SPHGB_ERR_STATE, "no state bound");
    if (ctx->n == 0) return SPHGB_OK;
    cudaStream_t st = as_stream(stream);
    // the latest step's result: the output buffers when bound, else the state
    const bool sep = ctx->out_pos != nullptr;
    k_slot_of<<<blocks(ctx->n), kBlock, 0, st>>>(ctx->d_pbegin, ctx->n_scenes, ctx->n,
                                                 sep ? ctx->out_pid : ctx->pidA, ctx->slot_of);
    k_store_aos<<<blocks(ctx->n), kBlock, 0, st>>>(
        ctx->d_scenes, ctx->d_pbegin, ctx->n_scenes, ctx->n, sep ? ctx->out_pos : ctx->posA,
        sep ? ctx->out_vel : ctx->velA, ctx->rho, ctx->slot_of,
        sep ? ctx->out_pos64 : ctx->pos64A, d_pos_aos, d_vel_aos, d_rho);
    SPHGB_CUDA(cudaGetLastError());
    return SPHGB_OK;
}

int sphgb_ctx_step(SphgbCtx* ctx, int n_steps, int use_graph, void* stream) {
    if (!ctx) return fail(SPHGB_ERR_INVALID, "ctx is null");
    if (!ctx->bound) return fail(SPHGB_ERR_STATE, "no state bound");
    if (n_steps < 0) return fail(SPHGB_ERR_INVALID, "n_steps < 0");
    if (n_steps == 0 || ctx->n == 0) return SPHGB_OK;
    cudaStream_t st = as_stream(stream);
    if (!use_graph) {
        for (int i = 0; i < n_steps; ++i) {
            int rc = enqueue_step(ctx, st);
            if (rc) return rc;
        }
        return SPHGB_OK;
    }
    auto it = ctx->graphs.find(n_steps);
    if (it == ctx->graphs.end()) {
        SPHGB_CUDA(cudaStreamBeginCapture(ctx->cap_stream, cudaStreamCaptureModeThreadLocal));
        int rc = SPHGB_OK;
        for (int i = 0; i < n_steps && rc == SPHGB_OK; ++i) rc = enqueue_step(ctx, ctx->cap_stream);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(ctx->cap_stream, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
        cudaGraphExec_t ex = nullptr;
        e = cudaGraphInstantiate(&ex, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
        it = ctx->graphs.emplace(n_steps, ex).first;
    }
    SPHGB_CUDA(cudaGraphLaunch(it->second, st));
    return SPHGB_OK;
}

int sphgb_ctx_step_profiled(SphgbCtx* ctx, int n_steps, void* stream, float* h_stage_ms) {
    if (!ctx) return fail(SPHGB_ERR_INVALID, "ctx is null");
    if (!ctx->bound) return fail(SPHGB_ERR_STATE, "no state bound");
    if (n_steps < 0 || !h_stage_ms) return fail(SPHGB_ERR_INVALID, "bad arguments");
    for (int i = 0; i < SPHGB_PROFILE_STAGES; ++i) h_stage_ms[i] = 0.0f;
    if (n_steps == 0 || ctx->n == 0) return SPHGB_OK;
    cudaStream_t st = as_stream(stream);
    std::vector<cudaEvent_t> ev((size_t)n_steps * 8, nullptr);
    int rc = SPHGB_OK;
    for (auto& e : ev) {
        cudaError_t err = cudaEventCreate(&e);
        if (err != cudaSuccess) { rc = cuda_fail(err, "cudaEventCreate"); break; }
    }
    for (int i = 0; i < n_steps && rc == SPHGB_OK; ++i) rc = enqueue_step(ctx, st, &ev[(size_t)i * 8]);
    if (rc == SPHGB_OK) {
        cudaError_t err = cudaStreamSynchronize(st);
        if (err != cudaSuccess) rc = cuda_fail(err, "cudaStreamSynchronize");
    }
    for (int i = 0; i < n_steps && rc == SPHGB_OK; ++i)
        for (int k = 0; k < SPHGB_PROFILE_STAGES; ++k) {
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, ev[(size_t)i * 8 + k], ev[(size_t)i * 8 + k + 1]);
            h_stage_ms[k] += ms / (float)n_steps;
        }
    for (auto& e : ev)
        if (e) cudaEventDestroy(e);
    return rc;
}

namespace {
// ---- pipelined host entry ---------------------------------------------------
// The density pass runs in kPipeK buckets of tasks, bucket b holding the
// tasks whose first particle falls in range b of the original indices; the
// force pass runs bucket by bucket over the same slots, in slot order, and
// writes each particle's FP64 rows by its id.  A voxel's slots are in id
// order, so a task's first particle has its smallest id and a particle of
// range r is in a task of bucket r or earlier; only the overflow entry
// (non-finite positions, arrival order) can put it in a later one.  Range r's
// rows are complete, and download, once force buckets 0..max(r, dl[r]) are
// done, dl[r] being the latest bucket of an overflow task holding a particle
// of range r.  Force bucket b needs the densities and force
// records of every neighbour of its particles, all of which lie in the 27
// walk voxels around their voxels: dep[b] is the latest bucket of any task in
// those voxels, and force bucket b starts as soon as density buckets
// 0..dep[b] and their velocity gathers are done, while later buckets are
// still in the density pass.  When particle ids follow space (a lattice in
// index order), dep[b] is about b + 1 and the downloads overlap most of the
// density pass; when they do not, dep[b] is the last bucket and the downloads
// wait for the whole density pass.
// pipe_i layout (kPipeK entries each): task counts per bucket, task fill
// counters, task counters of the density launches, dep, task offsets, slot
// counts, slot fill counters, slot offsets, dl.
constexpr int kPipeK = kPipeRanges;
constexpr int kPipeInts = 9 * kPipeK;
// The first buckets run while the velocities are still on the host link and
// are gathered by their own kernel; later buckets wait for the upload (done
// by then at 4M) and gather their velocities in the density pass itself.
constexpr int kPipeGathered = 2;

// Range r of the original indices is [b[r], b[r + 1]).  The last ranges are
// smaller: the force buckets and downloads that must wait for the end of the
// density pass are short.  Relative sizes of the ranges:
constexpr int kPipeWeight[kPipeK] = {4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 2, 1, 1};
struct PipeBounds {
    int32_t b[kPipeK + 1];
};

PipeBounds pipe_bounds(int n) {
    int64_t total = 0;
    for (int w : kPipeWeight) total += w;
    PipeBounds pb;
    int64_t acc = 0;
    pb.b[0] = 0;
    for (int r = 0; r < kPipeK; ++r) {
        acc += kPipeWeight[r];
        pb.b[r + 1] = (int32_t)((int64_t)n * acc / total);
    }
    return pb;
}

__device__ __forceinline__ int range_of(int i, const PipeBounds& pb) {
    int r = 0;
    while (r + 1 < kPipeK && i >= pb.b[r + 1]) ++r;
    return r;
}

// slots of a task: a run of at most kTaskRun from its first slot, within its voxel
__device__ __forceinline__ int task_size(int2 t, const int32_t* __restrict__ vstart,
                                         const int32_t* __restrict__ vcount) {
    return min(kTaskRun, __ldg(vstart + t.x) + __ldg(vcount + t.x) - t.y);
}

// The bucket kernels aggregate per block in shared memory: one global atomic
// per bucket and block, not one per task on kPipeK shared addresses.
__global__ void k_bucket_count(const int2* __restrict__ tasks, const int32_t* __restrict__ task_count,
                               const int32_t* __restrict__ pid, const int32_t* __restrict__ vstart,
                               const int32_t* __restrict__ vcount, PipeBounds pb,
                               int32_t* __restrict__ pi) {
    __shared__ int h[kPipeK], hs[kPipeK];
    if (threadIdx.x < kPipeK) h[threadIdx.x] = hs[threadIdx.x] = 0;
    __syncthreads();
    const int m = *task_count;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
        const int2 t = tasks[k];
        const int b = range_of(pid[t.y], pb);
        atomicAdd(h + b, 1);
        atomicAdd(hs + b, task_size(t, vstart, vcount));
    }
    __syncthreads();
    if (threadIdx.x < kPipeK && h[threadIdx.x]) {
        atomicAdd(pi + threadIdx.x, h[threadIdx.x]);
        atomicAdd(pi + 5 * kPipeK + threadIdx.x, hs[threadIdx.x]);
    }
}

// Each block places a block-sized run of tasks per round, so a bucket keeps
// the tasks' voxel order up to the order in which blocks take their places.
__global__ void k_bucket_scatter(const int2* __restrict__ tasks, const int32_t* __restrict__ task_count,
                                 const int32_t* __restrict__ pid, const int32_t* __restrict__ vstart,
                                 const int32_t* __restrict__ vcount, PipeBounds pb,
                                 int32_t* __restrict__ pi,
                                 int2* __restrict__ tasks_b, int32_t* __restrict__ slots_b,
                                 int32_t* __restrict__ vbucket) {
    __shared__ int cnt[kPipeK], scnt[kPipeK], base[kPipeK], sbase[kPipeK];
    int off[kPipeK], soff[kPipeK];
    int acc = 0, sacc = 0;
    for (int b = 0; b < kPipeK; ++b) {
        off[b] = acc;
        soff[b] = sacc;
        acc += pi[b];
        sacc += pi[5 * kPipeK + b];
    }
    if (blockIdx.x == 0 && threadIdx.x < kPipeK) {
        pi[4 * kPipeK + threadIdx.x] = off[threadIdx.x];
        pi[7 * kPipeK + threadIdx.x] = soff[threadIdx.x];
    }
    const int m = *task_count;
    for (int k0 = blockIdx.x * blockDim.x; k0 < m; k0 += gridDim.x * blockDim.x) {
        const int k = k0 + threadIdx.x;
        if (threadIdx.x < kPipeK) cnt[threadIdx.x] = scnt[threadIdx.x] = 0;
        __syncthreads();
        int2 t = make_int2(0, 0);
        int b = -1, local = 0, slocal = 0, sz = 0;
        if (k < m) {
            t = tasks[k];
            b = range_of(pid[t.y], pb);
            sz = task_size(t, vstart, vcount);
            local = atomicAdd(cnt + b, 1);
            slocal = atomicAdd(scnt + b, sz);
        }
        __syncthreads();
        if (threadIdx.x < kPipeK && cnt[threadIdx.x]) {
            base[threadIdx.x] = atomicAdd(pi + kPipeK + threadIdx.x, cnt[threadIdx.x]);
            sbase[threadIdx.x] = atomicAdd(pi + 6 * kPipeK + threadIdx.x, scnt[threadIdx.x]);
        }
        __syncthreads();
        if (b >= 0) {
            tasks_b[off[b] + base[b] + local] = t;
            int32_t* dst = slots_b + soff[b] + sbase[b] + slocal;
            for (int j = 0; j < sz; ++j) dst[j] = t.y + j;
            atomicMax(vbucket + t.x, b);
        }
        __syncthreads();
    }
}

// dep[b] = max over the tasks of bucket b of the latest bucket in the task
// voxel's 27 walk voxels (one scene, walk dims = table dims); dl[r] = max
// bucket of an overflow task holding a particle of range r
__global__ void k_bucket_deps(const SceneDev* __restrict__ scenes, const int2* __restrict__ tasks,
                              const int32_t* __restrict__ task_count,
                              const int32_t* __restrict__ pid, const int32_t* __restrict__ vstart,
                              const int32_t* __restrict__ vcount,
                              const int32_t* __restrict__ vbucket, PipeBounds pb,
                              int32_t* __restrict__ pi) {
    __shared__ int dep[kPipeK], dl[kPipeK];
    if (threadIdx.x < kPipeK) dep[threadIdx.x] = dl[threadIdx.x] = -1;
    __syncthreads();
    const SceneDev& sc = scenes[0];
    const int m = *task_count;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
        const int2 t = tasks[k];
        const int vid = t.x;
        const int b = range_of(pid[t.y], pb);
        int need = vbucket[vid];
        const int local = vid - sc.v_begin;
        if (local == sc.v_count) {      // the overflow entry: no neighbours, ids unordered
            const int end = t.y + task_size(t, vstart, vcount);
            for (int d = t.y; d < end; ++d) atomicMax(dl + range_of(pid[d], pb), b);
        } else {
            const Udiv q0{sc.div_m[0], sc.div_s[0]}, q1{sc.div_m[1], sc.div_s[1]};
            int vx, vy, vz;
            if (sc.tiled) {
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
            for (int w = 0; w < 27; ++w) {
                const int nx = vx + w / 9 - 1, ny = vy + (w / 3) % 3 - 1, nz = vz + w % 3 - 1;
                if (nx < 0 || nx >= sc.wdims[0] || ny < 0 || ny >= sc.wdims[1] || nz < 0 ||
                    nz >= sc.wdims[2])
                    continue;
                const int u = sc.v_begin + voxel_index(nx, ny, nz, sc.tiled, sc.wdims[0],
                                                       sc.wdims[1], sc.nt0, sc.nt1);
                need = max(need, vbucket[u]);
            }
        }
        atomicMax(dep + b, need);
    }
    __syncthreads();
    if (threadIdx.x < kPipeK && dep[threadIdx.x] >= 0)
        atomicMax(pi + 3 * kPipeK + threadIdx.x, dep[threadIdx.x]);
    if (threadIdx.x < kPipeK && dl[threadIdx.x] >= 0)
        atomicMax(pi + 8 * kPipeK + threadIdx.x, dl[threadIdx.x]);
}

// One scene with a neighbour list the warp kernel builds, enough particles
// for the buckets, and no step limits (a frozen scene has no density tasks,
// and the force pass runs only the tasks' slots).
bool pipelined_eligible(const SphgbCtx* c) {
    return c->n_scenes == 1 && !c->h_scenes[0].walk_trunc && c->h_scenes[0].cap <= kListCap &&
           c->density_variant == SPHGB_DENSITY_WARP && c->n >= 32 * kPipeK && !c->step_limit;
}

int ensure_pipelined(SphgbCtx* c) {
    const size_t N = (size_t)c->n, V = (size_t)c->v_total;
    if (c->cap_tasks_b < N) {
        if (c->tasks_b) cudaFree(c->tasks_b);
        if (c->slots_b) cudaFree(c->slots_b);
        c->tasks_b = nullptr;
        c->slots_b = nullptr;
        c->cap_tasks_b = 0;
        int rc = dalloc(&c->tasks_b, N);
        if (!rc) rc = dalloc(&c->slots_b, N);
        if (rc) return rc;
        c->cap_tasks_b = N;
    }
    if (c->cap_vbucket < V) {
        if (c->vbucket) cudaFree(c->vbucket);
        c->vbucket = nullptr;
        c->cap_vbucket = 0;
        int rc = dalloc(&c->vbucket, V);
        if (rc) return rc;
        c->cap_vbucket = V;
    }
    if (!c->pipe_i) {
        int rc = dalloc(&c->pipe_i, (size_t)kPipeInts);
        if (rc) return rc;
    }
    if (!c->h_pipe) SPHGB_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&c->h_pipe),
                                             sizeof(int32_t) * kPipeInts, cudaHostAllocDefault));
    if (!c->host_stream3) {
        // the gathers and force buckets go ahead of the density buckets when
        // both have blocks waiting for an SM
        int least = 0, greatest = 0;
        SPHGB_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        SPHGB_CUDA(cudaStreamCreateWithPriority(&c->host_stream3, cudaStreamNonBlocking, greatest));
    }
    if (!c->host_stream4)
        SPHGB_CUDA(cudaStreamCreateWithFlags(&c->host_stream4, cudaStreamNonBlocking));
    for (cudaEvent_t& e : c->pipe_ev)
        if (!e) SPHGB_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return SPHGB_OK;
}

// The host entry after the positions have been hashed (st) and the
// velocities uploaded (st2, event e_vel): the step with its force pass and
// downloads pipelined behind the density pass (see kPipeK above).  st sorts,
// buckets the tasks and runs the density buckets; st3, which has the
// greatest priority, builds the slot map, gathers the first buckets'
// velocities and runs the force buckets, each after the density buckets it
// depends on; st4 reads the counts and dependencies back and downloads each
// range's rows.
int host_step_pipelined(SphgbCtx* c, cudaEvent_t e_vel, double* sp, double* sv, double* sr,
                        double* h_pos_out, double* h_vel_out, double* h_rho_out) {
    const size_t N = (size_t)c->n;
    cudaStream_t st = c->host_stream, st3 = c->host_stream3, st4 = c->host_stream4;
    cudaEvent_t e_org = c->pipe_ev[0], e_bk = c->pipe_ev[1], e_dep = c->pipe_ev[2];
    cudaEvent_t* e_bucket = c->pipe_ev + 3;
    cudaEvent_t* e_range = c->pipe_ev + 3 + kPipeK;
    const Launch L = c->launch(st);
    const Launch L3 = c->launch(st3);
    double* p64A = c->any_pipe ? c->pos64A : nullptr;
    double* p64B = c->any_pipe ? c->pos64B : nullptr;
    // sort (the velocities follow bucket by bucket: gathered into slot order
    // by the density buckets themselves, or for the first buckets by a kernel
    // of their own on st3)
    int rc = enqueue_organize(c, L, c->posA, nullptr, c->pidA, p64A, c->posB, c->velB, c->pidB,
                              p64B, c->vstart, c->vcount, nullptr, true, true);
    if (rc) return rc;
    SPHGB_CUDA(cudaEventRecord(e_org, st));
    // st3 after the sort and the velocity upload: the gathers and the
    // density buckets read the upload's FP64 rows, and a force bucket
    // overwrites only the rows of its own particles, whose velocities its
    // density bucket (or gather) has already read
    SPHGB_CUDA(cudaStreamWaitEvent(st3, e_org, 0));
    SPHGB_CUDA(cudaStreamWaitEvent(st3, e_vel, 0));
    // buckets and dependencies
    int32_t* pi = c->pipe_i;
    const int32_t* n_tasks = c->big_count + 1;
    const int grid = device_sm_count() * 4;
    SPHGB_CUDA(cudaMemsetAsync(pi, 0, sizeof(int32_t) * kPipeInts, st));
    SPHGB_CUDA(cudaMemsetAsync(c->vbucket, 0xff, sizeof(int32_t) * c->v_total, st));
    const PipeBounds pb = pipe_bounds(c->n);
    k_bucket_count<<<grid, kBlock, 0, st>>>(c->tasks, n_tasks, c->pidB, c->vstart, c->vcount, pb,
                                            pi);
    k_bucket_scatter<<<grid, kBlock, 0, st>>>(c->tasks, n_tasks, c->pidB, c->vstart, c->vcount,
                                              pb, pi, c->tasks_b, c->slots_b, c->vbucket);
    SPHGB_CUDA(cudaGetLastError());
    SPHGB_CUDA(cudaEventRecord(e_bk, st));
    // st4: the dependencies, which only the host's ordering of the force
    // buckets needs, while st goes on with the density buckets; then the
    // counts, offsets and dependencies to the host
    SPHGB_CUDA(cudaStreamWaitEvent(st4, e_bk, 0));
    k_bucket_deps<<<grid, kBlock, 0, st4>>>(c->d_scenes, c->tasks_b, n_tasks, c->pidB, c->vstart,
                                            c->vcount, c->vbucket, pb, pi);
    SPHGB_CUDA(cudaGetLastError());
    SPHGB_CUDA(cudaMemcpyAsync(c->h_pipe, pi, sizeof(int32_t) * kPipeInts,
                               cudaMemcpyDeviceToHost, st4));
    SPHGB_CUDA(cudaEventRecord(e_dep, st4));
    // The density buckets, one after another on st.  From bucket
    // kPipeGathered on they wait for the velocity upload and gather their
    // velocities themselves.
    VelRows vrows;
    vrows.vel64 = sv;
    vrows.pid = c->pidB;
    vrows.vel_out = c->velB;
    for (int b = 0; b < kPipeK; ++b) {
        if (b == kPipeGathered) SPHGB_CUDA(cudaStreamWaitEvent(st, e_vel, 0));
        SPHGB_CUDA(launch_density_wc(L, c->posB, nullptr, c->vstart, c->vcount, c->rho, c->fin,
                                     c->nbr, c->tasks_b, pi + b, pi + 2 * kPipeK + b,
                                     pi + 4 * kPipeK + b,
                                     b >= kPipeGathered ? vrows : VelRows{}));
        SPHGB_CUDA(cudaEventRecord(e_bucket[b], st));
    }
    c->nbr_valid = true;
    // the slot counts and the dependencies are needed on the host to launch
    // and order the force buckets
    SPHGB_CUDA(cudaEventSynchronize(e_dep));
    const int32_t* h_dep = c->h_pipe + 3 * kPipeK;
    const int32_t* h_slots = c->h_pipe + 5 * kPipeK;
    const int32_t* h_soff = c->h_pipe + 7 * kPipeK;
    const int32_t* h_dl = c->h_pipe + 8 * kPipeK;
    int gathered = 0;   // buckets whose velocities are in slot order, as seen from st3
    auto gather_through = [&](int last) -> int {
        for (; gathered <= last; ++gathered) {
            SPHGB_CUDA(cudaStreamWaitEvent(st3, e_bucket[gathered], 0));
            if (gathered < kPipeGathered)
                SPHGB_CUDA(launch_gather_vel_tasks(L3, c->pidB, c->tasks_b, pi + gathered,
                                                   pi + 4 * kPipeK + gathered, c->vstart,
                                                   c->vcount, sv, c->rho, c->velB, c->fin));
        }
        return SPHGB_OK;
    };
    // range r downloads once force bucket max(r, dl[r]) is done (each force
    // bucket writes the FP64 rows of its particles)
    int next_r = 0;
    auto download_through = [&](int b) -> int {
        for (; next_r < kPipeK && std::max(next_r, (int)h_dl[next_r]) <= b; ++next_r) {
            SPHGB_CUDA(cudaStreamWaitEvent(st4, e_range[b], 0));
            const size_t i0 = (size_t)pb.b[next_r], i1 = (size_t)pb.b[next_r + 1];
            SPHGB_CUDA(cudaMemcpyAsync(h_pos_out + 3 * i0, sp + 3 * i0,
                                       sizeof(double) * 3 * (i1 - i0), cudaMemcpyDeviceToHost,
                                       st4));
            SPHGB_CUDA(cudaMemcpyAsync(h_vel_out + 3 * i0, sv + 3 * i0,
                                       sizeof(double) * 3 * (i1 - i0), cudaMemcpyDeviceToHost,
                                       st4));
            SPHGB_CUDA(cudaMemcpyAsync(h_rho_out + i0, sr + i0, sizeof(double) * (i1 - i0),
                                       cudaMemcpyDeviceToHost, st4));
        }
        return SPHGB_OK;
    };
    size_t listed = 0;
    for (int b = 0; b < kPipeK; ++b) {
        rc = gather_through(std::min(std::max(h_dep[b], b), kPipeK - 1));
        if (rc) return rc;
        if (h_slots[b] < 0 || h_soff[b] < 0 || (size_t)h_soff[b] + h_slots[b] > N)
            return fail(SPHGB_ERR_STATE, "pipelined step: bucket slot counts out of range");
        listed += (size_t)h_slots[b];
        PidRange range;
        range.slots = c->slots_b + h_soff[b];
        range.n_slots = h_slots[b];
        range.pos = sp;
        range.vel = sv;
        range.rho = sr;
        rc = enqueue_forces(c, L3, &range, b);
        if (rc) return rc;
        SPHGB_CUDA(cudaEventRecord(e_range[b], st3));
        rc = download_through(b);
        if (rc) return rc;
    }
    if (next_r != kPipeK) return fail(SPHGB_ERR_STATE, "pipelined step: range left undownloaded");
    // every bucket gathered (the slot-order velocities are complete), then
    // the checks and the step counter
    rc = gather_through(kPipeK - 1);
    if (rc) return rc;
    rc = enqueue_checks(c, st3);
    if (rc) return rc;
    k_step_counter<<<blocks(c->n_scenes, 128), 128, 0, st3>>>(c->scene_step, c->n_scenes,
                                                                c->step_limit);
    SPHGB_CUDA(cudaGetLastError());
    SPHGB_CUDA(cudaStreamSynchronize(st4));
    SPHGB_CUDA(cudaStreamSynchronize(st3));
    SPHGB_CUDA(cudaStreamSynchronize(st));
    // every slot was in exactly one bucket
    if (listed != N) return fail(SPHGB_ERR_STATE, "pipelined step: buckets missed particles");
    return SPHGB_OK;
}

// Force-pass order of the next host-entry call.  AUTO: calls 1 to 3 run slot
// order, particle order and the pipelined order (when the context allows it)
// once each, for their allocations and first kernel loads; calls 4 to 6 run
// them again and are timed, and later calls take the fastest order the
// context allows.
constexpr int kAutoTimedFirst = 3;   // index of the first timed call
int host_order_for_call(const SphgbCtx* c) {
    const bool pipe_ok = pipelined_eligible(c);
    if (c->host_order != SPHGB_HOST_ORDER_AUTO) {
        if (c->host_order == SPHGB_HOST_ORDER_PIPELINED && !pipe_ok) return SPHGB_HOST_ORDER_PARTICLE;
        return c->host_order;
    }
    if (c->host_calls < 2 * kAutoTimedFirst) {
        const int k = c->host_calls % kAutoTimedFirst;
        if (k == 0) return SPHGB_HOST_ORDER_SLOT;
        if (k == 1 || !pipe_ok) return SPHGB_HOST_ORDER_PARTICLE;
        return SPHGB_HOST_ORDER_PIPELINED;
    }
    int best = SPHGB_HOST_ORDER_SLOT;
    for (int o = SPHGB_HOST_ORDER_PARTICLE; o <= SPHGB_HOST_ORDER_PIPELINED; ++o)
        if (c->host_ms[o] > 0.0 && c->host_ms[o] < c->host_ms[best] &&
            (o != SPHGB_HOST_ORDER_PIPELINED || pipe_ok))
            best = o;
    return best;
}
}  // namespace

static int host_entry(SphgbCtx* ctx, const double* h_pos, const double* h_vel,
                      double* h_pos_out, double* h_vel_out, double* h_rho_out) {
    if (!ctx) return fail(SPHGB_ERR_INVALID, "ctx is null");
    if (ctx->n_scenes != 1) return fail(SPHGB_ERR_INVALID, "host entry needs a one-scene context");
    const size_t N = (size_t)ctx->n;
    if (N > 0 && (!h_pos || !h_vel || !h_pos_out || !h_vel_out || !h_rho_out))
        return fail(SPHGB_ERR_INVALID, "null host buffer");
    if (!ctx->bound) {
        // own state: pos, vel (float4), rho, pid, pos64, scene_step
        const size_t bytes = N * 16 * 2 + N * 4 * 2 + (ctx->any_pipe ? N * 24 : 0) + 16;
        if (!ctx->owned) {
            cudaError_t e = cudaMalloc(&ctx->owned, bytes);
            if (e != cudaSuccess) {
                ctx->owned = nullptr;
                return fail(SPHGB_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
            }
            SPHGB_CUDA(cudaMemset(ctx->owned, 0, bytes));
        }
        char* b = static_cast<char*>(ctx->owned);
        float* pos = reinterpret_cast<float*>(b);
        float* vel = reinterpret_cast<float*>(b + N * 16);
        float* rho = reinterpret_cast<float*>(b + N * 32);
        int32_t* pid = reinterpret_cast<int32_t*>(b + N * 36);
        double* pos64 = ctx->any_pipe ? reinterpret_cast<double*>(b + N * 40) : nullptr;
        int32_t* step = reinterpret_cast<int32_t*>(b + N * 40 + (ctx->any_pipe ? N * 24 : 0));
        int rc = sphgb_ctx_bind_state(ctx, pos, vel, rho, pid, pos64, step);
        if (rc) return rc;
    }
    if (N == 0) return SPHGB_OK;
    if (!ctx->stage) {
        cudaError_t e = cudaMalloc(&ctx->stage, sizeof(double) * N * 7);
        if (e != cudaSuccess) {
            ctx->stage = nullptr;
            return fail(SPHGB_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        }
    }
    cudaStream_t st = ctx->host_stream, st2 = ctx->host_stream2;
    cudaEvent_t e_start = ctx->host_ev[0], e_vel = ctx->host_ev[2],
                e_rho = ctx->host_ev[3], e_slot = ctx->host_ev[4], e_done = ctx->host_ev[5];
    double* sp = ctx->stage;
    double* sv = ctx->stage + 3 * N;
    double* sr = ctx->stage + 6 * N;
    const size_t b3 = sizeof(double) * 3 * N;
    const int nb = blocks(ctx->n);
    // Two streams.  st2 uploads: the positions in kHostPosChunks parts, then
    // the velocities.  st runs the step: each part of the positions is
    // converted and hashed as soon as it is in (the voxel histogram fills in
    // parts while the rest is in flight), then the voxel sort and the density
    // pass, which need positions only, run while the velocities are still on
    // the host link; the step gathers them into slot order after the density
    // pass.  Once the state is voxel-sorted, st2 builds the map from
    // original index to slot; once the density pass is done, it downloads the
    // densities, which overlaps the force pass.  The next positions and
    // velocities are downloaded whole from st after the force pass (slot
    // order), or range by range from st2 while st computes the next range
    // (particle order).  Results are the same bits as the one-stream sequence.
    SPHGB_CUDA(cudaEventRecord(e_start, st));
    SPHGB_CUDA(cudaStreamWaitEvent(st2, e_start, 0));
    if (ctx->v_total > 0)
        SPHGB_CUDA(cudaMemsetAsync(ctx->vcount, 0, sizeof(int32_t) * ctx->v_total, st));
    SPHGB_CUDA(cudaMemsetAsync(ctx->big_count, 0, kCounters * sizeof(int32_t), st));
    {
        const Launch L = ctx->launch(st);
        // parts start on whole warps (the hash aggregates its atomics per warp)
        auto bound = [&](int q) {
            return (int)std::min(N, ((N * q / kHostPosChunks) + 31) & ~(size_t)31);
        };
        for (int k = 0; k < kHostPosChunks; ++k) {
            const int i0 = bound(k);
            const int i1 = k + 1 == kHostPosChunks ? (int)N : bound(k + 1);
            if (i1 <= i0) continue;
            cudaEvent_t e_part = ctx->host_ev[kHostFirstChunkEvent + k];
            SPHGB_CUDA(cudaMemcpyAsync(sp + 3 * (size_t)i0, h_pos + 3 * (size_t)i0,
                                       sizeof(double) * 3 * (i1 - i0), cudaMemcpyHostToDevice,
                                       st2));
            SPHGB_CUDA(cudaEventRecord(e_part, st2));
            SPHGB_CUDA(cudaStreamWaitEvent(st, e_part, 0));
            k_load_aos<<<blocks(i1 - i0), kBlock, 0, st>>>(ctx->d_scenes, ctx->d_pbegin,
                                                            ctx->n_scenes, i0, i1, sp, nullptr,
                                                            ctx->posA, ctx->velA, ctx->pidA,
                                                            ctx->pos64A);
            SPHGB_CUDA(cudaGetLastError());
            SPHGB_CUDA(launch_hash_count(L, ctx->posA, ctx->cell, ctx->slot, ctx->vcount, i0, i1));
        }
    }
    const int order = host_order_for_call(ctx);
    SPHGB_CUDA(cudaMemcpyAsync(sv, h_vel, b3, cudaMemcpyHostToDevice, st2));
    // the pipelined order gathers from the FP64 rows bucket by bucket
    if (order != SPHGB_HOST_ORDER_PIPELINED) {
        k_load_aos<<<nb, kBlock, 0, st2>>>(ctx->d_scenes, ctx->d_pbegin, ctx->n_scenes, 0, ctx->n,
                                           nullptr, sv, ctx->posA, ctx->velA, ctx->pidA, nullptr);
        SPHGB_CUDA(cudaGetLastError());
    }
    SPHGB_CUDA(cudaEventRecord(e_vel, st2));
    const auto t0 = std::chrono::steady_clock::now();
    auto record_time = [&]() {
        const double ms = std::chrono::duration<double, std::milli>(
                              std::chrono::steady_clock::now() - t0).count();
        // calls 4 to 6 time the three orders (calls 1 to 3 warm them up)
        if (ctx->host_order == SPHGB_HOST_ORDER_AUTO && ctx->host_calls >= kAutoTimedFirst &&
            ctx->host_calls < 2 * kAutoTimedFirst)
            ctx->host_ms[order] = ms;
        if (ctx->host_calls < 1000) ++ctx->host_calls;
    };
    if (order == SPHGB_HOST_ORDER_PIPELINED) {
        int rc = ensure_pipelined(ctx);
        if (!rc) rc = host_step_pipelined(ctx, e_vel, sp, sv, sr, h_pos_out, h_vel_out, h_rho_out);
        if (rc) return rc;
        record_time();
        return SPHGB_OK;
    }
    cudaEvent_t e_org = ctx->host_ev[kHostOrganizedEvent];
    int rc = enqueue_step(ctx, st, nullptr, e_vel, e_rho, order == SPHGB_HOST_ORDER_SLOT, true,
                          e_org);
    if (rc) return rc;
    // st2: original index -> slot (from the sorted ids, which the force pass
    // copies to the output unchanged) during the density pass, then the
    // densities in original order
    SPHGB_CUDA(cudaStreamWaitEvent(st2, e_org, 0));
    k_slot_of<<<nb, kBlock, 0, st2>>>(ctx->d_pbegin, ctx->n_scenes, ctx->n, ctx->pidB,
                                      ctx->slot_of);
    SPHGB_CUDA(cudaGetLastError());
    SPHGB_CUDA(cudaEventRecord(e_slot, st2));
    SPHGB_CUDA(cudaStreamWaitEvent(st2, e_rho, 0));
    k_store_aos<<<nb, kBlock, 0, st2>>>(ctx->d_scenes, ctx->d_pbegin, ctx->n_scenes, ctx->n,
                                        nullptr, nullptr, ctx->rho, ctx->slot_of, nullptr,
                                        nullptr, nullptr, sr);
    SPHGB_CUDA(cudaGetLastError());
    SPHGB_CUDA(cudaMemcpyAsync(h_rho_out, sr, sizeof(double) * N, cudaMemcpyDeviceToHost, st2));
    if (order == SPHGB_HOST_ORDER_SLOT) {
        // st: positions and velocities in original order once the step is
        // done and the slot map is ready, then downloaded whole
        SPHGB_CUDA(cudaEventRecord(e_done, st2));
        SPHGB_CUDA(cudaStreamWaitEvent(st, e_done, 0));
        const bool sep = ctx->out_pos != nullptr;
        k_store_aos<<<nb, kBlock, 0, st>>>(ctx->d_scenes, ctx->d_pbegin, ctx->n_scenes, ctx->n,
                                           sep ? ctx->out_pos : ctx->posA,
                                           sep ? ctx->out_vel : ctx->velA, nullptr, ctx->slot_of,
                                           sep ? ctx->out_pos64 : ctx->pos64A, sp, sv, nullptr);
        SPHGB_CUDA(cudaGetLastError());
        SPHGB_CUDA(cudaMemcpyAsync(h_pos_out, sp, b3, cudaMemcpyDeviceToHost, st));
        SPHGB_CUDA(cudaMemcpyAsync(h_vel_out, sv, b3, cudaMemcpyDeviceToHost, st));
    } else {
        // st: the force pass in original particle order, kHostRanges ranges;
        // st2 downloads each range's rows while st computes the next
        SPHGB_CUDA(cudaStreamWaitEvent(st, e_slot, 0));
        const Launch L = ctx->launch(st);
        for (int r = 0; r < kHostRanges; ++r) {
            PidRange range;
            range.slot_of = ctx->slot_of;
            range.i0 = (int)(N * r / kHostRanges);
            range.i1 = (int)(N * (r + 1) / kHostRanges);
            range.pos = sp;
            range.vel = sv;
            rc = enqueue_forces(ctx, L, &range, r);
            if (rc) return rc;
            SPHGB_CUDA(cudaEventRecord(ctx->host_ev[kHostFirstRangeEvent + r], st));
            SPHGB_CUDA(cudaStreamWaitEvent(st2, ctx->host_ev[kHostFirstRangeEvent + r], 0));
            const size_t off = 3 * (size_t)range.i0, len = sizeof(double) * 3 * (range.i1 - range.i0);
            SPHGB_CUDA(cudaMemcpyAsync(h_pos_out + off, sp + off, len, cudaMemcpyDeviceToHost, st2));
            SPHGB_CUDA(cudaMemcpyAsync(h_vel_out + off, sv + off, len, cudaMemcpyDeviceToHost, st2));
        }
        rc = enqueue_checks(ctx, st);
        if (rc) return rc;
        k_step_counter<<<blocks(ctx->n_scenes, 128), 128, 0, st>>>(ctx->scene_step, ctx->n_scenes,
                                                                    ctx->step_limit);
        SPHGB_CUDA(cudaGetLastError());
        SPHGB_CUDA(cudaEventRecord(e_done, st2));
        SPHGB_CUDA(cudaStreamWaitEvent(st, e_done, 0));
    }
    SPHGB_CUDA(cudaStreamSynchronize(st));
    record_time();
    return SPHGB_OK;
}

int sphgb_compute_next_state_host(SphgbCtx* ctx, const double* h_pos, const double* h_vel,
                                  double* h_pos_out, double* h_vel_out, double* h_rho_out) {
    const int rc = host_entry(ctx, h_pos, h_vel, h_pos_out, h_vel_out, h_rho_out);
    if (rc && ctx) {
        // a failed call returns only once nothing it enqueued still runs: no
        // copy into the caller's host buffers outlives the call
        for (cudaStream_t s : {ctx->host_stream, ctx->host_stream2, ctx->host_stream3,
                               ctx->host_stream4})
            if (s) cudaStreamSynchronize(s);
    }
    return rc;
}

int sphgb_ctx_set_host_order(SphgbCtx* ctx, int order) {
    if (!ctx) return fail(SPHGB_ERR_INVALID, "ctx is null");
    if (order != SPHGB_HOST_ORDER_AUTO && order != SPHGB_HOST_ORDER_SLOT &&
        order != SPHGB_HOST_ORDER_PARTICLE && order != SPHGB_HOST_ORDER_PIPELINED)
        return fail(SPHGB_ERR_INVALID,
                    "order must be SPHGB_HOST_ORDER_AUTO, _SLOT, _PARTICLE or _PIPELINED");
    ctx->host_order = order;
    ctx->host_calls = 0;
    ctx->host_ms[1] = ctx->host_ms[2] = ctx->host_ms[3] = 0.0;
    return SPHGB_OK;
}

int sphgb_ctx_conservation(SphgbCtx* ctx, double* d_out, void* stream) {
    if (!ctx) return fail(SPHGB_ERR_INVALID, "ctx is null");
    if (!ctx->bound) return fail(SPHGB_ERR_STATE, "no state bound");
    if (!d_out) return fail(SPHGB_ERR_INVALID, "d_out is null");
    cudaStream_t st = as_stream(stream);
    if (ctx->n_chunks > 0)
        k_cons_partial<<<ctx->n_chunks, kConsThreads, 0, st>>>(ctx->d_scenes, ctx->d_chunks,
                                                               ctx->posA, ctx->velA, ctx->pos64A,
                                                               ctx->d_partials);
    k_cons_final<<<blocks(ctx->n_scenes * 32, 128), 128, 0, st>>>(ctx->d_chunks, ctx->n_chunks,
                                                            ctx->d_partials, ctx->d_scenes,
                                                            ctx->n_scenes, d_out);
    SPHGB_CUDA(cudaGetLastError());
    return SPHGB_OK;
}

int sphgb_ctx_neighbour_counts(SphgbCtx* ctx, int32_t* d_capped, int32_t* d_uncapped, void* stream) {
    if (!ctx) return fail(SPHGB_ERR_INVALID, "ctx is null");
    if (!ctx->bound) return fail(SPHGB_ERR_STATE, "no state bound");
    cudaStream_t st = as_stream(stream);
    Launch L = ctx->launch(st);
    L.step_limit = nullptr;   // counts of every scene, frozen or not
    int rc = enqueue_organize(ctx, L, ctx->posA, ctx->velA, ctx->pidA,
                              ctx->any_pipe ? ctx->pos64A : nullptr, ctx->posB, ctx->velB,
                              ctx->pidB, ctx->any_pipe ? ctx->pos64B : nullptr, ctx->vstart,
                              ctx->vcount);
    ctx->nbr_valid = false;
    if (rc) return rc;
    // per sorted slot into the scratch id buffers, then to original order
    SPHGB_CUDA(launch_neighbours(L, ctx->posB, ctx->vstart, ctx->vcount, nullptr, 0, ctx->cell,
                                 ctx->slot));
    k_by_pid<<<blocks(ctx->n), kBlock, 0, st>>>(ctx->d_pbegin, ctx->n_scenes, ctx->n, ctx->pidB,
                                                ctx->cell, ctx->slot, d_capped, d_uncapped);
    SPHGB_CUDA(cudaGetLastError());
    return SPHGB_OK;
}

int sphgb_ctx_step_neighbours(SphgbCtx* ctx, int32_t* d_list, int32_t* d_count, void* stream) {
    if (!ctx) return fail(SPHGB_ERR_INVALID, "ctx is null");
    if (!d_list && !d_count) return fail(SPHGB_ERR_INVALID, "d_list and d_count are both null");
    if (!ctx->nbr_valid)
        return fail(SPHGB_ERR_STATE, "no step has run since the context was configured or re-sorted");
    if (ctx->n == 0) return SPHGB_OK;
    cudaStream_t st = as_stream(stream);
    k_export_neighbours<<<blocks(ctx->n), kBlock, 0, st>>>(ctx->d_pbegin, ctx->n_scenes, ctx->n,
                                                           ctx->pidB, ctx->nbr, d_list, d_count);
    SPHGB_CUDA(cudaGetLastError());
    return SPHGB_OK;
}

int sphgb_ctx_set_step_limits(SphgbCtx* ctx, const int32_t* d_limits) {
    if (!ctx) return fail(SPHGB_ERR_INVALID, "ctx is null");
    if (d_limits) {
        // the kernels read it at every step: a host pointer would fault there
        cudaPointerAttributes a{};
        const cudaError_t e = cudaPointerGetAttributes(&a, d_limits);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(SPHGB_ERR_INVALID, "d_limits is not a device pointer");
        }
        if (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged)
            return fail(SPHGB_ERR_INVALID, "d_limits is not device or managed memory");
        if ((reinterpret_cast<uintptr_t>(d_limits) & 3u) != 0)
            return fail(SPHGB_ERR_INVALID, "d_limits is not 4-byte aligned");
    }
    if (d_limits != ctx->step_limit) {
        // captured step graphs hold the old pointer
        for (auto& kv : ctx->graphs) cudaGraphExecDestroy(kv.second);
        ctx->graphs.clear();
    }
    ctx->step_limit = d_limits;
    return SPHGB_OK;
}

int sphgb_ctx_set_checks(SphgbCtx* ctx, int enable) {
    if (!ctx) return fail(SPHGB_ERR_INVALID, "ctx is null");
    const bool on = enable != 0;
    if (on && !ctx->d_check) {
        int rc = dalloc(&ctx->d_check, 3);
        if (rc) return rc;
        const uint32_t init[3] = {0u, 0xffffffffu, 0u};
        SPHGB_CUDA(cudaMemcpy(ctx->d_check, init, sizeof(init), cudaMemcpyHostToDevice));
    }
    if (on != ctx->checks) {
        // captured step graphs hold the old sequence
        for (auto& kv : ctx->graphs) cudaGraphExecDestroy(kv.second);
        ctx->graphs.clear();
    }
    ctx->checks = on;
    return SPHGB_OK;
}

int sphgb_ctx_check_word(SphgbCtx* ctx, uint32_t* h_word, int clear, void* stream) {
    if (!ctx) return fail(SPHGB_ERR_INVALID, "ctx is null");
    if (!h_word) return fail(SPHGB_ERR_INVALID, "h_word is null");
    if (!ctx->d_check) {
        h_word[0] = 0u;
        h_word[1] = 0xffffffffu;
        h_word[2] = 0u;
        return SPHGB_OK;
    }
    cudaStream_t st = as_stream(stream);
    uint32_t w[3];
    SPHGB_CUDA(cudaMemcpyAsync(w, ctx->d_check, sizeof(w), cudaMemcpyDeviceToHost, st));
    SPHGB_CUDA(cudaStreamSynchronize(st));
    h_word[0] = w[0];
    h_word[1] = w[1];
    h_word[2] = w[2];
    if (clear) {   // {0, 0xffffffff, 0}, ordered on the caller's stream
        SPHGB_CUDA(cudaMemsetAsync(ctx->d_check, 0, 3 * sizeof(uint32_t), st));
        SPHGB_CUDA(cudaMemsetAsync(ctx->d_check + 1, 0xff, sizeof(uint32_t), st));
    }
    return SPHGB_OK;
}

int sphgb_assign_voxels(SphgbCtx* ctx, const float* d_pos, int32_t* d_voxel_out, void* stream) {
    if (!ctx) return fail(SPHGB_ERR_INVALID, "ctx is null");
    if (ctx->n > 0 && (!d_pos || !d_voxel_out)) return fail(SPHGB_ERR_INVALID, "null buffer");
    cudaStream_t st = as_stream(stream);
    const Launch L = ctx->launch(st, true);
    if (L.v_total > 0) SPHGB_CUDA(cudaMemsetAsync(ctx->vcount, 0, sizeof(int32_t) * L.v_total, st));
    SPHGB_CUDA(launch_hash_count(L, reinterpret_cast<const float4*>(d_pos), d_voxel_out, ctx->slot,
                                 ctx->vcount));
    return SPHGB_OK;
}

int sphgb_organize_voxels(SphgbCtx* ctx, const float* d_pos, const float* d_vel,
                          const int32_t* d_pid, const double* d_pos64, float* d_pos_out,
                          float* d_vel_out, int32_t* d_pid_out, double* d_pos64_out,
                          int32_t* d_voxel_start, int32_t* d_voxel_count, void* stream) {
    if (!ctx) return fail(SPHGB_ERR_INVALID, "ctx is null");
    if (ctx->n > 0 && (!d_pos || !d_vel || !d_pid || !d_pos_out || !d_vel_out || !d_pid_out))
        return fail(SPHGB_ERR_INVALID, "null buffer");
    if (!d_voxel_start || !d_voxel_count) return fail(SPHGB_ERR_INVALID, "null voxel table");
    if ((d_pos64 == nullptr) != (d_pos64_out == nullptr))
        return fail(SPHGB_ERR_INVALID, "pass both FP64 position buffers or neither");
    cudaStream_t st = as_stream(stream);
    const Launch L = ctx->launch(st, true);
    return enqueue_organize(ctx, L, reinterpret_cast<const float4*>(d_pos),
                            reinterpret_cast<const float4*>(d_vel), d_pid, d_pos64,
                            reinterpret_cast<float4*>(d_pos_out),
                            reinterpret_cast<float4*>(d_vel_out), d_pid_out, d_pos64_out,
                            d_voxel_start, d_voxel_count);
}

int sphgb_neighbours(SphgbCtx* ctx, const float* d_pos_sorted, const int32_t* d_voxel_start,
                     const int32_t* d_voxel_count, int32_t* d_list, int list_stride,
                     int32_t* d_count_capped, int32_t* d_count_uncapped, void* stream) {
    if (!ctx) return fail(SPHGB_ERR_INVALID, "ctx is null");
    if (d_list && list_stride <= 0) return fail(SPHGB_ERR_INVALID, "list_stride must be > 0");
    cudaStream_t st = as_stream(stream);
    SPHGB_CUDA(launch_neighbours(ctx->launch(st, true), reinterpret_cast<const float4*>(d_pos_sorted),
                                 d_voxel_start, d_voxel_count, d_list, list_stride, d_count_capped,
                                 d_count_uncapped));
    return SPHGB_OK;
}

int sphgb_density(SphgbCtx* ctx, const float* d_pos_sorted, const int32_t* d_voxel_start,
                  const int32_t* d_voxel_count, float* d_rho_out, void* stream) {
    if (!ctx) return fail(SPHGB_ERR_INVALID, "ctx is null");
    if (ctx->n > 0 && (!d_pos_sorted || !d_rho_out)) return fail(SPHGB_ERR_INVALID, "null buffer");
    cudaStream_t st = as_stream(stream);
    SPHGB_CUDA(launch_density(ctx->launch(st, true), reinterpret_cast<const float4*>(d_pos_sorted),
                              nullptr, d_voxel_start, d_voxel_count, d_rho_out, nullptr,
                              NbrList{}));
    return SPHGB_OK;
}

int sphgb_forces(SphgbCtx* ctx, const float* d_pos_sorted, const float* d_vel_sorted,
                 const float* d_rho_sorted, const int32_t* d_voxel_start,
                 const int32_t* d_voxel_count, float* d_pressure_out, float* d_viscosity_out,
                 void* stream) {
    if (!ctx) return fail(SPHGB_ERR_INVALID, "ctx is null");
    if (ctx->n > 0 && (!d_pos_sorted || !d_vel_sorted || !d_rho_sorted || !d_pressure_out ||
                       !d_viscosity_out))
        return fail(SPHGB_ERR_INVALID, "null buffer");
    cudaStream_t st = as_stream(stream);
    const Launch L = ctx->launch(st, true);
    SPHGB_CUDA(launch_force_inputs(L, reinterpret_cast<const float4*>(d_pos_sorted),
                                   reinterpret_cast<const float4*>(d_vel_sorted), d_rho_sorted,
                                   ctx->fin));
    SPHGB_CUDA(launch_forces(L, reinterpret_cast<const float4*>(d_pos_sorted),
                             reinterpret_cast<const float4*>(d_vel_sorted), d_rho_sorted, ctx->fin,
                             d_voxel_start, d_voxel_count, reinterpret_cast<float4*>(d_pressure_out),
                             reinterpret_cast<float4*>(d_viscosity_out)));
    return SPHGB_OK;
}

int sphgb_integrate(SphgbCtx* ctx, const float* d_pos_sorted, const float* d_vel_sorted,
                    const float* d_rho_sorted, const int32_t* d_pid_sorted,
                    const double* d_pos64_sorted, const int32_t* d_voxel_start,
                    const int32_t* d_voxel_count, const int32_t* d_scene_step, float* d_pos_out,
                    float* d_vel_out, int32_t* d_pid_out, double* d_pos64_out, float* d_force_out,
                    void* stream) {
    if (!ctx) return fail(SPHGB_ERR_INVALID, "ctx is null");
    if (ctx->n > 0 && (!d_pos_sorted || !d_vel_sorted || !d_rho_sorted || !d_pid_sorted ||
                       !d_pos_out || !d_vel_out || !d_pid_out || !d_scene_step))
        return fail(SPHGB_ERR_INVALID, "null buffer");
    if (ctx->any_pipe && ctx->n > 0 && (!d_pos64_sorted || !d_pos64_out))
        return fail(SPHGB_ERR_INVALID, "pipe scenes need the FP64 position buffers");
    cudaStream_t st = as_stream(stream);
    const Launch L = ctx->launch(st, true);
    SPHGB_CUDA(launch_force_inputs(L, reinterpret_cast<const float4*>(d_pos_sorted),
                                   reinterpret_cast<const float4*>(d_vel_sorted), d_rho_sorted,
                                   ctx->fin));
    SPHGB_CUDA(launch_integrate(L, reinterpret_cast<const float4*>(d_pos_sorted),
                                reinterpret_cast<const float4*>(d_vel_sorted), d_rho_sorted,
                                ctx->fin, d_pid_sorted, d_pos64_sorted, d_voxel_start,
                                d_voxel_count, d_scene_step, NbrList{},
                                reinterpret_cast<float4*>(d_pos_out),
                                reinterpret_cast<float4*>(d_vel_out), d_pid_out, d_pos64_out,
                                reinterpret_cast<float4*>(d_force_out)));
    return SPHGB_OK;
}

int sphgb_pipe_find_segment(const double* d_pos, int n, const double* d_pipe, int pipe_rows,
                            int32_t* d_seg_out, void* stream) {
    if (n < 0 || pipe_rows < 2) return fail(SPHGB_ERR_INVALID, "bad size");
    if (n == 0) return SPHGB_OK;
    k_pipe_find<<<blocks(n), kBlock, 0, as_stream(stream)>>>(d_pos, n, d_pipe, pipe_rows, d_seg_out);
    SPHGB_CUDA(cudaGetLastError());
    return SPHGB_OK;
}

int sphgb_pipe_is_out(const double* d_pos, const int32_t* d_seg, int n, const double* d_pipe,
                      int pipe_rows, int32_t* d_out, double* d_radius_out, void* stream) {
    if (n < 0 || pipe_rows < 2) return fail(SPHGB_ERR_INVALID, "bad size");
    if (n == 0) return SPHGB_OK;
    k_pipe_is_out<<<blocks(n), kBlock, 0, as_stream(stream)>>>(d_pos, d_seg, n, d_pipe, pipe_rows,
                                                               d_out, d_radius_out);
    SPHGB_CUDA(cudaGetLastError());
    return SPHGB_OK;
}

int sphgb_pipe_x_at_segment_beginning(const int32_t* d_seg, int n, const double* d_pipe,
                                      int pipe_rows, double* d_out, void* stream) {
    if (n < 0 || pipe_rows < 1) return fail(SPHGB_ERR_INVALID, "bad size");
    if (n == 0) return SPHGB_OK;
    k_pipe_xbegin<<<blocks(n), kBlock, 0, as_stream(stream)>>>(d_seg, n, d_pipe, pipe_rows, d_out);
    SPHGB_CUDA(cudaGetLastError());
    return SPHGB_OK;
}

int sphgb_pipe_solve_collision(double* d_pos, double* d_vel, int n, const double* d_pipe,
                               int pipe_rows, int32_t* d_seg_out, void* stream) {
    if (n < 0 || pipe_rows < 2) return fail(SPHGB_ERR_INVALID, "bad size");
    if (n == 0) return SPHGB_OK;
    k_pipe_solve<<<blocks(n), kBlock, 0, as_stream(stream)>>>(d_pos, d_vel, n, d_pipe, pipe_rows,
                                                              d_seg_out);
    SPHGB_CUDA(cudaGetLastError());
    return SPHGB_OK;
}

int sphgb_philox_uniform(uint64_t seed, const int32_t* d_pid, int n, int step, int draw,
                         double* d_out, void* stream) {
    if (n < 0) return fail(SPHGB_ERR_INVALID, "bad size");
    if (n == 0) return SPHGB_OK;
    k_philox<<<blocks(n), kBlock, 0, as_stream(stream)>>>(seed, d_pid, n, step, draw, d_out);
    SPHGB_CUDA(cudaGetLastError());
    return SPHGB_OK;
}

int sphgb_generator_size(void) { return (int)sizeof(SphgbGenerator); }

int sphgb_generate(const SphgbGenerator* g, const double* d_pipe, int pipe_rows, int64_t n,
                   double* d_pos, double* d_vel, void* stream) {
    if (!g) return fail(SPHGB_ERR_INVALID, "null generator");
    if (n < 0 || n > (int64_t)INT32_MAX) return fail(SPHGB_ERR_RANGE, "particle count out of range");
    if (n > 0 && (!d_pos || !d_vel)) return fail(SPHGB_ERR_INVALID, "null output");
    switch (g->kind) {
    case SPHGB_GEN_LATTICE:
        if (g->lattice[0] <= 0 || g->lattice[1] <= 0 || g->lattice[2] <= 0 ||
            (int64_t)g->lattice[0] * g->lattice[1] * g->lattice[2] != n)
            return fail(SPHGB_ERR_INVALID, "lattice nx*ny*nz must equal n");
        break;
    case SPHGB_GEN_BOX_WALL:
        break;
    case SPHGB_GEN_PIPE_FILL:
        if (!d_pipe || pipe_rows < 2)
            return fail(SPHGB_ERR_INVALID, "pipe fill needs a pipe table of >= 2 rows");
        break;
    default:
        return fail(SPHGB_ERR_INVALID, "unknown generator kind");
    }
    SPHGB_CUDA(launch_generate(*g, d_pipe, pipe_rows, n, d_pos, d_vel, as_stream(stream)));
    return SPHGB_OK;
}

int sphgb_point_field(const float* d_pos, int pos_stride, const float* d_rho, int64_t n,
                      const float* h_proj, const float* h_model, const float* h_view,
                      float* d_clip_out, float* d_colour_out, float* d_size_out, void* stream) {
    if (n < 0) return fail(SPHGB_ERR_INVALID, "bad size");
    if (pos_stride < 3) return fail(SPHGB_ERR_INVALID, "position stride below 3 floats");
    if (!h_proj || !h_model || !h_view) return fail(SPHGB_ERR_INVALID, "null matrix");
    if (n > 0 && (!d_pos || !d_rho || !d_clip_out || !d_colour_out || !d_size_out))
        return fail(SPHGB_ERR_INVALID, "null buffer");
    SPHGB_CUDA(launch_point_field(d_pos, pos_stride, d_rho, n, h_proj, h_model, h_view, d_clip_out,
                                  d_colour_out, d_size_out, as_stream(stream)));
    return SPHGB_OK;
}

}  // extern "C"

// ---- voxel organisation without allocation --------------------------------
//
// For callers that cannot allocate device memory (cudaMalloc is forbidden in
// their process, or they run inside a host allocator of their own and may not
// add allocations behind its back): the same kernels as
// sphgb_organize_voxels, with every scratch buffer in one file-scope
// __device__ array of fixed size.  Each GPU that loads this library holds the
// array (about 3.2 MB) until the process exits.
namespace {

constexpr int kNoAllocMaxParticles = 262144;
constexpr int kNoAllocMaxVoxels = 4194304;   // voxel-table entries, overflow entry included
constexpr int kNoAllocMaxTiles = (kNoAllocMaxVoxels + 4095) / 4096;

struct NoAllocScratch {
    SceneDev scene;
    int32_t pbegin[2];
    int32_t counters[2];
    int32_t tile_sums[kNoAllocMaxTiles];
    int32_t cell[kNoAllocMaxParticles];
    int32_t slot[kNoAllocMaxParticles];
    alignas(16) int32_t tmp_pid[kNoAllocMaxParticles + 4];   // + 4: see k_rank_gather
    int32_t big_list[kNoAllocMaxParticles / kBigVoxel + 1];
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

// device address of g_noalloc_scratch per device ordinal, looked up once
std::mutex g_noalloc_mutex;
constexpr int kNoAllocMaxDevices = 64;
NoAllocScratch* g_noalloc_addr[kNoAllocMaxDevices] = {};

// Writes the call's scene descriptor and particle range into the shared
// array and clears its counters.  The values travel as kernel arguments, which
// are copied when the launch is enqueued, so no host buffer has to outlive
// this call (a memcpy from the caller's stack would read it later).
__global__ void k_noalloc_setup(NoAllocScratch* S, SceneDev scene, int n) {
    if (threadIdx.x == 0) {
        S->scene = scene;
        S->pbegin[0] = 0;
        S->pbegin[1] = n;
        S->counters[0] = 0;
        S->counters[1] = 0;
    }
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

int noalloc_scratch(NoAllocScratch** out) {
    int dev = 0;
    SPHGB_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices)
        return fail(SPHGB_ERR_RANGE, "device ordinal beyond the no-alloc table");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_noalloc_addr[dev] = static_cast<NoAllocScratch*>(p);
    }
    *out = g_noalloc_addr[dev];
    return SPHGB_OK;
}

}  // namespace

extern "C" int sphgb_organize_voxels_noalloc(const SphgbSceneParams* scene, const float* d_pos,
                                             const float* d_vel, const int32_t* d_pid,
                                             float* d_pos_out, float* d_vel_out,
                                             int32_t* d_pid_out, int32_t* d_voxel_start,
                                             int32_t* d_voxel_count, void* stream) {
    if (!scene) return fail(SPHGB_ERR_INVALID, "scene is null");
    if (scene->particle_count > kNoAllocMaxParticles)
        return fail(SPHGB_ERR_RANGE, "particle_count " + std::to_string(scene->particle_count) +
                                         " exceeds the no-alloc limit of " +
                                         std::to_string(kNoAllocMaxParticles));
    SceneDev d;
    // pipe rows are not used by this stage: accept the scene's own range
    int rc = build_scene(*scene, (int)(scene->pipe_row_offset + scene->pipe_rows), d);
    if (rc) return rc;
    if ((int64_t)d.v_count + 1 > kNoAllocMaxVoxels)
        return fail(SPHGB_ERR_RANGE, "voxel table of " + std::to_string((int64_t)d.v_count + 1) +
                                         " entries exceeds the no-alloc limit of " +
                                         std::to_string(kNoAllocMaxVoxels));
    const int n = (int)scene->particle_count;
    if (n > 0 && (!d_pos || !d_vel || !d_pid || !d_pos_out || !d_vel_out || !d_pid_out))
        return fail(SPHGB_ERR_INVALID, "null buffer");
    if (!d_voxel_start || !d_voxel_count) return fail(SPHGB_ERR_INVALID, "null voxel table");
    // the kernels move positions and velocities as float4 and the voxel table
    // in 16-byte quads: a sub-allocated buffer must keep that alignment
    const void* bufs[] = {d_pos, d_vel, d_pid, d_pos_out, d_vel_out, d_pid_out, d_voxel_start,
                          d_voxel_count};
    const char* names[] = {"d_pos", "d_vel", "d_pid", "d_pos_out", "d_vel_out", "d_pid_out",
                           "d_voxel_start", "d_voxel_count"};
    for (int i = 0; i < 8; ++i)
        if (!aligned16(bufs[i]))
            return fail(SPHGB_ERR_INVALID, std::string(names[i]) + " is not 16-byte aligned");
    NoAllocScratch* S = nullptr;
    rc = noalloc_scratch(&S);
    if (rc) return rc;
    d.p_begin = 0;
    d.p_count = n;
    d.v_begin = 0;
    cudaStream_t st = as_stream(stream);
    // the scene descriptor and the counters live in the shared array too: a
    // later call overwrites them, so calls that overlap on the GPU race
    k_noalloc_setup<<<1, 32, 0, st>>>(S, d, n);
    SPHGB_CUDA(cudaGetLastError());
    const int v_total = d.v_count + 1;
    SPHGB_CUDA(cudaMemsetAsync(d_voxel_count, 0, sizeof(int32_t) * v_total, st));
    if (n == 0) {
        SPHGB_CUDA(cudaMemsetAsync(d_voxel_start, 0, sizeof(int32_t) * v_total, st));
        return SPHGB_OK;
    }
    Launch L;
    L.scenes = &S->scene;
    L.pbegin = S->pbegin;
    L.n_scenes = 1;
    L.n = n;
    L.v_total = v_total;
    L.pipe = nullptr;
    L.pipe_scenes = false;
    L.stream = st;
    const float4* pos = reinterpret_cast<const float4*>(d_pos);
    SPHGB_CUDA(launch_hash_count(L, pos, S->cell, S->slot, d_voxel_count));
    SPHGB_CUDA(launch_scan(L, d_voxel_count, d_voxel_start, S->tile_sums, scan_tiles(v_total)));
    SPHGB_CUDA(launch_scatter(L, S->cell, S->slot, d_pid, d_voxel_start, d_voxel_count, S->tmp_pid,
                              S->big_list, &S->counters[0]));
    SPHGB_CUDA(launch_sort_big(L, S->big_list, &S->counters[0], d_voxel_start, d_voxel_count,
                               S->tmp_pid));
    SPHGB_CUDA(launch_rank_gather(L, S->cell, S->slot, d_pid, S->tmp_pid, d_voxel_start, d_voxel_count, pos,
                                  reinterpret_cast<const float4*>(d_vel), nullptr,
                                  reinterpret_cast<float4*>(d_pos_out),
                                  reinterpret_cast<float4*>(d_vel_out), d_pid_out, nullptr));
    return SPHGB_OK;
}
