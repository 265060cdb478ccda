// sort.cu -- voxel hash, counting sort and voxel table.
//
// Replaces the host-side voxel organisation of the reference
// (sim/src/sph/strategies/voxel_sph_strategy.py:65-107: GPU hash, copy to the
// host, numpy structured sort by (voxel_id, particle_id), Python loop building
// voxel_begin) with four device passes:
//   1. hash: voxel id per particle + atomic histogram (slot = arrival rank;
//      one atomic per run of lanes in the same voxel);
//   2. scan: exclusive prefix of the histogram = voxel_start (tile sums; each
//      tile adds up the sums before it, or one block scans them for large
//      tables; tile-local warp-shuffle scans);
//   3. scatter: particle id of each particle to voxel_start + slot;
//   4. rank-gather: each particle's final slot = voxel_start + number of
//      members of its voxel with a smaller particle id; the state is gathered
//      into that slot.  The result is the reference's (voxel, particle id)
//      order exactly, independent of atomic arrival order and of the input
//      order of the state.
// Voxels with more than kBigVoxel members (dense clusters, the overflow bucket
// of non-finite particles) have their member ids sorted by one block each
// between 3 and 4, and the rank is a binary search, so the pass stays
// O(n log n) however the particles cluster.
#include "sphgb_internal.cuh"

namespace sphgb {

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;  // 4096 voxels per tile

__device__ __forceinline__ int warp_incl_scan(int v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// exclusive scan of one int per thread across the block; `total` receives the
// block total.  Safe to call repeatedly if the caller synchronises between calls.
__device__ __forceinline__ int block_excl_scan(int v, int& total) {
    constexpr int kWarps = kScanThreads / 32;
    __shared__ int warp_off[kWarps];
    __shared__ int block_total;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int incl = warp_incl_scan(v);
    if (lane == 31) warp_off[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        const int w = lane < kWarps ? warp_off[lane] : 0;
        const int wi = warp_incl_scan(w);
        if (lane < kWarps) warp_off[lane] = wi - w;
        if (lane == kWarps - 1) block_total = wi;
    }
    __syncthreads();
    total = block_total;
    return incl - v + warp_off[wid];
}

__global__ void __launch_bounds__(512)
k_hash_count(const SceneDev* __restrict__ scenes, const int32_t* __restrict__ pbegin, int n_scenes,
             int i0, int i1, const float4* __restrict__ pos, int32_t* __restrict__ cell,
             int32_t* __restrict__ slot, int32_t* __restrict__ vcount) {
    const int s = i0 + blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const bool valid = s < i1;
    int vid = -1;
    if (valid) {
        const SceneDev& sc = scenes[scene_of(s, pbegin, n_scenes)];
        const float4 p = __ldg(pos + s);
        if (finite3(p)) {
            const int vx = voxel_coord(p.x, sc.vs[0], sc.dims[0]);
            const int vy = voxel_coord(p.y, sc.vs[1], sc.dims[1]);
            const int vz = voxel_coord(p.z, sc.vs[2], sc.dims[2]);
            vid = sc.v_begin + voxel_index(vx, vy, vz, sc.tiled, sc.dims[0], sc.dims[1], sc.nt0, sc.nt1);
            cell[s] = vid;
        } else {
            vid = sc.v_begin + sc.v_count;   // overflow bucket
            cell[s] = ~vid;                  // negative: overflow bucket (no pid order needed)
        }
    }
    // Lanes of a run with the same voxel (sorted input holds whole voxels in
    // consecutive slots) take consecutive slots with one atomic by the run's
    // first lane.  Every lane of the warp takes part, in range or not.
    const unsigned full = 0xffffffffu;
    const int prev = __shfl_up_sync(full, vid, 1);
    const unsigned heads = __ballot_sync(full, !valid || lane == 0 || prev != vid);
    const unsigned le = (2u << lane) - 1u;
    const int leader = 31 - __clz(heads & le);
    int base = 0;
    if (valid && leader == lane) {
        const unsigned above = heads & ~le;
        const int next = above ? __ffs(above) - 1 : 32;
        base = atomicAdd(vcount + vid, next - lane);
    }
    base = __shfl_sync(full, base, leader);
    if (valid) slot[s] = base + (lane - leader);
}

__global__ void __launch_bounds__(kScanThreads)
k_tile_reduce(const int32_t* __restrict__ vcount, int v_total, int32_t* __restrict__ tile_sums) {
    const int base = blockIdx.x * kScanTile;
    int sum = 0;
    if (base + kScanTile <= v_total) {
        const int4* v4 = reinterpret_cast<const int4*>(vcount + base);
#pragma unroll
        for (int i = 0; i < kScanItems / 4; ++i) {
            int4 q = __ldg(v4 + threadIdx.x + i * kScanThreads);
            sum += q.x + q.y + q.z + q.w;
        }
    } else {
        for (int i = threadIdx.x; i < kScanTile; i += kScanThreads) {
            int k = base + i;
            if (k < v_total) sum += __ldg(vcount + k);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
    __shared__ int ws[kScanThreads / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = sum;
    __syncthreads();
    if (threadIdx.x < 32) {
        int v = threadIdx.x < kScanThreads / 32 ? ws[threadIdx.x] : 0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0) tile_sums[blockIdx.x] = v;
    }
}

// one block: exclusive scan of the tile sums in place
__global__ void __launch_bounds__(kScanThreads)
k_scan_tile_sums(int32_t* __restrict__ tile_sums, int n_tiles) {
    int carry = 0;
    for (int base = 0; base < n_tiles; base += kScanThreads) {
        const int i = base + threadIdx.x;
        const int v = i < n_tiles ? tile_sums[i] : 0;
        int total = 0;
        const int ex = block_excl_scan(v, total);
        if (i < n_tiles) tile_sums[i] = carry + ex;
        carry += total;
        __syncthreads();
    }
}

// Tables of at most this many tiles skip the one-block scan of the tile sums:
// each block of k_tile_scan adds up the sums of the tiles before it instead
// (at most kScanDirectTiles / kScanThreads loads per thread).
constexpr int kScanDirectTiles = 8192;

// sum of tile_sums[0 .. n) over the block (every thread gets it)
__device__ __forceinline__ int block_sum_before(const int32_t* __restrict__ tile_sums, int n) {
    __shared__ int ws[kScanThreads / 32];
    int v = 0;
    for (int i = threadIdx.x; i < n; i += kScanThreads) v += __ldg(tile_sums + i);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
    __syncthreads();
    int s = 0;
#pragma unroll
    for (int w = 0; w < kScanThreads / 32; ++w) s += ws[w];
    return s;
}

// tile_prefix: the exclusive scan of the tile sums, or (direct) the tile sums
// themselves, this block adding up those before it
template <bool kDirect>
__global__ void __launch_bounds__(kScanThreads)
k_tile_scan(const int32_t* __restrict__ vcount, int v_total, const int32_t* __restrict__ tile_prefix,
            int32_t* __restrict__ vstart) {
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int v[kScanItems];
    const bool full = (blockIdx.x + 1) * kScanTile <= v_total;
    if (full) {
        const int4* v4 = reinterpret_cast<const int4*>(vcount + base);
#pragma unroll
        for (int i = 0; i < kScanItems / 4; ++i) {
            int4 q = __ldg(v4 + i);
            v[4 * i] = q.x; v[4 * i + 1] = q.y; v[4 * i + 2] = q.z; v[4 * i + 3] = q.w;
        }
    } else {
#pragma unroll
        for (int i = 0; i < kScanItems; ++i) v[i] = base + i < v_total ? __ldg(vcount + base + i) : 0;
    }
    int tsum = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) tsum += v[i];
    int total = 0;
    const int before = kDirect ? block_sum_before(tile_prefix, blockIdx.x)
                               : __ldg(tile_prefix + blockIdx.x);
    int run = block_excl_scan(tsum, total) + before;
    int out[kScanItems];
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) { out[i] = run; run += v[i]; }
    if (full) {
        int4* o4 = reinterpret_cast<int4*>(vstart + base);
#pragma unroll
        for (int i = 0; i < kScanItems / 4; ++i)
            o4[i] = make_int4(out[4 * i], out[4 * i + 1], out[4 * i + 2], out[4 * i + 3]);
    } else {
#pragma unroll
        for (int i = 0; i < kScanItems; ++i) if (base + i < v_total) vstart[base + i] = out[i];
    }
}

__global__ void __launch_bounds__(512)
k_scatter(int n, const int32_t* __restrict__ cell, const int32_t* __restrict__ slot,
          const int32_t* __restrict__ pid, const int32_t* __restrict__ vstart,
          const int32_t* __restrict__ vcount, int32_t* __restrict__ tmp_pid,
          int32_t* __restrict__ big_list, int32_t* __restrict__ big_count, int big_voxel) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int code = cell[s];
    const int vid = code < 0 ? ~code : code;
    const int sl = slot[s];
    tmp_pid[__ldg(vstart + vid) + sl] = pid[s];
    // overflow buckets (non-finite particles, never walked) keep arrival order
    if (code >= 0 && sl == 0 && __ldg(vcount + vid) > big_voxel)
        big_list[atomicAdd(big_count, 1)] = vid;
}

// One block per big voxel (grid-stride over the list): sorts the voxel's
// member ids ascending with a bitonic network whose comparators all put the
// smaller value at the lower index, so the segment is padded to a power of
// two implicitly (comparators reaching past the end are no-ops).  Segments up
// to kSmemSort ids are sorted in shared memory, longer ones in place in global
// memory.
constexpr int kSortThreads = 1024;
constexpr int kSmemSort = 8192;

__device__ __forceinline__ void bitonic_pass(int32_t* a, int c, int n2, int k, int j) {
    const int half = n2 >> 1;
    for (int t = threadIdx.x; t < half; t += kSortThreads) {
        int i, p;
        if (j == (k >> 1)) {            // first step of a merge: mirror within the k-block
            i = (t / j) * k + (t % j);
            p = i ^ (k - 1);
        } else {                        // half-cleaner
            i = (t / j) * 2 * j + (t % j);
            p = i + j;
        }
        if (p < c) {
            const int32_t x = a[i], y = a[p];
            if (y < x) { a[i] = y; a[p] = x; }
        }
    }
}

__global__ void __launch_bounds__(kSortThreads)
k_sort_big(const int32_t* __restrict__ big_list, const int32_t* __restrict__ big_count,
           const int32_t* __restrict__ vstart, const int32_t* __restrict__ vcount,
           int32_t* __restrict__ tmp_pid) {
    __shared__ int32_t sm[kSmemSort];
    const int nb = *big_count;
    for (int b = blockIdx.x; b < nb; b += gridDim.x) {
        const int vid = big_list[b];
        const int st = vstart[vid], c = vcount[vid];
        int n2 = 1;
        while (n2 < c) n2 <<= 1;
        const bool in_smem = n2 <= kSmemSort;
        int32_t* a = in_smem ? sm : tmp_pid + st;
        if (in_smem)
            for (int i = threadIdx.x; i < c; i += kSortThreads) sm[i] = tmp_pid[st + i];
        __syncthreads();
        for (int k = 2; k <= n2; k <<= 1)
            for (int j = k >> 1; j > 0; j >>= 1) {
                bitonic_pass(a, c, n2, k, j);
                __syncthreads();
            }
        if (in_smem)
            for (int i = threadIdx.x; i < c; i += kSortThreads) tmp_pid[st + i] = sm[i];
        __syncthreads();
    }
}

__global__ void __launch_bounds__(512)
k_rank_gather(int n, const int32_t* __restrict__ cell, const int32_t* __restrict__ pid,
              const int32_t* __restrict__ tmp_pid, const int32_t* __restrict__ vstart,
              const int32_t* __restrict__ vcount, const float4* __restrict__ pos,
              const float4* __restrict__ vel, const double* __restrict__ pos64,
              float4* __restrict__ pos_out, float4* __restrict__ vel_out,
              int32_t* __restrict__ pid_out, double* __restrict__ pos64_out,
              int2* __restrict__ tasks, int32_t* __restrict__ task_count, int big_voxel,
              const int32_t* __restrict__ slot, const int32_t* __restrict__ pbegin, int n_scenes,
              const int32_t* __restrict__ step_limit, const int32_t* __restrict__ scene_step) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    if (step_limit && scene_frozen(step_limit, scene_step, scene_of(s, pbegin, n_scenes))) {
        // frozen scene: every particle keeps its slot, no density task
        pid_out[s] = pid[s];
        pos_out[s] = __ldg(pos + s);
        if (vel) vel_out[s] = __ldg(vel + s);
        if (pos64) {
            pos64_out[3 * s + 0] = pos64[3 * s + 0];
            pos64_out[3 * s + 1] = pos64[3 * s + 1];
            pos64_out[3 * s + 2] = pos64[3 * s + 2];
        }
        return;
    }
    const int code = cell[s];
    const int vid = code < 0 ? ~code : code;
    const int p = pid[s];
    const int st = __ldg(vstart + vid);
    const int c = __ldg(vcount + vid);
    int r = 0;
    if (code < 0) {
        r = slot[s];                    // overflow bucket: arrival order, no pid order
    } else if (c <= big_voxel) {
        // the voxel's ids four per load from the aligned quad at or before st;
        // entries outside [st, st + c) are masked (tmp_pid is 16-byte aligned
        // and padded by 4 entries, so the last quad stays inside it)
        const int e = st + c;
        for (int k = st & ~3; k < e; k += 4) {
            const int4 q = __ldg(reinterpret_cast<const int4*>(tmp_pid + k));
            r += (k >= st && q.x < p) + (k + 1 >= st && k + 1 < e && q.y < p) +
                 (k + 2 >= st && k + 2 < e && q.z < p) + (k + 3 < e && q.w < p);
        }
    } else {                            // sorted by k_sort_big: lower bound of p
        int lo = 0, hi = c;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (__ldg(tmp_pid + st + mid) < p) lo = mid + 1; else hi = mid;
        }
        r = lo;
    }
    const int d = st + r;
    if (tasks && (r % kTaskRun) == 0) tasks[atomicAdd(task_count, 1)] = make_int2(vid, d);
    pid_out[d] = p;
    pos_out[d] = __ldg(pos + s);
    if (vel) vel_out[d] = __ldg(vel + s);   // null: velocities gathered later
    if (pos64) {
        pos64_out[3 * d + 0] = pos64[3 * s + 0];
        pos64_out[3 * d + 1] = pos64[3 * s + 1];
        pos64_out[3 * d + 2] = pos64[3 * s + 2];
    }
}

}  // namespace

int scan_tiles(int v_total) { return (v_total + kScanTile - 1) / kScanTile; }

cudaError_t launch_hash_count(const Launch& L, const float4* pos, int32_t* cell, int32_t* slot,
                              int32_t* vcount, int i0, int i1) {
    if (i1 < 0) i1 = L.n;
    if (i0 < 0 || i1 > L.n || i0 > i1) return cudaErrorInvalidValue;
    if (i1 == i0) return cudaSuccess;
    const int b = L.sort_block;
    k_hash_count<<<(i1 - i0 + b - 1) / b, b, 0, L.stream>>>(L.scenes, L.pbegin, L.n_scenes, i0,
                                                            i1, pos, cell, slot, vcount);
    return cudaGetLastError();
}

cudaError_t launch_scan(const Launch& L, const int32_t* vcount, int32_t* vstart,
                        int32_t* tile_sums, int n_tiles) {
    if (L.v_total == 0) return cudaSuccess;
    k_tile_reduce<<<n_tiles, kScanThreads, 0, L.stream>>>(vcount, L.v_total, tile_sums);
    if (n_tiles <= kScanDirectTiles) {
        k_tile_scan<true><<<n_tiles, kScanThreads, 0, L.stream>>>(vcount, L.v_total, tile_sums,
                                                                   vstart);
    } else {
        k_scan_tile_sums<<<1, kScanThreads, 0, L.stream>>>(tile_sums, n_tiles);
        k_tile_scan<false><<<n_tiles, kScanThreads, 0, L.stream>>>(vcount, L.v_total, tile_sums,
                                                                    vstart);
    }
    return cudaGetLastError();
}

cudaError_t launch_scatter(const Launch& L, const int32_t* cell, const int32_t* slot,
                           const int32_t* pid, const int32_t* vstart, const int32_t* vcount,
                           int32_t* tmp_pid, int32_t* big_list, int32_t* big_count) {
    if (L.n == 0) return cudaSuccess;
    const int b = L.sort_block;
    k_scatter<<<(L.n + b - 1) / b, b, 0, L.stream>>>(L.n, cell, slot, pid, vstart, vcount, tmp_pid,
                                                     big_list, big_count, L.big_voxel);
    return cudaGetLastError();
}

cudaError_t launch_sort_big(const Launch& L, const int32_t* big_list, const int32_t* big_count,
                            const int32_t* vstart, const int32_t* vcount, int32_t* tmp_pid) {
    if (L.n == 0) return cudaSuccess;
    // one block per SM: enough for the rare big voxels, idle blocks exit at once
    k_sort_big<<<device_sm_count(), kSortThreads, 0, L.stream>>>(big_list, big_count, vstart,
                                                                 vcount, tmp_pid);
    return cudaGetLastError();
}

cudaError_t launch_rank_gather(const Launch& L, const int32_t* cell, const int32_t* slot,
                               const int32_t* pid, const int32_t* tmp_pid, const int32_t* vstart,
                               const int32_t* vcount, const float4* pos, const float4* vel,
                               const double* pos64, float4* pos_out, float4* vel_out,
                               int32_t* pid_out, double* pos64_out, int2* tasks,
                               int32_t* task_count) {
    if (L.n == 0) return cudaSuccess;
    const int b = L.sort_block;
    k_rank_gather<<<(L.n + b - 1) / b, b, 0, L.stream>>>(L.n, cell, pid, tmp_pid, vstart, vcount,
                                                         pos, vel, pos64, pos_out, vel_out,
                                                         pid_out, pos64_out, tasks, task_count,
                                                         L.big_voxel, slot, L.pbegin, L.n_scenes,
                                                         L.step_limit, L.scene_step);
    return cudaGetLastError();
}

}  // namespace sphgb
