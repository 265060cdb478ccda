/*
 * sphgb.h -- C ABI of the GB300 (sm_103a) SPH step library, libsphgb.so.
 *
 * The library replaces the per-step path of iwoplaza/cuda-sph's voxel strategy,
 * VoxelSPHStrategy.compute_next_state (sim/src/sph/strategies/
 * abstract_sph_strategy.py:31-46 with voxel_sph_strategy.py:20-116): voxel hash,
 * voxel sort and voxel_begin table, the 27-voxel neighbour walk, density,
 * pressure and viscosity terms, integration and the box or pipe wall response.
 *
 * Conventions
 *  - Every entry point returns an int status: SPHGB_OK (0) or a negative
 *    SPHGB_ERR_*; sphgb_last_error() returns a message for the calling thread.
 *    No C++ exception crosses this boundary.
 *  - Pointers named d_* are device pointers, h_* host pointers.  The library
 *    never frees caller memory.  Scratch buffers are owned by a context.
 *  - `stream` is a cudaStream_t passed as void* (0 = legacy default stream).
 *    Work is enqueued asynchronously unless the entry point says otherwise.
 *  - A context is not thread-safe; use one context per host thread.
 *  - Particle state on the device is FP32: position and velocity as float4
 *    (x, y, z, unused) per particle, density as float, particle ids as int32.
 *    Device state is kept in voxel-sorted order; d_pid[s] names the original
 *    particle at sorted slot s.  The stage entry points sort by the
 *    reference's row-major voxel ids; the context's own step may number the
 *    voxels of sparse scenes in 4x4x4 tiles instead, so the slot order of a
 *    bound state after sphgb_ctx_step is a permutation of that (same
 *    particles, same results in original order, read through d_pid).
 */
#ifndef SPHGB_H
#define SPHGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPHGB_ABI_VERSION 1

enum {
    SPHGB_OK = 0,
    SPHGB_ERR_INVALID = -1,   /* bad argument (null pointer, size, mode) */
    SPHGB_ERR_CUDA = -2,      /* a CUDA runtime call failed */
    SPHGB_ERR_NOMEM = -3,     /* device allocation failed */
    SPHGB_ERR_STATE = -4,     /* call out of order (e.g. step before bind) */
    SPHGB_ERR_RANGE = -5      /* a size is beyond a documented limit */
};

enum { SPHGB_MODE_BOX = 0, SPHGB_MODE_PIPE = 1 };      /* config.SIM_MODE (config.py:13) */
enum { SPHGB_WALK_CEIL = 0, SPHGB_WALK_TRUNCATED = 1 }; /* see walk_dims below */
/* sphgb_ctx_set_tuning */
enum { SPHGB_DENSITY_WARP = 0, SPHGB_DENSITY_THREAD = 1 };

/*
 * One scene: SimulationParameters (common/data_classes.py:70-78) plus the
 * physics constants the reference freezes from config.py:18-30 at JIT time.
 * Doubles are rounded to FP32 on the device; pass FP32-representable values for
 * bit-comparable results against an FP64 implementation.
 */
typedef struct SphgbSceneParams {
    int64_t particle_count;    /* SimulationParameters.particle_count */
    double space_size[3];      /* SimulationParameters.space_size (box extent) */
    double voxel_size[3];      /* SimulationParameters.voxel_size */
    double external_force[3];  /* SimulationParameters.external_force */
    double dt;                 /* 1 / fps (abstract_sph_strategy.py:20) */
    double mass;               /* MASS   (config.py:18) */
    double rho_0;              /* RHO_0  (config.py:19) */
    double inf_r;              /* INF_R  (config.py:20), the smoothing radius h */
    double visc;               /* VISC   (config.py:21) */
    double k;                  /* K      (config.py:22), gas constant */
    double damp;               /* DAMP   (config.py:23), wall restitution */
    int32_t max_neighbours;    /* MAX_NEIGHBOURS (config.py:30); <= 0 means no cap */
    int32_t mode;              /* SPHGB_MODE_BOX or SPHGB_MODE_PIPE */
    /* Voxel dims used by the neighbour walk.  The voxel table always uses
     * ceil(space/voxel) (voxel_sph_strategy.py:70-73).  SPHGB_WALK_CEIL walks
     * with the same dims.  SPHGB_WALK_TRUNCATED reproduces the reference's
     * walk exactly: it builds neighbour voxel ids with int(space/voxel)
     * (voxel_sph_strategy.py:110-116), which differ from the table's dims when
     * space is not a multiple of the voxel size. */
    int32_t walk_dims;
    int32_t pipe_rows;         /* rows of Pipe.to_numpy() (segments + 1); 0 in box mode */
    int64_t pipe_row_offset;   /* first row of this scene in the pipe table */
    uint64_t seed;             /* respawn random stream key (abstract_sph_strategy.py:27) */
} SphgbSceneParams;

#ifndef SPHGB_NO_FUNCTIONS

typedef struct SphgbCtx SphgbCtx;

/* ---- library ---------------------------------------------------------- */
int sphgb_abi_version(void);
/* sizeof(SphgbSceneParams), for binding checks. */
int sphgb_scene_params_size(void);
/* Message of the last failing call on this host thread ("" if none). */
const char* sphgb_last_error(void);

/* ---- context ----------------------------------------------------------
 * A context advances one or more independent scenes together.  With one
 * scene it is the reference's strategy object (AbstractSPHStrategy.__init__,
 * abstract_sph_strategy.py:18-29); with many it is the batched path.
 * pipe_rows_table: host doubles [total rows][5] in Pipe.to_numpy() layout
 * (common/data_classes.py:34-44); may be NULL when no scene is in pipe mode.
 * Allocates all scratch with cudaMalloc on the current device.  At most
 * SPHGB_MAX_PARTICLES particles over all scenes (SPHGB_ERR_RANGE beyond). */
#define SPHGB_MAX_PARTICLES (1 << 29)
int sphgb_ctx_create(const SphgbSceneParams* scenes, int n_scenes,
                     const double* pipe_rows_table, int n_pipe_rows_total,
                     SphgbCtx** out_ctx);
int sphgb_ctx_destroy(SphgbCtx* ctx);
/* Replace the context's scenes (same arguments as sphgb_ctx_create), reusing
 * every scratch buffer that is still large enough.  Synchronises the device.
 * Bound state and outputs are unbound: bind state for the new layout before
 * stepping.  Used by request servers whose scene set changes between batches;
 * the reference creates one strategy per run instead (state_generator.py:21-23). */
int sphgb_ctx_reconfigure(SphgbCtx* ctx, const SphgbSceneParams* scenes, int n_scenes,
                          const double* pipe_rows_table, int n_pipe_rows_total);
/* Launch tuning (results do not change): threads per block of the
 * per-particle sort kernels (128, 256, 512), the density kernel variant
 * (SPHGB_DENSITY_WARP: one warp per voxel run, one lane per candidate;
 * SPHGB_DENSITY_THREAD: one thread per particle) and the member count above which a voxel is sorted by
 * a block of its own (16..4096).  No counterpart in the reference (numba picks
 * one block size per device, thread_layout.py:27-33). */
int sphgb_ctx_set_tuning(SphgbCtx* ctx, int sort_block, int density_variant, int big_voxel);
/* Total particles / voxel-table entries over all scenes of the context.  A
 * scene's table has ceil(space/voxel) voxels plus one overflow entry (last)
 * that collects particles with non-finite coordinates; no walk visits it. */
int sphgb_ctx_sizes(const SphgbCtx* ctx, int64_t* n_particles, int64_t* n_voxels);

/* Bind caller-owned device state (voxel-sorted order, see conventions).
 * d_pos64 (3 doubles per particle) is required when any scene is in pipe mode
 * (FP64 position accumulator) and ignored otherwise.  d_scene_step: one int32
 * per scene, the number of steps each scene has taken. */
int sphgb_ctx_bind_state(SphgbCtx* ctx, float* d_pos, float* d_vel, float* d_rho,
                         int32_t* d_pid, double* d_pos64, int32_t* d_scene_step);

/* Optional: write the next state of every step to separate buffers instead
 * of back into the bound state, which is then left unchanged (repeated steps
 * all start from it).  Pass four NULLs to return to in-place stepping.
 * d_pos64_out is required when any scene is in pipe mode. */
int sphgb_ctx_bind_output(SphgbCtx* ctx, float* d_pos_out, float* d_vel_out, int32_t* d_pid_out,
                          double* d_pos64_out);

/* Load state from FP64 AoS arrays in original particle order (the layout of
 * SimulationState.position / .velocity, common/data_classes.py:81-85) already
 * on the device; sets pid = identity and the FP64 accumulator. */
int sphgb_ctx_load_aos_f64(SphgbCtx* ctx, const double* d_pos_aos, const double* d_vel_aos,
                           void* stream);
/* Write the latest state (the output buffers when bound with
 * sphgb_ctx_bind_output, else the bound state) as FP64 AoS in original
 * particle order; d_rho receives the density of the latest step. */
int sphgb_ctx_store_aos_f64(SphgbCtx* ctx, double* d_pos_aos, double* d_vel_aos,
                            double* d_rho, void* stream);

/* Optional per-scene step limits: d_limits holds one int32 per scene on the
 * device (NULL removes them).  A scene whose step counter (d_scene_step of
 * sphgb_ctx_bind_state) has reached its limit is frozen: later steps leave its
 * position, velocity, density, particle order and step counter unchanged
 * (its particles still pass through the voxel hash).  One launch, or one
 * captured graph, can so advance each scene of a batch by its own number of
 * steps.  The array is read on the device at every step, so new values need
 * no new call; a different pointer drops the context's captured graphs.
 * Reconfiguring the context removes the limits.  No counterpart in the
 * reference, which advances one scene per strategy object
 * (state_generator.py:21-23). */
int sphgb_ctx_set_step_limits(SphgbCtx* ctx, const int32_t* d_limits);

/* Advance every scene n_steps steps (compute_next_state, repeated) on the
 * bound state.  With use_graph != 0 the n_steps sequence is captured once
 * into a CUDA graph and replayed on later calls with the same n_steps. */
int sphgb_ctx_step(SphgbCtx* ctx, int n_steps, int use_graph, void* stream);

/* Advance n_steps steps without a graph, with a CUDA event after every
 * stage; synchronises the stream and writes the mean milliseconds per step of
 * each stage to h_stage_ms[SPHGB_PROFILE_STAGES]:
 * [hash+histogram (with the histogram clear), scan, scatter, rank-gather,
 *  density, force+integrate+wall, step counter]. */
#define SPHGB_PROFILE_STAGES 7
int sphgb_ctx_step_profiled(SphgbCtx* ctx, int n_steps, void* stream, float* h_stage_ms);

/* The reference's boundary with host buffers: FP64 AoS state in, next FP64
 * AoS state out, synchronous (AbstractSPHStrategy.compute_next_state,
 * abstract_sph_strategy.py:31-46, including its host<->device copies at
 * :65-74 and :77-84).  Context must hold exactly one scene.  Host buffers may
 * be pageable or page-locked (page-locked copies faster, and only they let
 * the copies overlap the step); they are copied through device staging
 * buffers.  A call that fails returns only after every copy it started has
 * finished. */
int sphgb_compute_next_state_host(SphgbCtx* ctx, const double* h_pos, const double* h_vel,
                                  double* h_pos_out, double* h_vel_out, double* h_rho_out);
/* Order in which sphgb_compute_next_state_host runs its force pass (results
 * do not change).  SPHGB_HOST_ORDER_SLOT: voxel-sorted order, then the next
 * state is downloaded whole.  SPHGB_HOST_ORDER_PARTICLE: original particle
 * order in ranges, each range's rows downloaded while the next range is
 * computed; faster when nearby particle ids are nearby in space, slower when
 * they are scattered.  SPHGB_HOST_ORDER_PIPELINED: the density pass in 16
 * buckets of tasks by the particle-id range of their first particle, the
 * force pass over each bucket's slots once every bucket its particles'
 * neighbours fall in is done, and each range's rows downloaded as soon as
 * the buckets holding its particles are, while later buckets are still
 * running (when ids follow space, most of the download overlaps the density
 * pass).  It needs one scene with a neighbour cap of at most 32, the
 * reference's walk dims set to SPHGB_WALK_CEIL, the warp density kernel, at
 * least 512 particles and no step limits, and is particle order otherwise.
 * SPHGB_HOST_ORDER_AUTO (default): calls 1 to 3 run the three orders once,
 * calls 4 to 6 time them and later calls take the fastest.
 * No counterpart in the reference (its step is synchronous,
 * abstract_sph_strategy.py:31-46). */
enum { SPHGB_HOST_ORDER_AUTO = 0, SPHGB_HOST_ORDER_SLOT = 1, SPHGB_HOST_ORDER_PARTICLE = 2,
       SPHGB_HOST_ORDER_PIPELINED = 3 };
int sphgb_ctx_set_host_order(SphgbCtx* ctx, int order);

/* Per-scene conservation sums in FP64, fixed summation order (identical for a
 * scene whether it runs alone or batched).  d_out: 8 doubles per scene:
 * [mass, px, py, pz, kinetic, potential, kinetic + potential, particles].
 * Potential energy is -m g.x with g = external_force. */
int sphgb_ctx_conservation(SphgbCtx* ctx, double* d_out, void* stream);

/* Neighbour statistics of the bound state at its current positions: capped
 * and uncapped neighbour counts (self included) per particle, in original
 * particle order (scene-concatenated).  Uses the context's scratch buffers. */
int sphgb_ctx_neighbour_counts(SphgbCtx* ctx, int32_t* d_capped, int32_t* d_uncapped,
                               void* stream);

/* The neighbour lists of the latest step of the context (sphgb_ctx_step or
 * sphgb_compute_next_state_host), as that step's density pass recorded them
 * and its force pass read them.  Row i (original particle order, scenes
 * concatenated; 32 int32 per particle) holds particle i's neighbours other
 * than itself in the reference's walk order, that is get_neighbours'
 * capped list (voxel_kernels.py:30-85) with the particle itself taken out, as
 * scene-local particle ids, -1 padded.  d_count[i] is their number, or -1
 * when there were more than 32 (a scene with no cap; that row is all -1).
 * Either pointer may be NULL.  SPHGB_ERR_STATE until a step has run, and
 * again after sphgb_ctx_neighbour_counts or a reconfiguration, which re-sort
 * the context's buffers. */
int sphgb_ctx_step_neighbours(SphgbCtx* ctx, int32_t* d_list, int32_t* d_count, void* stream);

/* Checked mode (off by default; no cost when off).  With enable != 0 every
 * later step runs one more kernel that validates what the step read and
 * wrote and ORs these bits into the context's error word.  The reference
 * leaves these cases undefined (voxel ids of particles outside the box,
 * voxel_kernels.py:10-17 and :89-105; never-written walk voxels and reads
 * past voxel_begin, :44, :64-65, :70); this library defines its behaviour
 * there (clamped voxel coordinates, an overflow entry for non-finite
 * positions) and the word reports that it happened.  The check
 * compares indices with their ranges before it uses them: bad data sets
 * bits, it never faults.  Toggling drops the context's captured graphs. */
enum {
    SPHGB_CHECK_NONFINITE_INPUT = 1,   /* a position or velocity of the step's input is NaN/inf */
    SPHGB_CHECK_OUT_OF_DOMAIN = 2,     /* a finite position outside [0, space_size) */
    SPHGB_CHECK_VOXEL_TABLE = 4,       /* a slot outside its voxel's range, ids out of order */
    SPHGB_CHECK_NEIGHBOUR_LIST = 8,    /* a list entry out of the scene, self, beyond h, or a
                                          count beyond the cap */
    SPHGB_CHECK_NONFINITE_OUTPUT = 16  /* density or next position/velocity is NaN/inf */
};
int sphgb_ctx_set_checks(SphgbCtx* ctx, int enable);
/* Reads the error word into h_word[3] = {bits, smallest original index of a
 * flagged particle (0xffffffff if none), flagged particle-steps}; with clear
 * != 0 resets it.  Synchronises the stream.  All zero (and 0xffffffff) when
 * checked mode was never enabled. */
int sphgb_ctx_check_word(SphgbCtx* ctx, uint32_t* h_word, int clear, void* stream);

/* ---- stages (each launches the same kernels sphgb_ctx_step uses) ------- */

/* assign_voxels_to_particles_kernel (voxel_kernels.py:89-105): voxel id of
 * each particle (ceil dims; coordinates clamped to the table).  A particle
 * with a non-finite coordinate gets ~id (negative) of its scene's overflow
 * entry, the last entry of the scene's voxel table. */
int sphgb_assign_voxels(SphgbCtx* ctx, const float* d_pos, int32_t* d_voxel_out, void* stream);

/* Voxel sort + voxel_begin (voxel_sph_strategy.py:65-107): stable counting
 * sort by (voxel id, particle id); particles of a scene's overflow entry
 * (non-finite coordinates, never walked) come last, in arrival order.  Reads state (d_pos, d_vel, d_pid) in any
 * order, writes it voxel-sorted to the *_out buffers, and writes the voxel
 * table: d_voxel_start[v] (first sorted slot) and d_voxel_count[v]. */
int sphgb_organize_voxels(SphgbCtx* ctx, const float* d_pos, const float* d_vel,
                          const int32_t* d_pid, const double* d_pos64,
                          float* d_pos_out, float* d_vel_out, int32_t* d_pid_out,
                          double* d_pos64_out, int32_t* d_voxel_start,
                          int32_t* d_voxel_count, void* stream);

/* The voxel organisation of sphgb_organize_voxels without any device
 * allocation, for callers that may not call cudaMalloc (their process forbids
 * it, or all device memory goes through an allocator of their own).  No
 * counterpart in the reference.  No context: the scene is passed directly
 * (one scene; pipe rows are not needed).  Scratch lives in one file-scope
 * __device__ array of fixed size (about 3.2 MB, held by every GPU that loads
 * the library until exit); limits: particle_count <= 262,144 and
 * ceil(space/voxel) voxels + 1 <= 4,194,304, else SPHGB_ERR_RANGE.  The first
 * call on a device looks the array up (cudaGetSymbolAddress) with that device
 * current; make it before any stream capture.  Every call shares the array and
 * it keeps the last call's contents: calls that overlap on the GPU (other
 * streams, other threads) race.  Outputs as sphgb_organize_voxels; the voxel
 * table has ceil dims + 1 entries.  Every buffer must be 16-byte aligned
 * (positions and velocities move as float4, the voxel table in int4 quads):
 * SPHGB_ERR_INVALID names the first one that is not, before any GPU work. */
int sphgb_organize_voxels_noalloc(const SphgbSceneParams* scene, const float* d_pos,
                                  const float* d_vel, const int32_t* d_pid, float* d_pos_out,
                                  float* d_vel_out, int32_t* d_pid_out, int32_t* d_voxel_start,
                                  int32_t* d_voxel_count, void* stream);

/* get_neighbours (voxel_kernels.py:30-85) for every sorted slot: the ordered,
 * capped neighbour list (sorted slots, -1 padded; d_list may be NULL) with
 * list_stride entries per particle, and the capped/uncapped counts. */
int sphgb_neighbours(SphgbCtx* ctx, const float* d_pos_sorted, const int32_t* d_voxel_start,
                     const int32_t* d_voxel_count, int32_t* d_list, int list_stride,
                     int32_t* d_count_capped, int32_t* d_count_uncapped, void* stream);

/* density_kernel (voxel_kernels.py:109-132) on sorted state. */
int sphgb_density(SphgbCtx* ctx, const float* d_pos_sorted, const int32_t* d_voxel_start,
                  const int32_t* d_voxel_count, float* d_rho_out, void* stream);

/* pressure_kernel + viscosity_kernel (voxel_kernels.py:136-211) on sorted
 * state: pressure and viscosity terms as float4 per particle. */
int sphgb_forces(SphgbCtx* ctx, const float* d_pos_sorted, const float* d_vel_sorted,
                 const float* d_rho_sorted, const int32_t* d_voxel_start,
                 const int32_t* d_voxel_count, float* d_pressure_out,
                 float* d_viscosity_out, void* stream);

/* Forces fused with integrating_kernel (base_kernels.py:30-53) and the wall
 * response (collision_kernel_box :75-98 or collision_kernel :56-72): reads
 * sorted state, writes the next state (same slot order) to the *_out buffers
 * and, if d_force_out is not NULL, result_force as float4.  step_index keys
 * the respawn random stream. */
int sphgb_integrate(SphgbCtx* ctx, const float* d_pos_sorted, const float* d_vel_sorted,
                    const float* d_rho_sorted, const int32_t* d_pid_sorted,
                    const double* d_pos64_sorted, const int32_t* d_voxel_start,
                    const int32_t* d_voxel_count, const int32_t* d_scene_step,
                    float* d_pos_out, float* d_vel_out, int32_t* d_pid_out,
                    double* d_pos64_out, float* d_force_out, void* stream);

/* ---- pipe geometry (sim/src/sph/kernels/util_kernels.py), FP64 --------
 * Batch wrappers over the device functions the pipe wall response uses, for
 * the reference's known-answer tests (sim/tests/test_collisions.py). */
int sphgb_pipe_find_segment(const double* d_pos, int n, const double* d_pipe, int pipe_rows,
                            int32_t* d_seg_out, void* stream);
int sphgb_pipe_is_out(const double* d_pos, const int32_t* d_seg, int n, const double* d_pipe,
                      int pipe_rows, int32_t* d_out, double* d_radius_out, void* stream);
int sphgb_pipe_x_at_segment_beginning(const int32_t* d_seg, int n, const double* d_pipe,
                                      int pipe_rows, double* d_out, void* stream);
/* In place: for each particle, find_segment; if out of the pipe, solve_collision. */
int sphgb_pipe_solve_collision(double* d_pos, double* d_vel, int n, const double* d_pipe,
                               int pipe_rows, int32_t* d_seg_out, void* stream);
/* Philox4x32-10 uniforms in [0,1) for (seed, pid, step, draw) -- the respawn stream. */
int sphgb_philox_uniform(uint64_t seed, const int32_t* d_pid, int n, int step, int draw,
                         double* d_out, void* stream);

#endif /* SPHGB_NO_FUNCTIONS */

/* ---- initial states on the device --------------------------------------
 * Replaces the host start-state loops of config.py:79-121
 * (__start_state_box_wall, __start_state_inside_pipe) and the reference's
 * spawn_particles_inside_pipe_kernel (sim/src/sph/kernels/base_kernels.py:
 * 130-143); LATTICE is the jittered dam-break block of the benchmark scenes.
 * Random numbers: Philox4x32-10 uniforms u(draw) = sphgb_philox_uniform(seed,
 * i, step = -1, draw) for particle i, so a state depends only on (generator,
 * n) and not on the launch shape.  Normal deviates use the Box-Muller
 * transform sqrt(-2 ln(1 - u(d))) cos(2 pi u(d + 1)).  Output: FP64 (n, 3)
 * position and velocity in particle-id order, ready for
 * sphgb_ctx_load_aos_f64. */
enum { SPHGB_GEN_LATTICE = 0, SPHGB_GEN_BOX_WALL = 1, SPHGB_GEN_PIPE_FILL = 2 };

typedef struct SphgbGenerator {
    int32_t kind;              /* SPHGB_GEN_* */
    int32_t lattice[3];        /* LATTICE: nx, ny, nz; n must be nx*ny*nz; particle
                                  i = (ix*ny + iy)*nz + iz (C order of the index grid) */
    double spacing;            /* LATTICE: p = origin + (idx + 0.5)*spacing + jitter*(2u - 1),
                                  u = draws 0, 1, 2 */
    double jitter;
    double origin[3];
    double extent[3];          /* BOX_WALL: p = u * extent, draws 0, 1, 2 (config.py:81-88 uses
                                  (0.1*space_x, space_y, space_z)) */
    double velocity[3];        /* every kind: base velocity */
    double velocity_spread;    /* BOX_WALL: v = velocity + (u - 0.5)*spread, draws 3, 4, 5
                                  (config.py:89-95: base (1.5, -5, -5), spread 1) */
    double velocity_sigma;     /* LATTICE, PIPE_FILL: v = velocity + sigma*N(0,1) per axis,
                                  normal draws (3,4), (5,6), (7,8); 0 = velocity exactly */
    double x_range[2];         /* PIPE_FILL: x = x0 + u*(x1 - x0), draw 0 (config.py:104: [0, length)) */
    double fill;               /* PIPE_FILL: r = sqrt(u)*R(x)*fill, draw 1, with R the pipe radius of
                                  calc_radius_in_position (util_kernels.py:56-69); theta =
                                  u*2*pi, draw 2; (y, z) = axis of row 0 + r (cos, sin) theta
                                  (config.py:107-111: fill 0.98; base_kernels.py:102-112: 1) */
    uint64_t seed;
} SphgbGenerator;

#ifndef SPHGB_NO_FUNCTIONS

int sphgb_generator_size(void);   /* sizeof(SphgbGenerator), for binding checks */
/* d_pipe / pipe_rows: the Pipe.to_numpy table on the device (PIPE_FILL only;
 * NULL / 0 otherwise).  x outside the table's rows takes the radius of the
 * first segment. */
int sphgb_generate(const SphgbGenerator* gen, const double* d_pipe, int pipe_rows, int64_t n,
                   double* d_pos, double* d_vel, void* stream);

/* ---- point-field vertex stage, headless --------------------------------
 * The arithmetic of the visualiser's shaders (vis/assets/point_field.vert:
 * 14-23, point_field.frag:5-9) per particle, written to device buffers
 * instead of a window: clip = (((P V) M) (x, y, z, 1)) with the 4x4 product
 * PVM = (P V) M formed once (column-major like GLSL uniforms, FP32, each
 * element summed k = 0..3 with one rounding per multiply and add);
 * t = min(rho / 10, 1); colour = (0.1, 0.7, 0.5)(1 - t) + (0.7 (0.3, 0.4, 1)) t,
 * alpha 0.5; point size = min(max(1, (40 + (1 - t) 20) / clip.z), 13).
 * min and max ignore a NaN operand (fminf / fmaxf).  d_pos has pos_stride
 * floats per particle (3 = packed vertex buffer, 4 = the library's float4). */
int sphgb_point_field(const float* d_pos, int pos_stride, const float* d_rho, int64_t n,
                      const float* h_proj, const float* h_model, const float* h_view,
                      float* d_clip_out, float* d_colour_out, float* d_size_out, void* stream);

#endif /* SPHGB_NO_FUNCTIONS */

#ifdef __cplusplus
}
#endif
#endif /* SPHGB_H */
