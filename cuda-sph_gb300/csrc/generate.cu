// generate.cu -- start states on the device and the headless point-field
// vertex stage, one thread per particle.
//
// Start states replace the host loops of the reference's config.py:79-121
// (__start_state_box_wall, __start_state_inside_pipe), which take minutes in
// Python at millions of particles, and its spawn_particles_inside_pipe_kernel
// (sim/src/sph/kernels/base_kernels.py:130-143).  Every draw is a
// counter-based Philox4x32-10 uniform keyed by (seed, particle id), so the
// state does not depend on the grid shape.
//
// The point-field stage is the per-vertex arithmetic of the visualiser
// (vis/assets/point_field.vert:14-23, point_field.frag:5-9) written to device
// buffers; there is no window or graphics API behind it.
#include <cmath>

#include "sphgb_internal.cuh"

#include "../../include/sphgb.h"

namespace sphgb {

namespace {

constexpr uint32_t kGenStep = 0xFFFFFFFFu;   // counter word 1 of every start-state draw
constexpr double kPi = 3.141592653589793;    // math.pi

__device__ __forceinline__ double gen_u(uint64_t seed, uint32_t id, uint32_t draw) {
    return philox_uniform(seed, id, kGenStep, draw);
}

// Box-Muller transform (Box and Muller, 1958) of draws d and d + 1; 1 - u
// lies in (0, 1], so the logarithm is finite
__device__ __forceinline__ double gen_normal(uint64_t seed, uint32_t id, uint32_t d) {
    const double u1 = __dsub_rn(1.0, gen_u(seed, id, d));
    const double u2 = gen_u(seed, id, d + 1);
    const double r = __dsqrt_rn(__dmul_rn(-2.0, log(u1)));
    return __dmul_rn(r, cos(__dmul_rn(__dmul_rn(u2, 2.0), kPi)));
}

__global__ void __launch_bounds__(kBlock)
k_generate(SphgbGenerator g, const double* __restrict__ pipe, int pipe_rows, int64_t n,
           double* __restrict__ pos, double* __restrict__ vel) {
    const PipeView P{pipe, pipe_rows};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t id = (uint32_t)i;
        double p[3], v[3];
        bool normal_v = false;
        if (g.kind == SPHGB_GEN_LATTICE) {
            const int64_t ny = g.lattice[1], nz = g.lattice[2];
            const int64_t idx[3] = {i / (ny * nz), (i / nz) % ny, i % nz};
            for (int a = 0; a < 3; ++a) {
                double base = __dmul_rn(__dadd_rn((double)idx[a], 0.5), g.spacing);
                base = __dadd_rn(g.origin[a], base);
                const double u = gen_u(g.seed, id, a);
                p[a] = __dadd_rn(base, __dmul_rn(g.jitter, __dsub_rn(__dmul_rn(2.0, u), 1.0)));
                v[a] = g.velocity[a];
            }
            normal_v = g.velocity_sigma != 0.0;
        } else if (g.kind == SPHGB_GEN_BOX_WALL) {
            // config.py:80-95
            for (int a = 0; a < 3; ++a) {
                p[a] = __dmul_rn(gen_u(g.seed, id, a), g.extent[a]);
                const double u = gen_u(g.seed, id, 3 + a);
                v[a] = __dadd_rn(g.velocity[a], __dmul_rn(__dsub_rn(u, 0.5), g.velocity_spread));
            }
        } else {
            // config.py:103-112 with rand_position_inside_pipe (base_kernels.py:102-112)
            const double u0 = gen_u(g.seed, id, 0);
            p[0] = __dadd_rn(g.x_range[0], __dmul_rn(u0, __dsub_rn(g.x_range[1], g.x_range[0])));
            p[1] = p[2] = 0.0;
            int seg = pipe_find_segment(p, P);
            if (seg < 0) seg = 0;
            const double R = pipe_radius(p, P, seg);
            const double r = __dmul_rn(__dmul_rn(__dsqrt_rn(gen_u(g.seed, id, 1)), R), g.fill);
            const double th = __dmul_rn(__dmul_rn(gen_u(g.seed, id, 2), 2.0), kPi);
            p[1] = __dadd_rn(P.at(0, 1), __dmul_rn(r, cos(th)));
            p[2] = __dadd_rn(P.at(0, 2), __dmul_rn(r, sin(th)));
            for (int a = 0; a < 3; ++a) v[a] = g.velocity[a];
            normal_v = g.velocity_sigma != 0.0;
        }
        if (normal_v)
            for (int a = 0; a < 3; ++a)
                v[a] = __dadd_rn(v[a], __dmul_rn(g.velocity_sigma, gen_normal(g.seed, id, 3 + 2 * a)));
        for (int a = 0; a < 3; ++a) {
            pos[3 * i + a] = p[a];
            vel[3 * i + a] = v[a];
        }
    }
}

struct Mat4 {
    float m[16];   // column-major: m[c * 4 + r]
};

// column-major product a * b, one rounding per multiply and add, k = 0..3
__device__ __forceinline__ float mat_elem(const float* a, const float* b, int r, int c) {
    float s = __fmul_rn(a[r], b[c * 4]);
#pragma unroll
    for (int k = 1; k < 4; ++k) s = __fadd_rn(s, __fmul_rn(a[k * 4 + r], b[c * 4 + k]));
    return s;
}

__global__ void __launch_bounds__(kBlock)
k_point_field(const float* __restrict__ pos, int stride, const float* __restrict__ rho, int64_t n,
              Mat4 proj, Mat4 model, Mat4 view, float4* __restrict__ clip,
              float4* __restrict__ colour, float* __restrict__ size) {
    // uProjMat * uViewMat * uModelMat * v evaluates as ((P V) M) v
    __shared__ float pv[16], pvm[16];
    if (threadIdx.x < 16) pv[threadIdx.x] = mat_elem(proj.m, view.m, threadIdx.x & 3, threadIdx.x >> 2);
    __syncthreads();
    if (threadIdx.x < 16) pvm[threadIdx.x] = mat_elem(pv, model.m, threadIdx.x & 3, threadIdx.x >> 2);
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float x[4] = {pos[i * stride], pos[i * stride + 1], pos[i * stride + 2], 1.0f};
        float c[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            float s = __fmul_rn(pvm[r], x[0]);
#pragma unroll
            for (int k = 1; k < 4; ++k) s = __fadd_rn(s, __fmul_rn(pvm[k * 4 + r], x[k]));
            c[r] = s;
        }
        clip[i] = make_float4(c[0], c[1], c[2], c[3]);
        const float t = fminf(__fdiv_rn(rho[i], 10.0f), 1.0f);
        const float omt = __fsub_rn(1.0f, t);
        // mix(a, b * 0.7, t) = a (1 - t) + (b * 0.7) t
        const float b0 = __fmul_rn(0.3f, 0.7f), b1 = __fmul_rn(0.4f, 0.7f), b2 = 0.7f;
        colour[i] = make_float4(__fadd_rn(__fmul_rn(0.1f, omt), __fmul_rn(b0, t)),
                                __fadd_rn(__fmul_rn(0.7f, omt), __fmul_rn(b1, t)),
                                __fadd_rn(__fmul_rn(0.5f, omt), __fmul_rn(b2, t)), 0.5f);
        const float big = __fadd_rn(40.0f, __fmul_rn(omt, 20.0f));
        size[i] = fminf(fmaxf(1.0f, __fdiv_rn(big, c[2])), 13.0f);
    }
}

// grid-stride launches: at most 64 blocks per SM
int grid_for(int64_t n) {
    const int64_t b = (n + kBlock - 1) / kBlock;
    const int64_t top = (int64_t)device_sm_count() * 64;
    return (int)(b < top ? b : top);
}

}  // namespace

cudaError_t launch_generate(const SphgbGenerator& g, const double* pipe, int pipe_rows, int64_t n,
                            double* pos, double* vel, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_generate<<<grid_for(n), kBlock, 0, st>>>(g, pipe, pipe_rows, n, pos, vel);
    return cudaGetLastError();
}

cudaError_t launch_point_field(const float* pos, int stride, const float* rho, int64_t n,
                               const float* proj16, const float* model16, const float* view16,
                               float* clip, float* colour, float* size, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    Mat4 P, M, V;
    for (int k = 0; k < 16; ++k) {
        P.m[k] = proj16[k];
        M.m[k] = model16[k];
        V.m[k] = view16[k];
    }
    k_point_field<<<grid_for(n), kBlock, 0, st>>>(pos, stride, rho, n, P, M, V,
                                                   reinterpret_cast<float4*>(clip),
                                                   reinterpret_cast<float4*>(colour), size);
    return cudaGetLastError();
}

}  // namespace sphgb
