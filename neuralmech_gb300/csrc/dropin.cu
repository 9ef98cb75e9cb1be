// Drop-ins for the reference's order-2 step kernels that store the field in
// reduced precision or in 1D (sm_103a): the same arguments, cells and storage
// formats as
//   mixed_step  (projects/18_simple_wave_fd/step2D_wave.cu:85-124): FP16 storage,
//   scaled_step (step2D_wave.cu:128-183): int16 with one FP32 scale per block of
//               32 values along a row, scale = block max / 32767,
//   step1D      (step1D_wave.cu:4-17): the 1D 3-point step.
// The arithmetic of every cell is the reference's expression in its operation
// order, in explicitly rounded IEEE operations (no contraction into FMAs, IEEE
// division), so the results equal a plain IEEE evaluation of the reference
// source value for value.
//
// The reference's row index i runs with dx and its column index j (fastest,
// M of them, padded to M_padded) with dy. Rows 0 and N - 1 and columns 0 and
// M - 1 are the fixed boundary.
#include "../../include/wavefd.h"
#include "common.cuh"
#include "internal.h"

namespace wfd {
namespace {

// u2 = -u0 + 2 u1 + k (lap_i / (dx dx) + lap_j / (dy dy)), k = dt dt c c, with
// lap = (a - 2 c) + b, evaluated left to right as the reference writes it.
__device__ __forceinline__ float update2d(float u0, float u1, float il, float ir, float jl, float jr,
                                          float k, float dx2, float dy2) {
    const float two_c = __fmul_rn(2.f, u1);
    const float li = __fadd_rn(__fsub_rn(il, two_c), ir);
    const float lj = __fadd_rn(__fsub_rn(jl, two_c), jr);
    const float lap = __fadd_rn(__fdiv_rn(li, dx2), __fdiv_rn(lj, dy2));
    return __fadd_rn(__fadd_rn(-u0, two_c), __fmul_rn(k, lap));
}

// 1D: one thread per cell of 0 < i < N - 1.
__global__ void step1d_kernel(const float* __restrict__ u0, const float* __restrict__ u1,
                              float* __restrict__ u2, float k, float dx2, int N) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i <= 0 || i >= N - 1) return;
    const float c = u1[i];
    const float lap = __fdiv_rn(__fadd_rn(__fsub_rn(u1[i - 1], __fmul_rn(2.f, c)), u1[i + 1]), dx2);
    u2[i] = __fadd_rn(__fadd_rn(-u0[i], __fmul_rn(2.f, c)), __fmul_rn(k, lap));
}

// FP16 storage: a thread owns the pair (j, j + 1), j even, of row i, loaded and
// stored as one __half2.
__global__ void mixed_kernel(const __half* __restrict__ u0, const __half* __restrict__ u1,
                             __half* __restrict__ u2, float k, float dx2, float dy2, int N, int M,
                             int Mp) {
    const int j = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i <= 0 || i >= N - 1 || j >= M) return;
    const size_t c = (size_t)i * Mp + j;
    const float2 a = __half22float2(*reinterpret_cast<const __half2*>(u0 + c));
    const float2 b = __half22float2(*reinterpret_cast<const __half2*>(u1 + c));
    const float2 up = __half22float2(*reinterpret_cast<const __half2*>(u1 + c - Mp));
    const float2 dn = __half22float2(*reinterpret_cast<const __half2*>(u1 + c + Mp));
    const float left = j > 0 ? __half2float(u1[c - 1]) : 0.f;
    const float right = __half2float(u1[c + 2]);
    const float v0 = update2d(a.x, b.x, up.x, dn.x, left, b.y, k, dx2, dy2);
    const float v1 = update2d(a.y, b.y, up.y, dn.y, b.x, right, k, dx2, dy2);
    if (j > 0 && j + 1 < M - 1) {
        *reinterpret_cast<__half2*>(u2 + c) = __floats2half2_rn(v0, v1);
    } else {
        if (j > 0 && j < M - 1) u2[c] = __float2half_rn(v0);
        if (j + 1 < M - 1) u2[c + 1] = __float2half_rn(v1);
    }
}

// Block-scaled int16: a thread owns 4 values (j .. j + 3, j a multiple of 4) of
// row i; the 8 lanes of an aligned lane octet hold one 32-value block and
// share its scale. Rows of the warp: a warp covers 128 columns of one row.
__global__ void scaled_kernel(const short* __restrict__ q0, const float* __restrict__ s0,
                              const short* __restrict__ q1, const float* __restrict__ s1,
                              short* __restrict__ q2, float* __restrict__ s2, float k, float dx2,
                              float dy2, int N, int M, int Mp) {
    const int j = 4 * (blockIdx.x * blockDim.x + threadIdx.x);
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i <= 0 || i >= N - 1) return;  // whole warps: blockDim.x is a multiple of 32
    const bool live = j < Mp;           // (Mp % 64 == 0: a lane octet is all live or all not)
    const int S = Mp / 32;              // blocks per row
    const size_t c = (size_t)i * Mp + j;
    const size_t b = (size_t)i * S + j / 32;
    float v[4] = {0.f, 0.f, 0.f, 0.f};
    if (live) {
        const short4 p0 = *reinterpret_cast<const short4*>(q0 + c);
        const short4 p1 = *reinterpret_cast<const short4*>(q1 + c);
        const short4 pu = *reinterpret_cast<const short4*>(q1 + c - Mp);
        const short4 pd = *reinterpret_cast<const short4*>(q1 + c + Mp);
        const float a0 = s0[b], a1 = s1[b], au = s1[b - S], ad = s1[b + S];
        const float u0v[4] = {a0 * p0.x, a0 * p0.y, a0 * p0.z, a0 * p0.w};
        const float u1v[4] = {a1 * p1.x, a1 * p1.y, a1 * p1.z, a1 * p1.w};
        const float uu[4] = {au * pu.x, au * pu.y, au * pu.z, au * pu.w};
        const float ud[4] = {ad * pd.x, ad * pd.y, ad * pd.z, ad * pd.w};
        // the neighbours j - 1 and j + 4, each decoded with its own block's scale
        const float left = j > 0 ? s1[(size_t)i * S + (j - 1) / 32] * q1[c - 1] : 0.f;
        const float right = j + 4 < Mp ? s1[(size_t)i * S + (j + 4) / 32] * q1[c + 4] : 0.f;
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const float jl = e > 0 ? u1v[e - 1] : left;
            const float jr = e < 3 ? u1v[e + 1] : right;
            const int je = j + e;
            v[e] = (je == 0 || je >= M - 1) ? 0.f  // boundary and padding stay zero
                                            : update2d(u0v[e], u1v[e], uu[e], ud[e], jl, jr, k, dx2, dy2);
        }
    }
    // encode: the largest magnitude of the block sets its scale
    float m = fmaxf(fmaxf(fabsf(v[0]), fabsf(v[1])), fmaxf(fabsf(v[2]), fabsf(v[3])));
#pragma unroll
    for (int o = 1; o < 8; o *= 2) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (!live) return;
    const float inv = m > 0.f ? __fdiv_rn(32767.f, m) : 0.f;
    *reinterpret_cast<short4*>(q2 + c) =
        make_short4(short(__float2int_rn(v[0] * inv)), short(__float2int_rn(v[1] * inv)),
                    short(__float2int_rn(v[2] * inv)), short(__float2int_rn(v[3] * inv)));
    if ((threadIdx.x & 7) == 0) s2[b] = __fdiv_rn(m, 32767.f);
}

float kcoef(float c, float dt) { return dt * dt * c * c; }  // as the reference: ((dt dt) c) c

}  // namespace
}  // namespace wfd

using namespace wfd;

extern "C" {

int wfd_step1d(const float* u0, const float* u1, float* u2, float wavespeed, float dt, float dx,
               int N, void* stream) {
    if (!u0 || !u1 || !u2) return set_error(WFD_ERR_INVALID, "NULL field");
    if (N < 3) return set_error(WFD_ERR_INVALID, "need N >= 3");
    const int blocks = (N + 255) / 256;
    step1d_kernel<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(u0, u1, u2, kcoef(wavespeed, dt),
                                                                          dx * dx, N);
    count_launch();
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? WFD_OK : set_error(WFD_ERR_CUDA, cudaGetErrorString(e));
}

int wfd_step2d_mixed(const void* u0, const void* u1, void* u2, float wavespeed, float dt, float dx,
                     float dy, int N, int M, int M_padded, void* stream) {
    if (!u0 || !u1 || !u2) return set_error(WFD_ERR_INVALID, "NULL field");
    if (N < 3 || M < 3 || M_padded < M + 1 || M_padded % 2)
        return set_error(WFD_ERR_INVALID, "need N, M >= 3 and an even M_padded > M");
    if (reinterpret_cast<uintptr_t>(u0) % 4 || reinterpret_cast<uintptr_t>(u1) % 4 ||
        reinterpret_cast<uintptr_t>(u2) % 4)
        return set_error(WFD_ERR_INVALID, "fields must be 4-byte aligned");
    if ((long long)N * M_padded >= (1ll << 31)) return set_error(WFD_ERR_INVALID, "grid too large");
    const dim3 block(128, 4), grid((M_padded / 2 + 127) / 128, (N + 3) / 4);
    mixed_kernel<<<grid, block, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const __half*>(u0), static_cast<const __half*>(u1), static_cast<__half*>(u2),
        kcoef(wavespeed, dt), dx * dx, dy * dy, N, M, M_padded);
    count_launch();
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? WFD_OK : set_error(WFD_ERR_CUDA, cudaGetErrorString(e));
}

int wfd_step2d_scaled(const int16_t* q0, const float* s0, const int16_t* q1, const float* s1,
                      int16_t* q2, float* s2, float wavespeed, float dt, float dx, float dy, int N,
                      int M, int M_padded, void* stream) {
    if (!q0 || !s0 || !q1 || !s1 || !q2 || !s2) return set_error(WFD_ERR_INVALID, "NULL field");
    if (N < 3 || M < 3 || M_padded < M || M_padded % 64)
        return set_error(WFD_ERR_INVALID, "need N, M >= 3 and M_padded >= M, a multiple of 64");
    for (const void* p : {(const void*)q0, (const void*)q1, (const void*)q2})
        if (reinterpret_cast<uintptr_t>(p) % 8) return set_error(WFD_ERR_INVALID, "q fields must be 8-byte aligned");
    if ((long long)N * M_padded >= (1ll << 31)) return set_error(WFD_ERR_INVALID, "grid too large");
    const dim3 block(64, 4), grid((M_padded / 4 + 63) / 64, (N + 3) / 4);
    scaled_kernel<<<grid, block, 0, static_cast<cudaStream_t>(stream)>>>(
        q0, s0, q1, s1, q2, s2, kcoef(wavespeed, dt), dx * dx, dy * dy, N, M, M_padded);
    count_launch();
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? WFD_OK : set_error(WFD_ERR_CUDA, cudaGetErrorString(e));
}

}  // extern "C"
