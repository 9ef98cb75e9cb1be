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

// FP32 storage with any row stride (padded_step / shared_step with M_padded,
// basic_step / coalesced_step with M_padded = M): a thread owns 4 consecutive
// cells j .. j + 3 of row i, read and written as scalars (rows need not be
// 16-byte aligned).
__global__ void exact_kernel(const float* __restrict__ u0, const float* __restrict__ u1,
                             float* __restrict__ u2, float k, float dx2, float dy2, int N, int M, int Mp) {
    const int j = 4 * (blockIdx.x * blockDim.x + threadIdx.x);
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i <= 0 || i >= N - 1 || j >= M - 1) return;
    const size_t c = (size_t)i * Mp + j;
    float w[6];  // u1 at j - 1 .. j + 4 of row i
#pragma unroll
    for (int e = 0; e < 6; ++e) w[e] = (j - 1 + e >= 0 && j - 1 + e < M) ? u1[c - 1 + e] : 0.f;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const int je = j + e;
        if (je == 0 || je >= M - 1) continue;  // the boundary columns (and beyond) stay untouched
        u2[c + e] = update2d(u0[c + e], w[e + 1], u1[c + e - Mp], u1[c + e + Mp], w[e], w[e + 2], k, dx2, dy2);
    }
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

// FP16 storage with pre-divided weights (the mixed_step update within FP32
// rounding, as the reference's --use_fast_math build computes it): a thread
// owns 8 consecutive values j .. j + 7 (j a multiple of 8) of row i, loaded
// and stored as 16 bytes; the left and right neighbours of the octet are two
// scalar loads. u2 = (2u - u0) + cx (u_{i-1} - 2u + u_{i+1}) + cy (u_{j-1} -
// 2u + u_{j+1}), cx = k / dx^2, cy = k / dy^2, rounded to FP16 once.
__global__ void mixed_fast_kernel(const __half* __restrict__ u0, const __half* __restrict__ u1,
                                  __half* __restrict__ u2, float cx, float cy, int N, int M, int Mp) {
    const int j = 8 * (blockIdx.x * blockDim.x + threadIdx.x);
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i <= 0 || i >= N - 1 || j >= M - 1) return;
    const size_t c = (size_t)i * Mp + j;
    const uint4 ra = *reinterpret_cast<const uint4*>(u0 + c);
    const uint4 rb = *reinterpret_cast<const uint4*>(u1 + c);
    const uint4 ru = *reinterpret_cast<const uint4*>(u1 + c - Mp);
    const uint4 rd = *reinterpret_cast<const uint4*>(u1 + c + Mp);
    float w[10];  // u1 at j - 1 .. j + 8 of row i
    w[0] = j > 0 ? __half2float(u1[c - 1]) : 0.f;
    w[9] = j + 8 < Mp ? __half2float(u1[c + 8]) : 0.f;  // (row i + 1 starts after the padding)
    const __half2* hb = reinterpret_cast<const __half2*>(&rb);
    const __half2* ha = reinterpret_cast<const __half2*>(&ra);
    const __half2* hu = reinterpret_cast<const __half2*>(&ru);
    const __half2* hd = reinterpret_cast<const __half2*>(&rd);
    float a[8], up[8], dn[8];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const float2 vb = __half22float2(hb[q]), va = __half22float2(ha[q]);
        const float2 vu = __half22float2(hu[q]), vd = __half22float2(hd[q]);
        w[1 + 2 * q] = vb.x;
        w[2 + 2 * q] = vb.y;
        a[2 * q] = va.x;
        a[2 * q + 1] = va.y;
        up[2 * q] = vu.x;
        up[2 * q + 1] = vu.y;
        dn[2 * q] = vd.x;
        dn[2 * q + 1] = vd.y;
    }
    float v[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        const float two_c = 2.f * w[e + 1];
        v[e] = fmaf(cx, (up[e] - two_c) + dn[e], fmaf(cy, (w[e] - two_c) + w[e + 2], two_c - a[e]));
    }
    if (j > 0 && j + 7 < M - 1) {
        uint4 o;
        __half2* ho = reinterpret_cast<__half2*>(&o);
#pragma unroll
        for (int q = 0; q < 4; ++q) ho[q] = __floats2half2_rn(v[2 * q], v[2 * q + 1]);
        *reinterpret_cast<uint4*>(u2 + c) = o;
    } else {
#pragma unroll
        for (int e = 0; e < 8; ++e)
            if (j + e > 0 && j + e < M - 1) u2[c + e] = __float2half_rn(v[e]);
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

// Eight steps per launch (temporal_step): a CTA stages both levels of a
// 160 x 48 window (a 144 x 32 output tile plus an 8-cell halo on every side)
// by TMA, advances them in shared memory, and writes the tile of both final
// levels. The cells a step can update shrink by one per step from the window
// edges (the halo is the step count); global boundary cells and cells outside
// the grid are never updated, exactly as eight padded_step launches.
constexpr int TT_TX = 144, TT_TZ = 32, TT_H = 8, TT_STEPS = 8;
constexpr int TT_W = TT_TX + 2 * TT_H;   // 160 staged columns (40 float4)
constexpr int TT_WZ = TT_TZ + 2 * TT_H;  // 48 staged rows
constexpr int TT_THREADS = 320;  // 8 rows x 40 float4 columns per pass
constexpr int TT_PASSES = TT_WZ / 8;  // 6 row passes per step
constexpr int TT_LEVEL = TT_WZ * TT_W * 4;  // bytes of one staged level
constexpr int TT_BYTES = 2 * TT_LEVEL + 16 + 128;

__global__ void __launch_bounds__(TT_THREADS)
    temporal_kernel(const __grid_constant__ CUtensorMap map_u0, const __grid_constant__ CUtensorMap map_u1,
                    float* __restrict__ v0, float* __restrict__ v1, float k, float dx2, float dy2, int N,
                    int M, int Mp) {
    extern __shared__ unsigned char smem_raw[];
    float* base = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    float* lev[2] = {base, base + TT_WZ * TT_W};
    uint64_t* bar = reinterpret_cast<uint64_t*>(base + 2 * TT_WZ * TT_W);
    const int tid = threadIdx.x;
    const int j0 = blockIdx.x * TT_TX - TT_H, i0 = blockIdx.y * TT_TZ - TT_H;  // window origin

    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();  // no thread polls the barrier before it is initialised
    grid_dependency_wait();
    if (tid == 0) {
        mbar_arrive_expect_tx(bar, 2u * TT_LEVEL);
        // (the maps are rank 3: x, rows, shot; one shot here)
        tma_load_3d(lev[0], &map_u0, j0, i0, 0, bar);  // cells outside the grid arrive as 0
        tma_load_3d(lev[1], &map_u1, j0, i0, 0, bar);
        launch_dependents();
    }
    mbar_wait(bar, 0);  // bounded; every thread goes on to the same barriers either way

    // a thread owns the float4 column tj of rows r0, r0 + 8, ..., r0 + 40
    const int tj = 4 * (tid % (TT_W / 4)), r0 = tid / (TT_W / 4);
    for (int st = 0; st < TT_STEPS; ++st) {
        float* old = lev[st & 1];              // u_{n-1}, overwritten by u_{n+1}
        const float* cur = lev[1 - (st & 1)];  // u_n
#pragma unroll 3
        for (int ps = 0; ps < TT_PASSES; ++ps) {
            const int ti = r0 + 8 * ps;
            const int i = i0 + ti;
            if (ti <= st || ti >= TT_WZ - 1 - st || i <= 0 || i >= N - 1) continue;
            const float* c = cur + ti * TT_W + tj;
            const float4 cv = *reinterpret_cast<const float4*>(c);
            const float4 up = *reinterpret_cast<const float4*>(c - TT_W);
            const float4 dn = *reinterpret_cast<const float4*>(c + TT_W);
            const float left = tj > 0 ? c[-1] : 0.f, right = tj + 4 < TT_W ? c[4] : 0.f;
            float4 ov = *reinterpret_cast<const float4*>(old + ti * TT_W + tj);
            const float cc[6] = {left, cv.x, cv.y, cv.z, cv.w, right};
            const float uu[4] = {up.x, up.y, up.z, up.w}, dd[4] = {dn.x, dn.y, dn.z, dn.w};
            float o[4] = {ov.x, ov.y, ov.z, ov.w};
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int te = tj + e, j = j0 + te;
                if (te > st && te < TT_W - 1 - st && j > 0 && j < M - 1)
                    o[e] = update2d(o[e], cc[e + 1], uu[e], dd[e], cc[e], cc[e + 2], k, dx2, dy2);
            }
            *reinterpret_cast<float4*>(old + ti * TT_W + tj) = make_float4(o[0], o[1], o[2], o[3]);
        }
        __syncthreads();
    }

    // after the eight steps lev[0] holds u_{n+7} and lev[1] u_{n+8}
    for (int g = tid; g < TT_TZ * (TT_TX / 4); g += TT_THREADS) {
        const int r = g / (TT_TX / 4), q = 4 * (g - r * (TT_TX / 4));
        const int i = i0 + TT_H + r, j = j0 + TT_H + q;
        if (i >= N || j >= M) continue;
        const float* a = lev[0] + (TT_H + r) * TT_W + TT_H + q;
        const float* b = lev[1] + (TT_H + r) * TT_W + TT_H + q;
        const size_t o = (size_t)i * Mp + j;
        if (j + 3 < M) {
            *reinterpret_cast<float4*>(v0 + o) = *reinterpret_cast<const float4*>(a);
            *reinterpret_cast<float4*>(v1 + o) = *reinterpret_cast<const float4*>(b);
        } else {
            for (int e = 0; j + e < M; ++e) {
                v0[o + e] = a[e];
                v1[o + e] = b[e];
            }
        }
    }
}

// Eight steps per launch with the window in registers (temporal_step's
// arguments and results). A CTA of 8 warps holds a 256-column x 40-row window:
// thread t owns column t, both levels of its 40 rows in registers. The
// vertical neighbours are registers of the same thread, the horizontal ones
// come from the neighbouring lanes by warp shuffles; at a warp's edge, lane 0
// and lane 31 read the neighbouring warp's edge column, which every warp
// publishes in shared memory at each step (double-buffered by step parity:
// one CTA barrier per step). The halo is 8 cells on every side, so the
// 240 x 24 inner tile is exact after the eight steps; the global boundary is
// never updated, as in temporal_step. Each cell is
// loaded and stored once per launch with coalesced row accesses (a warp reads
// 128 contiguous bytes of a row).
//   EXACT: the reference expression in IEEE operations (update2d), value for
//          value the reference's padded_step applied eight times;
//   else:  u_{n+1} = (2 u - u_{n-1}) + cx (u_{i-1} - 2u + u_{i+1}) + cy (...),
//          cx = k / dx^2, cy = k / dy^2 (fused multiply-adds, no division):
//          within FP32 rounding of the reference, as its own --use_fast_math
//          build (approximate division) is.
constexpr int TR_NW = 8;                    // warps per CTA
constexpr int TR_W = 32 * TR_NW;            // window columns, one per thread
constexpr int TR_H = 40;                    // window rows held by each thread
constexpr int TR_MINB = 2;                  // resident CTAs per SM the register budget allows
constexpr int TR_HALO = 8;                  // = steps per launch
constexpr int TR_OX = TR_W - 2 * TR_HALO;   // 240 output columns per CTA

// One step on the window: old <- the new level from (old, cur). GUARD: test
// every cell against the shrinking window and the global boundary (CTAs whose
// window reaches the boundary). Without it (windows inside the interior),
// every cell but the window's first and last rows is updated: the window's
// edge cells then take values from missing neighbours, but after s steps
// those spread s cells inwards at most, and the stored tile lies 8 cells in.
template <bool EXACT, bool GUARD, int H>
__device__ __forceinline__ void reg_step(float (&old)[H], const float (&cur)[H], float (*edge)[2][H], int warp,
                                         int lane, bool cupd, int rmin, int rmax, float k, float dx2, float dy2,
                                         float cx, float cy) {
    if (lane == 0 || lane == 31) {  // this warp's edge column, for the neighbouring warps
        float* dst = edge[warp][lane == 31 ? 1 : 0];
#pragma unroll
        for (int r = 0; r < H; ++r) dst[r] = cur[r];
    }
    __syncthreads();
    // lane 0: the previous warp's lane-31 column; lane 31: the next warp's
    // lane-0 column (the window's outer columns are never updated)
    const float* nb = lane == 31 ? edge[min(warp + 1, TR_NW - 1)][0] : edge[max(warp - 1, 0)][1];
#pragma unroll
    for (int r = 1; r < H - 1; ++r) {
        const float c = cur[r];
        float l = __shfl_up_sync(0xffffffffu, c, 1);
        float rr = __shfl_down_sync(0xffffffffu, c, 1);
        const float e = nb[r];
        if (lane == 0) l = e;
        if (lane == 31) rr = e;
        if (!GUARD || (cupd && r > rmin && r < rmax)) {
            if (EXACT) {
                old[r] = update2d(old[r], c, cur[r - 1], cur[r + 1], l, rr, k, dx2, dy2);
            } else {
                const float two_c = 2.f * c;
                old[r] = fmaf(cx, (cur[r - 1] - two_c) + cur[r + 1], fmaf(cy, (l - two_c) + rr, two_c - old[r]));
            }
        }
    }
}

// H window rows per thread (H - 16 output rows per CTA), MINB resident CTAs
// per SM for the register allocation.
template <bool EXACT, int H, int MINB>
__global__ void __launch_bounds__(TR_W, MINB)
    temporal_reg_kernel(const float* __restrict__ u0, const float* __restrict__ u1, float* __restrict__ v0,
                        float* __restrict__ v1, float k, float dx2, float dy2, float cx, float cy, int N, int M,
                        int Mp) {
    __shared__ float edge[2][TR_NW][2][H];  // [step parity][warp][lane 0 / lane 31][row]
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int j = blockIdx.x * TR_OX - TR_HALO + t;
    const int i0 = blockIdx.y * (H - 2 * TR_HALO) - TR_HALO;
    const bool jin = j >= 0 && j < M;
    float A[H], B[H];  // u_{n-1}, u_n; they trade roles every step
#pragma unroll
    for (int r = 0; r < H; ++r) {
        const int i = i0 + r;
        const bool in = jin && i >= 0 && i < N;  // cells outside the grid hold 0
        const long long c = (long long)i * Mp + j;
        A[r] = in ? __ldg(u0 + c) : 0.f;
        B[r] = in ? __ldg(u1 + c) : 0.f;
    }
    const bool jupd = j > 0 && j < M - 1;  // the boundary columns (and beyond) stay untouched
    const int j0 = blockIdx.x * TR_OX - TR_HALO;
    const bool inner = i0 >= 1 && i0 + H - 1 <= N - 2 && j0 >= 1 && j0 + TR_W - 1 <= M - 2;  // (CTA-uniform)
    for (int st = 0; st < TR_HALO; st += 2) {
        if (inner) {
            reg_step<EXACT, false, H>(A, B, edge[0], warp, lane, true, 0, 0, k, dx2, dy2, cx, cy);
            reg_step<EXACT, false, H>(B, A, edge[1], warp, lane, true, 0, 0, k, dx2, dy2, cx, cy);
            continue;
        }
        // updated rows: inside the shrinking window and inside (0, N - 1)
        for (int h = 0; h < 2; ++h) {
            const int s2 = st + h;
            const int rmin = max(s2, -i0), rmax = min(H - 1 - s2, N - 1 - i0);
            const bool cupd = jupd && t > s2 && t < TR_W - 1 - s2;
            if (h == 0)
                reg_step<EXACT, true, H>(A, B, edge[0], warp, lane, cupd, rmin, rmax, k, dx2, dy2, cx, cy);
            else
                reg_step<EXACT, true, H>(B, A, edge[1], warp, lane, cupd, rmin, rmax, k, dx2, dy2, cx, cy);
        }
    }
    // A holds u_{n+7}, B u_{n+8}
    if (t >= TR_HALO && t < TR_W - TR_HALO && j < M) {
#pragma unroll
        for (int r = TR_HALO; r < H - TR_HALO; ++r) {
            const int i = i0 + r;
            if (i < N) {
                const long long c = (long long)i * Mp + j;
                v0[c] = A[r];
                v1[c] = B[r];
            }
        }
    }
}

}  // namespace

// the staged window of temporal_kernel: TMA box (columns, rows)
void temporal_box(unsigned* cols, unsigned* rows) {
    *cols = TT_W;
    *rows = TT_WZ;
}

cudaError_t launch_temporal_reg(const float* u0, const float* u1, float* v0, float* v1, float wavespeed, float dt,
                                float dx, float dy, int N, int M, int Mp, bool exact, cudaStream_t s) {
    constexpr int OZ = TR_H - 2 * TR_HALO;
    const dim3 grid((M + TR_OX - 1) / TR_OX, (N + OZ - 1) / OZ);
    const float k = kcoef(wavespeed, dt), dx2 = dx * dx, dy2 = dy * dy;
    // a plain launch: the window's read-only loads of u0 and u1, the previous
    // launch's output, are ordered after it by the kernel boundary
    if (exact)
        temporal_reg_kernel<true, TR_H, TR_MINB><<<grid, TR_W, 0, s>>>(u0, u1, v0, v1, k, dx2, dy2, k / dx2, k / dy2,
                                                                     N, M, Mp);
    else
        temporal_reg_kernel<false, TR_H, TR_MINB><<<grid, TR_W, 0, s>>>(u0, u1, v0, v1, k, dx2, dy2, k / dx2, k / dy2,
                                                                      N, M, Mp);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_temporal(const CUtensorMap& m0, const CUtensorMap& m1, float* v0, float* v1, float wavespeed,
                            float dt, float dx, float dy, int N, int M, int Mp, cudaStream_t s) {
    static int configured_device = -1;
    int dev = 0;
    cudaGetDevice(&dev);
    if (configured_device != dev) {
        const cudaError_t e =
            cudaFuncSetAttribute(temporal_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, TT_BYTES);
        if (e != cudaSuccess) return e;
        configured_device = dev;
    }
    const dim3 grid((M + TT_TX - 1) / TT_TX, (N + TT_TZ - 1) / TT_TZ);
    const cudaError_t e = launch_pdl(temporal_kernel, grid, dim3(TT_THREADS), TT_BYTES, s, m0, m1, v0, v1,
                                     kcoef(wavespeed, dt), dx * dx, dy * dy, N, M, Mp);
    count_launch();
    return e != cudaSuccess ? e : cudaGetLastError();
}

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

int wfd_step2d_exact(const float* u0, const float* u1, float* u2, float wavespeed, float dt, float dx,
                     float dy, int N, int M, int M_padded, void* stream) {
    if (!u0 || !u1 || !u2) return set_error(WFD_ERR_INVALID, "NULL field");
    if (N < 3 || M < 3 || M_padded < M) return set_error(WFD_ERR_INVALID, "need N, M >= 3 and M_padded >= M");
    if ((long long)N * M_padded >= (1ll << 31)) return set_error(WFD_ERR_INVALID, "grid too large");
    if ((N + 3) / 4 > 65535) return set_error(WFD_ERR_INVALID, "N too large (more than 262140 rows)");
    const dim3 block(64, 4), grid(((M + 3) / 4 + 63) / 64, (N + 3) / 4);
    exact_kernel<<<grid, block, 0, static_cast<cudaStream_t>(stream)>>>(u0, u1, u2, kcoef(wavespeed, dt), dx * dx,
                                                                        dy * dy, N, M, M_padded);
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
    if ((N + 3) / 4 > 65535) return set_error(WFD_ERR_INVALID, "N too large (more than 262140 rows)");
    const dim3 block(128, 4), grid((M_padded / 2 + 127) / 128, (N + 3) / 4);
    mixed_kernel<<<grid, block, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const __half*>(u0), static_cast<const __half*>(u1), static_cast<__half*>(u2),
        kcoef(wavespeed, dt), dx * dx, dy * dy, N, M, M_padded);
    count_launch();
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? WFD_OK : set_error(WFD_ERR_CUDA, cudaGetErrorString(e));
}

int wfd_step2d_mixed_fast(const void* u0, const void* u1, void* u2, float wavespeed, float dt, float dx,
                          float dy, int N, int M, int M_padded, void* stream) {
    if (!u0 || !u1 || !u2) return set_error(WFD_ERR_INVALID, "NULL field");
    if (N < 3 || M < 3 || M_padded < M || M_padded % 8)
        return set_error(WFD_ERR_INVALID, "need N, M >= 3 and M_padded >= M, a multiple of 8");
    for (const void* p : {u0, u1, (const void*)u2})
        if (reinterpret_cast<uintptr_t>(p) % 16) return set_error(WFD_ERR_INVALID, "fields must be 16-byte aligned");
    if ((long long)N * M_padded >= (1ll << 31)) return set_error(WFD_ERR_INVALID, "grid too large");
    if ((N + 3) / 4 > 65535) return set_error(WFD_ERR_INVALID, "N too large (more than 262140 rows)");
    const float k = kcoef(wavespeed, dt);
    const dim3 block(64, 4), grid((M_padded / 8 + 63) / 64, (N + 3) / 4);
    mixed_fast_kernel<<<grid, block, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const __half*>(u0), static_cast<const __half*>(u1), static_cast<__half*>(u2), k / (dx * dx),
        k / (dy * dy), N, M, M_padded);
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
    if ((N + 3) / 4 > 65535) return set_error(WFD_ERR_INVALID, "N too large (more than 262140 rows)");
    const dim3 block(64, 4), grid((M_padded / 4 + 63) / 64, (N + 3) / 4);
    scaled_kernel<<<grid, block, 0, static_cast<cudaStream_t>(stream)>>>(
        q0, s0, q1, s1, q2, s2, kcoef(wavespeed, dt), dx * dx, dy * dy, N, M, M_padded);
    count_launch();
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? WFD_OK : set_error(WFD_ERR_CUDA, cudaGetErrorString(e));
}

}  // extern "C"
