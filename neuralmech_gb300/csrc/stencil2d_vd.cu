// Variable-density 2D time step (sm_103a): the conservative operator
//     u_{n+1} = g (2 u_n + k Lb u_n) - g^2 u_{n-1},   k = kappa dt^2 / dx^2,
//     Lb u = sum_k c_k (Fx_{x+k-1} - Fx_{x-k}) + sz sum_k c_k (Fz_{z+k-1} - Fz_{z-k}),
//     Fx_j = bx_j (Dx u)_j,  (Dx u)_j = sum_k c_k (u_{j+k} - u_{j-k+1})  at x = j + 1/2,
// b = 1 / rho, bx_j = (b_j + b_{j+1}) / 2 (likewise in z), c_k the order-2R
// staggered first-derivative weights, sz = (dx/dz)^2; fields and b are zero
// outside the grid. This is the two-phase medium of cuwave's AcousticWave
// (projects/8_physics_drivers/waveND.py:52-65), which interpolates 1/rho and
// 1/kappa between the phases (1_benchmark_2D/README.md:141-144).
//
// Per CTA (256 threads): a 128 x 16 tile of `shots_per_cta` shots. b on the
// tile (plus R rows and 8 columns) is staged once by TMA with the first shot;
// each shot's stage holds the field with a halo of 2R rows and 8 columns, the
// u_{n-1} tile and, in MODE_GRAD_U, the level u_k with the same halo. For a
// field, every thread forms the fluxes at its own half points (lanes 0 and 31
// and warps 0 .. 2R-2 also the tile's halo ones) into shared memory, then the
// divergence at its cells. MODE_GRAD_U does that for u_k (keeping L u_k and
// the raw differences Dx u_k, Dz u_k of its half points in registers), then
// for q_{k+1}, and accumulates
//     G   += q_{k+1} Lb u_k            (cells, dJ/dk = G / k),
//     Gbx -= (Dx q_{k+1}) (Dx u_k)     (half points (z, x + 1/2)),
//     Gbz -= sz (Dz q_{k+1}) (Dz u_k)  (half points (z + 1/2, x)).
// Sampling and injection are those of the constant-density kernel (k in the
// role of m).
#include <algorithm>

#include "common.cuh"
#include "internal.h"

namespace wfd {
namespace {

constexpr int VD_TX = 128, VD_TZ = 16, VD_RB = 2, VD_THREADS = 256;
constexpr int VD_W = VD_TX + 16;  // staged columns: x0 - 8 .. x0 + 135
constexpr int VD_FXW = VD_TX + 8; // flux columns: half points x0 - 4 .. x0 + 131

__host__ __device__ constexpr int al128(int v) { return (v + 127) / 128 * 128; }

template <int R, int MODE>
struct LayoutVD {
    static constexpr int FH = VD_TZ + 4 * R;      // staged field rows: z0 - 2R ..
    static constexpr int BH = VD_TZ + 2 * R + 1;  // staged b rows: z0 - R ..
    static constexpr int ZH = VD_TZ + 2 * R;      // flux rows in z: half rows z0 - R ..
    static constexpr int F = FH * VD_W * 4;
    // u_{n-1} tile: staged in the forward; the adjoint reads it from global
    // memory at the update, which keeps two adjoint CTAs within one SM
    static constexpr int O = MODE == MODE_GRAD_U ? 0 : VD_TZ * VD_TX * 4;
    static constexpr int U = MODE == MODE_GRAD_U ? F : 0;
    static constexpr int O_OFF = al128(F);
    static constexpr int U_OFF = O_OFF + al128(O);
    static constexpr int STAGE = U_OFF + al128(U);
    static constexpr int STAGES = 2;
    static constexpr int B_OFF = STAGES * STAGE;
    static constexpr int B = BH * VD_W * 4;
    static constexpr int FX_OFF = B_OFF + al128(B);
    static constexpr int FX = VD_TZ * VD_FXW * 4;
    static constexpr int FZ_OFF = FX_OFF + al128(FX);
    static constexpr int FZ = ZH * VD_TX * 4;
    static constexpr int BAR_OFF = FZ_OFF + al128(FZ);
    static constexpr int BYTES = BAR_OFF + 64 + 128;
};

__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void st4(float* p, const float4& v) { *reinterpret_cast<float4*>(p) = v; }

// Packed FP32x2 staggered sums, rounding as the scalar form
// s = fmaf(c_k, hi_k - lo_k, s), k = 1 .. R: each difference is one rounded
// subtraction (hi + (-1) lo, exact multiply), then a fused multiply-add.
__device__ __forceinline__ float2 psub(float2 hi, float2 lo) {
    return __ffma2_rn(lo, make_float2(-1.f, -1.f), hi);
}

// Raw staggered x differences at the 4 half points whose window w[12] spans
// the cells 4 left of the first half point's left cell to 7 right of it:
// (Dx f)_{j+e} = sum_k c_k (w[4 + e + k] - w[5 + e - k]), in pairs e, e + 1
// (the two operands of a pair sit one register apart, so the differences are
// scalar and the multiply-adds packed).
template <int R>
__device__ __forceinline__ float4 dx4(const float* w, const StepArgs& a) {
    float2 lo = make_float2(0.f, 0.f), hi = lo;
#pragma unroll
    for (int k = 1; k <= R; ++k) {
        lo = __ffma2_rn(a.csp[k - 1], make_float2(w[4 + k] - w[5 - k], w[5 + k] - w[6 - k]), lo);
        hi = __ffma2_rn(a.csp[k - 1], make_float2(w[6 + k] - w[7 - k], w[7 + k] - w[8 - k]), hi);
    }
    return make_float4(lo.x, lo.y, hi.x, hi.y);
}

__device__ __forceinline__ float2 lo2v(const float4& v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2v(const float4& v) { return make_float2(v.z, v.w); }

template <int R, int MODE>
__global__ void __launch_bounds__(VD_THREADS, 2)
    step2d_vd_kernel(const __grid_constant__ CUtensorMap map_f, const __grid_constant__ CUtensorMap map_o,
                     const __grid_constant__ CUtensorMap map_u, const __grid_constant__ CUtensorMap map_b,
                     const StepArgs a) {
    using L = LayoutVD<R, MODE>;
    extern __shared__ unsigned char smem_raw[];
    unsigned char* base = reinterpret_cast<unsigned char*>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    uint64_t* bars = reinterpret_cast<uint64_t*>(base + L::BAR_OFF);
    const float* B = reinterpret_cast<const float*>(base + L::B_OFF);
    float* FX = reinterpret_cast<float*>(base + L::FX_OFF);
    float* FZ = reinterpret_cast<float*>(base + L::FZ_OFF);

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int tile = blockIdx.x;
    const int ntiles = a.tiles_x * a.tiles_z;
    const int x0 = (tile % a.tiles_x) * VD_TX, z0 = (tile / a.tiles_x) * VD_TZ;
    const int s0 = blockIdx.y * a.shots_per_cta;
    const int ns = min(a.nshot - s0, a.shots_per_cta);
    if (ns <= 0) return;

    auto stage = [&](int b) { return base + b * L::STAGE; };
    auto issue = [&](int i) {  // thread 0 only
        const int b = i % L::STAGES;
        mbar_arrive_expect_tx(&bars[b], uint32_t(L::F + L::O + L::U + (i == 0 ? L::B : 0)));
        tma_load_3d(stage(b), &map_f, x0 - 8, z0 - 2 * R, s0 + i, &bars[b]);
        if (MODE != MODE_GRAD_U) tma_load_3d(stage(b) + L::O_OFF, &map_o, x0, z0, s0 + i, &bars[b]);
        if (MODE == MODE_GRAD_U) tma_load_3d(stage(b) + L::U_OFF, &map_u, x0 - 8, z0 - 2 * R, s0 + i, &bars[b]);
        if (i == 0) tma_load_2d(const_cast<float*>(B), &map_b, x0 - 8, z0 - R, &bars[b]);
    };

    __shared__ int2 smp_range[T2_MAX_SPC], inj_range[T2_MAX_SPC];
    // launched as a programmatic dependent: every global access comes after the wait
    if (tid == 0) {
        for (int b = 0; b < L::STAGES; ++b) mbar_init(&bars[b], 1);
        fence_mbar_init();
    }
    grid_dependency_wait();
    // the first stages are issued before the point-list ranges are read, so
    // that the two memory latencies overlap
    if (tid == 0) {
        for (int i = 0; i < min(ns, L::STAGES); ++i) issue(i);
        launch_dependents();
    }

    // ---- per-thread constants (loaded before the barrier below, so that their
    // latency overlaps the range reads)
    const int x = x0 + 4 * lane;
    const int zb = z0 + warp * VD_RB;
    float4 krow[VD_RB];
    float gzr[VD_RB];
    bool zin[VD_RB];
#pragma unroll
    for (int r = 0; r < VD_RB; ++r) {
        const int z = zb + r;
        krow[r] = (z < a.nz && x < a.ld) ? __ldg(reinterpret_cast<const float4*>(a.m + (long long)z * a.ld + x))
                                         : make_float4(0.f, 0.f, 0.f, 0.f);
        gzr[r] = (a.gz != nullptr && z < a.nz) ? __ldg(a.gz + z) : 1.f;
        zin[r] = z >= R && z < a.nz - R;
    }
    float gxe[4];
    bool xin[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        gxe[e] = (a.gx != nullptr && x + e < a.nx) ? __ldg(a.gx + x + e) : 1.f;
        xin[e] = x + e >= R && x + e < a.nx - R;
    }
    const bool all_x = xin[0] && xin[1] && xin[2] && xin[3];

    if (tid < ns) {
        const int k = (s0 + tid) * ntiles + tile;
        smp_range[tid] = a.smp.off ? make_int2(a.smp.off[k], a.smp.off[k + 1]) : make_int2(0, 0);
        inj_range[tid] = a.inj.off ? make_int2(a.inj.off[k], a.inj.off[k + 1]) : make_int2(0, 0);
    }
    __syncthreads();

    float4 gk[VD_RB], gbx[VD_RB], gbz[VD_RB];
#pragma unroll
    for (int r = 0; r < VD_RB; ++r) {
        gk[r] = make_float4(0.f, 0.f, 0.f, 0.f);
        gbx[r] = gk[r];
        gbz[r] = gk[r];
    }

    // Fluxes of the staged field T into FX / FZ; the raw differences of the
    // thread's own half points to dxr, dzr.
    auto fluxes = [&](const float* T, float4* dxr, float4* dzr) {
        auto trow = [&](int fr) { return T + fr * VD_W; };  // staged row of z = z0 - 2R + fr
        auto brow = [&](int br) { return B + br * VD_W; };  // staged b row of z = z0 - R + br
        // x: own half points x .. x + 3 of the rows zb, zb + 1
#pragma unroll
        for (int r = 0; r < VD_RB; ++r) {
            const int fr = warp * VD_RB + r + 2 * R, br = warp * VD_RB + r + R;
            const float4 p0 = ld4(trow(fr) + 4 * lane + 4), p1 = ld4(trow(fr) + 4 * lane + 8),
                         p2 = ld4(trow(fr) + 4 * lane + 12);
            const float w[12] = {p0.x, p0.y, p0.z, p0.w, p1.x, p1.y, p1.z, p1.w, p2.x, p2.y, p2.z, p2.w};
            const float4 d = dx4<R>(w, a);
            const float4 b0 = ld4(brow(br) + 4 * lane + 8), b1 = ld4(brow(br) + 4 * lane + 12);
            const float4 bx = make_float4(0.5f * (b0.x + b0.y), 0.5f * (b0.y + b0.z), 0.5f * (b0.z + b0.w),
                                          0.5f * (b0.w + b1.x));
            dxr[r] = d;
            st4(FX + (warp * VD_RB + r) * VD_FXW + 4 + 4 * lane,
                make_float4(bx.x * d.x, bx.y * d.y, bx.z * d.z, bx.w * d.w));
        }
        // the tile's halo half points x0 - 4 .. x0 - 1 and x0 + 128 .. x0 + 131 of
        // the warp's rows, one per lane of lanes 0 .. 8 RB - 1 (the same sums and
        // rounding as dx4): half point h of row r sits after the cell in staged
        // column sc
        if (lane < 8 * VD_RB) {
            const int r = lane >> 3, h = lane & 7;
            const int fr = warp * VD_RB + r + 2 * R, br = warp * VD_RB + r + R;
            const int sc = h < 4 ? 4 + h : 132 + h;
            const float* tr = trow(fr);
            float d = 0.f;
#pragma unroll
            for (int k = 1; k <= R; ++k) d = fmaf(a.cs[k - 1], tr[sc + k] - tr[sc - k + 1], d);
            const float bx = 0.5f * (brow(br)[sc] + brow(br)[sc + 1]);
            FX[(warp * VD_RB + r) * VD_FXW + (h < 4 ? h : VD_TX + h)] = bx * d;
        }
        // z: own half rows zb, zb + 1 from a window of field rows zb - R + 1 .. zb + R
        {
            float4 W[VD_RB + 2 * R - 1];
#pragma unroll
            for (int j = 0; j < VD_RB + 2 * R - 1; ++j) W[j] = ld4(trow(warp * VD_RB + R + 1 + j) + 8 + 4 * lane);
#pragma unroll
            for (int r = 0; r < VD_RB; ++r) {
                float2 dl = make_float2(0.f, 0.f), dh = dl;
#pragma unroll
                for (int k = 1; k <= R; ++k) {
                    const float4 up = W[r + R - 1 + k], dn = W[r + R - k];
                    dl = __ffma2_rn(a.csp[k - 1], psub(lo2v(up), lo2v(dn)), dl);
                    dh = __ffma2_rn(a.csp[k - 1], psub(hi2v(up), hi2v(dn)), dh);
                }
                const int br = warp * VD_RB + r + R;
                const float4 b0 = ld4(brow(br) + 8 + 4 * lane), b1 = ld4(brow(br + 1) + 8 + 4 * lane);
                dzr[r] = make_float4(dl.x, dl.y, dh.x, dh.y);
                const float2 h = make_float2(0.5f, 0.5f);
                const float2 fl = __fmul2_rn(__fmul2_rn(h, __fadd2_rn(lo2v(b0), lo2v(b1))), dl);
                const float2 fh = __fmul2_rn(__fmul2_rn(h, __fadd2_rn(hi2v(b0), hi2v(b1))), dh);
                st4(FZ + (warp * VD_RB + r + R) * VD_TX + 4 * lane, make_float4(fl.x, fl.y, fh.x, fh.y));
            }
        }
        // z halo half rows: FZ rows 0 .. R-1 (warps 0 .. R-1) and VD_TZ + R .. VD_TZ + 2R - 2
        if (warp < 2 * R - 1) {
            const int f = warp < R ? warp : VD_TZ + warp;  // FZ row: half row z0 - R + f
            float2 dl = make_float2(0.f, 0.f), dh = dl;
#pragma unroll
            for (int k = 1; k <= R; ++k) {
                const float4 up = ld4(trow(f + R + k) + 8 + 4 * lane), dn = ld4(trow(f + R + 1 - k) + 8 + 4 * lane);
                dl = __ffma2_rn(a.csp[k - 1], psub(lo2v(up), lo2v(dn)), dl);
                dh = __ffma2_rn(a.csp[k - 1], psub(hi2v(up), hi2v(dn)), dh);
            }
            const float4 b0 = ld4(brow(f) + 8 + 4 * lane), b1 = ld4(brow(f + 1) + 8 + 4 * lane);
            const float2 h = make_float2(0.5f, 0.5f);
            const float2 fl = __fmul2_rn(__fmul2_rn(h, __fadd2_rn(lo2v(b0), lo2v(b1))), dl);
            const float2 fh = __fmul2_rn(__fmul2_rn(h, __fadd2_rn(hi2v(b0), hi2v(b1))), dh);
            st4(FZ + f * VD_TX + 4 * lane, make_float4(fl.x, fl.y, fh.x, fh.y));
        }
    };

    // Lb of the fluxes at the thread's cells (rows zb, zb + 1)
    auto divergence = [&](float4* out) {
        float4 Z[VD_RB + 2 * R - 1];  // FZ rows warp RB .. (half rows zb - R .. zb + RB + R - 2)
#pragma unroll
        for (int j = 0; j < VD_RB + 2 * R - 1; ++j) Z[j] = ld4(FZ + (warp * VD_RB + j) * VD_TX + 4 * lane);
#pragma unroll
        for (int r = 0; r < VD_RB; ++r) {
            const float* fx = FX + (warp * VD_RB + r) * VD_FXW + 4 * lane;
            const float4 p0 = ld4(fx), p1 = ld4(fx + 4), p2 = ld4(fx + 8);
            const float w[12] = {p0.x, p0.y, p0.z, p0.w, p1.x, p1.y, p1.z, p1.w, p2.x, p2.y, p2.z, p2.w};
            // l = sz * (sum_k c_k (Z up - Z down)) + sum_k c_k (w right - w left), in pairs
            float2 xl = make_float2(0.f, 0.f), xh = xl, zl = xl, zh = xl;
#pragma unroll
            for (int k = 1; k <= R; ++k) {
                xl = __ffma2_rn(a.csp[k - 1], make_float2(w[3 + k] - w[4 - k], w[4 + k] - w[5 - k]), xl);
                xh = __ffma2_rn(a.csp[k - 1], make_float2(w[5 + k] - w[6 - k], w[6 + k] - w[7 - k]), xh);
                const float4 up = Z[r + R + k - 1], dn = Z[r + R - k];
                zl = __ffma2_rn(a.csp[k - 1], psub(lo2v(up), lo2v(dn)), zl);
                zh = __ffma2_rn(a.csp[k - 1], psub(hi2v(up), hi2v(dn)), zh);
            }
            const float2 szp = make_float2(a.vd_sz, a.vd_sz);
            const float2 ll = __ffma2_rn(szp, zl, xl), lh = __ffma2_rn(szp, zh, xh);
            out[r] = make_float4(ll.x, ll.y, lh.x, lh.y);
        }
    };

    for (int i = 0; i < ns; ++i) {
        const int s = s0 + i, b = i % L::STAGES;
        if (!mbar_wait(&bars[b], (i / L::STAGES) & 1)) report(a.err, DEV_ERR_TMA_TIMEOUT);
        const float* F = reinterpret_cast<const float*>(stage(b));
        const float* O = reinterpret_cast<const float*>(stage(b) + L::O_OFF);
        float* un = a.u_new + (long long)s * a.shot_stride;

        float4 lbu[MODE == MODE_GRAD_U ? VD_RB : 1], dxu[MODE == MODE_GRAD_U ? VD_RB : 1],
            dzu[MODE == MODE_GRAD_U ? VD_RB : 1];
        if (MODE == MODE_GRAD_U) {
            fluxes(reinterpret_cast<const float*>(stage(b) + L::U_OFF), dxu, dzu);
            __syncthreads();
            divergence(lbu);
            __syncthreads();  // the flux buffers are free again
            // G += q_{k+1} Lb u_k now, so that Lb u_k is no longer live
#pragma unroll
            for (int r = 0; r < VD_RB; ++r) {
                if (!zin[r]) continue;
                const float4 cv = ld4(F + (warp * VD_RB + r + 2 * R) * VD_W + 8 + 4 * lane);
                gk[r].x += xin[0] ? cv.x * lbu[r].x : 0.f;
                gk[r].y += xin[1] ? cv.y * lbu[r].y : 0.f;
                gk[r].z += xin[2] ? cv.z * lbu[r].z : 0.f;
                gk[r].w += xin[3] ? cv.w * lbu[r].w : 0.f;
            }
        }
        float4 dxq[VD_RB], dzq[VD_RB], lb[VD_RB];
        fluxes(F, dxq, dzq);
        if (MODE == MODE_GRAD_U) {  // the half-point terms now: the four differences die here
#pragma unroll
            for (int r = 0; r < VD_RB; ++r) {
                gbx[r].x -= dxq[r].x * dxu[r].x;
                gbx[r].y -= dxq[r].y * dxu[r].y;
                gbx[r].z -= dxq[r].z * dxu[r].z;
                gbx[r].w -= dxq[r].w * dxu[r].w;
                gbz[r].x -= a.vd_sz * dzq[r].x * dzu[r].x;
                gbz[r].y -= a.vd_sz * dzq[r].y * dzu[r].y;
                gbz[r].z -= a.vd_sz * dzq[r].z * dzu[r].z;
                gbz[r].w -= a.vd_sz * dzq[r].w * dzu[r].w;
            }
        }
        __syncthreads();
        // MODE_GRAD_U: u_{n-1} comes from global memory (plain loads: u_new is
        // this level's buffer, each cell read here and written below); issued
        // before the divergence so that their latency overlaps it
        float4 ovg[MODE == MODE_GRAD_U ? VD_RB : 1];
        if (MODE == MODE_GRAD_U) {
#pragma unroll
            for (int r = 0; r < VD_RB; ++r)
                ovg[r] = (zb + r < a.nz && x < a.ld)
                             ? *reinterpret_cast<const float4*>(un + (long long)(zb + r) * a.ld + x)
                             : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        divergence(lb);

#pragma unroll
        for (int r = 0; r < VD_RB; ++r) {
            const int z = zb + r;
            const float4 cv = ld4(F + (warp * VD_RB + r + 2 * R) * VD_W + 8 + 4 * lane);
            const long long off = (long long)z * a.ld + x;
            const float4 ov = MODE != MODE_GRAD_U ? ld4(O + (warp * VD_RB + r) * VD_TX + 4 * lane) : ovg[r];
            float nv[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const float g = gzr[r] * gxe[e];
                nv[e] = g * fmaf(comp(krow[r], e), comp(lb[r], e), 2.f * comp(cv, e)) - (g * g) * comp(ov, e);
            }
            if (zin[r] && all_x) {
                st4(un + off, make_float4(nv[0], nv[1], nv[2], nv[3]));
            } else if (a.zero_ring) {
                if (z < a.nz && x < a.ld)
                    st4(un + off, make_float4(zin[r] && xin[0] ? nv[0] : 0.f, zin[r] && xin[1] ? nv[1] : 0.f,
                                              zin[r] && xin[2] ? nv[2] : 0.f, zin[r] && xin[3] ? nv[3] : 0.f));
            } else if (zin[r]) {
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (xin[e]) un[off + e] = nv[e];
            }
        }

        // sampling of the staged level (receivers of the previous step, or the
        // adjoint field at the sources)
        {
            const int lo = smp_range[i].x, hi = smp_range[i].y;
            for (int j = lo + tid; j < hi; j += VD_THREADS) {
                const int2 en = a.smp.ent[j];
                const int z = en.x / a.ld, xx = en.x - z * a.ld;
                float v = F[(z - z0 + 2 * R) * VD_W + (xx - x0 + 8)] * a.smp_scale;
                if (a.smp_div_m) v /= a.m[en.x];
                a.smp_out[((long long)s * a.smp_nt + a.smp_t) * a.smp_np + en.y] = v;
            }
        }
        __syncthreads();  // stage b fully read, fluxes consumed, this shot's stores done
        if (tid == 0 && i + L::STAGES < ns) {
            fence_proxy_async_smem();
            issue(i + L::STAGES);
        }
        {
            const int lo = inj_range[i].x, hi = inj_range[i].y;
            for (int j = lo + tid; j < hi; j += VD_THREADS) {
                const int2 en = a.inj.ent[j];
                const int z = en.x / a.ld, xx = en.x - z * a.ld;
                float v = a.inj_val[((long long)s * a.inj_nt + a.inj_t) * a.inj_np + en.y] * a.inj_scale;
                if (a.inj_times_m) v *= a.m[en.x];
                const float g = (a.gz ? a.gz[z] : 1.f) * (a.gx ? a.gx[xx] : 1.f);
                atomicAdd(un + en.x, g * v);
            }
        }
    }

    if (MODE == MODE_GRAD_U) {
#pragma unroll
        for (int r = 0; r < VD_RB; ++r) {
            const int z = zb + r;
            if (z >= a.nz || x >= a.ld) continue;
            const long long off = (long long)z * a.ld + x;
            atomicAdd(reinterpret_cast<float4*>(a.grad + off), gk[r]);
            atomicAdd(reinterpret_cast<float4*>(a.grad_bx + off), gbx[r]);
            atomicAdd(reinterpret_cast<float4*>(a.grad_bz + off), gbz[r]);
        }
    }
}

template <int R, int MODE>
cudaError_t launch_impl(const CUtensorMap& mf, const CUtensorMap& mo, const CUtensorMap& mu,
                        const CUtensorMap& mb, const StepArgs& a, cudaStream_t s) {
    using L = LayoutVD<R, MODE>;
    static int configured_device = -1;
    int dev = 0;
    cudaGetDevice(&dev);
    if (configured_device != dev) {
        cudaError_t e = cudaFuncSetAttribute(step2d_vd_kernel<R, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             L::BYTES);
        if (e != cudaSuccess) return e;
        configured_device = dev;
    }
    const dim3 grid(a.tiles_x * a.tiles_z, (a.nshot + a.shots_per_cta - 1) / a.shots_per_cta);
    const cudaError_t e = launch_pdl(step2d_vd_kernel<R, MODE>, grid, dim3(VD_THREADS), L::BYTES, s, mf, mo, mu, mb,
                                      with_weight_pairs(a));
    count_launch();
    return e != cudaSuccess ? e : cudaGetLastError();
}

template <int R>
cudaError_t dispatch(int mode, const CUtensorMap& mf, const CUtensorMap& mo, const CUtensorMap& mu,
                     const CUtensorMap& mb, const StepArgs& a, cudaStream_t s) {
    switch (mode) {
        case MODE_PLAIN: return launch_impl<R, MODE_PLAIN>(mf, mo, mu, mb, a, s);
        case MODE_GRAD_U: return launch_impl<R, MODE_GRAD_U>(mf, mo, mu, mb, a, s);
        default: return cudaErrorInvalidValue;
    }
}

// k = kappa dt^2 / dx^2 and b = 1 / rho on [nz][ld] (0 in the row padding).
__global__ void vd_params_kernel(const float* kappa, const float* rho, float* k, float* b, int nz, int nx, int ld,
                                 float scale) {
    const long long n = (long long)nz * ld;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long z = i / ld;
        const int x = int(i - z * ld);
        const long long c = z * nx + x;
        k[i] = x < nx ? kappa[c] * scale : 0.f;
        b[i] = x < nx ? 1.f / rho[c] : 0.f;
    }
}

// dJ/dkappa = G / k * scale on the interior; dJ/drho = -(Gbx_{x-1} + Gbx_x + Gbz_{z-1} + Gbz_z) / 2 / rho^2.
__global__ void vd_finalize_kernel(const float* G, const float* Gbx, const float* Gbz, const float* k,
                                   const float* rho, float* gkap, float* grho, int nz, int nx, int ld, int R,
                                   float scale) {
    const long long n = (long long)nz * nx;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int z = int(i / nx), x = int(i - (long long)z * nx);
        const long long c = (long long)z * ld + x;
        const bool in = z >= R && z < nz - R && x >= R && x < nx - R;
        gkap[i] = in ? G[c] / k[c] * scale : 0.f;
        const float db = 0.5f * ((x > 0 ? Gbx[c - 1] : 0.f) + Gbx[c] + (z > 0 ? Gbz[c - ld] : 0.f) + Gbz[c]);
        grho[i] = -db / (rho[i] * rho[i]);
    }
}

int blocks_for(long long n) { return (int)std::min<long long>(std::max<long long>((n + 255) / 256, 1), 152LL * 32); }

}  // namespace

cudaError_t launch_step2d_vd(int R, int mode, const CUtensorMap& map_f, const CUtensorMap& map_o,
                             const CUtensorMap& map_u, const CUtensorMap& map_b, const StepArgs& a, cudaStream_t s) {
    switch (R) {
        case 1: return dispatch<1>(mode, map_f, map_o, map_u, map_b, a, s);
        case 2: return dispatch<2>(mode, map_f, map_o, map_u, map_b, a, s);
        case 4: return dispatch<4>(mode, map_f, map_o, map_u, map_b, a, s);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_vd_params(const float* kappa, const float* rho, float* k, float* b, int nz, int nx, int ld,
                             float scale, cudaStream_t s) {
    vd_params_kernel<<<blocks_for((long long)nz * ld), 256, 0, s>>>(kappa, rho, k, b, nz, nx, ld, scale);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_vd_finalize(const float* G, const float* Gbx, const float* Gbz, const float* k, const float* rho,
                               float* gkap, float* grho, int nz, int nx, int ld, int R, float scale, cudaStream_t s) {
    vd_finalize_kernel<<<blocks_for((long long)nz * nx), 256, 0, s>>>(G, Gbx, Gbz, k, rho, gkap, grho, nz, nx, ld, R,
                                                                      scale);
    count_launch();
    return cudaGetLastError();
}

}  // namespace wfd
