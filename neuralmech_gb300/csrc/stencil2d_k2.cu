// Two-step-blocked 2D time-step kernel of the acoustic wave path (sm_103a).
//
// One launch advances every shot by two steps (or one, `two_steps == 0`):
//   u_{n+1} = g (2 u_n + m L u_n) - g^2 u_{n-1},
//   u_{n+2} = g (2 u_{n+1} + m L u_{n+1}) - g^2 u_n,
// reading u_{n-1}, u_n and writing u_{n+1}, u_{n+2} to two other buffers.
// That saves the HBM round trip of u_{n+1}: about 8 instead of 12 bytes of
// field traffic per cell-update. This is the reference's temporal blocking
// (projects/18_simple_wave_fd/step2D_wave.cu:244-304, 8 steps of a 5-point
// stencil in one tile) for the order-2R stencil, at depth 2: each extra step
// widens the halo by R.
//
// Per CTA (256 threads, one shot): tile T = 120 x 32 cells. Shared memory
// holds:
//   U  = u_n on T plus a halo of 2R rows and 8 columns (136 x (32 + 4R), TMA),
//   O  = u_{n-1} on E = T plus R rows and 4 columns (128 x (32 + 2R), TMA); step 1
//        overwrites it in place with u_{n+1} on E,
//   M  = m on E (TMA),
//   L1, L2 (MODE_GRAD) = the stored L u tiles of the two steps (TMA).
// Step 1 runs over E with lane l owning E columns 4l..4l+3 (32 lanes x float4
// = 128 columns) and warp w owning E rows. Then the injections of step n that
// fall in E (also those owned by neighbouring tiles) are added in shared
// memory. Step 2 runs over T with lanes 1..30, the same column ownership.
// MODE_SAVE_LAP stores L u of both steps; MODE_GRAD accumulates
// q_{k+1} L u_k + q_k L u_{k-1} per cell and adds it once per launch.
#include "common.cuh"
#include "internal.h"

namespace wfd {
namespace {

__host__ __device__ constexpr int al128(int v) { return (v + 127) / 128 * 128; }

template <int R, int MODE>
struct LayoutK2 {
    static constexpr int EH = K2_TZ + 2 * R;  // E rows
    static constexpr int UH = K2_TZ + 4 * R;  // U rows
    static constexpr int U_BYTES = UH * K2_UW * 4;
    static constexpr int E_BYTES = EH * K2_EW * 4;
    static constexpr int L_BYTES = K2_TZ * K2_TX * 4;
    static constexpr int O_OFF = al128(U_BYTES);
    static constexpr int M_OFF = O_OFF + al128(E_BYTES);
    static constexpr int L1_OFF = M_OFF + al128(E_BYTES);
    static constexpr int L2_OFF = L1_OFF + (MODE == MODE_GRAD ? al128(L_BYTES) : 0);
    static constexpr int BAR_OFF = L2_OFF + (MODE == MODE_GRAD ? al128(L_BYTES) : 0);
    static constexpr int BYTES = BAR_OFF + 64 + 128;
    static constexpr int RB1 = (EH + 7) / 8;  // E rows per warp in step 1
    static constexpr int RB2 = K2_TZ / 8;     // T rows per warp in step 2
};

__device__ __forceinline__ float comp(const float4& v, int e) {
    return e == 0 ? v.x : e == 1 ? v.y : e == 2 ? v.z : v.w;
}
__device__ __forceinline__ float4 f4(const float* p) { return *reinterpret_cast<const float4*>(p); }

template <int R, int MODE>
__global__ void __launch_bounds__(K2_THREADS, 2)
    step2d_k2_kernel(const __grid_constant__ CUtensorMap map_u, const __grid_constant__ CUtensorMap map_o,
                     const __grid_constant__ CUtensorMap map_m, const __grid_constant__ CUtensorMap map_l1,
                     const __grid_constant__ CUtensorMap map_l2, const Step2Args p) {
    using L = LayoutK2<R, MODE>;
    const StepArgs& a = p.a;
    extern __shared__ unsigned char smem_raw[];
    unsigned char* base = reinterpret_cast<unsigned char*>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    float* U = reinterpret_cast<float*>(base);
    float* O = reinterpret_cast<float*>(base + L::O_OFF);  // u_{n-1}, then u_{n+1}, on E
    const float* M = reinterpret_cast<const float*>(base + L::M_OFF);
    const unsigned char* L1 = base + L::L1_OFF;
    const unsigned char* L2 = base + L::L2_OFF;
    uint64_t* bar = reinterpret_cast<uint64_t*>(base + L::BAR_OFF);

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int tile = blockIdx.x, s = blockIdx.y;
    const int ntiles = a.tiles_x * a.tiles_z;
    const int x0 = (tile % a.tiles_x) * K2_TX;
    const int z0 = (tile / a.tiles_x) * K2_TZ;
    const int two = p.two_steps;

    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (tid == 0) {
        const uint32_t lb = MODE == MODE_GRAD ? uint32_t(K2_TZ * K2_TX * (a.lap_bf16 ? 2 : 4)) : 0u;
        mbar_arrive_expect_tx(bar, uint32_t(L::U_BYTES + 2 * L::E_BYTES) + lb * (two ? 2u : 1u));
        tma_load_3d(U, &map_u, x0 - 8, z0 - 2 * R, s, bar);
        tma_load_3d(O, &map_o, x0 - 4, z0 - R, s, bar);
        tma_load_2d(const_cast<float*>(M), &map_m, x0 - 4, z0 - R, bar);
        if (MODE == MODE_GRAD) {
            tma_load_3d(const_cast<unsigned char*>(L1), &map_l1, x0, z0, s, bar);
            if (two) tma_load_3d(const_cast<unsigned char*>(L2), &map_l2, x0, z0, s, bar);
        }
    }
    // per-thread constants and point-list ranges while the tiles land: every
    // global read the CTA depends on is issued here, before the TMA wait
    __shared__ int2 rng[4];  // sampling, step-1 (extended) injection, step-2 injection
    if (tid < 3) {
        const PointLists& pl = tid == 0 ? a.smp : tid == 1 ? p.inj_e : a.inj;
        const int k = s * ntiles + tile;
        rng[tid] = pl.off != nullptr ? make_int2(pl.off[k], pl.off[k + 1]) : make_int2(0, 0);
    }
    const int ex = x0 - 4 + 4 * lane;  // global x of this lane's first E column
    float gz1[L::RB1], gz2[L::RB2];
#pragma unroll
    for (int r = 0; r < L::RB1; ++r) {
        const int z = z0 - R + warp * L::RB1 + r;
        gz1[r] = (a.gz != nullptr && z >= 0 && z < a.nz) ? __ldg(a.gz + z) : 1.f;
    }
#pragma unroll
    for (int r = 0; r < L::RB2; ++r) {
        const int z = z0 + warp * L::RB2 + r;
        gz2[r] = (a.gz != nullptr && z < a.nz) ? __ldg(a.gz + z) : 1.f;
    }
    float gxe[4];
    bool xin[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const int xx = ex + e;
        gxe[e] = (a.gx != nullptr && xx >= 0 && xx < a.nx) ? __ldg(a.gx + xx) : 1.f;
        xin[e] = xx >= R && xx < a.nx - R;
    }
    const bool all_x = xin[0] && xin[1] && xin[2] && xin[3];
    const bool t_lane = lane >= 1 && lane <= K2_TX / 4;  // lanes owning tile columns
    float* u_mid = p.u_mid + (long long)s * a.shot_stride;
    float* u_out = a.u_new + (long long)s * a.shot_stride;
    const long long lap_shot = (long long)s * a.shot_stride;

    if (!mbar_wait(bar, 0)) report(a.err, DEV_ERR_TMA_TIMEOUT);
    __syncthreads();  // rng visible to every thread

    // ---------------------------------------------------------------- step 1 on E
    {
        const int er0 = warp * L::RB1;
        float4 V[L::RB1 + 2 * R];
#pragma unroll
        for (int j = 0; j < L::RB1 + 2 * R; ++j) {
            const int ur = er0 + j;  // U row (E row er sits at U row er + R)
            V[j] = ur < L::UH ? f4(U + ur * K2_UW + 4 + 4 * lane) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int r = 0; r < L::RB1; ++r) {
            const int er = er0 + r;
            if (er >= L::EH) break;
            const int z = z0 - R + er;
            const float* urow = U + (er + R) * K2_UW + 4 * lane;
            const float4 lv = f4(urow), cv = V[r + R], rv = f4(urow + 8);
            const float w[12] = {lv.x, lv.y, lv.z, lv.w, cv.x, cv.y, cv.z, cv.w, rv.x, rv.y, rv.z, rv.w};
            float* orow = O + er * K2_EW + 4 * lane;
            const float4 ov = f4(orow);
            const float4 mv = f4(M + er * K2_EW + 4 * lane);
            const bool zin = z >= R && z < a.nz - R;
            const float gz = gz1[r];
            float nv[4], lap[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                float acc = a.c0 * w[4 + e];
#pragma unroll
                for (int k = 1; k <= R; ++k) {
                    acc = fmaf(a.cx[k - 1], w[4 + e - k] + w[4 + e + k], acc);
                    acc = fmaf(a.cz[k - 1], comp(V[r + R - k], e) + comp(V[r + R + k], e), acc);
                }
                lap[e] = acc;
                const float g = gz * gxe[e];
                nv[e] = (zin && xin[e]) ? g * fmaf(comp(mv, e), acc, 2.f * w[4 + e]) - (g * g) * comp(ov, e)
                                        : w[4 + e];  // fixed ring / outside the grid keep u_n
            }
            *reinterpret_cast<float4*>(orow) = make_float4(nv[0], nv[1], nv[2], nv[3]);
            if (MODE == MODE_SAVE_LAP && zin && t_lane && er >= R && er < R + K2_TZ) {
                const long long off = lap_shot + (long long)z * a.ld + ex;
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (xin[e]) {
                        if (a.lap_bf16)
                            static_cast<__nv_bfloat16*>(p.lap1)[off + e] = __float2bfloat16_rn(lap[e]);
                        else
                            static_cast<float*>(p.lap1)[off + e] = lap[e];
                    }
            }
        }
    }
    // sampling of u_n (receivers owned by this tile)
    if (p.smp_t1 >= 0) {
        const int lo = rng[0].x, hi = rng[0].y;
        for (int j = lo + tid; j < hi; j += K2_THREADS) {
            const int2 en = a.smp.ent[j];
            const int z = en.x / a.ld, xx = en.x - z * a.ld;
            float v = U[(z - z0 + 2 * R) * K2_UW + (xx - x0 + 8)] * a.smp_scale;
            if (a.smp_div_m) v /= a.m[en.x];
            a.smp_out[((long long)s * a.smp_nt + p.smp_t1) * a.smp_np + en.y] = v;
        }
    }
    __syncthreads();  // u_{n+1} on E complete in O
    // injection of step n into u_{n+1}, every point inside E (neighbours' too)
    if (p.inj_t1 >= 0 && rng[1].y > rng[1].x) {
        const int lo = rng[1].x, hi = rng[1].y;
        for (int j = lo + tid; j < hi; j += K2_THREADS) {
            const int2 en = p.inj_e.ent[j];
            const int z = en.x / a.ld, xx = en.x - z * a.ld;
            const int ez = z - (z0 - R), exx = xx - (x0 - 4);
            float v = a.inj_val[((long long)s * a.inj_nt + p.inj_t1) * a.inj_np + en.y] * a.inj_scale;
            if (a.inj_times_m) v *= M[ez * K2_EW + exx];
            const float g = (a.gz ? a.gz[z] : 1.f) * (a.gx ? a.gx[xx] : 1.f);
            atomicAdd(&O[ez * K2_EW + exx], g * v);
        }
        __syncthreads();
    }

    // ---------------------------------------------------------------- tile pass
    // store u_{n+1} on T; step 2 on T; gradient terms of both steps
    float4 gacc[L::RB2];
#pragma unroll
    for (int r = 0; r < L::RB2; ++r) gacc[r] = make_float4(0.f, 0.f, 0.f, 0.f);
    const int tr0 = warp * L::RB2;
    if (t_lane) {
        float4 V[L::RB2 + 2 * R];
        if (two) {
#pragma unroll
            for (int j = 0; j < L::RB2 + 2 * R; ++j) V[j] = f4(O + (tr0 + j) * K2_EW + 4 * lane);
        }
#pragma unroll
        for (int r = 0; r < L::RB2; ++r) {
            const int tr = tr0 + r, er = tr + R, z = z0 + tr;
            const bool zin = z >= R && z < a.nz - R;
            const float4 c1 = f4(O + er * K2_EW + 4 * lane);          // u_{n+1}
            const float4 c0 = f4(U + (tr + 2 * R) * K2_UW + 4 + 4 * lane);  // u_n
            const long long off = (long long)z * a.ld + ex;
            if (zin) {
                if (all_x)
                    *reinterpret_cast<float4*>(u_mid + off) = c1;
                else
#pragma unroll
                    for (int e = 0; e < 4; ++e)
                        if (xin[e]) u_mid[off + e] = comp(c1, e);
            }
            if (MODE == MODE_GRAD && zin) {
                const int li = tr * K2_TX + 4 * (lane - 1);
                const float4 l1 = a.lap_bf16 ? unpack_bf16x4(*reinterpret_cast<const uint2*>(
                                                   reinterpret_cast<const __nv_bfloat16*>(L1) + li))
                                             : f4(reinterpret_cast<const float*>(L1) + li);
                gacc[r].x += c0.x * l1.x;  // q_{k+1} L u_k
                gacc[r].y += c0.y * l1.y;
                gacc[r].z += c0.z * l1.z;
                gacc[r].w += c0.w * l1.w;
            }
            if (!two) continue;
            const float* nrow = O + er * K2_EW + 4 * lane;
            const float4 lv = f4(nrow - 4), rv = f4(nrow + 4);
            const float w[12] = {lv.x, lv.y, lv.z, lv.w, c1.x, c1.y, c1.z, c1.w, rv.x, rv.y, rv.z, rv.w};
            const float4 mv = f4(M + er * K2_EW + 4 * lane);
            const float gz = gz2[r];
            float nv[4], lap[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                float acc = a.c0 * w[4 + e];
#pragma unroll
                for (int k = 1; k <= R; ++k) {
                    acc = fmaf(a.cx[k - 1], w[4 + e - k] + w[4 + e + k], acc);
                    acc = fmaf(a.cz[k - 1], comp(V[r + R - k], e) + comp(V[r + R + k], e), acc);
                }
                lap[e] = acc;
                const float g = gz * gxe[e];
                nv[e] = g * fmaf(comp(mv, e), acc, 2.f * w[4 + e]) - (g * g) * comp(c0, e);
            }
            if (zin) {
                if (all_x) {
                    *reinterpret_cast<float4*>(u_out + off) = make_float4(nv[0], nv[1], nv[2], nv[3]);
                } else {
#pragma unroll
                    for (int e = 0; e < 4; ++e)
                        if (xin[e]) u_out[off + e] = nv[e];
                }
            }
            if (MODE == MODE_SAVE_LAP && zin) {
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (xin[e]) {
                        if (a.lap_bf16)
                            static_cast<__nv_bfloat16*>(a.lap)[lap_shot + off + e] = __float2bfloat16_rn(lap[e]);
                        else
                            static_cast<float*>(a.lap)[lap_shot + off + e] = lap[e];
                    }
            }
            if (MODE == MODE_GRAD && zin) {
                const int li = tr * K2_TX + 4 * (lane - 1);
                const float4 l2 = a.lap_bf16 ? unpack_bf16x4(*reinterpret_cast<const uint2*>(
                                                   reinterpret_cast<const __nv_bfloat16*>(L2) + li))
                                             : f4(reinterpret_cast<const float*>(L2) + li);
                gacc[r].x += c1.x * l2.x;  // q_k L u_{k-1}
                gacc[r].y += c1.y * l2.y;
                gacc[r].z += c1.z * l2.z;
                gacc[r].w += c1.w * l2.w;
            }
        }
    }
    if (two) {
        // sampling of u_{n+1} (receivers of this tile), from shared memory
        if (a.smp_t >= 0) {
            const int lo = rng[0].x, hi = rng[0].y;
            for (int j = lo + tid; j < hi; j += K2_THREADS) {
                const int2 en = a.smp.ent[j];
                const int z = en.x / a.ld, xx = en.x - z * a.ld;
                float v = O[(z - z0 + R) * K2_EW + (xx - x0 + 4)] * a.smp_scale;
                if (a.smp_div_m) v /= a.m[en.x];
                a.smp_out[((long long)s * a.smp_nt + a.smp_t) * a.smp_np + en.y] = v;
            }
        }
        __syncthreads();  // every u_{n+2} store of the tile is done
        if (a.inj_t >= 0) {
            const int lo = rng[2].x, hi = rng[2].y;
            for (int j = lo + tid; j < hi; j += K2_THREADS) {
                const int2 en = a.inj.ent[j];
                const int z = en.x / a.ld, xx = en.x - z * a.ld;
                float v = a.inj_val[((long long)s * a.inj_nt + a.inj_t) * a.inj_np + en.y] * a.inj_scale;
                if (a.inj_times_m) v *= a.m[en.x];
                const float g = (a.gz ? a.gz[z] : 1.f) * (a.gx ? a.gx[xx] : 1.f);
                atomicAdd(u_out + en.x, g * v);
            }
        }
    }
    if (MODE == MODE_GRAD && t_lane) {
#pragma unroll
        for (int r = 0; r < L::RB2; ++r) {
            const int z = z0 + tr0 + r;
            if (z < R || z >= a.nz - R) continue;
            float* gp = a.grad + (long long)z * a.ld + ex;
            if (all_x) {
                atomicAdd(reinterpret_cast<float4*>(gp), gacc[r]);
            } else {
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (xin[e]) atomicAdd(gp + e, comp(gacc[r], e));
            }
        }
    }
}

template <int R, int MODE>
cudaError_t launch_impl(const CUtensorMap& mu, const CUtensorMap& mo, const CUtensorMap& mm,
                        const CUtensorMap& l1, const CUtensorMap& l2, const Step2Args& p,
                        cudaStream_t s) {
    using L = LayoutK2<R, MODE>;
    static int configured_device = -1;
    int dev = 0;
    cudaGetDevice(&dev);
    if (configured_device != dev) {
        cudaError_t e = cudaFuncSetAttribute(step2d_k2_kernel<R, MODE>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, L::BYTES);
        if (e != cudaSuccess) return e;
        configured_device = dev;
    }
    const dim3 grid(p.a.tiles_x * p.a.tiles_z, p.a.nshot);
    step2d_k2_kernel<R, MODE><<<grid, K2_THREADS, L::BYTES, s>>>(mu, mo, mm, l1, l2, p);
    count_launch();
    return cudaGetLastError();
}

template <int R>
cudaError_t dispatch(int mode, const CUtensorMap& mu, const CUtensorMap& mo, const CUtensorMap& mm,
                     const CUtensorMap& l1, const CUtensorMap& l2, const Step2Args& p, cudaStream_t s) {
    switch (mode) {
        case MODE_PLAIN: return launch_impl<R, MODE_PLAIN>(mu, mo, mm, l1, l2, p, s);
        case MODE_SAVE_LAP: return launch_impl<R, MODE_SAVE_LAP>(mu, mo, mm, l1, l2, p, s);
        case MODE_GRAD: return launch_impl<R, MODE_GRAD>(mu, mo, mm, l1, l2, p, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace

cudaError_t launch_step2d_k2(int R, int mode, const CUtensorMap& map_u, const CUtensorMap& map_o,
                             const CUtensorMap& map_m, const CUtensorMap& map_l1,
                             const CUtensorMap& map_l2, const Step2Args& p, cudaStream_t s) {
    if (p.a.nshot > 65535) return cudaErrorInvalidValue;
    switch (R) {
        case 1: return dispatch<1>(mode, map_u, map_o, map_m, map_l1, map_l2, p, s);
        case 2: return dispatch<2>(mode, map_u, map_o, map_m, map_l1, map_l2, p, s);
        case 4: return dispatch<4>(mode, map_u, map_o, map_m, map_l1, map_l2, p, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace wfd
