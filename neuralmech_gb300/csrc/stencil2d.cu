// 2D time-step kernel of the acoustic wave path (sm_103a).
//
// One launch advances every shot of a batch by one step:
//   u_{n+1} = g (2 u_n + m L u_n) - g^2 u_{n-1}    on the interior,
// with m = (v dt / dx)^2, L the order-2R central Laplacian (per-axis weights
// pre-scaled by (dx/h)^2) and g = gz[z] gx[x] the sponge factor. It replaces
// the reference's padded_step (projects/18_simple_wave_fd/step2D_wave.cu:59-81),
// which is the R = 1, g = 1, constant-m case.
//
// Layout in HBM: each field is [shot][z][ld] FP32, ld a multiple of 8; the
// model m is [z][ld], shared by all shots. u_{n+1} overwrites u_{n-1} in place
// (or goes to a fresh buffer: the kernel writes every cell of its tile, the
// fixed ring as 0).
//
// Per CTA (256 threads): a 128 x TZ tile (TZ = 32 or 16 rows) of one shot at a time, over
// `shots_per_cta` shots of the batch. For each shot a TMA bulk-tensor load
// brings u_n with a halo of R rows and 4 columns and the u_{n-1} tile into
// shared memory; two stages are in flight so the next shot's tiles load while
// this one computes. m, the sponge factors and the gradient accumulator stay
// in registers across the shots, so m is read once per tile per step and the
// gradient written once per tile per step. Lane l owns x = x0 + 4l .. +3
// (float4 loads/stores); warp w owns rows z0 + RB w .. + RB - 1, with the
// vertical taps held in a register window.
//
// Fused per-step point work, bucketed by tile (PointLists):
//   * sampling of the staged u_n at receivers (traces of the previous step),
//   * injection into u_{n+1} (sources, or m-scaled residuals in the adjoint),
//   * MODE_SAVE_LAP: L u_n stored (FP32 or BF16) for the adjoint's imaging term,
//   * MODE_GRAD: q_{k+1} L u_k accumulated into the gradient;
//   * MODE_GRAD_U: the same with u_k staged (with its halo) instead of L u_k,
//     and L u_k formed in the kernel: the recompute then stores nothing but
//     the levels it writes anyway. This mode runs on 16-row tiles: with the
//     third tile, two stages of 32-row tiles would leave one CTA per SM.
//   * MODE_GRAD_U16: MODE_GRAD_U for a level kept in block floating point
//     (int16 mantissas, one exponent byte per 4 cells: 2.25 bytes per cell),
//     each thread decoding the blocks it reads.
//
// MODE_SUMMED advances the same recursion in its summed (increment) form
// (P. Henrici, Discrete Variable Methods in Ordinary Differential Equations,
// 1962): the state is u_n and the increment d_n = u_n - u_{n-1}, and
//   d_{n+1} = g^2 d_n - (1 - g)^2 u_n + g m L u_n,   u_{n+1} = u_n + d_{n+1},
// which is u_{n+1} = g (2 u_n + m L u_n) - g^2 u_{n-1} rearranged. In FP32 the
// increment, about (omega dt) |u| in size, keeps its own low bits. The
// leapfrog form instead feeds the rounding of two stored levels of size |u|
// into the velocity u_n - u_{n-1} at every step, where the recursion
// amplifies it by about 1 / (omega dt). The Laplacian of this mode is formed
// from neighbour differences (lap_row_diff), whose rounding is relative to
// the differences rather than to |u|: with the increment rounded on its own
// scale, the Laplacian's rounding is the next largest term. The staged "old" tile is d_n;
// d_{n+1} is written over it in place (each cell is read and written by its
// own thread) and u_{n+1} goes to u_new. 4 more bytes per update than the
// leapfrog step (the d write).
#include "common.cuh"
#include "internal.h"

namespace wfd {
namespace {

__host__ __device__ constexpr int align_up(int v, int a) { return (v + a - 1) / a * a; }

template <int R, int MODE, int RB>
struct Layout2D {
    static constexpr int TZ = 8 * RB;  // tile rows: 8 warps x RB rows
    static constexpr int H = TZ + 2 * R;
    static constexpr int CUR = H * T2_W * 4;  // TMA box bytes of u_n
    static constexpr int OLD = TZ * T2_TX * 4;
    // MODE_GRAD_U16: u_k's int16 mantissas (144 columns from x0 - 8) and
    // exponent bytes (64, one per 4 cells from x0 - 64)
    static constexpr int Q16 = H * (T2_TX + 16) * 2;
    static constexpr int E8 = H * 64;
    static constexpr int LAP = MODE == MODE_GRAD     ? TZ * T2_TX * 4
                               : MODE == MODE_GRAD_U ? H * T2_W * 4
                               : MODE == MODE_GRAD_U16 ? align_up(Q16, 128) + E8
                                                       : 0;
    // every TMA destination starts on a 128-byte boundary
    static constexpr int CUR_AL = align_up(CUR, 128);
    static constexpr int OLD_AL = align_up(OLD, 128);
    static constexpr int STAGE = align_up(CUR_AL + OLD_AL + LAP, 128);
    // TMA stages in flight per CTA: three for the u-store adjoint, whose three
    // tiles per shot make a stage the longest to arrive
    static constexpr bool GU = MODE == MODE_GRAD_U || MODE == MODE_GRAD_U16;
    static constexpr int STAGES = GU ? 3 : T2_STAGES;
    static constexpr int BYTES = STAGES * STAGE + 64 + 128;  // + barriers + alignment slack
};

template <int R, int MODE, int RB>
__global__ void __launch_bounds__(T2_THREADS, (RB == 2 && !Layout2D<R, MODE, RB>::GU && MODE != MODE_SUMMED) ? 3 : 2)
    step2d_kernel(const __grid_constant__ CUtensorMap map_cur,
                  const __grid_constant__ CUtensorMap map_old,
                  const __grid_constant__ CUtensorMap map_lap,
                  const __grid_constant__ CUtensorMap map_lx, const StepArgs a) {
    using L = Layout2D<R, MODE, RB>;
    constexpr int TZ = L::TZ;
    extern __shared__ unsigned char smem_raw[];
    unsigned char* base = reinterpret_cast<unsigned char*>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    uint64_t* bars = reinterpret_cast<uint64_t*>(base + L::STAGES * L::STAGE);

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int tile = blockIdx.x;
    const int ntiles = a.tiles_x * a.tiles_z;
    const int x0 = (tile % a.tiles_x) * T2_TX;
    const int z0 = (tile / a.tiles_x) * TZ;
    const int s0 = blockIdx.y * a.shots_per_cta;
    const int ns = min(a.nshot - s0, a.shots_per_cta);
    if (ns <= 0) return;

    const uint32_t lap_bytes =
        MODE == MODE_GRAD       ? uint32_t(TZ * T2_TX * (a.lap_bf16 ? 2 : 4))
        : MODE == MODE_GRAD_U   ? uint32_t(L::CUR)
        : MODE == MODE_GRAD_U16 ? uint32_t(L::Q16 + L::E8)
                                : 0u;
    const uint32_t stage_tx = uint32_t(L::CUR + L::OLD) + lap_bytes;
    auto cur_buf = [&](int b) { return reinterpret_cast<float*>(base + b * L::STAGE); };
    auto old_buf = [&](int b) { return reinterpret_cast<float*>(base + b * L::STAGE + L::CUR_AL); };
    auto lap_buf = [&](int b) { return base + b * L::STAGE + L::CUR_AL + L::OLD_AL; };

    auto issue = [&](int i) {  // called by thread 0 only
        const int b = i % L::STAGES;
        mbar_arrive_expect_tx(&bars[b], stage_tx);
        tma_load_3d(cur_buf(b), &map_cur, x0 - T2_XH, z0 - R, s0 + i, &bars[b]);
        tma_load_3d(old_buf(b), &map_old, x0, z0, s0 + i, &bars[b]);
        if (MODE == MODE_GRAD) tma_load_3d(lap_buf(b), &map_lap, x0, z0, s0 + i, &bars[b]);
        if (MODE == MODE_GRAD_U)  // u_k with the halo of u_n
            tma_load_3d(lap_buf(b), &map_lap, x0 - T2_XH, z0 - R, s0 + i, &bars[b]);
        if (MODE == MODE_GRAD_U16) {  // its mantissas and exponents (16-byte aligned x: x0 - 8, x0/4 - 16)
            tma_load_3d(lap_buf(b), &map_lap, x0 - 8, z0 - R, s0 + i, &bars[b]);
            tma_load_3d(lap_buf(b) + align_up(L::Q16, 128), &map_lx, x0 / 4 - 16, z0 - R, s0 + i, &bars[b]);
        }
    };

    // point-list ranges of this tile for every shot of the CTA, staged once
    // (one global read each instead of a dependent read per shot and list)
    __shared__ int2 smp_range[T2_MAX_SPC], inj_range[T2_MAX_SPC];
    // launched as a programmatic dependent: everything above touches only
    // registers and shared memory; every global access comes after the wait
    if (tid == 0) {
        for (int b = 0; b < L::STAGES; ++b) mbar_init(&bars[b], 1);
        fence_mbar_init();
    }
    grid_dependency_wait();
    // the first stages are issued before the point-list ranges are read, so
    // that the two memory latencies overlap
    if (tid == 0) {
        for (int i = 0; i < min(ns, L::STAGES); ++i) issue(i);
        launch_dependents();  // the next step's CTAs may take SM slots this grid frees
    }
    // ---- per-thread constants, reused for every shot of the CTA (loaded before
    // the barrier below, so that their latency overlaps the range reads)
    const int x = x0 + 4 * lane;
    const int zb = z0 + warp * RB;
    float4 mrow[RB];
    float gzr[RB];
    bool zin[RB];
#pragma unroll
    for (int r = 0; r < RB; ++r) {
        const int z = zb + r;
        if (a.m != nullptr && z < a.nz && x < a.ld)
            mrow[r] = __ldg(reinterpret_cast<const float4*>(a.m + (long long)z * a.ld + x));
        else
            mrow[r] = make_float4(a.m_const, a.m_const, a.m_const, a.m_const);
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

    float4 gacc[RB];
#pragma unroll
    for (int r = 0; r < RB; ++r) gacc[r] = make_float4(0.f, 0.f, 0.f, 0.f);

    for (int i = 0; i < ns; ++i) {
        const int s = s0 + i, b = i % L::STAGES;
        if (!mbar_wait(&bars[b], (i / L::STAGES) & 1)) report(a.err, DEV_ERR_TMA_TIMEOUT);
        const float* cur = cur_buf(b);
        const float* old = old_buf(b);
        float* un = a.u_new + (long long)s * a.shot_stride;

        // MODE_GRAD_U: L u_k of this thread's cells from the staged u_k tile,
        // times q_{k+1} at the cells into the gradient sum (before the q
        // window is loaded, so that the two register windows never coexist).
        // MODE_GRAD_U16 decodes each 4-cell block it reads from the staged
        // mantissas (144 columns from x0 - 8) and exponents (from x0 - 64).
        if (L::GU) {
            // staged row j, 4-cell block c (cells x0 - 4 + 4 c, the u_n box's column 4 c)
            auto u4 = [&](int j, int c) -> float4 {
                if constexpr (MODE == MODE_GRAD_U16) {
                    const unsigned char* st = lap_buf(b);
                    const uint2 q = *reinterpret_cast<const uint2*>(st + (j * (T2_TX + 16) + 4 + 4 * c) * 2);
                    return bfp4_decode(q, st[align_up(L::Q16, 128) + j * 64 + 15 + c]);
                } else {
                    return *reinterpret_cast<const float4*>(reinterpret_cast<const float*>(lap_buf(b)) + j * T2_W +
                                                            4 * c);
                }
            };
            float4 W[RB + 2 * R];
#pragma unroll
            for (int j = 0; j < RB + 2 * R; ++j) W[j] = u4(warp * RB + j, lane + 1);
#pragma unroll
            for (int r = 0; r < RB; ++r) {
                if (!zin[r]) continue;
                const float4 lv = u4(warp * RB + r + R, lane);
                const float4 cv = W[r + R];
                const float4 rv = u4(warp * RB + r + R, lane + 2);
                const float4 qv =
                    *reinterpret_cast<const float4*>(cur + (warp * RB + r + R) * T2_W + T2_XH + 4 * lane);
                const float4 lu = lap_row<R>(lv, cv, rv, W, r + R, a);
                float l4[4];
#pragma unroll
                for (int e = 0; e < 4; ++e) l4[e] = xin[e] ? comp(qv, e) * comp(lu, e) : 0.f;
                gacc[r].x += l4[0];
                gacc[r].y += l4[1];
                gacc[r].z += l4[2];
                gacc[r].w += l4[3];
            }
        }

        float4 V[RB + 2 * R];
#pragma unroll
        for (int j = 0; j < RB + 2 * R; ++j)
            V[j] = *reinterpret_cast<const float4*>(cur + (warp * RB + j) * T2_W + T2_XH +
                                                    4 * lane);
#pragma unroll
        for (int r = 0; r < RB; ++r) {
            const int z = zb + r;
            const float* row = cur + (warp * RB + r + R) * T2_W + 4 * lane;
            const float4 lv = *reinterpret_cast<const float4*>(row);
            const float4 cv = V[r + R];
            const float4 rv = *reinterpret_cast<const float4*>(row + 2 * T2_XH);
            const float4 ov =
                *reinterpret_cast<const float4*>(old + (warp * RB + r) * T2_TX + 4 * lane);
            const float4 l = MODE == MODE_SUMMED ? lap_row_diff<R>(lv, cv, rv, V, r + R, a)
                                                 : lap_row<R>(lv, cv, rv, V, r + R, a);
            float lap[4], nv[4], dv[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const float acc = comp(l, e);
                lap[e] = acc;
                const float g = gzr[r] * gxe[e];
                const float c = comp(cv, e);
                if (MODE == MODE_SUMMED) {  // ov is d_n; g = 1 gives d_n + m L u_n
                    const float omg = 1.f - g;
                    dv[e] = fmaf(g * comp(mrow[r], e), acc, fmaf(g * g, comp(ov, e), -(omg * omg) * c));
                    nv[e] = c + dv[e];
                } else {
                    nv[e] = g * fmaf(comp(mrow[r], e), acc, 2.f * c) - (g * g) * comp(ov, e);
                }
            }
            const long long off = (long long)z * a.ld + x;
            float* dn = MODE == MODE_SUMMED ? a.d_new + (long long)s * a.shot_stride : nullptr;
            if (zin[r] && all_x) {
                *reinterpret_cast<float4*>(un + off) = make_float4(nv[0], nv[1], nv[2], nv[3]);
                if (MODE == MODE_SUMMED)
                    *reinterpret_cast<float4*>(dn + off) = make_float4(dv[0], dv[1], dv[2], dv[3]);
            } else if (a.zero_ring) {
                // the fixed ring (and the row padding) as 0, so that a level
                // written to a fresh buffer needs no separate clearing
                if (z < a.nz && x < a.ld) {  // (ld is a multiple of 8: x + 3 < ld)
                    *reinterpret_cast<float4*>(un + off) =
                        make_float4(zin[r] && xin[0] ? nv[0] : 0.f, zin[r] && xin[1] ? nv[1] : 0.f,
                                    zin[r] && xin[2] ? nv[2] : 0.f, zin[r] && xin[3] ? nv[3] : 0.f);
                    if (MODE == MODE_SUMMED)
                        *reinterpret_cast<float4*>(dn + off) =
                            make_float4(zin[r] && xin[0] ? dv[0] : 0.f, zin[r] && xin[1] ? dv[1] : 0.f,
                                        zin[r] && xin[2] ? dv[2] : 0.f, zin[r] && xin[3] ? dv[3] : 0.f);
                }
            } else if (zin[r]) {
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (xin[e]) {
                        un[off + e] = nv[e];
                        if (MODE == MODE_SUMMED) dn[off + e] = dv[e];
                    }
            }
            if (MODE == MODE_SAVE_LAP && zin[r]) {
                const long long lo = (long long)s * a.shot_stride + off;
                const float4 lp = make_float4(lap[0], lap[1], lap[2], lap[3]);
                if (all_x) {
                    if (a.lap_bf16)
                        *reinterpret_cast<uint2*>(static_cast<__nv_bfloat16*>(a.lap) + lo) =
                            pack_bf16x4(lp);
                    else
                        *reinterpret_cast<float4*>(static_cast<float*>(a.lap) + lo) = lp;
                } else {
#pragma unroll
                    for (int e = 0; e < 4; ++e)
                        if (xin[e]) {
                            if (a.lap_bf16)
                                static_cast<__nv_bfloat16*>(a.lap)[lo + e] =
                                    __float2bfloat16_rn(lap[e]);
                            else
                                static_cast<float*>(a.lap)[lo + e] = lap[e];
                        }
                }
            }
            if (MODE == MODE_GRAD && zin[r]) {
                const unsigned char* lb = lap_buf(b);
                const int li = (warp * RB + r) * T2_TX + 4 * lane;
                const float4 lu =
                    a.lap_bf16 ? unpack_bf16x4(*reinterpret_cast<const uint2*>(
                                     reinterpret_cast<const __nv_bfloat16*>(lb) + li))
                               : *reinterpret_cast<const float4*>(
                                     reinterpret_cast<const float*>(lb) + li);
                gacc[r].x += xin[0] ? cv.x * lu.x : 0.f;
                gacc[r].y += xin[1] ? cv.y * lu.y : 0.f;
                gacc[r].z += xin[2] ? cv.z * lu.z : 0.f;
                gacc[r].w += xin[3] ? cv.w * lu.w : 0.f;
            }
        }

        // sampling of the staged level u_n (receivers of the previous step,
        // or the adjoint field at the sources)
        {
            const int lo = smp_range[i].x, hi = smp_range[i].y;
            for (int j = lo + tid; j < hi; j += T2_THREADS) {
                const int2 en = a.smp.ent[j];
                const int z = en.x / a.ld, xx = en.x - z * a.ld;
                float v = cur[(z - z0 + R) * T2_W + (xx - x0 + T2_XH)] * a.smp_scale;
                if (a.smp_div_m) v /= (a.m != nullptr ? a.m[en.x] : a.m_const);
                a.smp_out[((long long)s * a.smp_nt + a.smp_t) * a.smp_np + en.y] = v;
            }
        }
        __syncthreads();  // stage b fully read; this shot's u_{n+1} stores done
        if (tid == 32 * (i % (T2_THREADS / 32)) && i + L::STAGES < ns) {  // (issuing warp rotates)
            fence_proxy_async_smem();
            issue(i + L::STAGES);
        }
        // injection into u_{n+1}, after every store of this shot
        {
            const int lo = inj_range[i].x, hi = inj_range[i].y;
            for (int j = lo + tid; j < hi; j += T2_THREADS) {
                const int2 en = a.inj.ent[j];
                const int z = en.x / a.ld, xx = en.x - z * a.ld;
                float v = a.inj_val[((long long)s * a.inj_nt + a.inj_t) * a.inj_np + en.y] *
                          a.inj_scale;
                if (a.inj_times_m) v *= (a.m != nullptr ? a.m[en.x] : a.m_const);
                const float g = (a.gz ? a.gz[z] : 1.f) * (a.gx ? a.gx[xx] : 1.f);
                atomicAdd(un + en.x, g * v);
                if (MODE == MODE_SUMMED) atomicAdd(a.d_new + (long long)s * a.shot_stride + en.x, g * v);
            }
        }
    }

    if (MODE == MODE_GRAD || L::GU) {
#pragma unroll
        for (int r = 0; r < RB; ++r) {
            if (!zin[r]) continue;
            float* gp = a.grad + (long long)(zb + r) * a.ld + x;
            if (all_x) {
                atomicAdd(reinterpret_cast<float4*>(gp), gacc[r]);  // one 16-byte reduction
            } else {
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (xin[e]) atomicAdd(gp + e, comp(gacc[r], e));
            }
        }
    }
}

template <int R, int MODE, int RB>
cudaError_t launch_impl(const CUtensorMap& mc, const CUtensorMap& mo, const CUtensorMap& ml,
                        const CUtensorMap& mx, const StepArgs& a_in, cudaStream_t s) {
    const StepArgs a = with_weight_pairs(a_in);
    using L = Layout2D<R, MODE, RB>;
    static int configured_device = -1;
    int dev = 0;
    cudaGetDevice(&dev);
    if (configured_device != dev) {
        cudaError_t e = cudaFuncSetAttribute(step2d_kernel<R, MODE, RB>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, L::BYTES);
        if (e != cudaSuccess) return e;
        configured_device = dev;
    }
    const dim3 grid(a.tiles_x * a.tiles_z, (a.nshot + a.shots_per_cta - 1) / a.shots_per_cta);
    const cudaError_t e =
        launch_pdl(step2d_kernel<R, MODE, RB>, grid, dim3(T2_THREADS), L::BYTES, s, mc, mo, ml, mx, a);
    count_launch();
    return e != cudaSuccess ? e : cudaGetLastError();
}

template <int R, int RB>
cudaError_t dispatch_mode(int mode, const CUtensorMap& mc, const CUtensorMap& mo, const CUtensorMap& ml,
                          const CUtensorMap& mx, const StepArgs& a, cudaStream_t s) {
    switch (mode) {
        case MODE_PLAIN: return launch_impl<R, MODE_PLAIN, RB>(mc, mo, ml, mx, a, s);
        case MODE_SAVE_LAP: return launch_impl<R, MODE_SAVE_LAP, RB>(mc, mo, ml, mx, a, s);
        case MODE_GRAD: return launch_impl<R, MODE_GRAD, RB>(mc, mo, ml, mx, a, s);
        case MODE_GRAD_U: return launch_impl<R, MODE_GRAD_U, RB>(mc, mo, ml, mx, a, s);
        case MODE_SUMMED: return launch_impl<R, MODE_SUMMED, RB>(mc, mo, ml, mx, a, s);
        // (the u-store adjoint runs on 16-row tiles)
        case MODE_GRAD_U16: return RB == 2 ? launch_impl<R, MODE_GRAD_U16, 2>(mc, mo, ml, mx, a, s)
                                           : cudaErrorInvalidValue;
        default: return cudaErrorInvalidValue;
    }
}

template <int RB>
cudaError_t dispatch_r(int R, int mode, const CUtensorMap& mc, const CUtensorMap& mo, const CUtensorMap& ml,
                       const CUtensorMap& mx, const StepArgs& a, cudaStream_t s) {
    switch (R) {
        case 1: return dispatch_mode<1, RB>(mode, mc, mo, ml, mx, a, s);
        case 2: return dispatch_mode<2, RB>(mode, mc, mo, ml, mx, a, s);
        case 4: return dispatch_mode<4, RB>(mode, mc, mo, ml, mx, a, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace

cudaError_t launch_step2d(int R, int mode, int tile_rows, const CUtensorMap& mc,
                          const CUtensorMap& mo, const CUtensorMap& ml, const StepArgs& a,
                          cudaStream_t s, const CUtensorMap* mx) {
    if (mode == MODE_GRAD_U16 && !mx) return cudaErrorInvalidValue;
    const CUtensorMap& x = mx ? *mx : ml;
    switch (tile_rows) {
        case 16: return dispatch_r<2>(R, mode, mc, mo, ml, x, a, s);
        case 32: return dispatch_r<4>(R, mode, mc, mo, ml, x, a, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace wfd
