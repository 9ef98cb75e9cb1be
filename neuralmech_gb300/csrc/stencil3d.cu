// 3D time-step kernel of the acoustic wave path (sm_103a).
//
// Same update as the 2D kernel,
//   u_{n+1} = g (2 u_n + m L u_n) - g^2 u_{n-1},  g = gz[z] gy[y] gx[x],
// on fields [shot][z][y][ld] FP32 (x fastest, ld a multiple of 8).
//
// Per CTA (256 threads = 16 lanes along x x 16 rows along y): one shot, one
// 64 x 16 (x, y) column, marching along z through T3_ZCHUNK output planes.
// The shot is the fastest grid index: the CTAs of all shots of one column run
// together, so m and (MODE_GRAD) the gradient tile are read from DRAM once
// per column and served from L2 to the other shots.
//   * u_n planes, each with a halo of R rows in y and 4 columns in x, arrive by
//     TMA (cp.async.bulk.tensor.4d) into a ring of NB = 4 + R shared-memory
//     buffers, four planes ahead of use. A thread keeps the 2R + 1 z-taps of
//     its 4 cells in a register queue; the x and y taps come from the staged
//     plane of the output z.
//   * u_{n-1}, m and (MODE_GRAD) the stored L u of output plane zr arrive by
//     TMA into a ring of NBO = 4 buffers, on the mbarrier of staged plane
//     zr + 2R (the plane that output first needs): one wait per plane.
//   * All mbarrier waits are bounded (status bit on give-up, never a trap).
//   * Point lists are bucketed by (z chunk, y tile, x tile). At each output
//     plane the CTA samples receivers from the staged u_n plane, and after its
//     stores injects into u_{n+1}.
//   * MODE_SAVE_LAP stores L u_n; MODE_GRAD adds q_{k+1} L u_k into the
//     gradient with 16-byte vector atomics.
//   * MODE_SUMMED is the summed (increment) form of the 2D kernel's mode of
//     that name: the staged output-plane tile is d_n = u_n - u_{n-1} instead
//     of u_{n-1}, d_{n+1} = g^2 d_n - (1 - g)^2 u_n + g m L u_n goes to d_new
//     in place and u_{n+1} = u_n + d_{n+1} to u_new (the Laplacian keeps the
//     centre-weight form: this kernel is issue-bound).
#include "common.cuh"
#include "internal.h"

namespace wfd {
namespace {

__host__ __device__ constexpr int align3(int v, int a) { return (v + a - 1) / a * a; }

constexpr int NBO = 4;  // u_{n-1} / m / L u tile ring (the u_n ring has NBO + R buffers)
constexpr int LANES_X = T3_TX / 4;  // 16

template <int R, int MODE>
struct Layout3D {
    static constexpr int NB = NBO + R;  // u_n plane ring
    static constexpr int H = T3_TY + 2 * R;
    static constexpr int CUR = H * T3_W * 4;  // TMA box bytes of one u_n plane
    static constexpr int CUR_AL = align3(CUR, 128);
    static constexpr int TILE = T3_TY * T3_TX * 4;  // one FP32 output-plane tile
    static constexpr int OLD_GROUP = 2 * TILE + (MODE == MODE_GRAD ? TILE : 0);  // old, m, lap
    static constexpr int BYTES = NB * CUR_AL + NBO * OLD_GROUP + NB * 8 + T3_ZCHUNK * 4 + 128;
};

__device__ __forceinline__ float2 lo2(const float4& v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(const float4& v) { return make_float2(v.z, v.w); }

template <int R, int MODE, int TR>
__global__ void __launch_bounds__(LANES_X * T3_TY / TR, 2)
    step3d_kernel(const __grid_constant__ CUtensorMap map_cur,
                  const __grid_constant__ CUtensorMap map_old,
                  const __grid_constant__ CUtensorMap map_lap,
                  const __grid_constant__ CUtensorMap map_m, const StepArgs a) {
    using L = Layout3D<R, MODE>;
    constexpr int NB = L::NB;
    constexpr int Q = 2 * R + 1;                 // z taps held in registers per row
    constexpr int NTH = LANES_X * T3_TY / TR;    // threads
    constexpr int YW = TR + 2 * R;               // staged rows a thread reads for its y taps
    extern __shared__ unsigned char smem_raw[];
    unsigned char* base = reinterpret_cast<unsigned char*>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    unsigned char* cur_ring = base;
    unsigned char* old_ring = base + NB * L::CUR_AL;
    uint64_t* bc = reinterpret_cast<uint64_t*>(old_ring + NBO * L::OLD_GROUP);
    float* gzs = reinterpret_cast<float*>(bc + NB);  // gz of the CTA's output planes

    const int tid = threadIdx.x, lane = tid % LANES_X;
    const int yr0 = (tid / LANES_X) * TR;  // first tile row of this thread
    const int s = blockIdx.x;
    const int tile = blockIdx.y;
    const int ntiles = a.tiles_x * a.tiles_y * a.tiles_z;
    const int tx_i = tile % a.tiles_x;
    const int ty_i = (tile / a.tiles_x) % a.tiles_y;
    const int tz_i = tile / (a.tiles_x * a.tiles_y);
    const int x0 = tx_i * T3_TX, y0 = ty_i * T3_TY, z0 = tz_i * T3_ZCHUNK;
    const int zc = min(T3_ZCHUNK, a.nz - z0);  // output planes of this CTA
    const int total = zc + 2 * R;               // u_n planes it stages

    const uint32_t lap_bytes = MODE == MODE_GRAD ? uint32_t(T3_TY * T3_TX * (a.lap_bf16 ? 2 : 4)) : 0u;
    auto cur_buf = [&](int p) { return reinterpret_cast<float*>(cur_ring + (p % NB) * L::CUR_AL); };
    auto old_buf = [&](int zr) { return reinterpret_cast<float*>(old_ring + (zr % NBO) * L::OLD_GROUP); };
    auto m_buf = [&](int zr) { return reinterpret_cast<float*>(old_ring + (zr % NBO) * L::OLD_GROUP + L::TILE); };
    auto lap_buf = [&](int zr) { return old_ring + (zr % NBO) * L::OLD_GROUP + 2 * L::TILE; };

    // staged plane p holds u_n at z = z0 - R + p; old group zr holds output
    // plane z0 + zr and travels with staged plane zr + 2R (p < total <=> zr < zc)
    auto issue = [&](int p) {
        uint64_t* bar = &bc[p % NB];
        const int zr = p - 2 * R;
        mbar_arrive_expect_tx(bar, uint32_t(L::CUR) + (zr >= 0 ? uint32_t(2 * L::TILE) + lap_bytes : 0u));
        tma_load_4d(cur_buf(p), &map_cur, x0 - T3_XH, y0 - R, z0 - R + p, s, bar);
        if (zr >= 0) {
            tma_load_4d(old_buf(zr), &map_old, x0, y0, z0 + zr, s, bar);
            tma_load_3d(m_buf(zr), &map_m, x0, y0, z0 + zr, bar);
            if (MODE == MODE_GRAD) tma_load_4d(lap_buf(zr), &map_lap, x0, y0, z0 + zr, s, bar);
        }
    };

    if (tid == 0) {
        for (int b = 0; b < NB; ++b) mbar_init(&bc[b], 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (tid == 0)
        for (int p = 0; p < min(NB, total); ++p) issue(p);
    if (tid < zc) gzs[tid] = a.gz != nullptr ? __ldg(a.gz + z0 + tid) : 1.f;

    // ---- per-thread constants
    const int x = x0 + 4 * lane;
    float gxe[4];
    bool xin[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        gxe[e] = (a.gx != nullptr && x + e < a.nx) ? __ldg(a.gx + x + e) : 1.f;
        xin[e] = x + e >= R && x + e < a.nx - R;
    }
    const bool all_x = xin[0] && xin[1] && xin[2] && xin[3];
    bool yin[TR];
    float gyv[TR];
#pragma unroll
    for (int t = 0; t < TR; ++t) {
        const int y = y0 + yr0 + t;
        yin[t] = y >= R && y < a.ny - R;
        gyv[t] = (a.gy != nullptr && y < a.ny) ? __ldg(a.gy + y) : 1.f;
    }
    float* un = a.u_new + (long long)s * a.shot_stride;
    float* dnw = MODE == MODE_SUMMED ? a.d_new + (long long)s * a.shot_stride : nullptr;
    const int col = T3_XH + 4 * lane;  // staged column of this thread's first cell

    // ---- register queues of the z taps, one per row: V[t][j] = u_n of row
    // yr0 + t at z = zout - R + j
    float4 V[TR][Q];
#pragma unroll
    for (int p = 0; p < 2 * R; ++p) {
        if (!mbar_wait(&bc[p % NB], (p / NB) & 1)) report(a.err, DEV_ERR_TMA_TIMEOUT);
#pragma unroll
        for (int t = 0; t < TR; ++t)
            V[t][p + 1] = *reinterpret_cast<const float4*>(cur_buf(p) + (yr0 + t + R) * T3_W + col);
    }
    __syncthreads();  // planes 0 .. R-1 are consumed
    if (tid == 0) {
        for (int p = NB; p < min(NB + R, total); ++p) issue(p);
    }

    const int lo_s = a.smp.off ? a.smp.off[s * ntiles + tile] : 0;
    const int hi_s = a.smp.off ? a.smp.off[s * ntiles + tile + 1] : 0;
    const int lo_i = a.inj.off ? a.inj.off[s * ntiles + tile] : 0;
    const int hi_i = a.inj.off ? a.inj.off[s * ntiles + tile + 1] : 0;

    for (int zr = 0; zr < zc; ++zr) {
        const int z = z0 + zr;
        const int pn = zr + 2 * R;  // newest staged plane needed
        if (!mbar_wait(&bc[pn % NB], (pn / NB) & 1)) report(a.err, DEV_ERR_TMA_TIMEOUT);
#pragma unroll
        for (int t = 0; t < TR; ++t) {
#pragma unroll
            for (int j = 0; j < 2 * R; ++j) V[t][j] = V[t][j + 1];
            V[t][2 * R] = *reinterpret_cast<const float4*>(cur_buf(pn) + (yr0 + t + R) * T3_W + col);
        }

        const float* pl = cur_buf(zr + R);  // u_n at the output plane, with halo
        // y taps: staged rows yr0 .. yr0 + TR + 2R - 1 (tile rows yr0 - R ..);
        // the thread's own rows come from the queues
        float4 Y[YW];
#pragma unroll
        for (int j = 0; j < YW; ++j) {
            if (j >= R && j < R + TR)
                Y[j] = V[j - R][R];
            else
                Y[j] = *reinterpret_cast<const float4*>(pl + (yr0 + j) * T3_W + col);
        }
        const float gz = gzs[zr];
        const bool zin = z >= R && z < a.nz - R;
#pragma unroll
        for (int t = 0; t < TR; ++t) {
            const float* prow = pl + (yr0 + t + R) * T3_W + 4 * lane;
            const float4 lv = *reinterpret_cast<const float4*>(prow);
            const float4 cv = V[t][R];
            const float4 rv = *reinterpret_cast<const float4*>(prow + 2 * T3_XH);
            const float w[12] = {lv.x, lv.y, lv.z, lv.w, cv.x, cv.y, cv.z, cv.w, rv.x, rv.y, rv.z, rv.w};
            // L u in packed pairs: (c0 u + sum_k cx_k (x taps)) + sum_k cy_k (y taps)
            // + sum_k cz_k (z taps), the three sums in independent chains
            float2 lo = __fmul2_rn(a.c0p, lo2(cv));
            float2 hi = __fmul2_rn(a.c0p, hi2(cv));
            float2 loy = make_float2(0.f, 0.f), hiy = loy, loz = loy, hiz = loy;
#pragma unroll
            for (int k = 1; k <= R; ++k) {
                float2 xl, xh;
                if (k % 2 == 0) {  // the x taps form aligned register pairs
                    xl = __fadd2_rn(make_float2(w[4 - k], w[5 - k]), make_float2(w[4 + k], w[5 + k]));
                    xh = __fadd2_rn(make_float2(w[6 - k], w[7 - k]), make_float2(w[6 + k], w[7 + k]));
                } else {
                    xl = make_float2(w[4 - k] + w[4 + k], w[5 - k] + w[5 + k]);
                    xh = make_float2(w[6 - k] + w[6 + k], w[7 - k] + w[7 + k]);
                }
                lo = __ffma2_rn(a.cxp[k - 1], xl, lo);
                hi = __ffma2_rn(a.cxp[k - 1], xh, hi);
                const float4 ym = Y[R + t - k], yp = Y[R + t + k];
                loy = __ffma2_rn(a.cyp[k - 1], __fadd2_rn(lo2(ym), lo2(yp)), loy);
                hiy = __ffma2_rn(a.cyp[k - 1], __fadd2_rn(hi2(ym), hi2(yp)), hiy);
                const float4 zm = V[t][R - k], zp = V[t][R + k];
                loz = __ffma2_rn(a.czp[k - 1], __fadd2_rn(lo2(zm), lo2(zp)), loz);
                hiz = __ffma2_rn(a.czp[k - 1], __fadd2_rn(hi2(zm), hi2(zp)), hiz);
            }
            lo = __fadd2_rn(__fadd2_rn(lo, loy), loz);
            hi = __fadd2_rn(__fadd2_rn(hi, hiy), hiz);
            const int ti = (yr0 + t) * T3_TX + 4 * lane;
            const float4 ov = *reinterpret_cast<const float4*>(old_buf(zr) + ti);
            const float4 mv = *reinterpret_cast<const float4*>(m_buf(zr) + ti);
            // u_{n+1} = g (m L u + 2 u) - g^2 u_{n-1}
            const float gyz = gz * gyv[t];
            const float2 gl = __fmul2_rn(make_float2(gyz, gyz), make_float2(gxe[0], gxe[1]));
            const float2 gh = __fmul2_rn(make_float2(gyz, gyz), make_float2(gxe[2], gxe[3]));
            float2 nl, nh, dl, dh;
            if (MODE == MODE_SUMMED) {  // ov is d_n: d = g m L u + (g^2 d - (1 - g)^2 u), u + d
                const float2 one = make_float2(1.f, 1.f);
                const float2 ol = __fadd2_rn(one, make_float2(-gl.x, -gl.y)), oh = __fadd2_rn(one, make_float2(-gh.x, -gh.y));
                const float2 il = __ffma2_rn(__fmul2_rn(gl, gl), lo2(ov),
                                             make_float2(-(ol.x * ol.x) * cv.x, -(ol.y * ol.y) * cv.y));
                const float2 ih = __ffma2_rn(__fmul2_rn(gh, gh), hi2(ov),
                                             make_float2(-(oh.x * oh.x) * cv.z, -(oh.y * oh.y) * cv.w));
                dl = __ffma2_rn(__fmul2_rn(gl, lo2(mv)), lo, il);
                dh = __ffma2_rn(__fmul2_rn(gh, hi2(mv)), hi, ih);
                nl = __fadd2_rn(lo2(cv), dl);
                nh = __fadd2_rn(hi2(cv), dh);
            } else {
                const float2 tl = __ffma2_rn(lo2(mv), lo, __fadd2_rn(lo2(cv), lo2(cv)));
                const float2 th = __ffma2_rn(hi2(mv), hi, __fadd2_rn(hi2(cv), hi2(cv)));
                nl = __ffma2_rn(gl, tl, __fmul2_rn(__fmul2_rn(gl, gl), make_float2(-ov.x, -ov.y)));
                nh = __ffma2_rn(gh, th, __fmul2_rn(__fmul2_rn(gh, gh), make_float2(-ov.z, -ov.w)));
            }
            const float nv[4] = {nl.x, nl.y, nh.x, nh.y};
            const float lap[4] = {lo.x, lo.y, hi.x, hi.y};

            const bool rin = yin[t] && zin;
            const long long off = (long long)z * a.plane + (long long)(y0 + yr0 + t) * a.ld + x;
            if (rin && all_x) {
                *reinterpret_cast<float4*>(un + off) = make_float4(nv[0], nv[1], nv[2], nv[3]);
                if (MODE == MODE_SUMMED) *reinterpret_cast<float4*>(dnw + off) = make_float4(dl.x, dl.y, dh.x, dh.y);
            } else if (rin) {
                const float dv[4] = {dl.x, dl.y, dh.x, dh.y};
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (xin[e]) {
                        un[off + e] = nv[e];
                        if (MODE == MODE_SUMMED) dnw[off + e] = dv[e];
                    }
            }
            if (MODE == MODE_SAVE_LAP && rin) {
                const long long lo_i64 = (long long)s * a.shot_stride + off;
                const float4 lp = make_float4(lap[0], lap[1], lap[2], lap[3]);
                if (all_x) {
                    if (a.lap_bf16)
                        *reinterpret_cast<uint2*>(static_cast<__nv_bfloat16*>(a.lap) + lo_i64) = pack_bf16x4(lp);
                    else
                        *reinterpret_cast<float4*>(static_cast<float*>(a.lap) + lo_i64) = lp;
                } else {
#pragma unroll
                    for (int e = 0; e < 4; ++e)
                        if (xin[e]) {
                            if (a.lap_bf16)
                                static_cast<__nv_bfloat16*>(a.lap)[lo_i64 + e] = __float2bfloat16_rn(lap[e]);
                            else
                                static_cast<float*>(a.lap)[lo_i64 + e] = lap[e];
                        }
                }
            }
            if (MODE == MODE_GRAD && rin) {
                const unsigned char* lb = lap_buf(zr);
                const float4 lu = a.lap_bf16
                                      ? unpack_bf16x4(*reinterpret_cast<const uint2*>(
                                            reinterpret_cast<const __nv_bfloat16*>(lb) + ti))
                                      : *reinterpret_cast<const float4*>(reinterpret_cast<const float*>(lb) + ti);
                float* gp = a.grad + off;
                if (all_x) {
                    const float2 pl2 = __fmul2_rn(lo2(cv), lo2(lu)), ph2 = __fmul2_rn(hi2(cv), hi2(lu));
                    atomicAdd(reinterpret_cast<float4*>(gp), make_float4(pl2.x, pl2.y, ph2.x, ph2.y));
                } else {
#pragma unroll
                    for (int e = 0; e < 4; ++e)
                        if (xin[e]) atomicAdd(gp + e, comp(cv, e) * comp(lu, e));
                }
            }
        }
        // sampling of u_n at this plane
        for (int j = lo_s + tid; j < hi_s; j += NTH) {
            const int2 en = a.smp.ent[j];
            const int pz = en.x / int(a.plane);
            if (pz != z) continue;
            const int rem = en.x - pz * int(a.plane);
            const int py = rem / a.ld, px = rem - py * a.ld;
            float v = pl[(py - y0 + R) * T3_W + (px - x0 + T3_XH)] * a.smp_scale;
            if (a.smp_div_m) v /= a.m[en.x];
            a.smp_out[((long long)s * a.smp_nt + a.smp_t) * a.smp_np + en.y] = v;
        }
        __syncthreads();  // plane zr + R and old group zr fully read; stores of plane z done
        // the refill is issued by lane 0 of a warp that changes every plane, so
        // that no warp carries the extra work into every next barrier
        if (tid == 32 * (zr % (NTH / 32))) {
            fence_proxy_async_smem();
            if (zr + NB + R < total) issue(zr + NB + R);
        }
        for (int j = lo_i + tid; j < hi_i; j += NTH) {
            const int2 en = a.inj.ent[j];
            const int pz = en.x / int(a.plane);
            if (pz != z) continue;
            const int rem = en.x - pz * int(a.plane);
            const int py = rem / a.ld, px = rem - py * a.ld;
            float v = a.inj_val[((long long)s * a.inj_nt + a.inj_t) * a.inj_np + en.y] * a.inj_scale;
            if (a.inj_times_m) v *= a.m[en.x];
            const float g = (a.gz ? a.gz[pz] : 1.f) * (a.gy ? a.gy[py] : 1.f) * (a.gx ? a.gx[px] : 1.f);
            atomicAdd(un + en.x, g * v);
            if (MODE == MODE_SUMMED) atomicAdd(dnw + en.x, g * v);
        }
    }
}

template <int R, int MODE>
cudaError_t launch_impl(const CUtensorMap& mc, const CUtensorMap& mo, const CUtensorMap& ml,
                        const CUtensorMap& mm, const StepArgs& a, cudaStream_t s) {
    using L = Layout3D<R, MODE>;
    static int configured_device = -1;
    int dev = 0;
    cudaGetDevice(&dev);
    if (configured_device != dev) {
        cudaError_t e = cudaFuncSetAttribute(step3d_kernel<R, MODE, T3_ROWS>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, L::BYTES);
        if (e != cudaSuccess) return e;
        configured_device = dev;
    }
    const dim3 grid(a.nshot, a.tiles_x * a.tiles_y * a.tiles_z);
    step3d_kernel<R, MODE, T3_ROWS><<<grid, T3_THREADS, L::BYTES, s>>>(mc, mo, ml, mm, with_weight_pairs(a));
    count_launch();
    return cudaGetLastError();
}

template <int R>
cudaError_t dispatch(int mode, const CUtensorMap& mc, const CUtensorMap& mo, const CUtensorMap& ml,
                     const CUtensorMap& mm, const StepArgs& a, cudaStream_t s) {
    switch (mode) {
        case MODE_PLAIN: return launch_impl<R, MODE_PLAIN>(mc, mo, ml, mm, a, s);
        case MODE_SAVE_LAP: return launch_impl<R, MODE_SAVE_LAP>(mc, mo, ml, mm, a, s);
        case MODE_GRAD: return launch_impl<R, MODE_GRAD>(mc, mo, ml, mm, a, s);
        case MODE_SUMMED: return launch_impl<R, MODE_SUMMED>(mc, mo, ml, mm, a, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace

bool step3d_available() { return true; }

cudaError_t launch_step3d(int R, int mode, const CUtensorMap& mc, const CUtensorMap& mo,
                          const CUtensorMap& ml, const CUtensorMap& mm, const StepArgs& a,
                          cudaStream_t s) {
    if ((long long)a.tiles_x * a.tiles_y * a.tiles_z > 65535) return cudaErrorInvalidValue;
    switch (R) {
        case 1: return dispatch<1>(mode, mc, mo, ml, mm, a, s);
        case 2: return dispatch<2>(mode, mc, mo, ml, mm, a, s);
        case 4: return dispatch<4>(mode, mc, mo, ml, mm, a, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace wfd
