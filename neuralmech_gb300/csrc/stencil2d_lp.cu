// 2D time step with the wavefields stored in reduced precision (sm_103a):
// FP16, or int16 with one FP32 scale per block of 32 cells along x (u = s q,
// s = block max / 32767), the storage formats of the reference's mixed_step
// and scaled_step (projects/18_simple_wave_fd/step2D_wave.cu:85-183) carried
// over to the order-2R, sponge, multi-shot wave path. The arithmetic is FP32
// (the packed row stencil of the FP32 kernel); only the stored levels are
// rounded. A forward-only mode: 6 instead of 12 bytes of field traffic per
// cell-update.
//
// Per CTA (256 threads): a 128 x 32 tile of `shots_per_cta` shots, one after
// the other, with three TMA stages in flight. A stage holds the 16-bit u_n
// tile with a halo of R rows and 8 columns (the 16-byte TMA granule), the
// u_{n-1} tile, and for int16 their scale rows. Lane l owns x = x0 + 4l .. +3,
// warp w rows z0 + 4w .. +3; staged rows are decoded into a rolling window of
// FP32 rows. m and the sponge factors stay in registers across the shots.
// Each shot's source samples are added to u_{n+1} in FP32 before it is
// rounded for storage; receivers then sample the stored u_{n+1}.
#include <algorithm>

#include "../../include/wavefd.h"
#include "common.cuh"
#include "internal.h"

namespace wfd {
namespace {

constexpr int LP_TX = 128, LP_RB = 4, LP_TZ = 32, LP_THREADS = 256;
constexpr int LP_XH = 8;               // halo columns: 16 bytes of 16-bit cells, as TMA wants
constexpr int LP_W = LP_TX + 2 * LP_XH;  // 144 staged columns of u_n
constexpr int LP_CSB = 12;             // scale blocks staged per row of u_n: 4t - 4 .. 4t + 7
constexpr int LP_OSB = LP_TX / 32;     // scale blocks per row of u_{n-1}
constexpr int LP_STAGES = 3;

__host__ __device__ constexpr int al128(int v) { return (v + 127) / 128 * 128; }

template <int R, int FMT>
struct LayoutLP {
    static constexpr int H = LP_TZ + 2 * R;
    static constexpr int CUR = H * LP_W * 2;
    static constexpr int OLD = LP_TZ * LP_TX * 2;
    static constexpr int CS = FMT == WFD_FIELD_I16 ? H * LP_CSB * 4 : 0;
    static constexpr int OS = FMT == WFD_FIELD_I16 ? LP_TZ * LP_OSB * 4 : 0;
    static constexpr int OLD_OFF = al128(CUR);
    static constexpr int CS_OFF = OLD_OFF + al128(OLD);
    static constexpr int OS_OFF = CS_OFF + al128(CS);
    static constexpr int STAGE = OS_OFF + al128(OS);
    static constexpr int BYTES = LP_STAGES * STAGE + 64 + 128;
};

// 4 cells (8 bytes) of a staged 16-bit row as FP32; sc is the row's scale
// for the int16 format.
union Bits64 {  // one 8-byte load or store of 4 16-bit cells
    uint2 u;
    __half2 h[2];
};

// int16 <-> FP32 on the FMA/ALU pipes: 1.5 * 2^23 + q has the bit pattern
// 0x4B400000 + q for |q| < 2^22, so the conversions are an integer add and an
// exact FP32 subtraction (decode), or an FP32 add that rounds to the nearest
// integer, ties to even, and an integer subtraction (encode).
constexpr float kMagic = 12582912.0f;
__device__ __forceinline__ float s16_to_f(unsigned bits16) {
    const int q = (int)(short)(unsigned short)bits16;
    return __fsub_rn(__int_as_float(0x4B400000 + q), kMagic);
}
__device__ __forceinline__ unsigned f_to_s16(float v) {  // v rounded to the nearest integer, |v| <= 32767
    return unsigned(__float_as_int(__fadd_rn(v, kMagic)) - 0x4B400000) & 0xffffu;
}

template <int FMT>
__device__ __forceinline__ float4 dec4(const unsigned char* row, int c, float sc) {
    Bits64 w;
    w.u = *reinterpret_cast<const uint2*>(row + 2 * c);
    if (FMT == WFD_FIELD_FP16) {
        const float2 a = __half22float2(w.h[0]), b = __half22float2(w.h[1]);
        return make_float4(a.x, a.y, b.x, b.y);
    }
    return make_float4(sc * s16_to_f(w.u.x & 0xffffu), sc * s16_to_f(w.u.x >> 16), sc * s16_to_f(w.u.y & 0xffffu),
                       sc * s16_to_f(w.u.y >> 16));
}

// 4 values rounded to FP16 (nearest even), packed for one 8-byte store.
__device__ __forceinline__ uint2 pack_half4(float v0, float v1, float v2, float v3) {
    Bits64 w;
    w.h[0] = __floats2half2_rn(v0, v1);
    w.h[1] = __floats2half2_rn(v2, v3);
    return w.u;
}

// 4 stored cells at x..x+3 of row z (x a multiple of 4), through L2 (the
// level was written in this launch).
template <int FMT>
__device__ __forceinline__ float load4_l2(const LpArgs& p, int s, int z, int x, int e) {
    const long long c = (long long)s * p.a.shot_stride + (long long)z * p.a.ld + x;
    const uint2 w = __ldcg(reinterpret_cast<const uint2*>(static_cast<const short*>(p.nw) + c));
    const unsigned word = e < 2 ? w.x : w.y;
    const unsigned short bits = (unsigned short)((e & 1) ? word >> 16 : word & 0xffffu);
    if (FMT == WFD_FIELD_FP16)
        return __half2float(__ushort_as_half(bits));
    return __ldcg(p.snw + (long long)s * p.sstride + (long long)z * p.nblk + (x >> 5)) * (float)(short)bits;
}

template <int R, int FMT>
__global__ void __launch_bounds__(LP_THREADS, 2)
    step2d_lp_kernel(const __grid_constant__ CUtensorMap map_cur, const __grid_constant__ CUtensorMap map_old,
                     const __grid_constant__ CUtensorMap map_cs, const __grid_constant__ CUtensorMap map_os,
                     const LpArgs p) {
    using L = LayoutLP<R, FMT>;
    const StepArgs& a = p.a;
    extern __shared__ unsigned char smem_raw[];
    unsigned char* base = reinterpret_cast<unsigned char*>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    uint64_t* bars = reinterpret_cast<uint64_t*>(base + LP_STAGES * L::STAGE);

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int tile = blockIdx.x;
    const int ntiles = a.tiles_x * a.tiles_z;
    const int x0 = (tile % a.tiles_x) * LP_TX, z0 = (tile / a.tiles_x) * LP_TZ;
    const int s0 = blockIdx.y * a.shots_per_cta;
    const int ns = min(a.nshot - s0, a.shots_per_cta);
    if (ns <= 0) return;

    auto stage = [&](int b) { return base + b * L::STAGE; };
    auto issue = [&](int i) {  // thread 0 only
        const int b = i % LP_STAGES;
        mbar_arrive_expect_tx(&bars[b], uint32_t(L::CUR + L::OLD + L::CS + L::OS));
        tma_load_3d(stage(b), &map_cur, x0 - LP_XH, z0 - R, s0 + i, &bars[b]);
        tma_load_3d(stage(b) + L::OLD_OFF, &map_old, x0, z0, s0 + i, &bars[b]);
        if (FMT == WFD_FIELD_I16) {
            tma_load_3d(stage(b) + L::CS_OFF, &map_cs, x0 / 32 - 4, z0 - R, s0 + i, &bars[b]);
            tma_load_3d(stage(b) + L::OS_OFF, &map_os, x0 / 32, z0, s0 + i, &bars[b]);
        }
    };

    __shared__ int2 smp_range[T2_MAX_SPC], inj_range[T2_MAX_SPC];
    // launched as a programmatic dependent: every global access comes after the wait
    if (tid == 0) {
        for (int b = 0; b < LP_STAGES; ++b) mbar_init(&bars[b], 1);
        fence_mbar_init();
    }
    grid_dependency_wait();
    // the first stages are issued before the point-list ranges are read, so
    // that the two memory latencies overlap
    if (tid == 0) {
        for (int i = 0; i < min(ns, LP_STAGES); ++i) issue(i);
        launch_dependents();
    }

    // ---- per-thread constants (loaded before the barrier below, so that their
    // latency overlaps the range reads)
    const int x = x0 + 4 * lane;
    const int zb = z0 + warp * LP_RB;
    float4 mrow[LP_RB];
    float gzr[LP_RB];
    bool zin[LP_RB];
#pragma unroll
    for (int r = 0; r < LP_RB; ++r) {
        const int z = zb + r;
        mrow[r] = (a.m != nullptr && z < a.nz && x < a.ld)
                      ? __ldg(reinterpret_cast<const float4*>(a.m + (long long)z * a.ld + x))
                      : make_float4(a.m_const, a.m_const, a.m_const, a.m_const);
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
    const bool x_ok = x < a.ld;

    if (tid < ns) {
        const int k = (s0 + tid) * ntiles + tile;
        smp_range[tid] = a.smp.off ? make_int2(a.smp.off[k], a.smp.off[k + 1]) : make_int2(0, 0);
        inj_range[tid] = a.inj.off ? make_int2(a.inj.off[k], a.inj.off[k + 1]) : make_int2(0, 0);
    }
    __syncthreads();

    // staged columns of this lane: centre 8 + 4l, left 4 + 4l, right 12 + 4l;
    // their scale blocks in the staged scale rows (block 4t - 4 at index 0)
    const int cc = LP_XH + 4 * lane;
    const int bl = ((cc - 4 - LP_XH) >> 5) + 4, bc = ((cc - LP_XH) >> 5) + 4, br = ((cc + 4 - LP_XH) >> 5) + 4;

    for (int i = 0; i < ns; ++i) {
        const int s = s0 + i, b = i % LP_STAGES;
        if (!mbar_wait(&bars[b], (i / LP_STAGES) & 1)) report(a.err, DEV_ERR_TMA_TIMEOUT);
        const unsigned char* cur = stage(b);
        const unsigned char* old = stage(b) + L::OLD_OFF;
        const float* cs = reinterpret_cast<const float*>(stage(b) + L::CS_OFF);
        const float* os = reinterpret_cast<const float*>(stage(b) + L::OS_OFF);
        auto crow = [&](int j) { return cur + j * (LP_W * 2); };
        auto cscale = [&](int j, int blk) { return FMT == WFD_FIELD_I16 ? cs[j * LP_CSB + blk] : 0.f; };
        const int ilo = inj_range[i].x, ihi = inj_range[i].y;

        float4 V[LP_RB + 2 * R];
        const int j0 = warp * LP_RB;  // staged row of z = zb - R
#pragma unroll
        for (int j = 0; j < 2 * R; ++j) V[j] = dec4<FMT>(crow(j0 + j), cc, cscale(j0 + j, bc));
#pragma unroll
        for (int r = 0; r < LP_RB; ++r) {
            const int z = zb + r, jr = j0 + r + R;
            V[r + 2 * R] = dec4<FMT>(crow(j0 + r + 2 * R), cc, cscale(j0 + r + 2 * R, bc));
            const float4 cv = V[r + R];
            const float4 lv = dec4<FMT>(crow(jr), cc - 4, cscale(jr, bl));
            const float4 rv = dec4<FMT>(crow(jr), cc + 4, cscale(jr, br));
            const float4 ov = dec4<FMT>(old + (warp * LP_RB + r) * (LP_TX * 2), 4 * lane,
                                        FMT == WFD_FIELD_I16 ? os[(warp * LP_RB + r) * LP_OSB + (lane >> 3)] : 0.f);
            const float4 l = lap_row<R>(lv, cv, rv, V, r + R, a);
            float nv[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const float g = gzr[r] * gxe[e];
                nv[e] = (zin[r] && xin[e])
                            ? g * fmaf(comp(mrow[r], e), comp(l, e), 2.f * comp(cv, e)) - (g * g) * comp(ov, e)
                            : 0.f;  // the fixed ring and the row padding are stored as 0
            }
            // this step's sources at the thread's cells, in FP32 before rounding
            // (summed per cell in a float4 first: an array updated inside the
            // runtime loop would live in local memory)
            if (ihi > ilo) {
                float4 add = make_float4(0.f, 0.f, 0.f, 0.f);
                for (int j = ilo; j < ihi; ++j) {
                    const int2 en = a.inj.ent[j];
                    const int ez = en.x / a.ld, e = en.x - ez * a.ld - x;
                    if (ez != z || e < 0 || e >= 4) continue;
                    const float v = a.inj_val[((long long)s * a.inj_nt + a.inj_t) * a.inj_np + en.y] * a.inj_scale;
                    add.x += e == 0 ? v : 0.f;
                    add.y += e == 1 ? v : 0.f;
                    add.z += e == 2 ? v : 0.f;
                    add.w += e == 3 ? v : 0.f;
                }
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const float v = a.inj_times_m ? comp(add, e) * comp(mrow[r], e) : comp(add, e);
                    nv[e] += gzr[r] * gxe[e] * v;
                }
            }
            // store u_{n+1}
            const bool row_ok = z < a.nz;
            const long long c = (long long)s * a.shot_stride + (long long)z * a.ld + x;
            if (FMT == WFD_FIELD_FP16) {
                if (row_ok && x_ok) *reinterpret_cast<uint2*>(static_cast<__half*>(p.nw) + c) = pack_half4(nv[0], nv[1], nv[2], nv[3]);
            } else {
                // the 8 lanes of an aligned octet hold one 32-cell block
                float mx = (row_ok && x_ok) ? fmaxf(fmaxf(fabsf(nv[0]), fabsf(nv[1])),
                                                    fmaxf(fabsf(nv[2]), fabsf(nv[3])))
                                            : 0.f;
#pragma unroll
                for (int o = 1; o < 8; o *= 2) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
                if (mx < 1e-30f) mx = 0.f;  // (32767 / max must stay finite: such blocks are stored as 0)
                if (row_ok && x_ok) {
                    const float inv = mx > 0.f ? 32767.f / mx : 0.f;
                    unsigned q[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e) q[e] = f_to_s16(__fmul_rn(nv[e], inv));
                    *reinterpret_cast<uint2*>(static_cast<short*>(p.nw) + c) =
                        make_uint2(q[0] | (q[1] << 16), q[2] | (q[3] << 16));
                    if ((lane & 7) == 0)
                        p.snw[(long long)s * p.sstride + (long long)z * p.nblk + (x >> 5)] = mx / 32767.f;
                }
            }
        }
        __syncthreads();  // stage b fully read; this shot's u_{n+1} stored
        if (tid == 0 && i + LP_STAGES < ns) {
            fence_proxy_async_smem();
            issue(i + LP_STAGES);
        }
        // receivers sample the stored u_{n+1}
        {
            const int lo = smp_range[i].x, hi = smp_range[i].y;
            for (int j = lo + tid; j < hi; j += LP_THREADS) {
                const int2 en = a.smp.ent[j];
                const int z = en.x / a.ld, xx = en.x - z * a.ld;
                a.smp_out[((long long)s * a.smp_nt + a.smp_t) * a.smp_np + en.y] =
                    load4_l2<FMT>(p, s, z, xx & ~3, xx & 3) * a.smp_scale;
            }
        }
    }
}

template <int R, int FMT>
cudaError_t launch_impl(const CUtensorMap& mc, const CUtensorMap& mo, const CUtensorMap& mcs,
                        const CUtensorMap& mos, const LpArgs& p_in, cudaStream_t s) {
    using L = LayoutLP<R, FMT>;
    static int configured_device = -1;
    int dev = 0;
    cudaGetDevice(&dev);
    if (configured_device != dev) {
        cudaError_t e = cudaFuncSetAttribute(step2d_lp_kernel<R, FMT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             L::BYTES);
        if (e != cudaSuccess) return e;
        configured_device = dev;
    }
    LpArgs p = p_in;
    p.a = with_weight_pairs(p_in.a);
    const dim3 grid(p.a.tiles_x * p.a.tiles_z, (p.a.nshot + p.a.shots_per_cta - 1) / p.a.shots_per_cta);
    const cudaError_t e = launch_pdl(step2d_lp_kernel<R, FMT>, grid, dim3(LP_THREADS), L::BYTES, s, mc, mo, mcs, mos, p);
    count_launch();
    return e != cudaSuccess ? e : cudaGetLastError();
}

template <int FMT>
__global__ void decode_kernel(const void* f, const float* sc, float* out, long long nrows, int nx, int ld,
                              int nblk) {
    const long long n = nrows * (long long)nx;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const long long row = i / nx;
        const int xx = int(i - row * nx);
        const long long c = row * ld + xx;
        out[i] = FMT == WFD_FIELD_FP16 ? __half2float(static_cast<const __half*>(f)[c])
                                       : sc[row * nblk + (xx >> 5)] * static_cast<const short*>(f)[c];
    }
}

}  // namespace

cudaError_t launch_step2d_lp(int R, int fmt, const CUtensorMap& map_cur, const CUtensorMap& map_old,
                             const CUtensorMap& map_cs, const CUtensorMap& map_os, const LpArgs& p,
                             cudaStream_t s) {
    if (p.a.shots_per_cta < 1 || p.a.shots_per_cta > T2_MAX_SPC) return cudaErrorInvalidValue;
    if (fmt != WFD_FIELD_FP16 && fmt != WFD_FIELD_I16) return cudaErrorInvalidValue;
    const CUtensorMap &mc = map_cur, &mo = map_old, &mcs = map_cs, &mos = map_os;
    const bool h = fmt == WFD_FIELD_FP16;
    switch (R) {
        case 1: return h ? launch_impl<1, WFD_FIELD_FP16>(mc, mo, mcs, mos, p, s)
                         : launch_impl<1, WFD_FIELD_I16>(mc, mo, mcs, mos, p, s);
        case 2: return h ? launch_impl<2, WFD_FIELD_FP16>(mc, mo, mcs, mos, p, s)
                         : launch_impl<2, WFD_FIELD_I16>(mc, mo, mcs, mos, p, s);
        case 4: return h ? launch_impl<4, WFD_FIELD_FP16>(mc, mo, mcs, mos, p, s)
                         : launch_impl<4, WFD_FIELD_I16>(mc, mo, mcs, mos, p, s);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_decode_field(int fmt, const void* f, const float* sc, float* out, long long nrows, int nx,
                                int ld, int nblk, cudaStream_t s) {
    const long long n = nrows * (long long)nx;
    if (n <= 0) return cudaSuccess;
    const int blocks = (int)std::min<long long>((n + 255) / 256, 152LL * 32);
    if (fmt == WFD_FIELD_FP16)
        decode_kernel<WFD_FIELD_FP16><<<blocks, 256, 0, s>>>(f, sc, out, nrows, nx, ld, nblk);
    else
        decode_kernel<WFD_FIELD_I16><<<blocks, 256, 0, s>>>(f, sc, out, nrows, nx, ld, nblk);
    count_launch();
    return cudaGetLastError();
}

}  // namespace wfd
