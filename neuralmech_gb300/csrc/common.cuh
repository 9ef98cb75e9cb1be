// Shared device helpers: mbarrier + TMA (cp.async.bulk.tensor) inline PTX for
// sm_103a, bounded waits, error codes. No CUTLASS/CuTe: everything is written
// here against the public PTX ISA.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <utility>

#include "internal.h"

namespace wfd {

// Upper bound on mbarrier try_wait polls before a wait is declared lost. One
// poll suspends for at most a few microseconds, so this is well under a second
// of waiting, far beyond any legitimate TMA latency.
constexpr uint32_t kMaxWaitPolls = 1u << 18;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
                 : "memory");
}

// Makes the mbarrier initialisation visible to the async (TMA) proxy.
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Orders this thread's earlier generic-proxy shared-memory accesses before
// later async-proxy (TMA) writes into the same buffer.
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}

// Programmatic dependent launch (sm_90+): a kernel launched with programmatic
// stream serialisation may start while the previous kernel of the stream
// finishes. grid_dependency_wait() blocks the calling thread until that kernel
// has completed and its memory is visible; launch_dependents() lets the next
// kernel of the stream start its CTAs once every CTA of this grid has called
// it (or exited).
__device__ __forceinline__ void grid_dependency_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Host side: launch `kernel` with programmatic stream serialisation allowed
// (the kernel must call grid_dependency_wait() before its first global access).
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// Bounded wait on phase `parity`; false when it gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    for (uint32_t i = 0; i < kMaxWaitPolls; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// 2D / 3D tiled TMA loads global -> shared, completing on `bar`. The innermost
// coordinate x must be a multiple of 16 bytes / element size (checked by the
// launchers, which only pass x0 - 4 with x0 a multiple of 128 for FP32 and a
// multiple of 128 for BF16).
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z,
                                            uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, int x, int y, int z,
                                            int w, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(w),
        "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ void report(unsigned* err, unsigned bits) {
    if (err) atomicOr(err, bits);
}

// 4 x FP32 <-> 4 x BF16 (round to nearest even), packed in a uint2.
__device__ __forceinline__ uint2 pack_bf16x4(float4 v) {
    __nv_bfloat162 lo = __floats2bfloat162_rn(v.x, v.y);
    __nv_bfloat162 hi = __floats2bfloat162_rn(v.z, v.w);
    uint2 r;
    r.x = *reinterpret_cast<uint32_t*>(&lo);
    r.y = *reinterpret_cast<uint32_t*>(&hi);
    return r;
}

__device__ __forceinline__ float4 unpack_bf16x4(uint2 p) {
    __nv_bfloat162 lo = *reinterpret_cast<__nv_bfloat162*>(&p.x);
    __nv_bfloat162 hi = *reinterpret_cast<__nv_bfloat162*>(&p.y);
    float2 a = __bfloat1622float2(lo), b = __bfloat1622float2(hi);
    return make_float4(a.x, a.y, b.x, b.y);
}

// ---------------------------------------------------------------- 2D stencil rows
// The launchers' copy of the arguments with the duplicated weight pairs set.
inline StepArgs with_weight_pairs(StepArgs a) {
    a.c0p = make_float2(a.c0, a.c0);
    for (int k = 0; k < 4; ++k) {
        a.czp[k] = make_float2(a.cz[k], a.cz[k]);
        a.cyp[k] = make_float2(a.cy[k], a.cy[k]);
        a.csp[k] = make_float2(a.cs[k], a.cs[k]);
        a.cxp[k] = make_float2(a.cx[k], a.cx[k]);
    }
    return a;
}

// A thread owns 4 consecutive cells of a row (a float4); lv and rv are the
// float4s to its left and right, V a register window of the rows above and
// below.
__device__ __forceinline__ float comp(const float4& v, int e) {
    return e == 0 ? v.x : e == 1 ? v.y : e == 2 ? v.z : v.w;
}

// Block floating point of 4 cells (WFD_LEVEL_BFP16): mantissas q and one
// exponent byte t with v = q 2^(t - 141), t the FP32 exponent field of the
// block's largest magnitude M. M < 2^(t - 126) makes |v 2^(141 - t)| < 2^15, so
// q = rint(v 2^(141 - t)) clamped to +-32767 keeps every value within 2^-15 of
// 2^(t - 126). Both scalings are exact powers of two; blocks with t < 15
// (M < 2^-112) are stored as 0, which keeps 2^(t - 141) a normal FP32 number.
// A mantissa is stored as the 16 bits u = q + 32768. Both directions go
// through FP32 values of exponent 23, whose low mantissa bits hold an integer
// (B = 2^23 + 32768): rint(x) + B is fma(x, 1, B) rounded to the nearest
// integer, ties to even, and the float with the bits 0x4B00 0000 | u is
// 2^23 + u, so q 2^k = fma(2^23 + u, 2^k, -B 2^k) exactly. No integer/float
// conversion instruction is involved.
__device__ __forceinline__ void bfp4_encode(const float4& v, uint2& q, unsigned& t) {
    const float M = fmaxf(fmaxf(fabsf(v.x), fabsf(v.y)), fmaxf(fabsf(v.z), fabsf(v.w)));
    const int e = (__float_as_int(M) >> 23) & 0xff;
    if (e < 15) {
        q = make_uint2(0x80008000u, 0x80008000u);  // q = 0
        t = 0u;
        return;
    }
    const float inv = __int_as_float((268 - e) << 23);  // 2^(141 - e)
    constexpr float B = 8421376.f;                        // 2^23 + 32768
    auto m16 = [&](float x) { return __float_as_uint(fminf(fmaxf(fmaf(x, inv, B), B - 32767.f), B + 32767.f)); };
    q = make_uint2(__byte_perm(m16(v.x), m16(v.y), 0x5410), __byte_perm(m16(v.z), m16(v.w), 0x5410));
    t = unsigned(e);
}

__device__ __forceinline__ float4 bfp4_decode(uint2 q, unsigned t) {
    const float sc = t ? __int_as_float(int(t - 14u) << 23) : 0.f;  // 2^(t - 141)
    const float2 s2 = make_float2(sc, sc), c2 = make_float2(-8421376.f * sc, -8421376.f * sc);
    auto f = [](unsigned w, unsigned sel) { return __uint_as_float(__byte_perm(w, 0x4B000000u, sel)); };
    const float2 lo = __ffma2_rn(make_float2(f(q.x, 0x7610), f(q.x, 0x7632)), s2, c2);
    const float2 hi = __ffma2_rn(make_float2(f(q.y, 0x7610), f(q.y, 0x7632)), s2, c2);
    return make_float4(lo.x, lo.y, hi.x, hi.y);
}

// L u at the four cells of a row: horizontal taps from (lv, cv, rv), vertical
// taps from the register window V (centre row C). The cells go in pairs
// through the packed FP32x2 arithmetic of sm_100+, with the operations and
// their order of the scalar form c0 u + sum_k cx_k (u_{x-k} + u_{x+k}) +
// cz_k (u_{z-k} + u_{z+k}), accumulated k = 1 .. R with x before z.
template <int R, int N>
__device__ __forceinline__ float4 lap_row(const float4& lv, const float4& cv, const float4& rv,
                                          const float4 (&V)[N], int C, const StepArgs& a) {
    const float w[12] = {lv.x, lv.y, lv.z, lv.w, cv.x, cv.y, cv.z, cv.w, rv.x, rv.y, rv.z, rv.w};
    float2 lo = __fmul2_rn(a.c0p, make_float2(cv.x, cv.y));
    float2 hi = __fmul2_rn(a.c0p, make_float2(cv.z, cv.w));
#pragma unroll
    for (int k = 1; k <= R; ++k) {
        const float2 cx = a.cxp[k - 1];
        const float2 cz = a.czp[k - 1];
        float2 xl, xh;
        if (k % 2 == 0) {  // the x taps form aligned register pairs
            xl = __fadd2_rn(make_float2(w[4 - k], w[5 - k]), make_float2(w[4 + k], w[5 + k]));
            xh = __fadd2_rn(make_float2(w[6 - k], w[7 - k]), make_float2(w[6 + k], w[7 + k]));
        } else {
            xl = make_float2(w[4 - k] + w[4 + k], w[5 - k] + w[5 + k]);
            xh = make_float2(w[6 - k] + w[6 + k], w[7 - k] + w[7 + k]);
        }
        lo = __ffma2_rn(cx, xl, lo);
        hi = __ffma2_rn(cx, xh, hi);
        const float4 up = V[C - k], dn = V[C + k];
        lo = __ffma2_rn(cz, __fadd2_rn(make_float2(up.x, up.y), make_float2(dn.x, dn.y)), lo);
        hi = __ffma2_rn(cz, __fadd2_rn(make_float2(up.z, up.w), make_float2(dn.z, dn.w)), hi);
    }
    return make_float4(lo.x, lo.y, hi.x, hi.y);
}

// L u at the four cells of a row as sums of neighbour differences,
// sum_k cx_k ((u_{x-k} - u) + (u_{x+k} - u)) + cz_k ((u_{z-k} - u) + (u_{z+k} - u)),
// accumulated k = 1 .. R with x before z (the centre weight is -2 sum_k (cx_k +
// cz_k), so this is L u). Each difference of neighbouring values of a smooth
// field is exact or nearly so in FP32, and the sum's rounding is relative to
// the differences instead of to |u| times the centre weight. Packed FP32x2
// pairs as lap_row.
template <int R, int N>
__device__ __forceinline__ float4 lap_row_diff(const float4& lv, const float4& cv, const float4& rv,
                                               const float4 (&V)[N], int C, const StepArgs& a) {
    const float w[12] = {lv.x, lv.y, lv.z, lv.w, cv.x, cv.y, cv.z, cv.w, rv.x, rv.y, rv.z, rv.w};
    // minus the centre values: x - u as one packed add of -u (the negation is exact)
    const float2 nl = make_float2(-cv.x, -cv.y), nh = make_float2(-cv.z, -cv.w);
    float2 lo = make_float2(0.f, 0.f), hi = make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 1; k <= R; ++k) {
        const float2 cx = a.cxp[k - 1];
        const float2 cz = a.czp[k - 1];
        const float2 xl = __fadd2_rn(__fadd2_rn(make_float2(w[4 - k], w[5 - k]), nl),
                                     __fadd2_rn(make_float2(w[4 + k], w[5 + k]), nl));
        const float2 xh = __fadd2_rn(__fadd2_rn(make_float2(w[6 - k], w[7 - k]), nh),
                                     __fadd2_rn(make_float2(w[6 + k], w[7 + k]), nh));
        lo = __ffma2_rn(cx, xl, lo);
        hi = __ffma2_rn(cx, xh, hi);
        const float4 up = V[C - k], dn = V[C + k];
        lo = __ffma2_rn(cz, __fadd2_rn(__fadd2_rn(make_float2(up.x, up.y), nl), __fadd2_rn(make_float2(dn.x, dn.y), nl)),
                        lo);
        hi = __ffma2_rn(cz, __fadd2_rn(__fadd2_rn(make_float2(up.z, up.w), nh), __fadd2_rn(make_float2(dn.z, dn.w), nh)),
                        hi);
    }
    return make_float4(lo.x, lo.y, hi.x, hi.y);
}

// u_{n+1} = m L u_n + 2 u_n - u_{n-1} at 4 interior cells outside the sponge
// (g = 1), in packed pairs: the general update g (m L u + 2 u) - g^2 u_{n-1}
// with g = 1, value for value.
__device__ __forceinline__ float4 leap_plain(const float4& m, const float4& l, const float4& c,
                                             const float4& o) {
    const float2 lo = __fadd2_rn(__ffma2_rn(make_float2(m.x, m.y), make_float2(l.x, l.y),
                                            __fadd2_rn(make_float2(c.x, c.y), make_float2(c.x, c.y))),
                                 make_float2(-o.x, -o.y));
    const float2 hi = __fadd2_rn(__ffma2_rn(make_float2(m.z, m.w), make_float2(l.z, l.w),
                                            __fadd2_rn(make_float2(c.z, c.w), make_float2(c.z, c.w))),
                                 make_float2(-o.z, -o.w));
    return make_float4(lo.x, lo.y, hi.x, hi.y);
}

// A compile-time flag for generic lambdas (the plain-tile and general bodies).
template <bool B>
struct Flag {
    static constexpr bool value = B;
};

}  // namespace wfd
