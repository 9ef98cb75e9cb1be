// Two-step-blocked 2D time-step kernel of the acoustic wave path (sm_103a).
//
// One launch advances every shot by two steps (or one, `two_steps == 0`):
//   u_{n+1} = g (2 u_n + m L u_n) - g^2 u_{n-1},
//   u_{n+2} = g (2 u_{n+1} + m L u_{n+1}) - g^2 u_n,
// reading u_{n-1}, u_n and writing u_{n+1}, u_{n+2} to two other buffers.
// That saves the HBM round trip of u_{n+1}: 8 instead of 12 bytes of field
// traffic per cell-update. This is the reference's temporal blocking
// (projects/18_simple_wave_fd/step2D_wave.cu:244-304, 8 steps of a 5-point
// stencil in one tile) for the order-2R stencil, at depth 2: each extra step
// widens the halo by R.
//
// Per CTA (256 threads): tile T = 120 x 24 cells of `shots_per_cta` shots,
// one shot after the other, with two TMA stages in flight so that the next
// shot's tiles land while this one computes. A stage holds
//   U = u_n on T plus a halo of 2R rows and 8 columns (136 x (24 + 4R)),
//   O = u_{n-1} on E = T plus R rows and 4 columns (128 x (24 + 2R)); step 1
//       overwrites it in place with u_{n+1} on E.
// m on E is staged once per CTA (TMA, with the first shot's stage) and serves
// all its shots; the sponge factors sit in registers. Two CTAs fit an SM.
// Step 1 runs over E with lane l owning E columns 4l..4l+3 (32 lanes x float4
// = 128 columns) and warp w owning E rows; then the injections of step n that
// fall in E (also those owned by neighbouring tiles) are added in shared
// memory. Step 2 runs over T with lanes 1..30, the same column ownership.
// Both steps form L u with the packed FP32x2 row stencil of the one-step kernel.
//
// SUMMED: the same two steps in the summed (increment) form of the one-step
// kernel's MODE_SUMMED, state (u_n, d_n = u_n - u_{n-1}):
//   d_{n+1} = g^2 d_n - (1 - g)^2 u_n + g m L u_n,  u_{n+1} = u_n + d_{n+1},
// L in the centre-weight form of the leapfrog steps: this kernel is bound by
// its instruction count, and the neighbour-difference form that the memory-
// bound one-step kernel uses for its rounding costs 41% more instructions
// (the gradient of the 2-shot fwi1024 case: 4.7e-4 against 3.8e-4 vs FP64,
// both within 1e-3). O stages d_n on E; step 1 writes u_{n+1} over
// it and d_{n+1} into a fourth E buffer D1; step 2 reads both on the tile.
// Only u_{n+2} and d_{n+2} leave the CTA, to buffers the launch does not read
// (d_n is read with a halo by the neighbouring tiles, so d is double-
// buffered): 16 field bytes per two updates instead of 40 for two summed
// one-step launches. The intermediate level is written only on request.
#include "common.cuh"
#include "internal.h"

namespace wfd {
namespace {

__host__ __device__ constexpr int al128(int v) { return (v + 127) / 128 * 128; }

template <int R, bool SUMMED = false>
struct LayoutK2 {
    static constexpr int EH = K2_TZ + 2 * R;  // E rows
    static constexpr int UH = K2_TZ + 4 * R;  // U rows
    static constexpr int U_BYTES = UH * K2_UW * 4;
    static constexpr int E_BYTES = EH * K2_EW * 4;
    static constexpr int O_OFF = al128(U_BYTES);
    static constexpr int STAGE = O_OFF + al128(E_BYTES);
    static constexpr int STAGES = 2;
    static constexpr int M_OFF = STAGES * STAGE;  // m on E, once per CTA
    static constexpr int D1_OFF = M_OFF + al128(E_BYTES);  // summed: d_{n+1} on E
    static constexpr int BAR_OFF = D1_OFF + (SUMMED ? al128(E_BYTES) : 0);
    static constexpr int BYTES = BAR_OFF + 64 + 128;  // + barriers + alignment slack
    static constexpr int RB1 = (EH + 7) / 8;  // E rows per warp in step 1
    static constexpr int RB2 = K2_TZ / 8;     // T rows per warp in step 2
};

__device__ __forceinline__ float4 f4(const float* p) { return *reinterpret_cast<const float4*>(p); }

// Stores a level's 4 cells at p (row z < nz, x = p's column): the interior
// cells, and with zero_ring the fixed ring and row padding as 0.
__device__ __forceinline__ void store_level(float* p, const float4& v, bool zin, const bool* xin,
                                            bool all_x, int zero_ring, bool x_ok) {
    if (zin && all_x) {
        *reinterpret_cast<float4*>(p) = v;
    } else if (zero_ring) {
        if (x_ok)
            *reinterpret_cast<float4*>(p) = make_float4(zin && xin[0] ? v.x : 0.f, zin && xin[1] ? v.y : 0.f,
                                                        zin && xin[2] ? v.z : 0.f, zin && xin[3] ? v.w : 0.f);
    } else if (zin) {
#pragma unroll
        for (int e = 0; e < 4; ++e)
            if (xin[e]) p[e] = comp(v, e);
    }
}

// A kept level's 4 cells at (shot base q, e; in-shot offset off = z ld + x, x a
// multiple of 4) in block floating point; with ring, the fixed ring and row
// padding (cells outside xin / zin) as 0, as store_level writes them.
__device__ __forceinline__ void store_bfp(short* q, unsigned char* e, long long off, int z, int x, int eld,
                                          float4 v, bool ring, bool zin, const bool* xin) {
    if (ring)
        v = make_float4(zin && xin[0] ? v.x : 0.f, zin && xin[1] ? v.y : 0.f, zin && xin[2] ? v.z : 0.f,
                        zin && xin[3] ? v.w : 0.f);
    uint2 qv;
    unsigned t;
    bfp4_encode(v, qv, t);
    *reinterpret_cast<uint2*>(q + off) = qv;
    e[(long long)z * eld + (x >> 2)] = (unsigned char)t;
}

// The summed update of 4 cells: (d_new, u_new) from (u, d, m, L u, g), the
// one-step kernel's expression; g = 1 gives d + m L u.
__device__ __forceinline__ void summed4(const float4& u, const float4& d, const float4& m, const float4& l,
                                        const float* g, float4& dn, float4& un) {
    float dd[4], uu[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const float omg = 1.f - g[e];
        dd[e] = fmaf(g[e] * comp(m, e), comp(l, e), fmaf(g[e] * g[e], comp(d, e), -(omg * omg) * comp(u, e)));
        uu[e] = comp(u, e) + dd[e];
    }
    dn = make_float4(dd[0], dd[1], dd[2], dd[3]);
    un = make_float4(uu[0], uu[1], uu[2], uu[3]);
}

// summed4 with g = 1 (cells outside the sponge), in packed pairs:
// d_{n+1} = m L u + d_n, u_{n+1} = u_n + d_{n+1}. summed4's value there: g m = m,
// g^2 d = d and (1 - g)^2 u = 0 leave the same sums (up to the sign of a zero).
__device__ __forceinline__ void summed4_plain(const float4& u, const float4& d, const float4& m, const float4& l,
                                              float4& dn, float4& un) {
    const float2 dl = __ffma2_rn(make_float2(m.x, m.y), make_float2(l.x, l.y), make_float2(d.x, d.y));
    const float2 dh = __ffma2_rn(make_float2(m.z, m.w), make_float2(l.z, l.w), make_float2(d.z, d.w));
    const float2 ul = __fadd2_rn(make_float2(u.x, u.y), dl);
    const float2 uh = __fadd2_rn(make_float2(u.z, u.w), dh);
    dn = make_float4(dl.x, dl.y, dh.x, dh.y);
    un = make_float4(ul.x, ul.y, uh.x, uh.y);
}

template <int R, bool SUMMED, bool LVL16 = false>
__global__ void __launch_bounds__(K2_THREADS, 2)
    step2d_k2_kernel(const __grid_constant__ CUtensorMap map_u, const __grid_constant__ CUtensorMap map_o,
                     const __grid_constant__ CUtensorMap map_m, const Step2Args p) {
    using L = LayoutK2<R, SUMMED>;
    const StepArgs& a = p.a;
    extern __shared__ unsigned char smem_raw[];
    unsigned char* base = reinterpret_cast<unsigned char*>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    uint64_t* bars = reinterpret_cast<uint64_t*>(base + L::BAR_OFF);
    float* M = reinterpret_cast<float*>(base + L::M_OFF);
    float* D1 = reinterpret_cast<float*>(base + L::D1_OFF);  // (summed only)

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int tile = blockIdx.x;
    const int ntiles = a.tiles_x * a.tiles_z;
    const int x0 = (tile % a.tiles_x) * K2_TX;
    const int z0 = (tile / a.tiles_x) * K2_TZ;
    const int s0 = blockIdx.y * a.shots_per_cta;
    const int ns = min(a.nshot - s0, a.shots_per_cta);
    if (ns <= 0) return;
    const int two = p.two_steps;

    auto U_of = [&](int b) { return reinterpret_cast<float*>(base + b * L::STAGE); };
    auto O_of = [&](int b) { return reinterpret_cast<float*>(base + b * L::STAGE + L::O_OFF); };
    auto issue = [&](int i) {  // thread 0 only: u_n and u_{n-1} of shot s0 + i (+ m with the first)
        const int b = i % L::STAGES;
        mbar_arrive_expect_tx(&bars[b], uint32_t(L::U_BYTES + L::E_BYTES * (i == 0 ? 2 : 1)));
        tma_load_3d(U_of(b), &map_u, x0 - 8, z0 - 2 * R, s0 + i, &bars[b]);
        tma_load_3d(O_of(b), &map_o, x0 - 4, z0 - R, s0 + i, &bars[b]);
        if (i == 0) tma_load_2d(M, &map_m, x0 - 4, z0 - R, &bars[b]);
    };

    // point-list ranges of this tile for every shot of the CTA, staged once:
    // sampling, step-1 (extended region) injection, step-2 injection
    __shared__ int2 smp_rng[T2_MAX_SPC], inje_rng[T2_MAX_SPC], inj_rng[T2_MAX_SPC];
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
    if (tid < ns) {
        const int k = (s0 + tid) * ntiles + tile;
        smp_rng[tid] = a.smp.off ? make_int2(a.smp.off[k], a.smp.off[k + 1]) : make_int2(0, 0);
        inje_rng[tid] = p.inj_e.off ? make_int2(p.inj_e.off[k], p.inj_e.off[k + 1]) : make_int2(0, 0);
        inj_rng[tid] = a.inj.off ? make_int2(a.inj.off[k], a.inj.off[k + 1]) : make_int2(0, 0);
    }
    __syncthreads();

    // ---- per-thread constants, reused for every shot of the CTA
    const int ex = x0 - 4 + 4 * lane;  // global x of this lane's first E column
    const int er0 = warp * L::RB1;      // first E row of this warp (step 1)
    const int tr0 = warp * L::RB2;      // first T row of this warp (step 2)
    float gz1[L::RB1], gz2[L::RB2];
#pragma unroll
    for (int r = 0; r < L::RB1; ++r) {
        const int z = z0 - R + er0 + r;
        gz1[r] = (a.gz != nullptr && z >= 0 && z < a.nz) ? __ldg(a.gz + z) : 1.f;
    }
#pragma unroll
    for (int r = 0; r < L::RB2; ++r) {
        const int z = z0 + tr0 + r;
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
    const bool x_ok = ex >= 0 && ex < a.ld;
    // plain tile: every cell of E in the interior and outside the sponge (no
    // ring to keep, g = 1); its shots take the branch-free update
    bool mine = all_x;
#pragma unroll
    for (int e = 0; e < 4; ++e) mine = mine && gxe[e] == 1.f;
#pragma unroll
    for (int r = 0; r < L::RB1; ++r) {
        const int z = z0 - R + er0 + r;
        if (er0 + r < L::EH) mine = mine && z >= R && z < a.nz - R && gz1[r] == 1.f;
    }
    const bool plain = __syncthreads_and(mine) != 0;

    for (int i = 0; i < ns; ++i) {
        const int s = s0 + i, b = i % L::STAGES;
        if (!mbar_wait(&bars[b], (i / L::STAGES) & 1)) report(a.err, DEV_ERR_TMA_TIMEOUT);
        const float* U = U_of(b);
        float* O = O_of(b);  // u_{n-1}, then u_{n+1}, on E
        float* u_mid = p.u_mid + (long long)s * a.shot_stride;
        float* u_out = a.u_new + (long long)s * a.shot_stride;
        float* d_mid = SUMMED && p.d_mid ? p.d_mid + (long long)s * a.shot_stride : nullptr;
        float* d_out = SUMMED ? p.d_out + (long long)s * a.shot_stride : nullptr;
        const bool mid = !two || p.write_mid;  // (summed: the intermediate level leaves the CTA)
        // block-floating-point copies of kept levels (summed form)
        // (LVL16: the launch writes at least one of them)
        short* lq_mid = LVL16 && p.lq_mid ? p.lq_mid + (long long)s * a.shot_stride : nullptr;
        short* lq_out = LVL16 && p.lq_out ? p.lq_out + (long long)s * a.shot_stride : nullptr;
        unsigned char* le_mid = lq_mid ? p.le_mid + (long long)s * a.nz * p.eld : nullptr;
        unsigned char* le_out = lq_out ? p.le_out + (long long)s * a.nz * p.eld : nullptr;

        // ------------------------------------------------------------ step 1 on E
        auto step1 = [&](auto plain_c) {
            constexpr bool PLAIN = decltype(plain_c)::value;
            // vertical taps: a window of U rows er0 .. er0 + RB1 + 2R - 1 (E row er
            // sits at U row er + R), each row loaded just before its first use so
            // that only 2R + 1 rows are live at a time
            float4 V[L::RB1 + 2 * R];
            // (rows past U, read by the last warp when 8 RB1 > EH, lie inside the
            // stage and feed only E rows >= EH, which are skipped)
            auto urow_c = [&](int ur) { return f4(U + ur * K2_UW + 4 + 4 * lane); };
#pragma unroll
            for (int j = 0; j < 2 * R; ++j) V[j] = urow_c(er0 + j);
#pragma unroll
            for (int r = 0; r < L::RB1; ++r) {
                const int er = er0 + r;
                if (er >= L::EH) break;
                V[r + 2 * R] = urow_c(er0 + r + 2 * R);
                const int z = z0 - R + er;
                const float* urow = U + (er + R) * K2_UW + 4 * lane;
                const float4 lv = f4(urow), cv = V[r + R], rv = f4(urow + 8);
                float* orow = O + er * K2_EW + 4 * lane;
                const float4 ov = f4(orow);
                const float4 mv = f4(M + er * K2_EW + 4 * lane);
                const bool zin = z >= R && z < a.nz - R;
                if constexpr (SUMMED) {  // ov is d_n; O gets u_{n+1}, D1 d_{n+1}
                    const float4 l = lap_row<R>(lv, cv, rv, V, r + R, a);
                    float4 dn, un;
                    if constexpr (PLAIN) {
                        summed4_plain(cv, ov, mv, l, dn, un);
                    } else {
                        float g[4];
#pragma unroll
                        for (int e = 0; e < 4; ++e) g[e] = gz1[r] * gxe[e];
                        summed4(cv, ov, mv, l, g, dn, un);
                    }
                    if (!PLAIN) {  // fixed ring / outside the grid keep (u_n, d_n)
                        float uu[4], dd[4];
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            const bool in = zin && xin[e];
                            uu[e] = in ? comp(un, e) : comp(cv, e);
                            dd[e] = in ? comp(dn, e) : comp(ov, e);
                        }
                        un = make_float4(uu[0], uu[1], uu[2], uu[3]);
                        dn = make_float4(dd[0], dd[1], dd[2], dd[3]);
                    }
                    *reinterpret_cast<float4*>(orow) = un;
                    *reinterpret_cast<float4*>(D1 + er * K2_EW + 4 * lane) = dn;
                    continue;
                }
                const float4 l = lap_row<R>(lv, cv, rv, V, r + R, a);
                if constexpr (PLAIN) {
                    *reinterpret_cast<float4*>(orow) = leap_plain(mv, l, cv, ov);
                } else {
                    float nv[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const float g = gz1[r] * gxe[e];
                        const float c = comp(cv, e);
                        nv[e] = (zin && xin[e]) ? g * fmaf(comp(mv, e), comp(l, e), 2.f * c) - (g * g) * comp(ov, e)
                                                : c;  // fixed ring / outside the grid keep u_n
                    }
                    *reinterpret_cast<float4*>(orow) = make_float4(nv[0], nv[1], nv[2], nv[3]);
                }
            }
        };
        if (plain)
            step1(Flag<true>{});
        else
            step1(Flag<false>{});
        // sampling of u_n (receivers owned by this tile)
        if (p.smp_t1 >= 0) {
            const int lo = smp_rng[i].x, hi = smp_rng[i].y;
            for (int j = lo + tid; j < hi; j += K2_THREADS) {
                const int2 en = a.smp.ent[j];
                const int z = en.x / a.ld, xx = en.x - z * a.ld;
                float v = U[(z - z0 + 2 * R) * K2_UW + (xx - x0 + 8)] * a.smp_scale;
                if (a.smp_div_m) v /= (a.m != nullptr ? a.m[en.x] : a.m_const);
                a.smp_out[((long long)s * a.smp_nt + p.smp_t1) * a.smp_np + en.y] = v;
            }
        }
        __syncthreads();  // u_{n+1} on E complete in O
        // injection of step n into u_{n+1}, every point inside E (neighbours' too)
        if (p.inj_t1 >= 0 && inje_rng[i].y > inje_rng[i].x) {
            const int lo = inje_rng[i].x, hi = inje_rng[i].y;
            for (int j = lo + tid; j < hi; j += K2_THREADS) {
                const int2 en = p.inj_e.ent[j];
                const int z = en.x / a.ld, xx = en.x - z * a.ld;
                const int ez = z - (z0 - R), exx = xx - (x0 - 4);
                float v = a.inj_val[((long long)s * a.inj_nt + p.inj_t1) * a.inj_np + en.y] * a.inj_scale;
                if (a.inj_times_m) v *= (a.m != nullptr ? a.m[en.x] : a.m_const);
                const float g = (a.gz ? a.gz[z] : 1.f) * (a.gx ? a.gx[xx] : 1.f);
                atomicAdd(&O[ez * K2_EW + exx], g * v);
                if (SUMMED) atomicAdd(&D1[ez * K2_EW + exx], g * v);
            }
            __syncthreads();
        }

        // ------------------------------------------------------------ tile pass
        // store u_{n+1} on T; step 2 on T
        auto tile_pass = [&](auto plain_c) {
            constexpr bool PLAIN = decltype(plain_c)::value;
            // u_{n+1} rows tr0 .. tr0 + RB2 + 2R - 1 of E (T row tr is E row tr + R),
            // each loaded just before its first use
            float4 V[L::RB2 + 2 * R];
#pragma unroll
            for (int j = 0; j < 2 * R; ++j) V[j] = f4(O + (tr0 + j) * K2_EW + 4 * lane);
#pragma unroll
            for (int r = 0; r < L::RB2; ++r) {
                const int tr = tr0 + r, z = z0 + tr;
                if (z >= a.nz) break;
                V[r + 2 * R] = f4(O + (tr0 + r + 2 * R) * K2_EW + 4 * lane);
                const bool zin = z >= R && z < a.nz - R;
                const float4 c1 = V[r + R];  // u_{n+1}
                const long long off = (long long)z * a.ld + ex;
                if (!SUMMED || mid) {
                    if constexpr (PLAIN)
                        *reinterpret_cast<float4*>(u_mid + off) = c1;
                    else
                        store_level(u_mid + off, c1, zin, xin, all_x, a.zero_ring, x_ok);
                    if constexpr (SUMMED)
                        store_level(d_mid + off, f4(D1 + (tr + R) * K2_EW + 4 * lane), zin, xin, all_x,
                                    a.zero_ring, x_ok);
                }
                if (LVL16 && lq_mid && x_ok) store_bfp(lq_mid, le_mid, off, z, ex, p.eld, c1, !PLAIN, zin, xin);
                if (!two) continue;
                const float* nrow = O + (tr + R) * K2_EW + 4 * lane;
                const float4 lv = f4(nrow - 4), rv = f4(nrow + 4);
                if constexpr (SUMMED) {  // step 2 from (u_{n+1} in O, d_{n+1} in D1)
                    const float4 l = lap_row<R>(lv, c1, rv, V, r + R, a);
                    const float4 d1 = f4(D1 + (tr + R) * K2_EW + 4 * lane);
                    const float4 mv = f4(M + (tr + R) * K2_EW + 4 * lane);
                    float4 dn, un;
                    if constexpr (PLAIN) {
                        summed4_plain(c1, d1, mv, l, dn, un);
                    } else {
                        float g[4];
#pragma unroll
                        for (int e = 0; e < 4; ++e) g[e] = gz2[r] * gxe[e];
                        summed4(c1, d1, mv, l, g, dn, un);
                    }
                    if constexpr (PLAIN) {
                        *reinterpret_cast<float4*>(u_out + off) = un;
                        *reinterpret_cast<float4*>(d_out + off) = dn;
                    } else {
                        store_level(u_out + off, un, zin, xin, all_x, a.zero_ring, x_ok);
                        store_level(d_out + off, dn, zin, xin, all_x, a.zero_ring, x_ok);
                    }
                    // (blocks holding a source of step n + 1 are encoded again after the injection)
                    if (LVL16 && lq_out && x_ok) store_bfp(lq_out, le_out, off, z, ex, p.eld, un, !PLAIN, zin, xin);
                    continue;
                }
                const float4 l = lap_row<R>(lv, c1, rv, V, r + R, a);
                const float4 c0 = f4(U + (tr + 2 * R) * K2_UW + 4 + 4 * lane);  // u_n
                const float4 mv = f4(M + (tr + R) * K2_EW + 4 * lane);
                if constexpr (PLAIN) {
                    *reinterpret_cast<float4*>(u_out + off) = leap_plain(mv, l, c1, c0);
                } else {
                    float nv[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const float g = gz2[r] * gxe[e];
                        nv[e] = g * fmaf(comp(mv, e), comp(l, e), 2.f * comp(c1, e)) - (g * g) * comp(c0, e);
                    }
                    store_level(u_out + off, make_float4(nv[0], nv[1], nv[2], nv[3]), zin, xin, all_x,
                                a.zero_ring, x_ok);
                }
            }
        };
        if (t_lane) {
            if (plain)
                tile_pass(Flag<true>{});
            else
                tile_pass(Flag<false>{});
        }
        // sampling of u_{n+1} (receivers of this tile), from shared memory
        if (two && a.smp_t >= 0) {
            const int lo = smp_rng[i].x, hi = smp_rng[i].y;
            for (int j = lo + tid; j < hi; j += K2_THREADS) {
                const int2 en = a.smp.ent[j];
                const int z = en.x / a.ld, xx = en.x - z * a.ld;
                float v = O[(z - z0 + R) * K2_EW + (xx - x0 + 4)] * a.smp_scale;
                if (a.smp_div_m) v /= (a.m != nullptr ? a.m[en.x] : a.m_const);
                a.smp_out[((long long)s * a.smp_nt + a.smp_t) * a.smp_np + en.y] = v;
            }
        }
        __syncthreads();  // stage b fully read; this shot's stores done
        if (tid == 0 && i + L::STAGES < ns) {
            fence_proxy_async_smem();
            issue(i + L::STAGES);
        }
        // injection of step n + 1 into u_{n+2}, after every store of this shot
        if (two && a.inj_t >= 0) {
            const int lo = inj_rng[i].x, hi = inj_rng[i].y;
            for (int j = lo + tid; j < hi; j += K2_THREADS) {
                const int2 en = a.inj.ent[j];
                const int z = en.x / a.ld, xx = en.x - z * a.ld;
                float v = a.inj_val[((long long)s * a.inj_nt + a.inj_t) * a.inj_np + en.y] * a.inj_scale;
                if (a.inj_times_m) v *= (a.m != nullptr ? a.m[en.x] : a.m_const);
                const float g = (a.gz ? a.gz[z] : 1.f) * (a.gx ? a.gx[xx] : 1.f);
                atomicAdd(u_out + en.x, g * v);
                if (SUMMED) atomicAdd(d_out + en.x, g * v);
            }
            // the kept copy of u_{n+2}: the blocks of the injected cells again, from
            // u_{n+2} in global memory once every injection of the tile is in (the
            // condition is uniform over the CTA; a block's 4 cells lie in this tile)
            if (LVL16 && lq_out && inj_rng[i].y > inj_rng[i].x) {
                __syncthreads();
                for (int j = lo + tid; j < hi; j += K2_THREADS) {
                    const int2 en = a.inj.ent[j];
                    const int z = en.x / a.ld, xx = (en.x - z * a.ld) & ~3;
                    const long long off = (long long)z * a.ld + xx;
                    const float4 v = __ldcg(reinterpret_cast<const float4*>(u_out + off));
                    bool xi[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e) xi[e] = xx + e >= R && xx + e < a.nx - R;
                    store_bfp(lq_out, le_out, off, z, xx, p.eld, v, true, z >= R && z < a.nz - R, xi);
                }
            }
        }
    }
}

template <int R, bool SUMMED, bool LVL16 = false>
cudaError_t launch_impl(const CUtensorMap& mu, const CUtensorMap& mo, const CUtensorMap& mm, const Step2Args& p_in,
                        cudaStream_t s) {
    Step2Args p = p_in;
    p.a = with_weight_pairs(p_in.a);
    using L = LayoutK2<R, SUMMED>;
    static int configured_device = -1;
    int dev = 0;
    cudaGetDevice(&dev);
    if (configured_device != dev) {
        cudaError_t e = cudaFuncSetAttribute(step2d_k2_kernel<R, SUMMED, LVL16>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, L::BYTES);
        if (e != cudaSuccess) return e;
        configured_device = dev;
    }
    const dim3 grid(p.a.tiles_x * p.a.tiles_z, (p.a.nshot + p.a.shots_per_cta - 1) / p.a.shots_per_cta);
    const cudaError_t e =
        launch_pdl(step2d_k2_kernel<R, SUMMED, LVL16>, grid, dim3(K2_THREADS), L::BYTES, s, mu, mo, mm, p);
    count_launch();
    return e != cudaSuccess ? e : cudaGetLastError();
}

}  // namespace

cudaError_t launch_step2d_k2(int R, const CUtensorMap& map_u, const CUtensorMap& map_o,
                             const CUtensorMap& map_m, const Step2Args& p, cudaStream_t s) {
    if (p.a.shots_per_cta < 1 || p.a.shots_per_cta > T2_MAX_SPC) return cudaErrorInvalidValue;
    if (p.summed && (!p.d_out || (p.write_mid && !p.d_mid) || (!p.two_steps && !p.d_mid)))
        return cudaErrorInvalidValue;
    if (p.lq_mid || p.lq_out) {  // kept levels in block floating point (summed form only)
        if (!p.summed) return cudaErrorInvalidValue;
        switch (R) {
            case 1: return launch_impl<1, true, true>(map_u, map_o, map_m, p, s);
            case 2: return launch_impl<2, true, true>(map_u, map_o, map_m, p, s);
            case 4: return launch_impl<4, true, true>(map_u, map_o, map_m, p, s);
            default: return cudaErrorInvalidValue;
        }
    }
    switch (R * 2 + (p.summed ? 1 : 0)) {
        case 2: return launch_impl<1, false>(map_u, map_o, map_m, p, s);
        case 4: return launch_impl<2, false>(map_u, map_o, map_m, p, s);
        case 8: return launch_impl<4, false>(map_u, map_o, map_m, p, s);
        case 3: return launch_impl<1, true>(map_u, map_o, map_m, p, s);
        case 5: return launch_impl<2, true>(map_u, map_o, map_m, p, s);
        case 9: return launch_impl<4, true>(map_u, map_o, map_m, p, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace wfd
