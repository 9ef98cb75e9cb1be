// K time steps per launch of the 2D wave path at orders 2 and 4 (sm_103a).
//
// The step is the one-step kernel's,
//   u_{n+1} = g (2 u_n + m L u_n) - g^2 u_{n-1},  g = gz[z] gx[x],
// with its weights, operation order and source/receiver conventions (a source
// sample w_n goes into u_{n+1}; traces[n] = u_{n+1} at the receiver). This is
// the reference's temporal blocking (projects/18_simple_wave_fd/step2D_wave.cu:244-304:
// eight steps of the 5-point stencil in one tile) for the wave path's model
// field, sponge, sources and receivers: K = WR_HALO / R steps per launch, 8 at
// order 2 and 4 at order 4.
//
// Per CTA (256 threads): one shot and a window of 256 columns x 40 rows, the
// output tile (240 x 24) plus WR_HALO = 8 cells on every side. Each thread
// holds one column of the window in registers (the two levels u_{n-1}, u_n,
// which trade roles every step): the vertical taps are registers of the same
// thread, the horizontal ones come from neighbouring lanes by warp shuffles;
// the R edge columns of each warp go through shared memory (double-buffered
// by step parity: one CTA barrier per step). m of the window is staged in
// shared memory once per launch. A window cell at distance d from the window's
// edge has exact values for d / R steps; after K steps the output tile, 8
// cells in, is exact. Cells of the grid's fixed ring and outside the grid are
// never updated (the wave path keeps them at 0).
//
// Sources and receivers. At the start of a launch the CTA links the entries of
// its window's source list and its tile's receiver list into per-column lists
// in shared memory, so that after each step the thread owning a column adds
// the column's source samples into its new level and writes its receivers'
// samples. Entries past the lists' capacity are handled by every thread
// scanning them (correct for any number of points, slower).
#include "common.cuh"
#include "internal.h"

namespace wfd {
namespace {

constexpr int WR_NW = WR_W / 32;  // warps per CTA
constexpr int WR_CAP = 1024;      // source and receiver entries linked per CTA

template <int R>
struct LayoutWR {
    static constexpr int M_OFF = 0;                               // m on the window, [row][col]
    static constexpr int EDGE_OFF = M_OFF + WR_H * WR_W * 4;      // [parity][warp][side][k][row]
    static constexpr int EDGE = 2 * WR_NW * 2 * R * WR_H * 4;
    static constexpr int GZ_OFF = EDGE_OFF + EDGE;                // gz of the window rows
    static constexpr int LIST_OFF = GZ_OFF + WR_H * 4;            // heads, then entries (row, id, next)
    static constexpr int LISTS = 2 * WR_W * 4 + 2 * WR_CAP * 3 * 4;
    static constexpr int BYTES = LIST_OFF + LISTS;
};

// The thread's column's value at window row rr (a runtime index into a
// register array, by selection).
__device__ __forceinline__ float pick(const float (&v)[WR_H], int rr) {
    float out = 0.f;
#pragma unroll
    for (int r = 0; r < WR_H; ++r) out = (r == rr) ? v[r] : out;
    return out;
}

__device__ __forceinline__ void add_at(float (&v)[WR_H], int rr, float x) {
#pragma unroll
    for (int r = 0; r < WR_H; ++r)
        if (r == rr) v[r] += x;
}

// One step over the window: nxt (the level before cur) <- the level after cur.
// GUARD: update only cells of the grid's interior (windows that reach the
// grid's fixed ring or beyond); otherwise every row with its 2R vertical
// neighbours inside the window is updated. PLAIN: g = 1 on the whole window
// (no sponge there), where the update g (m L u + 2 u) - g^2 u_{n-1} is
// (m L u + 2 u) - u_{n-1}, value for value.
template <int R, bool GUARD, bool PLAIN>
__device__ __forceinline__ void wr_step(float (&nxt)[WR_H], const float (&cur)[WR_H], float* edge, const float* msh,
                                        const float* gzs, int t, int lane, int warp, float gxj, bool col_ok, int i0,
                                        const StepArgs& a) {
    if (lane < R) {
        float* d = edge + ((warp * 2 + 0) * R + lane) * WR_H;
#pragma unroll
        for (int r = 0; r < WR_H; ++r) d[r] = cur[r];
    }
    if (lane >= 32 - R) {
        float* d = edge + ((warp * 2 + 1) * R + (lane - (32 - R))) * WR_H;
#pragma unroll
        for (int r = 0; r < WR_H; ++r) d[r] = cur[r];
    }
    __syncthreads();
    // the neighbouring warps' edge column that lanes < k (left) and lanes
    // >= 32 - k (right) read for the tap at distance k: one shared-memory load
    // per row and tap through a per-lane pointer (the window's outermost
    // columns read their own warp's edge in place of a missing neighbour:
    // finite values that never reach the output tile)
    const int wl = max(warp - 1, 0), wr = min(warp + 1, WR_NW - 1);
    int nb[R];  // offsets into edge; lanes that use no edge value read an in-range slot
#pragma unroll
    for (int k = 1; k <= R; ++k)
        nb[k - 1] = lane < 16 ? ((wl * 2 + 1) * R + min(R - k + lane, R - 1)) * WR_H
                              : ((wr * 2 + 0) * R + min(max(lane + k - 32, 0), R - 1)) * WR_H;
#pragma unroll
    for (int r = R; r < WR_H - R; ++r) {
        const float c = cur[r];
        float acc = a.c0 * c;
#pragma unroll
        for (int k = 1; k <= R; ++k) {
            float l = __shfl_up_sync(0xffffffffu, c, k);
            float rr = __shfl_down_sync(0xffffffffu, c, k);
            const float e = edge[nb[k - 1] + r];
            if (lane < k) l = e;
            if (lane >= 32 - k) rr = e;
            acc = fmaf(a.cx[k - 1], l + rr, acc);
            acc = fmaf(a.cz[k - 1], cur[r - k] + cur[r + k], acc);
        }
        float nv;
        if (PLAIN) {
            nv = fmaf(msh[r * WR_W + t], acc, 2.f * c) - nxt[r];
        } else {
            const float g = gzs[r] * gxj;
            nv = g * fmaf(msh[r * WR_W + t], acc, 2.f * c) - (g * g) * nxt[r];
        }
        if (!GUARD || (col_ok && i0 + r >= R && i0 + r < a.nz - R)) nxt[r] = nv;
    }
}

template <int R>
__global__ void __launch_bounds__(WR_W, 2) wave_reg_kernel(const StepArgs a, const RegArgs q) {
    using L = LayoutWR<R>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float* msh = reinterpret_cast<float*>(smem_raw + L::M_OFF);
    float* edge_base = reinterpret_cast<float*>(smem_raw + L::EDGE_OFF);
    float* gzs = reinterpret_cast<float*>(smem_raw + L::GZ_OFF);
    int* shead = reinterpret_cast<int*>(smem_raw + L::LIST_OFF);  // sources, per column
    int* rhead = shead + WR_W;                                       // receivers, per column
    int* sent = rhead + WR_W;                                        // (row, id, next) x WR_CAP
    int* rent = sent + 3 * WR_CAP;

    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int shot = blockIdx.z;
    const int tile = blockIdx.y * a.tiles_x + blockIdx.x;
    const int ntiles = a.tiles_x * a.tiles_z;
    const int j0 = blockIdx.x * WR_OX - WR_HALO, i0 = blockIdx.y * WR_OZ - WR_HALO;
    const int jcol = j0 + t;
    const bool jin = jcol >= 0 && jcol < a.nx;
    const bool col_ok = jcol >= R && jcol < a.nx - R;
    const bool inner = i0 >= R && i0 + WR_H - 1 < a.nz - R && j0 >= R && j0 + WR_W - 1 < a.nx - R;  // (CTA-uniform)
    const long long sbase = (long long)shot * a.shot_stride;

    shead[t] = -1;
    rhead[t] = -1;
    float A[WR_H], B[WR_H];  // u_{n-1}, u_n; they trade roles every step
#pragma unroll
    for (int r = 0; r < WR_H; ++r) {
        const int i = i0 + r;
        const bool in = jin && i >= 0 && i < a.nz;
        const long long c = (long long)i * a.ld + jcol;
        A[r] = in ? __ldg(q.u0 + sbase + c) : 0.f;
        B[r] = in ? __ldg(q.u1 + sbase + c) : 0.f;
        msh[r * WR_W + t] = in ? __ldg(a.m + c) : 0.f;
    }
    if (t < WR_H) {
        const int i = i0 + t;
        gzs[t] = (a.gz != nullptr && i >= 0 && i < a.nz) ? __ldg(a.gz + i) : 1.f;
    }
    const float gxj = (a.gx != nullptr && jin) ? __ldg(a.gx + jcol) : 1.f;
    // g = 1 on the whole window: every column's gx and every row's gz is 1
    const bool g1 = gxj == 1.f && (t >= WR_H || gzs[t] == 1.f);
    const bool plain = __syncthreads_and(g1 ? 1 : 0) != 0;  // (also: list heads initialised)

    // link the window's sources and the tile's receivers into per-column lists
    const long long key = (long long)shot * ntiles + tile;
    const int s_lo = q.src.off ? q.src.off[key] : 0, s_hi = q.src.off ? q.src.off[key + 1] : 0;
    const int r_lo = (a.smp.off && a.smp_out) ? a.smp.off[key] : 0;
    const int r_hi = (a.smp.off && a.smp_out) ? a.smp.off[key + 1] : 0;
    // (a point outside the window, which the lists' geometry rules out, is
    // reported and skipped rather than indexed)
    auto in_window = [&](int z, int x) { return x - j0 >= 0 && x - j0 < WR_W && z - i0 >= 0 && z - i0 < WR_H; };
    for (int e = t; e < min(s_hi - s_lo, WR_CAP); e += WR_W) {
        const int2 en = q.src.ent[s_lo + e];
        const int z = en.x / a.ld, x = en.x - z * a.ld;
        if (!in_window(z, x)) {
            report(a.err, DEV_ERR_BAD_POSITION);
            continue;
        }
        sent[3 * e] = z - i0;
        sent[3 * e + 1] = en.y;
        sent[3 * e + 2] = atomicExch(&shead[x - j0], e);
    }
    for (int e = t; e < min(r_hi - r_lo, WR_CAP); e += WR_W) {
        const int2 en = a.smp.ent[r_lo + e];
        const int z = en.x / a.ld, x = en.x - z * a.ld;
        if (!in_window(z, x)) {
            report(a.err, DEV_ERR_BAD_POSITION);
            continue;
        }
        rent[3 * e] = z - i0;
        rent[3 * e + 1] = en.y;
        rent[3 * e + 2] = atomicExch(&rhead[x - j0], e);
    }
    __syncthreads();

    // after a step: the step's source samples into the new level, then its
    // receivers' samples of it
    auto points = [&](float (&nv)[WR_H], int n) {
        for (int e = shead[t]; e >= 0; e = sent[3 * e + 2]) {
            const int rr = sent[3 * e];
            const float v = a.inj_val[((long long)shot * a.inj_nt + n) * a.inj_np + sent[3 * e + 1]] * a.inj_scale;
            add_at(nv, rr, gzs[rr] * gxj * v);
        }
        for (int e = s_lo + WR_CAP; e < s_hi; ++e) {  // (beyond the linked capacity)
            const int2 en = q.src.ent[e];
            const int z = en.x / a.ld, x = en.x - z * a.ld;
            if (x != jcol || z - i0 < 0 || z - i0 >= WR_H) continue;
            const float v = a.inj_val[((long long)shot * a.inj_nt + n) * a.inj_np + en.y] * a.inj_scale;
            add_at(nv, z - i0, gzs[z - i0] * gxj * v);
        }
        for (int e = rhead[t]; e >= 0; e = rent[3 * e + 2])
            a.smp_out[((long long)shot * a.smp_nt + n) * a.smp_np + rent[3 * e + 1]] =
                pick(nv, rent[3 * e]) * a.smp_scale;
        for (int e = r_lo + WR_CAP; e < r_hi; ++e) {
            const int2 en = a.smp.ent[e];
            const int z = en.x / a.ld, x = en.x - z * a.ld;
            if (x != jcol || z - i0 < 0 || z - i0 >= WR_H) continue;
            a.smp_out[((long long)shot * a.smp_nt + n) * a.smp_np + en.y] = pick(nv, z - i0) * a.smp_scale;
        }
    };

    const int kind = inner ? (plain ? 0 : 1) : 2;  // (CTA-uniform)
    auto step = [&](float (&nxt)[WR_H], const float (&cur)[WR_H], float* edge) {
        if (kind == 0)
            wr_step<R, false, true>(nxt, cur, edge, msh, gzs, t, lane, warp, gxj, col_ok, i0, a);
        else if (kind == 1)
            wr_step<R, false, false>(nxt, cur, edge, msh, gzs, t, lane, warp, gxj, col_ok, i0, a);
        else
            wr_step<R, true, false>(nxt, cur, edge, msh, gzs, t, lane, warp, gxj, col_ok, i0, a);
    };
    for (int st = 0; st < q.ksteps; ++st) {
        float* edge = edge_base + (st & 1) * (WR_NW * 2 * R * WR_H);
        const int n = q.n0 + st;
        if ((st & 1) == 0) {
            step(A, B, edge);
            points(A, n);
        } else {
            step(B, A, edge);
            points(B, n);
        }
    }

    // the output tile: u_{n0+k-1} (the older level) and u_{n0+k}
    const bool odd = q.ksteps & 1;  // odd: A is u_{n0+k}, B the level before
    if (t >= WR_HALO && t < WR_W - WR_HALO && jin) {
#pragma unroll
        for (int r = WR_HALO; r < WR_H - WR_HALO; ++r) {
            const int i = i0 + r;
            if (i < a.nz) {
                const long long c = sbase + (long long)i * a.ld + jcol;
                q.v0[c] = odd ? B[r] : A[r];
                q.v1[c] = odd ? A[r] : B[r];
            }
        }
    }
}

template <int R>
cudaError_t launch_impl(const StepArgs& a, const RegArgs& q, cudaStream_t s) {
    using L = LayoutWR<R>;
    static int configured_device = -1;
    int dev = 0;
    cudaGetDevice(&dev);
    if (configured_device != dev) {
        const cudaError_t e =
            cudaFuncSetAttribute(wave_reg_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, L::BYTES);
        if (e != cudaSuccess) return e;
        configured_device = dev;
    }
    const dim3 grid(a.tiles_x, a.tiles_z, a.nshot);
    // a plain launch: the window's read-only loads of u0 and u1, the previous
    // launch's output, are ordered after it by the kernel boundary
    wave_reg_kernel<R><<<grid, WR_W, L::BYTES, s>>>(a, q);
    count_launch();
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_wave_reg(int R, const StepArgs& a, const RegArgs& q, cudaStream_t s) {
    if (q.ksteps < 1 || q.ksteps * R > WR_HALO || a.nshot > 65535 || a.tiles_z > 65535) return cudaErrorInvalidValue;
    switch (R) {
        case 1: return launch_impl<1>(a, q, s);
        case 2: return launch_impl<2>(a, q, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace wfd
