// Small helper kernels of the wave path: model conversion, per-tile point
// lists, gathers, checkpoint packing, FP64 misfit / norm reductions.
// All are launched once per call (or once per checkpoint), not per cell-step,
// except the checkpoint pack which runs every ckpt_every steps.
#include <algorithm>

#include "common.cuh"
#include "internal.h"

namespace wfd {
namespace {

__global__ void vel_to_m_kernel(const float* __restrict__ vel, float* __restrict__ m, int nz,
                                int ny, int nx, int ld, float scale) {
    const long long n = (long long)nz * ny * ld;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int x = int(i % ld);
        const long long zy = i / ld;
        float v = 0.f;
        if (x < nx) v = vel[zy * nx + x] * scale;
        m[i] = v * v;
    }
}

__device__ __forceinline__ bool decode(const int32_t* pos, int nz, int ny, int nx, int R, int& z,
                                       int& y, int& x) {
    z = pos[0];
    y = pos[1];
    x = pos[2];
    const bool zok = z >= R && z < nz - R, xok = x >= R && x < nx - R;
    const bool yok = ny == 1 ? y == 0 : (y >= R && y < ny - R);
    return zok && yok && xok;
}

// Range of tiles (along one axis) whose region [t*T - h, (t+1)*T + h) holds v.
__device__ __forceinline__ void tile_span(int v, int T, int h, int ntile, int& lo, int& hi) {
    lo = v - h >= 0 ? (v - h) / T : 0;                  // smallest t with (t+1) T + h > v
    hi = min(ntile - 1, (v + h) / T);                   // largest t with t T - h <= v
    if (h == 0) lo = hi = v / T;
}

__global__ void count_kernel(const int32_t* __restrict__ pos, int nshot, int np, int nz, int ny,
                             int nx, int R, int tz, int ty, int tx, int tiles_y, int tiles_x,
                             int ntiles, int* counts, unsigned* err, int hz, int hx) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= (long long)nshot * np) return;
    const int s = int(i / np);
    int z, y, x;
    if (!decode(pos + 3 * i, nz, ny, nx, R, z, y, x)) {
        report(err, DEV_ERR_BAD_POSITION);
        return;
    }
    int zl, zh, xl, xh;
    tile_span(z, tz, hz, (nz + tz - 1) / tz, zl, zh);
    tile_span(x, tx, hx, tiles_x, xl, xh);
    for (int a = zl; a <= zh; ++a)
        for (int b = xl; b <= xh; ++b) {
            const int t = (a * tiles_y + (y / ty)) * tiles_x + b;
            atomicAdd(&counts[(long long)s * ntiles + t], 1);
        }
}

// Exclusive scan of counts into off[0..n] in one block; counts reset to 0 so
// they serve as fill cursors.
__global__ void scan_kernel(int* counts, int* off, int n) {
    __shared__ int part[1024];
    const int t = threadIdx.x;
    const int per = (n + blockDim.x - 1) / blockDim.x;
    const int lo = min(n, t * per), hi = min(n, lo + per);
    int sum = 0;
    for (int i = lo; i < hi; ++i) sum += counts[i];
    part[t] = sum;
    __syncthreads();
    for (int d = 1; d < (int)blockDim.x; d <<= 1) {
        const int v = t >= d ? part[t - d] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    int run = part[t] - sum;  // exclusive prefix of this thread's chunk
    for (int i = lo; i < hi; ++i) {
        off[i] = run;
        run += counts[i];
        counts[i] = 0;
    }
    if (t == blockDim.x - 1) off[n] = part[t];
}

__global__ void fill_kernel(const int32_t* __restrict__ pos, int nshot, int np, int nz, int ny,
                            int nx, int ld, int R, int tz, int ty, int tx, int tiles_y,
                            int tiles_x, int ntiles, int* cursor, const int* off, int2* ent, int hz,
                            int hx) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= (long long)nshot * np) return;
    const int s = int(i / np), p = int(i % np);
    int z, y, x;
    if (!decode(pos + 3 * i, nz, ny, nx, R, z, y, x)) return;
    int zl, zh, xl, xh;
    tile_span(z, tz, hz, (nz + tz - 1) / tz, zl, zh);
    tile_span(x, tx, hx, tiles_x, xl, xh);
    for (int a = zl; a <= zh; ++a)
        for (int b = xl; b <= xh; ++b) {
            const long long key = (long long)s * ntiles + (a * tiles_y + (y / ty)) * tiles_x + b;
            const int slot = off[key] + atomicAdd(&cursor[key], 1);
            ent[slot] = make_int2(int(((long long)z * ny + y) * ld + x), p);
        }
}

__global__ void gather_kernel(const float* __restrict__ u, long long shot_stride, const int* off,
                              const int2* ent, int ntiles, int np, const float* m, float scale,
                              int div_m, float* out, int out_nt, int out_t) {
    const int s = blockIdx.y;
    const int lo = off[(long long)s * ntiles], hi = off[(long long)(s + 1) * ntiles];
    const int j = lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= hi) return;
    const int2 en = ent[j];
    float v = u[s * shot_stride + en.x] * scale;
    if (div_m) v /= m[en.x];
    out[((long long)s * out_nt + out_t) * np + en.y] = v;
}

__global__ void pack_kernel(const float4* __restrict__ src, void* dst, long long n4, int fmt) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n4;
         i += (long long)gridDim.x * blockDim.x) {
        const float4 v = src[i];
        if (fmt == 1)
            static_cast<uint2*>(dst)[i] = pack_bf16x4(v);
        else
            static_cast<float4*>(dst)[i] = v;
    }
}

// from[i] - v instead of v where `from` is given (from may not alias dst)
__device__ __forceinline__ float4 minus_from(const float4* __restrict__ from, long long i, float4 v) {
    if (!from) return v;
    const float4 f = from[i];
    return make_float4(f.x - v.x, f.y - v.y, f.z - v.z, f.w - v.w);
}

__global__ void unpack_kernel(const void* src, float4* __restrict__ dst, long long n4, int fmt,
                              const float4* __restrict__ from) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n4;
         i += (long long)gridDim.x * blockDim.x) {
        const float4 v = fmt == 1 ? unpack_bf16x4(static_cast<const uint2*>(src)[i])
                                  : static_cast<const float4*>(src)[i];
        dst[i] = minus_from(from, i, v);
    }
}

// Block-scaled int16: each block of 32 consecutive values (8 float4, 8 lanes)
// stores round(v * 32767 / max|v|) and one FP32 scale max|v| / 32767. A warp
// walks chunks of 32 float4 (4 blocks); the block max is a 3-step xor shuffle.
__global__ void pack_i16_kernel(const float4* __restrict__ src, short4* __restrict__ q,
                                float* __restrict__ scales, long long n4) {
    const int lane = threadIdx.x & 31;
    const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    const long long nchunks = (n4 + 31) / 32;
    for (long long c = warp; c < nchunks; c += nwarps) {
        const long long i = c * 32 + lane;
        const float4 v = i < n4 ? src[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        float m = fmaxf(fmaxf(fabsf(v.x), fabsf(v.y)), fmaxf(fabsf(v.z), fabsf(v.w)));
        m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, 1));
        m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, 2));
        m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, 4));
        const float inv = m > 0.f ? 32767.f / m : 0.f;
        if (i < n4) {
            q[i] = make_short4(short(__float2int_rn(v.x * inv)), short(__float2int_rn(v.y * inv)),
                               short(__float2int_rn(v.z * inv)), short(__float2int_rn(v.w * inv)));
            if ((lane & 7) == 0) scales[i / 8] = m / 32767.f;
        }
    }
}

__global__ void unpack_i16_kernel(const short4* __restrict__ q, const float* __restrict__ scales,
                                  float4* __restrict__ dst, long long n4, const float4* __restrict__ from) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n4;
         i += (long long)gridDim.x * blockDim.x) {
        const short4 v = q[i];
        const float sc = scales[i / 8];
        dst[i] = minus_from(from, i, make_float4(v.x * sc, v.y * sc, v.z * sc, v.w * sc));
    }
}

__device__ __forceinline__ double block_sum(double v) {
    __shared__ double warp_sums[32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) warp_sums[w] = v;
    __syncthreads();
    v = threadIdx.x < (blockDim.x >> 5) ? warp_sums[threadIdx.x] : 0.0;
    if (w == 0)
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// res = d - obs (FP32); misfit += 1/2 sum res^2 accumulated in FP64.
__global__ void residual_misfit_kernel(const float* __restrict__ d, const float* __restrict__ obs,
                                       float* __restrict__ res, long long n, double* misfit) {
    double acc = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float r = d[i] - obs[i];
        res[i] = r;
        acc += 0.5 * double(r) * double(r);
    }
    acc = block_sum(acc);
    if (threadIdx.x == 0) atomicAdd(misfit, acc);
}

__global__ void sum_sq_kernel(const float* __restrict__ x, long long n, double* out) {
    double acc = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        acc += double(x[i]) * double(x[i]);
    acc = block_sum(acc);
    if (threadIdx.x == 0) atomicAdd(out, acc);
}

// grad_vel = dJ/dv = (G / m) dm/dv = 2 G / v on the interior, 0 on the ring.
__global__ void grad_finalize_kernel(const float* __restrict__ G, const float* __restrict__ vel,
                                     float* __restrict__ gv, int nz, int ny, int nx, int ld,
                                     int R) {
    const long long n = (long long)nz * ny * nx;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int x = int(i % nx);
        const long long zy = i / nx;
        const int y = int(zy % ny), z = int(zy / ny);
        const bool in = z >= R && z < nz - R && x >= R && x < nx - R &&
                        (ny == 1 || (y >= R && y < ny - R));
        gv[i] = in ? 2.f * G[zy * ld + x] / vel[i] : 0.f;
    }
}

int grid_for(long long n, int block = 256) {
    long long g = (n + block - 1) / block;
    return int(g < 1 ? 1 : (g > 152 * 32 ? 152 * 32 : g));
}

}  // namespace

cudaError_t launch_vel_to_m(const float* vel, float* m, int nz, int ny, int nx, int ld,
                            float scale, cudaStream_t s) {
    vel_to_m_kernel<<<grid_for((long long)nz * ny * ld), 256, 0, s>>>(vel, m, nz, ny, nx, ld, scale);
    count_launch();
    return cudaGetLastError();
}

namespace {

// Copies the damped frame of nshot fields [z][ld] to (save) or from a compact
// store: rows [0, W) and [nz - W, nz) in full, the other rows' columns
// [0, cl) and [cr, ld).
__global__ void band_kernel(float* field, float* store, long long shot_stride, int nshot, int nz, int ld, int W,
                            int cl, int cr, int save) {
    const long long rows = 2LL * W * ld, side = (long long)(cl + ld - cr);
    const long long B = rows + (long long)(nz - 2 * W) * side;
    const long long n = B * nshot;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const long long s = i / B;
        long long j = i - s * B;
        int z, x;
        if (j < rows) {
            const int r = int(j / ld);
            x = int(j - (long long)r * ld);
            z = r < W ? r : nz - 2 * W + r;
        } else {
            j -= rows;
            const int r = int(j / side), c = int(j - (long long)r * side);
            z = W + r;
            x = c < cl ? c : cr + (c - cl);
        }
        float* f = field + s * shot_stride + (long long)z * ld + x;
        if (save)
            store[i] = *f;
        else
            *f = store[i];
    }
}

}  // namespace

long long band_cells(int nz, int ld, int W, int cl, int cr) {
    return 2LL * W * ld + (long long)(nz - 2 * W) * (cl + ld - cr);
}

cudaError_t launch_band(float* field, float* store, long long shot_stride, int nshot, int nz, int ld, int W,
                        int cl, int cr, bool save, cudaStream_t s) {
    const long long n = band_cells(nz, ld, W, cl, cr) * nshot;
    if (n <= 0) return cudaSuccess;
    const int blocks = (int)std::min<long long>((n + 255) / 256, 152LL * 16);
    band_kernel<<<blocks, 256, 0, s>>>(field, store, shot_stride, nshot, nz, ld, W, cl, cr, save ? 1 : 0);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_build_lists(const int32_t* pos, int nshot, int np, int nz, int ny, int nx,
                               int ld, int R, int tile_z, int tile_y, int tile_x, int tiles_z,
                               int tiles_y, int tiles_x, int* counts, int* off, int2* ent,
                               unsigned* err, cudaStream_t s, int halo_z, int halo_x) {
    const int ntiles = tiles_z * tiles_y * tiles_x;
    const long long nkeys = (long long)nshot * ntiles;
    cudaError_t e = cudaMemsetAsync(counts, 0, sizeof(int) * nkeys, s);
    if (e != cudaSuccess) return e;
    const long long npts = (long long)nshot * np;
    const int blocks = int((npts + 255) / 256);
    if (npts > 0) {
        count_kernel<<<blocks, 256, 0, s>>>(pos, nshot, np, nz, ny, nx, R, tile_z, tile_y, tile_x,
                                            tiles_y, tiles_x, ntiles, counts, err, halo_z, halo_x);
        count_launch();
    }
    scan_kernel<<<1, 1024, 0, s>>>(counts, off, int(nkeys));
    count_launch();
    if (npts > 0) {
        fill_kernel<<<blocks, 256, 0, s>>>(pos, nshot, np, nz, ny, nx, ld, R, tile_z, tile_y,
                                           tile_x, tiles_y, tiles_x, ntiles, counts, off, ent, halo_z,
                                           halo_x);
        count_launch();
    }
    return cudaGetLastError();
}

cudaError_t launch_gather(const float* u, long long shot_stride, PointLists lists, int ntiles,
                          int nshot, int np, const float* m, float scale, int div_m, float* out,
                          int out_nt, int out_t, cudaStream_t s) {
    if (np == 0 || nshot == 0) return cudaSuccess;
    const dim3 grid((np + 127) / 128, nshot);
    gather_kernel<<<grid, 128, 0, s>>>(u, shot_stride, lists.off, lists.ent, ntiles, np, m, scale,
                                       div_m, out, out_nt, out_t);
    count_launch();
    return cudaGetLastError();
}

size_t ckpt_bytes(int format, long long n) {
    if (format == 2) return (size_t)((n * 2 + 15) / 16 * 16) + (size_t)((n + 31) / 32) * 4;
    return (size_t)n * (format == 1 ? 2 : 4);
}

cudaError_t launch_pack(const float* src, void* dst, long long n, int format, cudaStream_t s) {
    if (format == 2) {
        short4* q = static_cast<short4*>(dst);
        float* sc = reinterpret_cast<float*>(static_cast<unsigned char*>(dst) + (n * 2 + 15) / 16 * 16);
        pack_i16_kernel<<<grid_for(n / 4), 256, 0, s>>>(reinterpret_cast<const float4*>(src), q, sc,
                                                        n / 4);
        count_launch();
    } else {
        pack_kernel<<<grid_for(n / 4), 256, 0, s>>>(reinterpret_cast<const float4*>(src), dst,
                                                    n / 4, format);
        count_launch();
    }
    return cudaGetLastError();
}

namespace {

cudaError_t unpack_impl(const void* src, const float* from, float* dst, long long n, int format,
                        cudaStream_t s) {
    const float4* f = reinterpret_cast<const float4*>(from);
    if (format == 2) {
        const short4* q = static_cast<const short4*>(src);
        const float* sc = reinterpret_cast<const float*>(static_cast<const unsigned char*>(src) +
                                                         (n * 2 + 15) / 16 * 16);
        unpack_i16_kernel<<<grid_for(n / 4), 256, 0, s>>>(q, sc, reinterpret_cast<float4*>(dst), n / 4, f);
        count_launch();
    } else {
        unpack_kernel<<<grid_for(n / 4), 256, 0, s>>>(src, reinterpret_cast<float4*>(dst), n / 4,
                                                      format, f);
        count_launch();
    }
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_unpack(const void* src, float* dst, long long n, int format, cudaStream_t s) {
    return unpack_impl(src, nullptr, dst, n, format, s);
}

cudaError_t launch_unpack_diff(const void* src, const float* from, float* dst, long long n, int format,
                               cudaStream_t s) {
    return unpack_impl(src, from, dst, n, format, s);
}

cudaError_t launch_residual_misfit(const float* d, const float* obs, float* res, long long n,
                                   double* misfit, cudaStream_t s) {
    residual_misfit_kernel<<<grid_for(n), 256, 0, s>>>(d, obs, res, n, misfit);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_sum_sq(const float* x, long long n, double* out, cudaStream_t s) {
    sum_sq_kernel<<<grid_for(n), 256, 0, s>>>(x, n, out);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_grad_finalize(const float* G, const float* vel, float* grad_vel, int nz,
                                 int ny, int nx, int ld, int R, cudaStream_t s) {
    grad_finalize_kernel<<<grid_for((long long)nz * ny * nx), 256, 0, s>>>(G, vel, grad_vel, nz,
                                                                         ny, nx, ld, R);
    count_launch();
    return cudaGetLastError();
}

}  // namespace wfd
