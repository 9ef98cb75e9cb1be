// C-ABI layer of the wave path (include/wavefd.h): argument checks, workspace
// layout, TMA descriptors, and the time loops of the forward, the
// checkpointed adjoint and the misfit gradient. Host code only; all device
// work is in stencil2d.cu / stencil3d.cu / aux.cu.
#include <nvtx3/nvToolsExt.h>

#include <atomic>
#include <cmath>
#include <map>
#include <mutex>
#include <utility>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/wavefd.h"
#include "internal.h"

using namespace wfd;

namespace {
std::atomic<uint64_t> g_launches{0};
}

void wfd::count_launch(int n) { g_launches.fetch_add((uint64_t)n, std::memory_order_relaxed); }

namespace {

thread_local std::string g_last_error;

// ------------------------------------------------------------------ phase timing
enum Phase { PH_FORWARD = 0, PH_RECOMPUTE = 1, PH_ADJOINT = 2 };
const char* const kPhaseName[3] = {"wfd forward", "wfd recompute", "wfd adjoint"};

struct PhaseRecord {
    int phase;
    cudaEvent_t start, stop;
    int launches;
};
thread_local bool g_profiling = false;
thread_local std::vector<PhaseRecord> g_records;

// Marks one phase: an NVTX range always, CUDA events on the stream while
// profiling is on.
class PhaseScope {
   public:
    PhaseScope(int phase, cudaStream_t s, int launches) : s_(s) {
        nvtxRangePushA(kPhaseName[phase]);
        if (g_profiling) {
            rec_.phase = phase;
            rec_.launches = launches;
            if (cudaEventCreate(&rec_.start) == cudaSuccess) {
                if (cudaEventCreate(&rec_.stop) == cudaSuccess) {
                    cudaEventRecord(rec_.start, s_);
                    active_ = true;
                } else {
                    cudaEventDestroy(rec_.start);
                }
            }
        }
    }
    ~PhaseScope() {
        if (active_) {
            cudaEventRecord(rec_.stop, s_);
            g_records.push_back(rec_);
        }
        nvtxRangePop();
    }

   private:
    cudaStream_t s_;
    PhaseRecord rec_{};
    bool active_ = false;
};

int fail(int status, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
int fail(int status, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return status;
}

}  // namespace

int wfd::set_error(int status, const char* message) { return fail(status, "%s", message); }

namespace {

#define WFD_CUDA(call)                                                                      \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess)                                                              \
            return fail(WFD_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));     \
    } while (0)

// ------------------------------------------------------------------ TMA maps
using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                 const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                 const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                 CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encoder() {
    static EncodeTiled fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(p);
    }
    return fn;
}

// Tiled map over a field buffer [nshot][nz][ny][ld] with extent nx in x
// (reads past nx, or past any edge, fill zeros).
int make_field_map(CUtensorMap* map, const void* base, bool bf16, int ndim, int nz, int ny,
                   int nx, int ld, int nshot, const cuuint32_t* box) {
    EncodeTiled enc = encoder();
    if (!enc) return fail(WFD_ERR_CUDA, "cuTensorMapEncodeTiled entry point unavailable");
    const cuuint64_t es = bf16 ? 2 : 4;
    cuuint64_t dims[4], strides[3];
    cuuint32_t estr[4] = {1, 1, 1, 1};
    int rank;
    if (ndim == 2) {
        rank = 3;
        dims[0] = nx; dims[1] = nz; dims[2] = nshot;
        strides[0] = ld * es;
        strides[1] = (cuuint64_t)nz * ld * es;
    } else {
        rank = 4;
        dims[0] = nx; dims[1] = ny; dims[2] = nz; dims[3] = nshot;
        strides[0] = ld * es;
        strides[1] = (cuuint64_t)ny * ld * es;
        strides[2] = (cuuint64_t)nz * ny * ld * es;
    }
    CUresult r = enc(map, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                     rank, const_cast<void*>(base), dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(WFD_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return WFD_OK;
}

// 3D tiled map (x fastest) of any element type, zero fill out of range.
int make_map3(CUtensorMap* map, const void* base, CUtensorMapDataType dt, const cuuint64_t* dims,
              const cuuint64_t* strides, const cuuint32_t* box) {
    EncodeTiled enc = encoder();
    if (!enc) return fail(WFD_ERR_CUDA, "cuTensorMapEncodeTiled entry point unavailable");
    const cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = enc(map, dt, 3, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(WFD_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return WFD_OK;
}

int scale_blocks(int ld) { return ((ld + 31) / 32 + 3) / 4 * 4; }  // per row, a multiple of 4

// ------------------------------------------------------------------ geometry
struct Geom {
    int ndim, R, nz, ny, nx, ld;
    int sb;                  // time steps per launch (2D: 1 or 2)
    long long plane, cells;  // z stride; cells per shot (padded)
    int tile_z, tile_y, tile_x, tiles_z, tiles_y, tiles_x, ntiles;
    int spc;                 // shots per CTA
    int K, nseg, k0_last;    // checkpoint interval, segments, first step of the last segment
    bool ustore;             // the adjoint forms L u_k from stored levels u_k (2D, one step)
    int jstore, k0_store;    // u store: the forward keeps the levels of segments >= jstore
    bool lvl16;              // ... in block floating point (WFD_LEVEL_BFP16), not as FP32 slots
    bool lap_bf16;           // stored L u_k in BF16 (when !ustore)
    float c0, cz[4], cy[4], cx[4];
    bool vd;                 // variable density (2D): 128 x 16 tiles, staggered operator
    bool recon;              // the reconstruction adjoint (time reversal, saved frames)
    int band_w, band_cl, band_cr;  // its damped frame: W rows / columns [0, cl), [cr, ld)
    float cs[4], vd_sz;      // staggered first-derivative weights, (dx/dz)^2
};

// Staggered first-derivative weights of order 2R on a unit grid:
// c_k = 1/(2k-1) prod_{m != k} (2m-1)^2 / ((2m-1)^2 - (2k-1)^2).
void stag_weights(int R, double* c) {
    for (int k = 1; k <= R; ++k) {
        double v = 1.0 / (2 * k - 1);
        for (int m = 1; m <= R; ++m)
            if (m != k) {
                const double a = (2 * m - 1) * (2 * m - 1), b = (2 * k - 1) * (2 * k - 1);
                v *= a / (a - b);
            }
        c[k] = v;
    }
}

int cdiv(long long a, long long b) { return int((a + b - 1) / b); }

void fd_weights(int order, double* a) {
    const int R = order / 2;
    auto fact = [](int n) { double f = 1; for (int i = 2; i <= n; ++i) f *= i; return f; };
    double s = 0;
    for (int k = 1; k <= R; ++k) {
        a[k] = 2.0 * ((k % 2) ? 1.0 : -1.0) * fact(R) * fact(R) /
               (double(k) * k * fact(R - k) * fact(R + k));
        s += a[k];
    }
    a[0] = -2.0 * s;
}

int check_problem(const wfd_problem* p) {
    if (!p) return fail(WFD_ERR_INVALID, "problem is NULL");
    if (p->ndim != 2 && p->ndim != 3) return fail(WFD_ERR_INVALID, "ndim must be 2 or 3");
    if (p->order != 2 && p->order != 4 && p->order != 8)
        return fail(WFD_ERR_INVALID, "order must be 2, 4 or 8");
    const int R = p->order / 2;
    if (p->ndim == 2 && p->ny != 1) return fail(WFD_ERR_INVALID, "2D problems need ny == 1");
    if (p->ndim == 3 && !step3d_available())
        return fail(WFD_ERR_INVALID, "3D kernel not built into this library");
    if (p->nz < 2 * R + 1 || p->nx < 2 * R + 1 || (p->ndim == 3 && p->ny < 2 * R + 1))
        return fail(WFD_ERR_INVALID, "grid too small for order %d", p->order);
    if (p->nx > (1 << 24) || p->nz > (1 << 24) || p->ny > (1 << 24))
        return fail(WFD_ERR_INVALID, "grid axis too large");
    if ((long long)p->nz * p->ny * (long long)(p->nx + 8) >= (1ll << 31))
        return fail(WFD_ERR_INVALID, "more than 2^31 cells per shot");
    if (p->nshot < 1 || p->nt < 1 || p->nsrc < 0 || p->nrec < 0)
        return fail(WFD_ERR_INVALID, "nshot, nt must be >= 1 and nsrc, nrec >= 0");
    if (p->nshot > 65535 || (p->ndim == 2 && p->nshot > 65535 * T2_MAX_SPC))
        return fail(WFD_ERR_INVALID, "too many shots");
    if (p->ndim == 3 && (long long)cdiv(p->nz, T3_ZCHUNK) * cdiv(p->ny, T3_TY) * cdiv(p->nx, T3_TX) > 65535)
        return fail(WFD_ERR_INVALID, "3D grid has more than 65535 (%d x %d x %d)-cell columns", T3_ZCHUNK,
                    T3_TY, T3_TX);
    if (!(p->dt > 0) || !(p->dx > 0) || !(p->dz > 0) || (p->ndim == 3 && !(p->dy > 0)))
        return fail(WFD_ERR_INVALID, "dt and spacings must be positive");
    if (p->ckpt_format < WFD_CKPT_FP32 || p->ckpt_format > WFD_CKPT_I16)
        return fail(WFD_ERR_INVALID, "unknown checkpoint format %d", p->ckpt_format);
    if (p->lap_store < WFD_LAP_AUTO || p->lap_store > WFD_LAP_FP32)
        return fail(WFD_ERR_INVALID, "unknown lap_store %d", p->lap_store);
    if (p->field_format < WFD_FIELD_FP32 || p->field_format > WFD_FIELD_I16)
        return fail(WFD_ERR_INVALID, "unknown field_format %d", p->field_format);
    if (p->field_format != WFD_FIELD_FP32 && (p->ndim != 2 || p->step_block == 2))
        return fail(WFD_ERR_INVALID, "reduced-precision fields: 2D, one step per launch only");
    if (p->adjoint_mode < WFD_ADJOINT_CHECKPOINT || p->adjoint_mode > WFD_ADJOINT_RECONSTRUCT)
        return fail(WFD_ERR_INVALID, "unknown adjoint_mode %d", p->adjoint_mode);
    if (p->adjoint_mode == WFD_ADJOINT_RECONSTRUCT &&
        (p->ndim != 2 || p->step_block == 2 || p->lap_store != WFD_LAP_AUTO || p->field_format != WFD_FIELD_FP32))
        return fail(WFD_ERR_INVALID, "the reconstruction adjoint: 2D, one step per launch, lap_store auto, FP32");
    if (p->update_form < WFD_UPDATE_AUTO || p->update_form > WFD_UPDATE_SUMMED)
        return fail(WFD_ERR_INVALID, "unknown update_form %d", p->update_form);
    if (p->update_form == WFD_UPDATE_SUMMED &&
        (p->field_format != WFD_FIELD_FP32 || p->lap_store != WFD_LAP_AUTO ||
         p->adjoint_mode != WFD_ADJOINT_CHECKPOINT))
        return fail(WFD_ERR_INVALID, "the summed update form: FP32 fields, lap_store auto, checkpoint adjoint");
    if (p->level_format < WFD_LEVEL_FP32 || p->level_format > WFD_LEVEL_BFP16)
        return fail(WFD_ERR_INVALID, "unknown level_format %d", p->level_format);
    if (p->level_format == WFD_LEVEL_BFP16 &&
        (p->ndim != 2 || p->step_block != 2 || p->update_form == WFD_UPDATE_LEAPFROG ||
         p->field_format != WFD_FIELD_FP32 || p->lap_store != WFD_LAP_AUTO ||
         p->adjoint_mode != WFD_ADJOINT_CHECKPOINT))
        return fail(WFD_ERR_INVALID,
                    "block-floating-point levels: 2D, step_block 2, the summed forward (FP32 fields, "
                    "lap_store auto, checkpoint adjoint)");
    if (p->recon_band < 0 || 2 * p->recon_band > std::min(p->nz, p->nx))
        return fail(WFD_ERR_INVALID, "recon_band must lie in [0, min(nz, nx) / 2]");
    if (p->tile_rows != 0 && p->tile_rows != 16 && p->tile_rows != 32)
        return fail(WFD_ERR_INVALID, "tile_rows must be 0, 16 or 32");
    if (p->step_block < 0 || (p->step_block > 2 && p->step_block != 4 && p->step_block != 8) ||
        (p->step_block == 2 && p->ndim != 2))
        return fail(WFD_ERR_INVALID, "step_block must be 0, 1, 2, 4 or 8 (2: 2D only)");
    if (p->step_block >= 4 && (p->ndim != 2 || p->order != (p->step_block == 8 ? 2 : 4) ||
                               p->field_format != WFD_FIELD_FP32 || p->update_form == WFD_UPDATE_SUMMED))
        return fail(WFD_ERR_INVALID,
                    "step_block %d: the 2D leapfrog forward at order %d with FP32 fields", p->step_block,
                    p->step_block == 8 ? 2 : 4);
    if (p->step_block == 2 && p->lap_store != WFD_LAP_AUTO)
        return fail(WFD_ERR_INVALID, "step_block 2 keeps the levels u_k: lap_store must be WFD_LAP_AUTO");
    if (p->ckpt_every < 0 || p->shots_per_cta < 0 || p->group_shots < 0 || p->store_levels < 0)
        return fail(WFD_ERR_INVALID,
                    "ckpt_every, shots_per_cta, group_shots and store_levels must be >= 0");
    if (p->vmax > 0) {
        double a[5];
        fd_weights(p->order, a);
        double S = std::fabs(a[0]);
        for (int k = 1; k <= R; ++k) S += 2 * std::fabs(a[k]);
        double inv2 = 1.0 / (p->dz * (double)p->dz) + 1.0 / (p->dx * (double)p->dx);
        if (p->ndim == 3) inv2 += 1.0 / (p->dy * (double)p->dy);
        const double lhs = p->vmax * (double)p->dt * std::sqrt(inv2 * S);
        if (lhs > 2.0)
            return fail(WFD_ERR_UNSTABLE, "vmax*dt = %g exceeds the CFL bound %g of order %d",
                        p->vmax * (double)p->dt, 2.0 / std::sqrt(inv2 * S), p->order);
    }
    return WFD_OK;
}

// tile_rows > 0 overrides the problem's 2D tile height and step_block >= 1
// its steps per launch (the u-store adjoint runs one step per launch on
// 16-row tiles: its third staged tile must leave room for the stages).
Geom make_geom(const wfd_problem* p, int tile_rows = 0, int step_block = 0, bool vd = false) {
    Geom g{};
    g.vd = vd;
    g.ndim = p->ndim;
    g.R = p->order / 2;
    g.nz = p->nz;
    g.ny = p->ndim == 3 ? p->ny : 1;
    g.nx = p->nx;
    g.ld = (p->nx + 7) / 8 * 8;
    g.plane = (long long)g.ny * g.ld;
    g.cells = (long long)g.nz * g.plane;
    const int sb = step_block > 0 ? step_block : p->step_block;
    g.sb = (p->ndim == 2 && (sb == 2 || (sb >= 4 && g.R * sb == WR_HALO))) ? sb : 1;
    if (vd) {
        g.sb = 1;
        g.tile_z = 16;  // the variable-density kernel's 128 x 16 tile
        g.tile_y = 1;
        g.tile_x = T2_TX;
    } else if (g.ndim == 2 && g.sb == 2) {
        g.tile_z = K2_TZ;
        g.tile_y = 1;
        g.tile_x = K2_TX;
    } else if (g.ndim == 2 && g.sb >= 4) {  // the register window's output tile
        g.tile_z = WR_OZ;
        g.tile_y = 1;
        g.tile_x = WR_OX;
    } else if (g.ndim == 2 && p->field_format != WFD_FIELD_FP32) {
        g.tile_z = 32;  // the reduced-precision kernel's 128 x 32 tile
        g.tile_y = 1;
        g.tile_x = T2_TX;
    } else if (g.ndim == 2) {
        g.tile_z = tile_rows > 0 ? tile_rows : p->tile_rows > 0 ? p->tile_rows : T2_TZ;
        g.tile_y = 1;
        g.tile_x = T2_TX;
    } else {
        g.tile_z = T3_ZCHUNK; g.tile_y = T3_TY; g.tile_x = T3_TX;
    }
    g.tiles_z = cdiv(g.nz, g.tile_z);
    g.tiles_y = cdiv(g.ny, g.tile_y);
    g.tiles_x = cdiv(g.nx, g.tile_x);
    g.ntiles = g.tiles_z * g.tiles_y * g.tiles_x;
    if (g.ndim == 3) {
        g.spc = 1;  // a 3D CTA works on one shot
    } else if (p->shots_per_cta > 0) {
        g.spc = std::min(std::min(p->shots_per_cta, p->nshot), T2_MAX_SPC);
    } else {
        // enough CTAs for ~6 waves of 2 resident CTAs on 152 SMs, otherwise
        // as many shots per CTA as possible (m and the gradient amortise over them)
        const long long target = 152LL * 2 * 6;
        long long spc = (long long)g.ntiles * p->nshot / target;
        int s = 1;
        while (2LL * s <= spc && 2 * s <= p->nshot) s *= 2;
        g.spc = std::min(s, T2_MAX_SPC);
    }
    // (the shot count is bounded so that nshot / T2_MAX_SPC CTA rows fit gridDim.y)
    g.K = p->ckpt_every > 0 ? std::min(p->ckpt_every, p->nt)
                            : std::max(1, (int)std::ceil(std::sqrt((double)p->nt)));
    g.nseg = cdiv(p->nt, g.K);
    g.k0_last = (g.nseg - 1) * g.K;
    g.ustore = g.ndim == 2 && p->lap_store == WFD_LAP_AUTO;
    g.jstore = g.nseg - 1;
    if (g.ustore && p->store_levels > g.K + 2)
        g.jstore = std::max(0, g.nseg - (p->store_levels - 2) / g.K);
    g.k0_store = g.jstore * g.K;
    g.lvl16 = g.ustore && !vd && p->level_format == WFD_LEVEL_BFP16;
    g.lap_bf16 = p->lap_store == WFD_LAP_BF16;
    g.recon = p->adjoint_mode == WFD_ADJOINT_RECONSTRUCT;
    if (g.recon) {
        g.band_w = p->recon_band;
        g.band_cl = (g.band_w + 3) / 4 * 4;
        g.band_cr = g.band_w == 0 ? g.ld : std::max(g.band_cl, (g.nx - g.band_w) / 4 * 4);
    }
    double a[5] = {0, 0, 0, 0, 0};
    fd_weights(p->order, a);
    const double sz = (double)p->dx * p->dx / ((double)p->dz * p->dz);
    const double sy = g.ndim == 3 ? (double)p->dx * p->dx / ((double)p->dy * p->dy) : 0.0;
    g.c0 = float(a[0] * (1.0 + sz + sy));
    for (int k = 1; k <= 4; ++k) {
        g.cz[k - 1] = k <= g.R ? float(a[k] * sz) : 0.f;
        g.cy[k - 1] = k <= g.R ? float(a[k] * sy) : 0.f;
        g.cx[k - 1] = k <= g.R ? float(a[k]) : 0.f;
    }
    if (vd) {
        double c[5] = {0, 0, 0, 0, 0};
        stag_weights(g.R, c);
        for (int k = 1; k <= 4; ++k) g.cs[k - 1] = k <= g.R ? float(c[k]) : 0.f;
        g.vd_sz = float(sz);
    }
    return g;
}

// Geometry of the adjoint launches: 16-row tiles for the u-store adjoint.
Geom adjoint_geom(const wfd_problem* p, const Geom& g) {
    return g.ustore && (g.tile_z != 16 || g.sb != 1) ? make_geom(p, 16, 1) : g;
}

// ------------------------------------------------------------------ workspace
struct Layout {
    int nbuf;  // forward field buffers: 2 (in place) or 4 (two-step blocking)
    size_t err, m, P[4], counts, src_off, src_ent, rec_off, rec_ent;
    size_t srce_off, srce_ent;  // extended-region source lists (two-step)
    size_t asrc_off, asrc_ent, arec_off, arec_ent;  // adjoint-geometry lists (u store)
    size_t Q[4], G, ckpt, lap, res, total;
    size_t field_bytes, ckpt_field_bytes, lap_field_bytes;
    size_t S[2], scale_bytes;  // reduced-precision fields: the int16 block scales
    size_t b, Gbx, Gbz;        // variable density: b = 1/rho, half-point gradient sums
    size_t frames, frame_bytes;  // reconstruction adjoint: the damped frame of u_1 .. u_nt
    size_t D;                  // summed form: the increment field d_n (0: leapfrog)
    int nlap;  // slots of the lap region: K stored L u_k, or levels u_k (u store): from
               // u_{k0_store - 1} to u_nt, and at least K + 2 for a recomputed segment
    // block-floating-point kept levels u_{k0_store} .. u_{nt-1} (level i = u_{k0_store + i}),
    // in the same region: the adjoint is done with them before a segment is recomputed
    int nlvl;
    size_t lvl_q_bytes, lvl_bytes;  // mantissas of a level; mantissas + exponents
};

size_t up256(size_t v) { return (v + 255) / 256 * 256; }

// Whether the forward runs in the summed form (state u_n, d_n): forced by
// WFD_UPDATE_SUMMED, or chosen by WFD_UPDATE_AUTO for a forward that saves the
// state of a gradient, on the 2D u-store path and in 3D (lap_store auto in both).
bool summed_forward(const wfd_problem* p, const Geom& g, bool save) {
    const bool avail = !g.vd && p->field_format == WFD_FIELD_FP32 && !g.recon &&
                       p->lap_store == WFD_LAP_AUTO && (g.ndim == 3 || g.ustore);
    return avail && (p->update_form == WFD_UPDATE_SUMMED || (p->update_form == WFD_UPDATE_AUTO && save));
}

Layout make_layout(const wfd_problem* p, const Geom& g, bool grad) {
    Layout L{};
    size_t o = 0;
    auto take = [&](size_t bytes) { size_t at = o; o = up256(o + bytes); return at; };
    const Geom ga = adjoint_geom(p, g);
    const bool alists = grad && (ga.tile_z != g.tile_z || ga.tile_x != g.tile_x);
    const size_t keys = (size_t)p->nshot * std::max(g.ntiles, alists ? ga.ntiles : 0);
    L.field_bytes = (size_t)p->nshot * g.cells * (p->field_format == WFD_FIELD_FP32 ? 4 : 2);
    L.nbuf = g.sb >= 2 ? 4 : 2;  // (K steps per launch: two pairs of levels, read one, write the other)
    L.err = take(256);
    L.m = take((size_t)g.cells * 4);
    if (g.vd) L.b = take((size_t)g.cells * 4);
    for (int b = 0; b < L.nbuf; ++b) L.P[b] = take(L.field_bytes);
    // the increment d_n; with two steps per launch d_n, d_{n+2} and d_{n+1}
    if (summed_forward(p, g, grad)) L.D = take((g.sb == 2 ? 3 : 1) * L.field_bytes);
    if (p->field_format == WFD_FIELD_I16) {
        L.scale_bytes = (size_t)p->nshot * g.nz * scale_blocks(g.ld) * 4;
        for (int b = 0; b < 2; ++b) L.S[b] = take(L.scale_bytes);
    }
    L.counts = take(keys * 4);
    L.src_off = take((keys + 1) * 4);
    L.src_ent = take((size_t)p->nshot * p->nsrc * 8 + 8);
    L.rec_off = take((keys + 1) * 4);
    L.rec_ent = take((size_t)p->nshot * p->nrec * 8 + 8);
    if (g.sb >= 2) {  // a point joins up to 4 extended tile regions (windows)
        L.srce_off = take((keys + 1) * 4);
        L.srce_ent = take((size_t)p->nshot * p->nsrc * 32 + 8);
    }
    if (alists) {
        const size_t akeys = (size_t)p->nshot * ga.ntiles;
        L.asrc_off = take((akeys + 1) * 4);
        L.asrc_ent = take((size_t)p->nshot * p->nsrc * 8 + 8);
        L.arec_off = take((akeys + 1) * 4);
        L.arec_ent = take((size_t)p->nshot * p->nrec * 8 + 8);
    }
    if (grad) {
        // per-field slots start on 256-byte boundaries (TMA bases, short4/float4 access)
        L.ckpt_field_bytes = up256(ckpt_bytes(p->ckpt_format, (long long)p->nshot * g.cells));
        L.lap_field_bytes = up256((size_t)p->nshot * g.cells * (g.lap_bf16 ? 2 : 4));
        L.nlap = g.recon ? 0 : g.lvl16 ? g.K + 2 : g.ustore ? std::max(g.K + 2, p->nt - g.k0_store + 2) : g.K;
        if (g.lvl16) {
            L.nlvl = p->nt - g.k0_store;
            L.lvl_q_bytes = up256((size_t)p->nshot * g.cells * 2);
            L.lvl_bytes = L.lvl_q_bytes + up256((size_t)p->nshot * g.nz * bfp_eld(g.ld));
        }
        for (int b = 0; b < 2; ++b) L.Q[b] = take(L.field_bytes);  // (the adjoint is one-step)
        L.G = take((size_t)g.cells * 4);
        if (g.vd) {
            L.Gbx = take((size_t)g.cells * 4);
            L.Gbz = take((size_t)g.cells * 4);
        }
        // (segments whose levels the forward keeps need no checkpoint)
        L.ckpt = take(g.recon ? 0 : (size_t)(g.ustore ? g.jstore : g.nseg) * 2 * L.ckpt_field_bytes);
        if (g.recon) {
            L.frame_bytes = up256((size_t)band_cells(g.nz, g.ld, g.band_w, g.band_cl, g.band_cr) * p->nshot * 4);
            L.frames = take((size_t)(p->nt + 1) * L.frame_bytes);
        }
        L.lap = take(std::max((size_t)L.nlap * L.lap_field_bytes, (size_t)L.nlvl * L.lvl_bytes));
        L.res = take((size_t)p->nshot * p->nt * p->nrec * 4 + 4);
    }
    L.total = o;
    return L;
}

struct Work {
    unsigned* err;
    float *m, *P[4], *Q[4], *G, *res;
    float* S[2];  // int16 block scales of P[0], P[1] (reduced-precision fields)
    float *b, *Gbx, *Gbz;  // variable density (workspace)
    float* D;              // summed form: the increment d_n, [nshot][cells] (null: leapfrog)
    const float* rho;      // variable density: the caller's rho, for setup and the gradient
    float* grad_rho;       // variable density: dJ/drho output
    unsigned char* frames; // reconstruction adjoint: frame n at frames + n frame_bytes
    int* counts;
    PointLists src, rec, src_e;
    PointLists src_a, rec_a;  // lists of the adjoint geometry (== src, rec unless u store)
    unsigned char *ckpt, *lap;
    bool own_alists;          // src_a / rec_a are separate lists that setup() builds
    float* slot(const Layout& L, int i) const {  // u-store level slot i
        return reinterpret_cast<float*>(lap + (size_t)i * L.lap_field_bytes);
    }
    short* lvl_q(const Layout& L, int i) const {  // block-floating-point level i: mantissas
        return reinterpret_cast<short*>(lap + (size_t)i * L.lvl_bytes);
    }
    unsigned char* lvl_e(const Layout& L, int i) const {  // ... and exponents
        return lap + (size_t)i * L.lvl_bytes + L.lvl_q_bytes;
    }
};

Work carve(void* ws, const Layout& L, bool grad) {
    unsigned char* b = static_cast<unsigned char*>(ws);
    Work w{};
    w.err = reinterpret_cast<unsigned*>(b + L.err);
    w.m = reinterpret_cast<float*>(b + L.m);
    if (L.b) w.b = reinterpret_cast<float*>(b + L.b);
    if (L.Gbx) {
        w.Gbx = reinterpret_cast<float*>(b + L.Gbx);
        w.Gbz = reinterpret_cast<float*>(b + L.Gbz);
    }
    for (int k = 0; k < L.nbuf; ++k) w.P[k] = reinterpret_cast<float*>(b + L.P[k]);
    if (L.D) w.D = reinterpret_cast<float*>(b + L.D);
    if (L.S[0])
        for (int k = 0; k < 2; ++k) w.S[k] = reinterpret_cast<float*>(b + L.S[k]);
    w.counts = reinterpret_cast<int*>(b + L.counts);
    w.src.off = reinterpret_cast<int*>(b + L.src_off);
    w.src.ent = reinterpret_cast<int2*>(b + L.src_ent);
    w.rec.off = reinterpret_cast<int*>(b + L.rec_off);
    w.rec.ent = reinterpret_cast<int2*>(b + L.rec_ent);
    if (L.nbuf == 4) {
        w.src_e.off = reinterpret_cast<int*>(b + L.srce_off);
        w.src_e.ent = reinterpret_cast<int2*>(b + L.srce_ent);
    }
    w.src_a = w.src;
    w.rec_a = w.rec;
    if (L.asrc_off) {
        w.own_alists = true;
        w.src_a.off = reinterpret_cast<int*>(b + L.asrc_off);
        w.src_a.ent = reinterpret_cast<int2*>(b + L.asrc_ent);
        w.rec_a.off = reinterpret_cast<int*>(b + L.arec_off);
        w.rec_a.ent = reinterpret_cast<int2*>(b + L.arec_ent);
    }
    if (grad) {
        for (int k = 0; k < 2; ++k) w.Q[k] = reinterpret_cast<float*>(b + L.Q[k]);
        w.G = reinterpret_cast<float*>(b + L.G);
        w.ckpt = b + L.ckpt;
        if (L.frames) w.frames = b + L.frames;
        w.lap = b + L.lap;
        w.res = reinterpret_cast<float*>(b + L.res);
    }
    return w;
}

int check_workspace(void* ws, size_t bytes, size_t need) {
    if (!ws) return fail(WFD_ERR_WORKSPACE, "workspace is NULL");
    if (reinterpret_cast<uintptr_t>(ws) % 256)
        return fail(WFD_ERR_WORKSPACE, "workspace must be 256-byte aligned");
    if (bytes < need)
        return fail(WFD_ERR_WORKSPACE, "workspace of %zu bytes, %zu needed", bytes, need);
    return WFD_OK;
}

bool aligned16(const void* p) { return reinterpret_cast<uintptr_t>(p) % 16 == 0; }

// ------------------------------------------------------------------ stepping
struct Stepper {
    const wfd_problem* p;
    Geom g;
    cudaStream_t s;
    unsigned* err;
    const float* m;
    const float *gz, *gy, *gx;
    CUtensorMap map_m{};  // 3D: tiles of the model m; 2D two-step: m on the extended tile

    const float* bfield = nullptr;  // variable density: b = 1/rho

    int init() {
        if (g.vd) {  // b on the tile with R rows / 8 columns of halo (and one more row)
            EncodeTiled enc = encoder();
            if (!enc) return fail(WFD_ERR_CUDA, "cuTensorMapEncodeTiled entry point unavailable");
            const cuuint64_t dims[2] = {(cuuint64_t)g.nx, (cuuint64_t)g.nz};
            const cuuint64_t strides[1] = {(cuuint64_t)g.ld * 4};
            const cuuint32_t box[2] = {T2_TX + 16, cuuint32_t(16 + 2 * g.R + 1)}, estr[2] = {1, 1};
            CUresult r = enc(&map_m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(bfield), dims,
                             strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
            if (r != CUDA_SUCCESS) return fail(WFD_ERR_CUDA, "cuTensorMapEncodeTiled (b) failed (%d)", (int)r);
            return WFD_OK;
        }
        if (g.ndim == 2 && g.sb == 2) {
            EncodeTiled enc = encoder();
            if (!enc) return fail(WFD_ERR_CUDA, "cuTensorMapEncodeTiled entry point unavailable");
            const cuuint64_t dims[2] = {(cuuint64_t)g.nx, (cuuint64_t)g.nz};
            const cuuint64_t strides[1] = {(cuuint64_t)g.ld * 4};
            const cuuint32_t box[2] = {K2_EW, cuuint32_t(K2_TZ + 2 * g.R)}, estr[2] = {1, 1};
            CUresult r = enc(&map_m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(m), dims,
                             strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
            if (r != CUDA_SUCCESS) return fail(WFD_ERR_CUDA, "cuTensorMapEncodeTiled (m) failed (%d)", (int)r);
            return WFD_OK;
        }
        if (g.ndim != 3) return WFD_OK;
        EncodeTiled enc = encoder();
        if (!enc) return fail(WFD_ERR_CUDA, "cuTensorMapEncodeTiled entry point unavailable");
        const cuuint64_t dims[3] = {(cuuint64_t)g.nx, (cuuint64_t)g.ny, (cuuint64_t)g.nz};
        const cuuint64_t strides[2] = {(cuuint64_t)g.ld * 4, (cuuint64_t)g.plane * 4};
        const cuuint32_t box[3] = {T3_TX, T3_TY, 1}, estr[3] = {1, 1, 1};
        CUresult r = enc(&map_m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(m), dims,
                         strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return fail(WFD_ERR_CUDA, "cuTensorMapEncodeTiled (m) failed (%d)", (int)r);
        return WFD_OK;
    }

    StepArgs base(float* u_new) const {
        StepArgs a{};
        a.u_new = u_new;
        a.m = m;
        a.m_const = 0.f;
        a.gz = gz;
        a.gy = gy;
        a.gx = gx;
        a.nz = g.nz; a.ny = g.ny; a.nx = g.nx; a.ld = g.ld;
        a.plane = g.plane;
        a.shot_stride = g.cells;
        a.nshot = p->nshot;
        a.shots_per_cta = g.spc;
        a.tiles_x = g.tiles_x; a.tiles_y = g.tiles_y; a.tiles_z = g.tiles_z;
        a.c0 = g.c0;
        for (int k = 0; k < 4; ++k) { a.cz[k] = g.cz[k]; a.cy[k] = g.cy[k]; a.cx[k] = g.cx[k]; }
        a.zero_ring = 1;  // the wave path's ring is 0 in every level
        if (g.vd) {
            for (int k = 0; k < 4; ++k) a.cs[k] = g.cs[k];
            a.vd_sz = g.vd_sz;
        }
        a.err = err;
        return a;
    }

    int map_pair(const float* cur, const float* old, CUtensorMap* mc, CUtensorMap* mo) const {
        int rc;
        if (g.vd) {  // the field with 2R rows / 8 columns of halo
            const cuuint32_t bc[3] = {T2_TX + 16, cuuint32_t(16 + 4 * g.R), 1};
            const cuuint32_t bo[3] = {T2_TX, 16, 1};
            if ((rc = make_field_map(mc, cur, false, 2, g.nz, 1, g.nx, g.ld, p->nshot, bc))) return rc;
            return make_field_map(mo, old, false, 2, g.nz, 1, g.nx, g.ld, p->nshot, bo);
        }
        if (g.ndim == 2) {
            const cuuint32_t bc[3] = {T2_W, cuuint32_t(g.tile_z + 2 * g.R), 1};
            const cuuint32_t bo[3] = {T2_TX, cuuint32_t(g.tile_z), 1};
            if ((rc = make_field_map(mc, cur, false, 2, g.nz, 1, g.nx, g.ld, p->nshot, bc))) return rc;
            return make_field_map(mo, old, false, 2, g.nz, 1, g.nx, g.ld, p->nshot, bo);
        }
        const cuuint32_t bc[4] = {T3_W, cuuint32_t(T3_TY + 2 * g.R), 1, 1};
        const cuuint32_t bo[4] = {T3_TX, T3_TY, 1, 1};
        if ((rc = make_field_map(mc, cur, false, 3, g.nz, g.ny, g.nx, g.ld, p->nshot, bc))) return rc;
        return make_field_map(mo, old, false, 3, g.nz, g.ny, g.nx, g.ld, p->nshot, bo);
    }

    int lap_map(const void* lap, bool bf16, CUtensorMap* ml) const {
        if (g.ndim == 2) {
            const cuuint32_t b[3] = {T2_TX, cuuint32_t(g.tile_z), 1};
            return make_field_map(ml, lap, bf16, 2, g.nz, 1, g.nx, g.ld, p->nshot, b);
        }
        const cuuint32_t b[4] = {T3_TX, T3_TY, 1, 1};
        return make_field_map(ml, lap, bf16, 3, g.nz, g.ny, g.nx, g.ld, p->nshot, b);
    }

    // two-step kernel: u_n box (2R rows / 8 columns of halo) and u_{n-1} box (R / 4)
    int map_k2(const float* buf, CUtensorMap* mu, CUtensorMap* mo) const {
        const cuuint32_t bu[3] = {K2_UW, cuuint32_t(K2_TZ + 4 * g.R), 1};
        const cuuint32_t bo[3] = {K2_EW, cuuint32_t(K2_TZ + 2 * g.R), 1};
        int rc;
        if ((rc = make_field_map(mu, buf, false, 2, g.nz, 1, g.nx, g.ld, p->nshot, bu))) return rc;
        return make_field_map(mo, buf, false, 2, g.nz, 1, g.nx, g.ld, p->nshot, bo);
    }

    int launch_k2(const CUtensorMap& mu, const CUtensorMap& mo, const Step2Args& q) const {
        cudaError_t e = launch_step2d_k2(g.R, mu, mo, map_m, q, s);
        if (e != cudaSuccess) return fail(WFD_ERR_CUDA, "two-step launch failed: %s", cudaGetErrorString(e));
        return WFD_OK;
    }

    int launch(int mode, const CUtensorMap& mc, const CUtensorMap& mo, const CUtensorMap& ml,
               const StepArgs& a, const CUtensorMap* mx = nullptr) const {
        cudaError_t e = g.vd           ? launch_step2d_vd(g.R, mode, mc, mo, ml, map_m, a, s)
                        : g.ndim == 2 ? launch_step2d(g.R, mode, g.tile_z, mc, mo, ml, a, s, mx)
                                      : launch_step3d(g.R, mode, mc, mo, ml, map_m, a, s);
        if (e != cudaSuccess) return fail(WFD_ERR_CUDA, "step launch failed: %s", cudaGetErrorString(e));
        return WFD_OK;
    }
};

int common_checks(const wfd_problem* p, const float* vel, const float* wavelet, const int32_t* src,
                  const int32_t* rec) {
    int rc = check_problem(p);
    if (rc) return rc;
    if (!vel) return fail(WFD_ERR_INVALID, "vel is NULL");
    if (p->nsrc > 0 && (!wavelet || !src)) return fail(WFD_ERR_INVALID, "wavelet/src is NULL");
    if (p->nrec > 0 && !rec) return fail(WFD_ERR_INVALID, "rec is NULL");
    return WFD_OK;
}

// Shots per sequential group (all of them when group_shots is 0 or >= nshot).
int group_size(const wfd_problem* p) {
    return (p->group_shots > 0 && p->group_shots < p->nshot) ? p->group_shots : p->nshot;
}

// The problem restricted to shots [g0, g0 + count).
wfd_problem group_problem(const wfd_problem* p, int g0) {
    wfd_problem q = *p;
    q.nshot = std::min(group_size(p), p->nshot - g0);
    q.group_shots = 0;
    return q;
}

int setup(const wfd_problem* p, const Geom& g, const Work& w, const float* vel,
          const int32_t* src, const int32_t* rec, cudaStream_t s, bool clear_status = true) {
    if (clear_status) WFD_CUDA(cudaMemsetAsync(w.err, 0, sizeof(unsigned), s));  // fresh status word
    if (g.vd)  // vel is kappa: k = kappa dt^2 / dx^2, b = 1 / rho
        WFD_CUDA(launch_vd_params(vel, w.rho, w.m, w.b, g.nz, g.nx, g.ld,
                                  float((double)p->dt * p->dt / ((double)p->dx * p->dx)), s));
    else
        WFD_CUDA(launch_vel_to_m(vel, w.m, g.nz, g.ny, g.nx, g.ld, p->dt / p->dx, s));
    WFD_CUDA(launch_build_lists(src, p->nshot, p->nsrc, g.nz, g.ny, g.nx, g.ld, g.R, g.tile_z,
                                g.tile_y, g.tile_x, g.tiles_z, g.tiles_y, g.tiles_x, w.counts,
                                const_cast<int*>(w.src.off), const_cast<int2*>(w.src.ent), w.err, s));
    WFD_CUDA(launch_build_lists(rec, p->nshot, p->nrec, g.nz, g.ny, g.nx, g.ld, g.R, g.tile_z,
                                g.tile_y, g.tile_x, g.tiles_z, g.tiles_y, g.tiles_x, w.counts,
                                const_cast<int*>(w.rec.off), const_cast<int2*>(w.rec.ent), w.err, s));
    if (g.sb >= 2) {  // points inside each tile's extended region (R rows, 4 columns) or window
        const int hz = g.sb == 2 ? g.R : WR_HALO, hx = g.sb == 2 ? 4 : WR_HALO;
        WFD_CUDA(launch_build_lists(src, p->nshot, p->nsrc, g.nz, g.ny, g.nx, g.ld, g.R, g.tile_z,
                                    g.tile_y, g.tile_x, g.tiles_z, g.tiles_y, g.tiles_x, w.counts,
                                    const_cast<int*>(w.src_e.off), const_cast<int2*>(w.src_e.ent),
                                    w.err, s, hz, hx));
    }
    if (w.own_alists) {  // the u-store adjoint's 16-row tiles
        const Geom a = adjoint_geom(p, g);
        WFD_CUDA(launch_build_lists(src, p->nshot, p->nsrc, a.nz, a.ny, a.nx, a.ld, a.R, a.tile_z,
                                    a.tile_y, a.tile_x, a.tiles_z, a.tiles_y, a.tiles_x, w.counts,
                                    const_cast<int*>(w.src_a.off), const_cast<int2*>(w.src_a.ent),
                                    w.err, s));
        WFD_CUDA(launch_build_lists(rec, p->nshot, p->nrec, a.nz, a.ny, a.nx, a.ld, a.R, a.tile_z,
                                    a.tile_y, a.tile_x, a.tiles_z, a.tiles_y, a.tiles_x, w.counts,
                                    const_cast<int*>(w.rec_a.off), const_cast<int2*>(w.rec_a.ent),
                                    w.err, s));
    }
    return WFD_OK;
}


// Forward time loop. With save: checkpoints every K steps and, for the
// adjoint's imaging term, either the kept levels (u store) or the L u store
// of the last segment (which the backward then does not recompute).
// final_buf (optional) receives the index of the buffer P[] that holds u_nt.
//
// Level u_k lives in P[k % nP]: nP = 2 with one step per launch (u_{k+1}
// overwrites u_{k-1} in place), nP = 4 with two (a launch reads u_{k-1}, u_k
// and writes u_{k+1}, u_{k+2}, none of which alias). With the u store the
// levels of the kept segments, from u_{k0_store - 1} on, go to the store's
// slots k - k0_store + 1 for the adjoint to read instead.
int run_forward_lp(const wfd_problem* p, const Geom& g, const Layout& L, const Work& w,
                   const Stepper& st, const float* wavelet, float* traces, int* final_buf);

// Forward of K = WR_HALO / R steps per launch (step_block 8 at order 2, 4 at
// order 4; leapfrog, no checkpoints): the levels (u_{n-1}, u_n) in one pair of
// buffers, P[2i] and P[2i + 1]; a launch of k steps writes (u_{n+k-1}, u_{n+k})
// to the other pair. The kernel samples the receivers after every step.
int run_forward_reg(const wfd_problem* p, const Geom& g, const Layout& L, const Work& w, const Stepper& st,
                    const float* wavelet, float* traces, int* final_buf) {
    cudaStream_t s = st.s;
    for (int b = 0; b < 4; ++b) WFD_CUDA(cudaMemsetAsync(w.P[b], 0, L.field_bytes, s));
    const int K = WR_HALO / g.R;
    int pair = 0;
    PhaseScope scope(PH_FORWARD, s, (p->nt + K - 1) / K);
    for (int n = 0; n < p->nt; n += K) {
        StepArgs a = st.base(nullptr);
        a.inj_val = wavelet;
        a.inj_np = p->nsrc; a.inj_nt = p->nt;
        a.inj_scale = p->src_scale;
        if (traces && p->nrec > 0) {
            a.smp = w.rec;
            a.smp_out = traces;
            a.smp_np = p->nrec; a.smp_nt = p->nt;
            a.smp_scale = 1.f;
        }
        RegArgs q{};
        q.u0 = w.P[2 * pair];
        q.u1 = w.P[2 * pair + 1];
        q.v0 = w.P[2 * (pair ^ 1)];
        q.v1 = w.P[2 * (pair ^ 1) + 1];
        if (p->nsrc > 0) q.src = w.src_e;
        q.n0 = n;
        q.ksteps = std::min(K, p->nt - n);
        const cudaError_t e = launch_wave_reg(g.R, a, q, s);
        if (e != cudaSuccess) return fail(WFD_ERR_CUDA, "multi-step launch failed: %s", cudaGetErrorString(e));
        pair ^= 1;
    }
    if (final_buf) *final_buf = 2 * pair + 1;
    return WFD_OK;
}

int run_forward(const wfd_problem* p, const Geom& g, const Layout& L, const Work& w,
                const Stepper& st, const float* wavelet, float* traces, bool save,
                int* final_buf = nullptr) {
    if (g.sb >= 4) {
        if (save) return fail(WFD_ERR_INVALID, "step_block %d is a forward-only mode", g.sb);
        return run_forward_reg(p, g, L, w, st, wavelet, traces, final_buf);
    }
    if (p->field_format != WFD_FIELD_FP32) {
        if (save) return fail(WFD_ERR_INVALID, "reduced-precision fields are a forward-only mode");
        return run_forward_lp(p, g, L, w, st, wavelet, traces, final_buf);
    }
    cudaStream_t s = st.s;
    const bool rc_mode = save && g.recon;  // reconstruction adjoint: frames, no checkpoints or slots
    const bool us = save && g.ustore && !rc_mode;
    // kept levels as block-floating-point copies beside the FP32 state (which then
    // stays in P), or as FP32 slots that the state itself runs through
    const bool keep16 = us && g.lvl16;
    const bool uslots = us && !g.lvl16;
    const int np = L.nbuf;
    const int nslot = uslots ? L.nlap : 0;
    auto loc = [&](int k) -> int {
        return uslots && k >= g.k0_store - 1 ? np + (k - g.k0_store + 1) : ((k % np) + np) % np;
    };
    auto kept16 = [&](int k) { return keep16 && k >= g.k0_store && k < p->nt; };
    std::vector<float*> buf(np + nslot);
    for (int b = 0; b < np; ++b) buf[b] = w.P[b];
    for (int i = 0; i < nslot; ++i) buf[np + i] = w.slot(L, i);
    if (final_buf) {
        if (us) return fail(WFD_ERR_INVALID, "internal: final level requested from a u-store forward");
        *final_buf = loc(p->nt);
    }
    // summed form: the state is (u_n, d_n); u_{n+1} still goes over u_{n-1}
    // (or to a slot), d_{n+1} over d_n
    const bool summed = summed_forward(p, g, save);
    if (summed && !w.D) return fail(WFD_ERR_INVALID, "internal: summed forward without its increment field");
    WFD_CUDA(cudaMemsetAsync(buf[loc(-1)], 0, L.field_bytes, s));
    WFD_CUDA(cudaMemsetAsync(buf[loc(0)], 0, L.field_bytes, s));
    // increment buffers: one step per launch D[0] (in place); two steps per
    // launch d_n in D[(n / 2) % 2], d_{n+2} in the other, d_{n+1} in D[2]
    float* D[3] = {w.D, nullptr, nullptr};
    if (summed && g.sb == 2)
        for (int k = 1; k < 3; ++k) D[k] = w.D + (size_t)k * (L.field_bytes / sizeof(float));
    if (summed) WFD_CUDA(cudaMemsetAsync(w.D, 0, L.field_bytes, s));  // d_0 = 0
    if (kept16(0)) WFD_CUDA(cudaMemsetAsync(w.lvl_q(L, 0), 0, L.lvl_bytes, s));  // u_0 = 0
    std::vector<CUtensorMap> mc(buf.size()), mo(buf.size());
    int rc;
    for (size_t b = 0; b < buf.size(); ++b)
        if ((rc = g.sb == 2 ? st.map_k2(buf[b], &mc[b], &mo[b]) : st.map_pair(buf[b], buf[b], &mc[b], &mo[b])))
            return rc;
    CUtensorMap mdc{}, mdo{};  // d_n as the staged "old" tile
    CUtensorMap mdu[2]{}, mde[2]{};  // two steps per launch: d_n on the extended region, per buffer
    if (summed && g.sb == 1 && (rc = st.map_pair(w.D, w.D, &mdc, &mdo))) return rc;
    if (summed && g.sb == 2)
        for (int k = 0; k < 2; ++k)
            if ((rc = st.map_k2(D[k], &mdu[k], &mde[k]))) return rc;
    const long long n_all = (long long)p->nshot * g.cells;
    // whether level k gets a checkpoint (the start of a segment the adjoint recomputes)
    auto ckpt_at = [&](int k) { return save && !rc_mode && k % g.K == 0 && !(us && k >= g.k0_store); };
    // (u_{n-1}, u_n) at the start of segment n / K; (d_n, u_n) in the summed form
    // (two steps per launch: d_n in dsrc)
    auto checkpoint = [&](int n, const float* dsrc) -> int {
        if (!ckpt_at(n)) return WFD_OK;  // (kept segments need none)
        unsigned char* slot = w.ckpt + (size_t)(n / g.K) * 2 * L.ckpt_field_bytes;
        WFD_CUDA(launch_pack(summed ? dsrc : buf[loc(n - 1)], slot, n_all, p->ckpt_format, s));
        WFD_CUDA(launch_pack(buf[loc(n)], slot + L.ckpt_field_bytes, n_all, p->ckpt_format, s));
        return WFD_OK;
    };
    PhaseScope scope(PH_FORWARD, s, g.sb == 2 ? (p->nt + 1) / 2 : p->nt);
    for (int n = 0; n < p->nt;) {
        if (g.sb == 2) {
            // u_{n+1} and u_{n+2} from (u_{n-1}, u_n); no buffer the launch reads is written
            const bool two = n + 1 < p->nt;
            Step2Args q{};
            q.a = st.base(buf[loc(two ? n + 2 : n + 1)]);
            q.u_mid = buf[loc(n + 1)];
            q.two_steps = two;
            q.inj_t1 = -1;
            q.a.inj_t = -1;
            if (p->nsrc > 0) {
                q.inj_e = w.src_e;
                q.inj_t1 = n;
                q.a.inj = w.src;
                q.a.inj_val = wavelet;
                q.a.inj_np = p->nsrc; q.a.inj_nt = p->nt; q.a.inj_t = two ? n + 1 : -1;
                q.a.inj_scale = p->src_scale;
            }
            q.smp_t1 = -1;
            q.a.smp_t = -1;
            if (traces && p->nrec > 0) {
                q.a.smp = w.rec;
                q.a.smp_out = traces;
                q.a.smp_np = p->nrec; q.a.smp_nt = p->nt;
                q.a.smp_scale = 1.f;
                q.smp_t1 = n - 1;
                q.a.smp_t = two ? n : -1;
            }
            if (summed) {
                // (u_n, d_n) -> (u_{n+2}, d_{n+2}); the intermediate level leaves the
                // CTAs only where a checkpoint or a kept level needs it
                const int din = (n / 2) & 1;
                q.summed = 1;
                q.d_out = D[din ^ 1];
                q.d_mid = two ? D[2] : D[din ^ 1];
                q.write_mid = !two || ckpt_at(n + 1) || (uslots && n + 1 >= g.k0_store - 1);
                q.eld = bfp_eld(g.ld);
                if (kept16(n + 1)) {
                    q.lq_mid = w.lvl_q(L, n + 1 - g.k0_store);
                    q.le_mid = w.lvl_e(L, n + 1 - g.k0_store);
                }
                if (two && kept16(n + 2)) {
                    q.lq_out = w.lvl_q(L, n + 2 - g.k0_store);
                    q.le_out = w.lvl_e(L, n + 2 - g.k0_store);
                }
                if ((rc = st.launch_k2(mc[loc(n)], mde[din], q))) return rc;
                if ((rc = checkpoint(n, D[din]))) return rc;
                if (two && (rc = checkpoint(n + 1, D[2]))) return rc;
                n += two ? 2 : 1;
                continue;
            }
            if ((rc = st.launch_k2(mc[loc(n)], mo[loc(n - 1)], q))) return rc;
            for (int k = n; k < n + (two ? 2 : 1); ++k)  // (every level read there is still held)
                if ((rc = checkpoint(k, nullptr))) return rc;
            n += two ? 2 : 1;
            continue;
        }
        if ((rc = checkpoint(n, w.D))) return rc;
        const int bo = loc(n - 1), bc = loc(n), bn = loc(n + 1);
        // (the summed forward stores no L u: the backward recomputes every segment)
        const bool lap = save && !g.ustore && !summed && n >= g.k0_last;
        StepArgs a = st.base(buf[bn]);
        a.inj = w.src;
        a.inj_val = wavelet;
        a.inj_np = p->nsrc; a.inj_nt = p->nt; a.inj_t = n;
        a.inj_scale = p->src_scale;
        if (p->nsrc == 0) a.inj.off = nullptr;
        if (traces && n >= 1 && p->nrec > 0) {
            a.smp = w.rec;
            a.smp_out = traces;
            a.smp_np = p->nrec; a.smp_nt = p->nt; a.smp_t = n - 1;
            a.smp_scale = 1.f;
        }
        if (lap) {
            a.lap = w.lap + (size_t)(n - g.k0_last) * L.lap_field_bytes;
            a.lap_bf16 = g.lap_bf16;
        }
        if (summed) {
            a.d_new = w.D;
            if ((rc = st.launch(MODE_SUMMED, mc[bc], mdo, mc[bc], a))) return rc;
        } else if ((rc = st.launch(lap ? MODE_SAVE_LAP : MODE_PLAIN, mc[bc], mo[bo], mc[bc], a))) {
            return rc;
        }
        if (rc_mode)  // the damped frame of u_{n+1} (sources included: after the launch)
            WFD_CUDA(launch_band(buf[bn], reinterpret_cast<float*>(w.frames + (size_t)(n + 1) * L.frame_bytes),
                                 g.cells, p->nshot, g.nz, g.ld, g.band_w, g.band_cl, g.band_cr, true, s));
        ++n;
    }
    if (traces && p->nrec > 0)
        WFD_CUDA(launch_gather(buf[loc(p->nt)], g.cells, w.rec, g.ntiles, p->nshot, p->nrec, nullptr,
                               1.f, 0, traces, p->nt, p->nt - 1, s));
    return WFD_OK;
}

// Forward with reduced-precision fields (FP16 or block-scaled int16): u_{n+1}
// over u_{n-1} in two buffers, the sources added and the receivers sampled in
// the step kernel (traces[n] = the stored u_{n+1}).
int run_forward_lp(const wfd_problem* p, const Geom& g, const Layout& L, const Work& w,
                   const Stepper& st, const float* wavelet, float* traces, int* final_buf) {
    cudaStream_t s = st.s;
    if (final_buf) *final_buf = p->nt & 1;
    const bool i16 = p->field_format == WFD_FIELD_I16;
    for (int b = 0; b < 2; ++b) {
        WFD_CUDA(cudaMemsetAsync(w.P[b], 0, L.field_bytes, s));
        if (i16) WFD_CUDA(cudaMemsetAsync(w.S[b], 0, L.scale_bytes, s));
    }
    const int nblk = scale_blocks(g.ld);
    CUtensorMap mcur[2], mold[2], mcs[2]{}, mos[2]{};
    // (int16 cells travel as 16-bit patterns: the copy does not look at them)
    const CUtensorMapDataType dt = i16 ? CU_TENSOR_MAP_DATA_TYPE_UINT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
    const cuuint64_t fdims[3] = {(cuuint64_t)g.nx, (cuuint64_t)g.nz, (cuuint64_t)p->nshot};
    const cuuint64_t fstr[2] = {(cuuint64_t)g.ld * 2, (cuuint64_t)g.nz * g.ld * 2};
    const cuuint64_t sdims[3] = {(cuuint64_t)nblk, (cuuint64_t)g.nz, (cuuint64_t)p->nshot};
    const cuuint64_t sstr[2] = {(cuuint64_t)nblk * 4, (cuuint64_t)g.nz * nblk * 4};
    const cuuint32_t bcur[3] = {144, cuuint32_t(32 + 2 * g.R), 1}, bold[3] = {128, 32, 1};
    const cuuint32_t bcs[3] = {12, cuuint32_t(32 + 2 * g.R), 1}, bos[3] = {4, 32, 1};
    int rc;
    for (int b = 0; b < 2; ++b) {
        if ((rc = make_map3(&mcur[b], w.P[b], dt, fdims, fstr, bcur))) return rc;
        if ((rc = make_map3(&mold[b], w.P[b], dt, fdims, fstr, bold))) return rc;
        if (i16) {
            if ((rc = make_map3(&mcs[b], w.S[b], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, sdims, sstr, bcs))) return rc;
            if ((rc = make_map3(&mos[b], w.S[b], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, sdims, sstr, bos))) return rc;
        }
    }
    PhaseScope scope(PH_FORWARD, s, p->nt);
    for (int n = 0; n < p->nt; ++n) {
        const int bc = n & 1, bn = (n + 1) & 1;
        LpArgs q{};
        q.a = st.base(nullptr);
        q.a.inj = w.src;
        q.a.inj_val = wavelet;
        q.a.inj_np = p->nsrc; q.a.inj_nt = p->nt; q.a.inj_t = n;
        q.a.inj_scale = p->src_scale;
        if (p->nsrc == 0) q.a.inj.off = nullptr;
        if (traces && p->nrec > 0) {
            q.a.smp = w.rec;
            q.a.smp_out = traces;
            q.a.smp_np = p->nrec; q.a.smp_nt = p->nt; q.a.smp_t = n;
            q.a.smp_scale = 1.f;
        }
        q.cur = w.P[bc];
        q.old = w.P[bn];
        q.nw = w.P[bn];
        if (i16) {
            q.scur = w.S[bc];
            q.sold = w.S[bn];
            q.snw = w.S[bn];
        }
        q.nblk = nblk;
        q.sstride = (long long)g.nz * nblk;
        cudaError_t e = launch_step2d_lp(g.R, p->field_format, mcur[bc], mold[bn], mcs[bc], mos[bn], q, s);
        if (e != cudaSuccess) return fail(WFD_ERR_CUDA, "reduced-precision step failed: %s", cudaGetErrorString(e));
    }
    return WFD_OK;
}

// A second stream and a pool of events per (device, primary stream), for the
// recompute that overlaps the adjoint (run_backward_ustore). They are created
// only outside a stream capture (a capture uses the ones an earlier eager call
// made), for at most AUX_MAX primary streams per process (they live as long as
// it does); without them the backward runs on the primary stream alone.
struct AuxStream {
    cudaStream_t r = nullptr;
    std::vector<cudaEvent_t> ev;
};
constexpr size_t AUX_MAX = 64;
std::mutex g_aux_mu;
std::map<std::pair<int, cudaStream_t>, AuxStream> g_aux;

const AuxStream* aux_stream(cudaStream_t s, size_t nev) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    std::lock_guard<std::mutex> lock(g_aux_mu);
    const std::pair<int, cudaStream_t> key{dev, s};
    if (g_aux.find(key) == g_aux.end() && g_aux.size() >= AUX_MAX) return nullptr;
    AuxStream& a = g_aux[key];
    if (a.r && a.ev.size() >= nev) return &a;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return nullptr;
    if (!a.r && cudaStreamCreateWithFlags(&a.r, cudaStreamNonBlocking) != cudaSuccess) {
        a.r = nullptr;
        return nullptr;
    }
    while (a.ev.size() < nev) {
        cudaEvent_t e;
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return nullptr;
        a.ev.push_back(e);
    }
    return &a;
}

// Adjoint with the u store (2D, one step per launch). The forward left the
// levels of segments >= jstore in the slots (u_k in slot k - k0_store + 1).
// Every earlier segment j restores (u_{k0-1}, u_k0) into slots 0 and 1 and
// recomputes u_{k0+1} .. u_{k1-1} into slots 2 .. k1 - k0 (each step writes a
// new slot: nothing else is stored). The adjoint step k stages u_k from its
// slot next to q_{k+1} and forms L u_k itself (MODE_GRAD_U) on 16-row tiles;
// the recompute runs on the forward's tiles.
//
// With two or more recomputed segments and room for two sets of K + 2 slots
// in the region the kept levels leave free, the recompute of segment j - 1
// runs on a second stream while the adjoint of segment j runs: recomputed
// segments alternate between slot sets [K + 2, 2K + 4) and [0, K + 2), the
// recompute of segment j waits for the adjoint of segment j + 2 (the last
// reader of its set: a kept segment or the recomputed one before), and the
// adjoint of segment j for its recompute. The recompute is latency-bound and
// the adjoint DRAM-bound, so together they fill the memory system better.
int run_backward_ustore(const wfd_problem* p, const Geom& g, const Layout& L, const Work& w,
                        const Stepper& st, const float* wavelet, const float* dtraces,
                        float* grad_vel, float* grad_wavelet, const float* vel, bool zero_G,
                        bool finalize) {
    cudaStream_t s = st.s;
    const Geom ga = adjoint_geom(p, g);
    Stepper sa = st;
    sa.g = ga;
    const bool summed = summed_forward(p, g, true);  // the checkpoints hold (d_k0, u_k0)
    WFD_CUDA(cudaMemsetAsync(w.Q[0], 0, L.field_bytes, s));
    WFD_CUDA(cudaMemsetAsync(w.Q[1], 0, L.field_bytes, s));
    if (zero_G) {
        WFD_CUDA(cudaMemsetAsync(w.G, 0, (size_t)g.cells * 4, s));
        if (g.vd) {
            WFD_CUDA(cudaMemsetAsync(w.Gbx, 0, (size_t)g.cells * 4, s));
            WFD_CUDA(cudaMemsetAsync(w.Gbz, 0, (size_t)g.cells * 4, s));
        }
    }
    int rc;
    CUtensorMap qc[2], qo[2];
    for (int b = 0; b < 2; ++b)
        if ((rc = sa.map_pair(w.Q[b], w.Q[b], &qc[b], &qo[b]))) return rc;
    // per slot: u_k as the recompute's u_n / u_{n-1} tiles and as the adjoint's staged u_k
    std::vector<CUtensorMap> uc(L.nlap), uo(L.nlap), ua(L.nlap), unused(L.nlap);
    for (int i = 0; i < L.nlap; ++i) {
        if ((rc = g.sb == 2 ? st.map_k2(w.slot(L, i), &uc[i], &uo[i])
                            : st.map_pair(w.slot(L, i), w.slot(L, i), &uc[i], &uo[i])))
            return rc;
        if ((rc = sa.map_pair(w.slot(L, i), w.slot(L, i), &ua[i], &unused[i]))) return rc;
    }
    // block-floating-point kept levels: mantissa and exponent tiles of the adjoint's
    // 16-row tiles (boxes at x0 - 8 and, in exponent bytes, x0/4 - 16)
    std::vector<CUtensorMap> lq(L.nlvl), le(L.nlvl);
    if (g.lvl16) {
        const int eld = bfp_eld(g.ld);
        const cuuint64_t qd[3] = {(cuuint64_t)g.nx, (cuuint64_t)g.nz, (cuuint64_t)p->nshot};
        const cuuint64_t qs[2] = {(cuuint64_t)g.ld * 2, (cuuint64_t)g.nz * g.ld * 2};
        const cuuint64_t ed[3] = {(cuuint64_t)(g.ld / 4), (cuuint64_t)g.nz, (cuuint64_t)p->nshot};
        const cuuint64_t es[2] = {(cuuint64_t)eld, (cuuint64_t)g.nz * eld};
        const cuuint32_t qb[3] = {T2_TX + 16, cuuint32_t(ga.tile_z + 2 * g.R), 1};
        const cuuint32_t eb[3] = {64, cuuint32_t(ga.tile_z + 2 * g.R), 1};
        for (int i = 0; i < L.nlvl; ++i) {
            if ((rc = make_map3(&lq[i], w.lvl_q(L, i), CU_TENSOR_MAP_DATA_TYPE_UINT16, qd, qs, qb))) return rc;
            if ((rc = make_map3(&le[i], w.lvl_e(L, i), CU_TENSOR_MAP_DATA_TYPE_UINT8, ed, es, eb))) return rc;
        }
    }
    const long long n_all = (long long)p->nshot * g.cells;

    // q_k from (q_{k+1}, q_{k+2}); with the gradient term q_{k+1} L u_k, u_k in slot
    // `slot` (FP32), or in block-floating-point level `slot` when lvl is set
    auto adjoint_step = [&](int k, int slot, bool lvl = false) -> int {
        const int bc = (k + 1) & 1, bn = k & 1;
        StepArgs a = sa.base(w.Q[bn]);
        if (p->nrec > 0) {
            a.inj = w.rec_a;
            a.inj_val = dtraces;
            a.inj_np = p->nrec; a.inj_nt = p->nt; a.inj_t = k - 1;
            a.inj_scale = 1.f;
            a.inj_times_m = 1;
        }
        if (grad_wavelet && k <= p->nt - 1 && p->nsrc > 0) {
            a.smp = w.src_a;
            a.smp_out = grad_wavelet;
            a.smp_np = p->nsrc; a.smp_nt = p->nt; a.smp_t = k;
            a.smp_scale = p->src_scale;
            a.smp_div_m = 1;
        }
        if (slot < 0) return sa.launch(MODE_PLAIN, qc[bc], qo[bn], qc[bc], a);
        a.grad = w.G;
        a.grad_bx = w.Gbx;
        a.grad_bz = w.Gbz;
        if (lvl) return sa.launch(MODE_GRAD_U16, qc[bc], qo[bn], lq[slot], a, &le[slot]);
        return sa.launch(MODE_GRAD_U, qc[bc], qo[bn], ua[slot], a);
    };

    {
        PhaseScope scope(PH_ADJOINT, s, 1);
        if ((rc = adjoint_step(p->nt, -1))) return rc;  // q_nt: its gradient term is 0
    }
    // the recompute on a second stream (see above), or on s
    const AuxStream* aux = (g.jstore >= 2 && L.nlap >= 2 * (g.K + 2)) ? aux_stream(s, 2 * (size_t)g.nseg + 1)
                                                                       : nullptr;
    const cudaStream_t r = aux ? aux->r : s;
    Stepper sr = st;
    sr.s = r;
    auto ev_adj = [&](int j) { return aux->ev[1 + j]; };
    auto ev_rec = [&](int j) { return aux->ev[1 + g.nseg + j]; };
    auto set_base = [&](int j) { return aux && ((g.jstore - 1 - j) % 2 == 0) ? g.K + 2 : 0; };
    if (aux) {  // (the second stream joins here: everything it reads is ready)
        WFD_CUDA(cudaEventRecord(aux->ev[0], s));
        WFD_CUDA(cudaStreamWaitEvent(r, aux->ev[0], 0));
    }
    // u_k0 .. u_{k1-1} of recomputed segment j into slots sb .. sb + k1 - k0 on stream r
    auto recompute = [&](int j) -> int {
        const int k0 = j * g.K, k1 = std::min(p->nt, k0 + g.K), sb = set_base(j);
        if (aux && j + 2 < g.nseg) WFD_CUDA(cudaStreamWaitEvent(r, ev_adj(j + 2), 0));
        PhaseScope scope(PH_RECOMPUTE, r, g.sb == 2 ? (k1 - k0) / 2 : k1 - k0 - 1);
        const unsigned char* ck = w.ckpt + (size_t)j * 2 * L.ckpt_field_bytes;
        WFD_CUDA(launch_unpack(ck + L.ckpt_field_bytes, w.slot(L, sb + 1), n_all, p->ckpt_format, r));
        if (summed)  // (d_k0, u_k0): u_{k0-1} = u_k0 - d_k0 for the leapfrog recompute
            WFD_CUDA(launch_unpack_diff(ck, w.slot(L, sb + 1), w.slot(L, sb), n_all, p->ckpt_format, r));
        else
            WFD_CUDA(launch_unpack(ck, w.slot(L, sb), n_all, p->ckpt_format, r));
        for (int k = k0; k + 1 < k1;) {  // u_{k+1} (and u_{k+2}) up to u_{k1-1}
            const int i = sb + k - k0 + 1;  // slot of u_k
            const bool two = g.sb == 2 && k + 2 < k1;
            if (g.sb == 2) {
                Step2Args q{};
                q.a = sr.base(w.slot(L, i + (two ? 2 : 1)));
                q.u_mid = w.slot(L, i + 1);
                q.two_steps = two;
                q.inj_t1 = -1;
                q.a.inj_t = -1;
                q.smp_t1 = -1;
                q.a.smp_t = -1;
                if (p->nsrc > 0) {
                    q.inj_e = w.src_e;
                    q.inj_t1 = k;
                    q.a.inj = w.src;
                    q.a.inj_val = wavelet;
                    q.a.inj_np = p->nsrc; q.a.inj_nt = p->nt; q.a.inj_t = two ? k + 1 : -1;
                    q.a.inj_scale = p->src_scale;
                }
                if ((rc = sr.launch_k2(uc[i], uo[i - 1], q))) return rc;
            } else {
                StepArgs a = sr.base(w.slot(L, i + 1));
                if (p->nsrc > 0) {
                    a.inj = w.src;
                    a.inj_val = wavelet;
                    a.inj_np = p->nsrc; a.inj_nt = p->nt; a.inj_t = k;
                    a.inj_scale = p->src_scale;
                }
                if ((rc = sr.launch(MODE_PLAIN, uc[i], uo[i - 1], uc[i], a))) return rc;
            }
            k += two ? 2 : 1;
        }
        if (aux) WFD_CUDA(cudaEventRecord(ev_rec(j), r));
        return WFD_OK;
    };
    for (int j = g.nseg - 1; j >= 0; --j) {
        const int k0 = j * g.K, k1 = std::min(p->nt, k0 + g.K);
        if (j < g.jstore) {
            if (!aux) {
                if ((rc = recompute(j))) return rc;
            } else {  // (issued with the segment after it, on r)
                WFD_CUDA(cudaStreamWaitEvent(s, ev_rec(j), 0));
            }
        }
        // the next segment's recompute, on r beside this adjoint
        if (aux && j - 1 >= 0 && j - 1 < g.jstore && (rc = recompute(j - 1))) return rc;
        {
            PhaseScope scope(PH_ADJOINT, s, k1 - std::max(k0, 1));
            // u_k: kept levels from slot k - k0_store + 1 (or block-floating-point
            // level k - k0_store), recomputed ones from slot set_base(j) + k - k0 + 1
            const bool lvl = g.lvl16 && j >= g.jstore;
            const int first = j >= g.jstore ? 1 - g.k0_store : set_base(j) + 1 - k0;
            for (int k = k1 - 1; k >= std::max(k0, 1); --k)
                if ((rc = lvl ? adjoint_step(k, k - g.k0_store, true) : adjoint_step(k, k + first))) return rc;
        }
        if (aux) WFD_CUDA(cudaEventRecord(ev_adj(j), s));
    }
    if (grad_wavelet && p->nsrc > 0)  // q_1 at the sources -> d J / d w_0
        WFD_CUDA(launch_gather(w.Q[1], ga.cells, w.src_a, ga.ntiles, p->nshot, p->nsrc, w.m,
                               p->src_scale, 1, grad_wavelet, p->nt, 0, s));
    if (finalize && g.vd)  // vel is kappa, grad_vel dJ/dkappa
        WFD_CUDA(launch_vd_finalize(w.G, w.Gbx, w.Gbz, w.m, w.rho, grad_vel, w.grad_rho, g.nz, g.nx, g.ld, g.R,
                                    float((double)p->dt * p->dt / ((double)p->dx * p->dx)), s));
    else if (finalize)
        WFD_CUDA(launch_grad_finalize(w.G, vel, grad_vel, g.nz, g.ny, g.nx, g.ld, g.R, s));
    return WFD_OK;
}

// Adjoint by time reversal (WFD_ADJOINT_RECONSTRUCT, 2D one step per launch).
// The forward leaves u_{nt-1}, u_nt in P[(nt-1) & 1], P[nt & 1] and the damped
// frame of every level in w.frames. Going back, u_k comes from inverting the
// forward step k + 1 where it is undamped,
//     u_k = 2 u_{k+1} + m L u_{k+1} + s w_{k+1} - u_{k+2}
// (the step kernel without sponge factors, in place of u_{k+2}), and the frame
// is restored from its copy; the adjoint step k then stages u_k as in the
// u-store adjoint. No checkpoints, no recomputed segments.
int run_backward_recon(const wfd_problem* p, const Geom& g, const Layout& L, const Work& w, const Stepper& st,
                       const float* wavelet, const float* dtraces, float* grad_vel, float* grad_wavelet,
                       const float* vel) {
    cudaStream_t s = st.s;
    const Geom ga = adjoint_geom(p, g);
    Stepper sa = st;
    sa.g = ga;
    Stepper rv = st;  // the reversal: no sponge factors
    rv.gz = rv.gy = rv.gx = nullptr;
    WFD_CUDA(cudaMemsetAsync(w.Q[0], 0, L.field_bytes, s));
    WFD_CUDA(cudaMemsetAsync(w.Q[1], 0, L.field_bytes, s));
    WFD_CUDA(cudaMemsetAsync(w.G, 0, (size_t)g.cells * 4, s));
    if (g.vd) {
        WFD_CUDA(cudaMemsetAsync(w.Gbx, 0, (size_t)g.cells * 4, s));
        WFD_CUDA(cudaMemsetAsync(w.Gbz, 0, (size_t)g.cells * 4, s));
    }
    int rc;
    CUtensorMap qc[2], qo[2], pc[2], po[2], pa[2], unused[2];
    for (int b = 0; b < 2; ++b) {
        if ((rc = sa.map_pair(w.Q[b], w.Q[b], &qc[b], &qo[b]))) return rc;
        if ((rc = rv.map_pair(w.P[b], w.P[b], &pc[b], &po[b]))) return rc;
        if ((rc = sa.map_pair(w.P[b], w.P[b], &pa[b], &unused[b]))) return rc;
    }
    auto adjoint_step = [&](int k, bool grad) -> int {  // q_k from (q_{k+1}, q_{k+2}); u_k in P[k & 1]
        const int bc = (k + 1) & 1, bn = k & 1;
        StepArgs a = sa.base(w.Q[bn]);
        if (p->nrec > 0) {
            a.inj = w.rec_a;
            a.inj_val = dtraces;
            a.inj_np = p->nrec; a.inj_nt = p->nt; a.inj_t = k - 1;
            a.inj_scale = 1.f;
            a.inj_times_m = 1;
        }
        if (grad_wavelet && k <= p->nt - 1 && p->nsrc > 0) {
            a.smp = w.src_a;
            a.smp_out = grad_wavelet;
            a.smp_np = p->nsrc; a.smp_nt = p->nt; a.smp_t = k;
            a.smp_scale = p->src_scale;
            a.smp_div_m = 1;
        }
        if (!grad) return sa.launch(MODE_PLAIN, qc[bc], qo[bn], qc[bc], a);
        a.grad = w.G;
        a.grad_bx = w.Gbx;
        a.grad_bz = w.Gbz;
        return sa.launch(MODE_GRAD_U, qc[bc], qo[bn], pa[k & 1], a);
    };
    {
        PhaseScope scope(PH_ADJOINT, s, 1);
        if ((rc = adjoint_step(p->nt, false))) return rc;
    }
    PhaseScope scope(PH_ADJOINT, s, 2 * (p->nt - 1));
    for (int k = p->nt - 1; k >= 1; --k) {
        if (k < p->nt - 1) {  // u_k into P[k & 1] (which holds u_{k+2})
            StepArgs a = rv.base(w.P[k & 1]);
            if (p->nsrc > 0) {
                a.inj = w.src;
                a.inj_val = wavelet;
                a.inj_np = p->nsrc; a.inj_nt = p->nt; a.inj_t = k + 1;
                a.inj_scale = p->src_scale;
            }
            if ((rc = rv.launch(MODE_PLAIN, pc[(k + 1) & 1], po[k & 1], pc[(k + 1) & 1], a))) return rc;
            WFD_CUDA(launch_band(w.P[k & 1], reinterpret_cast<float*>(w.frames + (size_t)k * L.frame_bytes), g.cells,
                                 p->nshot, g.nz, g.ld, g.band_w, g.band_cl, g.band_cr, false, s));
        }
        if ((rc = adjoint_step(k, true))) return rc;
    }
    if (grad_wavelet && p->nsrc > 0)  // q_1 at the sources -> d J / d w_0
        WFD_CUDA(launch_gather(w.Q[1], ga.cells, w.src_a, ga.ntiles, p->nshot, p->nsrc, w.m, p->src_scale, 1,
                               grad_wavelet, p->nt, 0, s));
    if (g.vd)
        WFD_CUDA(launch_vd_finalize(w.G, w.Gbx, w.Gbz, w.m, w.rho, grad_vel, w.grad_rho, g.nz, g.nx, g.ld, g.R,
                                    float((double)p->dt * p->dt / ((double)p->dx * p->dx)), s));
    else
        WFD_CUDA(launch_grad_finalize(w.G, vel, grad_vel, g.nz, g.ny, g.nx, g.ld, g.R, s));
    return WFD_OK;
}

// Adjoint of one (group of) shots. zero_G starts a new gradient sum; finalize
// turns the sum into dJ/dv (the last group of a grouped call).
int run_backward(const wfd_problem* p, const Geom& g, const Layout& L, const Work& w,
                 const Stepper& st, const float* wavelet, const float* dtraces, float* grad_vel,
                 float* grad_wavelet, const float* vel, bool zero_G = true, bool finalize = true) {
    if (g.recon) {
        if (!zero_G || !finalize)
            return fail(WFD_ERR_INVALID, "the reconstruction adjoint does not run in shot groups");
        return run_backward_recon(p, g, L, w, st, wavelet, dtraces, grad_vel, grad_wavelet, vel);
    }
    if (g.ustore)
        return run_backward_ustore(p, g, L, w, st, wavelet, dtraces, grad_vel, grad_wavelet, vel,
                                   zero_G, finalize);
    cudaStream_t s = st.s;
    WFD_CUDA(cudaMemsetAsync(w.Q[0], 0, L.field_bytes, s));
    WFD_CUDA(cudaMemsetAsync(w.Q[1], 0, L.field_bytes, s));
    if (zero_G) WFD_CUDA(cudaMemsetAsync(w.G, 0, (size_t)g.cells * 4, s));
    int rc;
    CUtensorMap pc[2], po[2], qc[2], qo[2];
    for (int b = 0; b < 2; ++b) {
        if ((rc = st.map_pair(w.P[b], w.P[b], &pc[b], &po[b]))) return rc;
        if ((rc = st.map_pair(w.Q[b], w.Q[b], &qc[b], &qo[b]))) return rc;
    }
    std::vector<CUtensorMap> lm(g.K);
    for (int k = 0; k < g.K; ++k)
        if ((rc = st.lap_map(w.lap + (size_t)k * L.lap_field_bytes, g.lap_bf16, &lm[k]))) return rc;
    const long long n_all = (long long)p->nshot * g.cells;

    auto adjoint_step = [&](int k, bool with_grad, int slot) -> int {
        const int bc = (k + 1) & 1, bn = k & 1;  // cur = q_{k+1}, new = q_k over q_{k+2}
        StepArgs a = st.base(w.Q[bn]);
        if (p->nrec > 0) {
            a.inj = w.rec;
            a.inj_val = dtraces;
            a.inj_np = p->nrec; a.inj_nt = p->nt; a.inj_t = k - 1;
            a.inj_scale = 1.f;
            a.inj_times_m = 1;
        }
        if (grad_wavelet && k <= p->nt - 1 && p->nsrc > 0) {
            a.smp = w.src;
            a.smp_out = grad_wavelet;
            a.smp_np = p->nsrc; a.smp_nt = p->nt; a.smp_t = k;
            a.smp_scale = p->src_scale;
            a.smp_div_m = 1;
        }
        int mode = MODE_PLAIN;
        if (with_grad) {
            mode = MODE_GRAD;
            a.lap = w.lap + (size_t)slot * L.lap_field_bytes;
            a.lap_bf16 = g.lap_bf16;
            a.grad = w.G;
        }
        return st.launch(mode, qc[bc], qo[bn], with_grad ? lm[slot] : qc[bc], a);
    };

    {
        PhaseScope scope(PH_ADJOINT, s, 1);
        if ((rc = adjoint_step(p->nt, false, 0))) return rc;
    }
    const bool summed = summed_forward(p, g, true);  // checkpoints (d_k0, u_k0), no forward L u store
    for (int j = g.nseg - 1; j >= 0; --j) {
        const int k0 = j * g.K, k1 = std::min(p->nt, k0 + g.K);
        if (j != g.nseg - 1 || summed) {
            PhaseScope scope(PH_RECOMPUTE, s, k1 - k0);
            const unsigned char* slot = w.ckpt + (size_t)j * 2 * L.ckpt_field_bytes;
            WFD_CUDA(launch_unpack(slot + L.ckpt_field_bytes, w.P[k0 & 1], n_all, p->ckpt_format, s));
            if (summed)  // u_{k0-1} = u_k0 - d_k0
                WFD_CUDA(launch_unpack_diff(slot, w.P[k0 & 1], w.P[(k0 + 1) & 1], n_all, p->ckpt_format, s));
            else
                WFD_CUDA(launch_unpack(slot, w.P[(k0 + 1) & 1], n_all, p->ckpt_format, s));
            for (int k = k0; k < k1; ++k) {
                const int bc = k & 1, bn = (k + 1) & 1;
                StepArgs a = st.base(w.P[bn]);
                if (p->nsrc > 0) {
                    a.inj = w.src;
                    a.inj_val = wavelet;
                    a.inj_np = p->nsrc; a.inj_nt = p->nt; a.inj_t = k;
                    a.inj_scale = p->src_scale;
                }
                a.lap = w.lap + (size_t)(k - k0) * L.lap_field_bytes;
                a.lap_bf16 = g.lap_bf16;
                if ((rc = st.launch(MODE_SAVE_LAP, pc[bc], po[bn], pc[bc], a))) return rc;
            }
        }
        PhaseScope scope(PH_ADJOINT, s, k1 - std::max(k0, 1));
        for (int k = k1 - 1; k >= std::max(k0, 1); --k)
            if ((rc = adjoint_step(k, true, k - k0))) return rc;
    }
    if (grad_wavelet && p->nsrc > 0)  // q_1 at the sources -> d J / d w_0
        WFD_CUDA(launch_gather(w.Q[1], g.cells, w.src, g.ntiles, p->nshot, p->nsrc, w.m,
                               p->src_scale, 1, grad_wavelet, p->nt, 0, s));
    if (finalize) WFD_CUDA(launch_grad_finalize(w.G, vel, grad_vel, g.nz, g.ny, g.nx, g.ld, g.R, s));
    return WFD_OK;
}

}  // namespace

extern "C" {

const char* wfd_strerror(int status) {
    switch (status) {
        case WFD_OK: return "ok";
        case WFD_ERR_INVALID: return "invalid argument";
        case WFD_ERR_WORKSPACE: return "workspace too small or misaligned";
        case WFD_ERR_CUDA: return "CUDA call failed";
        case WFD_ERR_UNSTABLE: return "time step violates the CFL bound";
        case WFD_ERR_POSITION: return "source or receiver outside the updated interior";
        case WFD_ERR_TIMEOUT: return "kernel timed out waiting for a TMA tile";
        case WFD_ERR_STATE: return "backward without a checkpointed forward";
        default: return "unknown status";
    }
}

const char* wfd_last_error(void) { return g_last_error.c_str(); }

int wfd_version(void) { return (3 << 16) | 1; }  // 3.0: update_form; 3.1: level_format

int wfd_workspace_bytes(const wfd_problem* p, int with_gradient, size_t* bytes) {
    int rc = check_problem(p);
    if (rc) return rc;
    if (!bytes) return fail(WFD_ERR_INVALID, "bytes is NULL");
    if (with_gradient && p->field_format != WFD_FIELD_FP32)
        return fail(WFD_ERR_INVALID, "reduced-precision fields are a forward-only mode");
    if (with_gradient && p->step_block >= 4)
        return fail(WFD_ERR_INVALID, "step_block %d is a forward-only mode", p->step_block);
    const wfd_problem q = group_problem(p, 0);  // the workspace serves one group at a time
    const Geom g = make_geom(&q);
    *bytes = make_layout(&q, g, with_gradient != 0).total;
    return WFD_OK;
}

int wfd_forward(const wfd_problem* p, const float* vel, const float* sponge_z,
                const float* sponge_y, const float* sponge_x, const float* wavelet,
                const int32_t* src, const int32_t* rec, float* traces, int save_checkpoints,
                void* workspace, size_t workspace_bytes, void* stream) {
    int rc = common_checks(p, vel, wavelet, src, rec);
    if (rc) return rc;
    const int G = group_size(p);
    if (save_checkpoints && G < p->nshot)
        return fail(WFD_ERR_INVALID, "a checkpointed forward cannot be split into shot groups");
    if (save_checkpoints && p->field_format != WFD_FIELD_FP32)
        return fail(WFD_ERR_INVALID, "reduced-precision fields are a forward-only mode");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // one layout, sized for a full group, serves every group
    const wfd_problem first = group_problem(p, 0);
    const Layout L = make_layout(&first, make_geom(&first), save_checkpoints != 0);
    if ((rc = check_workspace(workspace, workspace_bytes, L.total))) return rc;
    const Work w = carve(workspace, L, save_checkpoints != 0);
    for (int g0 = 0; g0 < p->nshot; g0 += G) {
        const wfd_problem q = group_problem(p, g0);
        const Geom g = make_geom(&q);
        if ((rc = setup(&q, g, w, vel, src + 3L * g0 * p->nsrc, rec + 3L * g0 * p->nrec, s, g0 == 0)))
            return rc;
        Stepper st{&q, g, s, w.err, w.m, sponge_z, p->ndim == 3 ? sponge_y : nullptr, sponge_x};
        if ((rc = st.init())) return rc;
        if ((rc = run_forward(&q, g, L, w, st, wavelet + (long long)g0 * p->nt * p->nsrc,
                              traces ? traces + (long long)g0 * p->nt * p->nrec : nullptr,
                              save_checkpoints != 0)))
            return rc;
    }
    return WFD_OK;
}

int wfd_forward_final(const wfd_problem* p, const float* vel, const float* sponge_z,
                      const float* sponge_y, const float* sponge_x, const float* wavelet,
                      const int32_t* src, const int32_t* rec, float* traces, float* u_final,
                      void* workspace, size_t workspace_bytes, void* stream) {
    int rc = common_checks(p, vel, wavelet, src, rec);
    if (rc) return rc;
    if (!u_final) return fail(WFD_ERR_INVALID, "u_final is NULL");
    if (group_size(p) < p->nshot) return fail(WFD_ERR_INVALID, "no shot groups with u_final");
    const Geom g = make_geom(p);
    const Layout L = make_layout(p, g, false);
    if ((rc = check_workspace(workspace, workspace_bytes, L.total))) return rc;
    const Work w = carve(workspace, L, false);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if ((rc = setup(p, g, w, vel, src, rec, s))) return rc;
    Stepper st{p, g, s, w.err, w.m, sponge_z, p->ndim == 3 ? sponge_y : nullptr, sponge_x};
    if ((rc = st.init())) return rc;
    int fb = 0;
    if ((rc = run_forward(p, g, L, w, st, wavelet, traces, false, &fb))) return rc;
    if (p->field_format != WFD_FIELD_FP32) {  // decode, rows of nx cells
        WFD_CUDA(launch_decode_field(p->field_format, w.P[fb], w.S[fb], u_final, (long long)p->nshot * g.nz,
                                     g.nx, g.ld, scale_blocks(g.ld), s));
        return WFD_OK;
    }
    // strip the row padding: rows of ld floats -> rows of nx floats
    WFD_CUDA(cudaMemcpy2DAsync(u_final, (size_t)g.nx * 4, w.P[fb], (size_t)g.ld * 4, (size_t)g.nx * 4,
                               (size_t)p->nshot * g.nz * g.ny, cudaMemcpyDeviceToDevice, s));
    return WFD_OK;
}

int wfd_backward(const wfd_problem* p, const float* vel, const float* sponge_z,
                 const float* sponge_y, const float* sponge_x, const float* wavelet,
                 const int32_t* src, const int32_t* rec, const float* dtraces, float* grad_vel,
                 float* grad_wavelet, void* workspace, size_t workspace_bytes, void* stream) {
    int rc = common_checks(p, vel, wavelet, src, rec);
    if (rc) return rc;
    if (!grad_vel || (p->nrec > 0 && !dtraces))
        return fail(WFD_ERR_INVALID, "grad_vel/dtraces is NULL");
    if (p->field_format != WFD_FIELD_FP32)
        return fail(WFD_ERR_INVALID, "reduced-precision fields are a forward-only mode");
    if (p->step_block >= 4) return fail(WFD_ERR_INVALID, "step_block %d is a forward-only mode", p->step_block);
    if (group_size(p) < p->nshot)
        return fail(WFD_ERR_INVALID, "wfd_backward cannot be split into shot groups");
    const Geom g = make_geom(p);
    const Layout L = make_layout(p, g, true);
    if ((rc = check_workspace(workspace, workspace_bytes, L.total))) return rc;
    const Work w = carve(workspace, L, true);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Stepper st{p, g, s, w.err, w.m, sponge_z, p->ndim == 3 ? sponge_y : nullptr, sponge_x};
    if ((rc = st.init())) return rc;
    return run_backward(p, g, L, w, st, wavelet, dtraces, grad_vel, grad_wavelet, vel);
}

namespace {

// The misfit gradient; when `observed_ready` is set, the stream waits for it
// just before the first read of `observed` (after the forward).
int misfit_gradient_impl(const wfd_problem* p, const float* vel, const float* sponge_z,
                         const float* sponge_y, const float* sponge_x, const float* wavelet,
                         const int32_t* src, const int32_t* rec, const float* observed,
                         cudaEvent_t observed_ready, float* traces, float* grad_vel, float* grad_wavelet,
                         double* misfit, void* workspace, size_t workspace_bytes, void* stream) {
    int rc = common_checks(p, vel, wavelet, src, rec);
    if (rc) return rc;
    if (!grad_vel || !misfit || (p->nrec > 0 && !observed))
        return fail(WFD_ERR_INVALID, "grad_vel/misfit/observed is NULL");
    if (p->field_format != WFD_FIELD_FP32)
        return fail(WFD_ERR_INVALID, "reduced-precision fields are a forward-only mode");
    if (p->step_block >= 4) return fail(WFD_ERR_INVALID, "step_block %d is a forward-only mode", p->step_block);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    WFD_CUDA(cudaMemsetAsync(misfit, 0, sizeof(double), s));
    const int G = group_size(p);
    // one layout, sized for a full group, serves every group (the gradient
    // accumulator keeps its address across groups)
    const wfd_problem first = group_problem(p, 0);
    const Layout L = make_layout(&first, make_geom(&first), true);
    if ((rc = check_workspace(workspace, workspace_bytes, L.total))) return rc;
    const Work w = carve(workspace, L, true);
    for (int g0 = 0; g0 < p->nshot; g0 += G) {
        // one group: forward with checkpoints, residual, adjoint; the gradient
        // and the misfit accumulate over the groups
        const wfd_problem q = group_problem(p, g0);
        const Geom g = make_geom(&q);
        const int32_t* gsrc = src + 3L * g0 * p->nsrc;
        const int32_t* grec = rec + 3L * g0 * p->nrec;
        const float* gwav = wavelet + (long long)g0 * p->nt * p->nsrc;
        const long long toff = (long long)g0 * p->nt * p->nrec;
        if ((rc = setup(&q, g, w, vel, gsrc, grec, s, g0 == 0))) return rc;
        Stepper st{&q, g, s, w.err, w.m, sponge_z, p->ndim == 3 ? sponge_y : nullptr, sponge_x};
        if ((rc = st.init())) return rc;
        float* d = traces ? traces + toff : w.res;
        if ((rc = run_forward(&q, g, L, w, st, gwav, d, true))) return rc;
        const long long ntr = (long long)q.nshot * q.nt * q.nrec;
        if (observed_ready && g0 == 0) WFD_CUDA(cudaStreamWaitEvent(s, observed_ready, 0));
        if (ntr > 0) WFD_CUDA(launch_residual_misfit(d, observed + toff, w.res, ntr, misfit, s));
        if ((rc = run_backward(&q, g, L, w, st, gwav, w.res, grad_vel,
                               grad_wavelet ? grad_wavelet + (long long)g0 * p->nt * p->nsrc : nullptr,
                               vel, g0 == 0, g0 + G >= p->nshot)))
            return rc;
    }
    return WFD_OK;
}

}  // namespace

int wfd_misfit_gradient(const wfd_problem* p, const float* vel, const float* sponge_z,
                        const float* sponge_y, const float* sponge_x, const float* wavelet,
                        const int32_t* src, const int32_t* rec, const float* observed,
                        float* traces, float* grad_vel, float* grad_wavelet, double* misfit,
                        void* workspace, size_t workspace_bytes, void* stream) {
    return misfit_gradient_impl(p, vel, sponge_z, sponge_y, sponge_x, wavelet, src, rec, observed, nullptr,
                                traces, grad_vel, grad_wavelet, misfit, workspace, workspace_bytes, stream);
}

int wfd_misfit_gradient_overlap(const wfd_problem* p, const float* vel, const float* sponge_z,
                                const float* sponge_y, const float* sponge_x, const float* wavelet,
                                const int32_t* src, const int32_t* rec, const float* observed,
                                void* observed_ready, float* traces, float* grad_vel, float* grad_wavelet,
                                double* misfit, void* workspace, size_t workspace_bytes, void* stream) {
    if (!observed_ready) return fail(WFD_ERR_INVALID, "observed_ready is NULL");
    return misfit_gradient_impl(p, vel, sponge_z, sponge_y, sponge_x, wavelet, src, rec, observed,
                                static_cast<cudaEvent_t>(observed_ready), traces, grad_vel, grad_wavelet, misfit,
                                workspace, workspace_bytes, stream);
}

// ------------------------------------------------------------------ variable density
namespace {

int vd_checks(const wfd_problem* p, const float* kappa, const float* rho, const float* wavelet,
              const int32_t* src, const int32_t* rec) {
    int rc = common_checks(p, kappa, wavelet, src, rec);
    if (rc) return rc;
    if (!rho) return fail(WFD_ERR_INVALID, "rho is NULL");
    if (p->ndim != 2 || p->step_block == 2 || p->lap_store != WFD_LAP_AUTO ||
        p->field_format != WFD_FIELD_FP32 || p->group_shots != 0)
        return fail(WFD_ERR_INVALID,
                    "variable density: 2D, one step per launch, lap_store auto, FP32 fields, no shot groups");
    if (p->update_form == WFD_UPDATE_SUMMED)
        return fail(WFD_ERR_INVALID, "variable density: the leapfrog update only");
    if (p->vmax > 0) {  // the staggered operator's bound: vmax dt sqrt((2 sum|c_k|)^2 sum 1/h^2) <= 2
        double c[5] = {0, 0, 0, 0, 0};
        stag_weights(p->order / 2, c);
        double S = 0;
        for (int k = 1; k <= p->order / 2; ++k) S += std::fabs(c[k]);
        S = 4 * S * S;
        const double inv2 = 1.0 / ((double)p->dz * p->dz) + 1.0 / ((double)p->dx * p->dx);
        if (p->vmax * (double)p->dt * std::sqrt(inv2 * S) > 2.0)
            return fail(WFD_ERR_UNSTABLE, "vmax*dt = %g exceeds the staggered CFL bound %g of order %d",
                        p->vmax * (double)p->dt, 2.0 / std::sqrt(inv2 * S), p->order);
    }
    return WFD_OK;
}

}  // namespace

int wfd_vd_workspace_bytes(const wfd_problem* p, int with_gradient, size_t* bytes) {
    int rc = check_problem(p);
    if (rc) return rc;
    if (!bytes) return fail(WFD_ERR_INVALID, "bytes is NULL");
    const Geom g = make_geom(p, 0, 0, true);
    *bytes = make_layout(p, g, with_gradient != 0).total;
    return WFD_OK;
}

int wfd_vd_forward(const wfd_problem* p, const float* kappa, const float* rho, const float* sponge_z,
                   const float* sponge_x, const float* wavelet, const int32_t* src, const int32_t* rec,
                   float* traces, void* workspace, size_t workspace_bytes, void* stream) {
    int rc = vd_checks(p, kappa, rho, wavelet, src, rec);
    if (rc) return rc;
    const Geom g = make_geom(p, 0, 0, true);
    const Layout L = make_layout(p, g, false);
    if ((rc = check_workspace(workspace, workspace_bytes, L.total))) return rc;
    Work w = carve(workspace, L, false);
    w.rho = rho;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if ((rc = setup(p, g, w, kappa, src, rec, s))) return rc;
    Stepper st{p, g, s, w.err, w.m, sponge_z, nullptr, sponge_x};
    st.bfield = w.b;
    if ((rc = st.init())) return rc;
    return run_forward(p, g, L, w, st, wavelet, traces, false);
}

int wfd_vd_forward_final(const wfd_problem* p, const float* kappa, const float* rho, const float* sponge_z,
                         const float* sponge_x, const float* wavelet, const int32_t* src, const int32_t* rec,
                         float* traces, float* u_final, void* workspace, size_t workspace_bytes, void* stream) {
    int rc = vd_checks(p, kappa, rho, wavelet, src, rec);
    if (rc) return rc;
    if (!u_final) return fail(WFD_ERR_INVALID, "u_final is NULL");
    const Geom g = make_geom(p, 0, 0, true);
    const Layout L = make_layout(p, g, false);
    if ((rc = check_workspace(workspace, workspace_bytes, L.total))) return rc;
    Work w = carve(workspace, L, false);
    w.rho = rho;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if ((rc = setup(p, g, w, kappa, src, rec, s))) return rc;
    Stepper st{p, g, s, w.err, w.m, sponge_z, nullptr, sponge_x};
    st.bfield = w.b;
    if ((rc = st.init())) return rc;
    int fb = 0;
    if ((rc = run_forward(p, g, L, w, st, wavelet, traces, false, &fb))) return rc;
    WFD_CUDA(cudaMemcpy2DAsync(u_final, (size_t)g.nx * 4, w.P[fb], (size_t)g.ld * 4, (size_t)g.nx * 4,
                               (size_t)p->nshot * g.nz, cudaMemcpyDeviceToDevice, s));
    return WFD_OK;
}

int wfd_vd_misfit_gradient(const wfd_problem* p, const float* kappa, const float* rho, const float* sponge_z,
                           const float* sponge_x, const float* wavelet, const int32_t* src, const int32_t* rec,
                           const float* observed, float* traces, float* grad_kappa, float* grad_rho,
                           float* grad_wavelet, double* misfit, void* workspace, size_t workspace_bytes,
                           void* stream) {
    int rc = vd_checks(p, kappa, rho, wavelet, src, rec);
    if (rc) return rc;
    if (!grad_kappa || !grad_rho || !misfit || (p->nrec > 0 && !observed))
        return fail(WFD_ERR_INVALID, "grad_kappa/grad_rho/misfit/observed is NULL");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    WFD_CUDA(cudaMemsetAsync(misfit, 0, sizeof(double), s));
    const Geom g = make_geom(p, 0, 0, true);
    const Layout L = make_layout(p, g, true);
    if ((rc = check_workspace(workspace, workspace_bytes, L.total))) return rc;
    Work w = carve(workspace, L, true);
    w.rho = rho;
    w.grad_rho = grad_rho;
    if ((rc = setup(p, g, w, kappa, src, rec, s))) return rc;
    Stepper st{p, g, s, w.err, w.m, sponge_z, nullptr, sponge_x};
    st.bfield = w.b;
    if ((rc = st.init())) return rc;
    float* d = traces ? traces : w.res;
    if ((rc = run_forward(p, g, L, w, st, wavelet, d, true))) return rc;
    const long long ntr = (long long)p->nshot * p->nt * p->nrec;
    if (ntr > 0) WFD_CUDA(launch_residual_misfit(d, observed, w.res, ntr, misfit, s));
    return run_backward(p, g, L, w, st, wavelet, w.res, grad_kappa, grad_wavelet, kappa, true, true);
}

int wfd_status(void* workspace, void* stream) {
    if (!workspace) return fail(WFD_ERR_WORKSPACE, "workspace is NULL");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned h = 0;
    WFD_CUDA(cudaMemcpyAsync(&h, workspace, sizeof h, cudaMemcpyDeviceToHost, s));
    WFD_CUDA(cudaStreamSynchronize(s));
    WFD_CUDA(cudaMemsetAsync(workspace, 0, sizeof h, s));
    if (h & DEV_ERR_TMA_TIMEOUT) return fail(WFD_ERR_TIMEOUT, "device: TMA wait timed out");
    if (h & DEV_ERR_BAD_POSITION)
        return fail(WFD_ERR_POSITION, "device: a source/receiver lies outside the interior");
    return WFD_OK;
}

uint64_t wfd_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }

int wfd_profile_begin(void) {
    for (auto& r : g_records) {
        cudaEventDestroy(r.start);
        cudaEventDestroy(r.stop);
    }
    g_records.clear();
    g_profiling = true;
    return WFD_OK;
}

int wfd_profile_end(wfd_phase_times* out) {
    g_profiling = false;
    if (!out) return fail(WFD_ERR_INVALID, "out is NULL");
    *out = wfd_phase_times{};
    int rc = WFD_OK;
    for (auto& r : g_records) {
        float ms = 0.f;
        if (cudaEventSynchronize(r.stop) != cudaSuccess ||
            cudaEventElapsedTime(&ms, r.start, r.stop) != cudaSuccess)
            rc = fail(WFD_ERR_CUDA, "phase event timing failed");
        out->ms[r.phase] += ms;
        out->launches[r.phase] += r.launches;
        cudaEventDestroy(r.start);
        cudaEventDestroy(r.stop);
    }
    g_records.clear();
    return rc;
}

int wfd_sum_sq(const float* x, int64_t n, double* out, void* stream) {
    if (!x || !out || n < 0) return fail(WFD_ERR_INVALID, "bad sum_sq arguments");
    WFD_CUDA(launch_sum_sq(x, n, out, static_cast<cudaStream_t>(stream)));
    return WFD_OK;
}

int wfd_analytic_signal(const float* traces, int64_t ntraces, int nt, const float* hilbert_kernel,
                        float* out, void* stream) {
    if (!traces || !hilbert_kernel || !out) return fail(WFD_ERR_INVALID, "NULL argument");
    if (ntraces < 0 || nt < 2 || nt > 18000) return fail(WFD_ERR_INVALID, "need 2 <= nt <= 18000");
    if (ntraces == 0) return WFD_OK;
    if (ntraces > 0x7fffffffLL) return fail(WFD_ERR_INVALID, "too many traces");
    if (reinterpret_cast<uintptr_t>(out) % 8) return fail(WFD_ERR_INVALID, "out must be 8-byte aligned");
    WFD_CUDA(launch_analytic(traces, ntraces, nt, hilbert_kernel, reinterpret_cast<float2*>(out),
                             static_cast<cudaStream_t>(stream)));
    return WFD_OK;
}

int wfd_tfm(const float* h, int E, const float* xe, const float* ye, int nt, float dt, float t0,
            float c, const float* xp, const float* yp, int npix, int reciprocity, float* image,
            void* stream) {
    if (!h || !xe || !ye || !xp || !yp || !image) return fail(WFD_ERR_INVALID, "NULL argument");
    if (E < 1 || E > 256 || nt < 2 || npix < 0) return fail(WFD_ERR_INVALID, "need 1 <= E <= 256, nt >= 2");
    if (!(dt > 0) || !(c > 0)) return fail(WFD_ERR_INVALID, "dt and c must be positive");
    if (reinterpret_cast<uintptr_t>(h) % 8) return fail(WFD_ERR_INVALID, "h must be 8-byte aligned");
    if (npix == 0) return WFD_OK;
    WFD_CUDA(launch_tfm(reinterpret_cast<const float2*>(h), E, xe, ye, nt, dt, t0, c, xp, yp, npix,
                        reciprocity, image, static_cast<cudaStream_t>(stream)));
    return WFD_OK;
}

int wfd_temporal_step(const float* u0, const float* u1, float* v0, float* v1, float wavespeed, float dt,
                      float dx, float dy, int N, int M, int M_padded, void* stream) {
    if (!u0 || !u1 || !v0 || !v1) return fail(WFD_ERR_INVALID, "NULL field");
    if (N < 3 || M < 3 || M_padded < M || M_padded % 4)
        return fail(WFD_ERR_INVALID, "need N, M >= 3 and M_padded >= M, M_padded %% 4 == 0");
    if (!aligned16(u0) || !aligned16(u1) || !aligned16(v0) || !aligned16(v1))
        return fail(WFD_ERR_INVALID, "fields must be 16-byte aligned");
    if ((long long)N * M_padded >= (1ll << 31)) return fail(WFD_ERR_INVALID, "grid too large");
    // neighbouring tiles read each other's halos, so the outputs must not overlap the inputs
    const uintptr_t n = (uintptr_t)N * M_padded * sizeof(float);
    auto overlap = [n](const void* a, const void* b) {
        const uintptr_t x = reinterpret_cast<uintptr_t>(a), y = reinterpret_cast<uintptr_t>(b);
        return x < y + n && y < x + n;
    };
    if (overlap(v0, u0) || overlap(v0, u1) || overlap(v1, u0) || overlap(v1, u1) || overlap(v0, v1))
        return fail(WFD_ERR_INVALID, "v0 and v1 must not overlap each other, u0 or u1");
    unsigned cols = 0, rows = 0;
    temporal_box(&cols, &rows);
    const cuuint32_t box[3] = {cols, rows, 1};
    CUtensorMap m0, m1;
    int rc;
    if ((rc = make_field_map(&m0, u0, false, 2, N, 1, M, M_padded, 1, box))) return rc;
    if ((rc = make_field_map(&m1, u1, false, 2, N, 1, M, M_padded, 1, box))) return rc;
    const cudaError_t e = launch_temporal(m0, m1, v0, v1, wavespeed, dt, dx, dy, N, M, M_padded,
                                          static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(WFD_ERR_CUDA, "temporal step launch failed: %s", cudaGetErrorString(e));
    return WFD_OK;
}

int wfd_temporal_step_fast(const float* u0, const float* u1, float* v0, float* v1, float wavespeed, float dt,
                           float dx, float dy, int N, int M, int M_padded, void* stream) {
    if (!u0 || !u1 || !v0 || !v1) return fail(WFD_ERR_INVALID, "NULL field");
    if (N < 3 || M < 3 || M_padded < M) return fail(WFD_ERR_INVALID, "need N, M >= 3 and M_padded >= M");
    if ((long long)N * M_padded >= (1ll << 31)) return fail(WFD_ERR_INVALID, "grid too large");
    if ((N + 31) / 32 > 65535) return fail(WFD_ERR_INVALID, "N too large");
    const uintptr_t n = (uintptr_t)N * M_padded * sizeof(float);
    auto overlap = [n](const void* a, const void* b) {
        const uintptr_t x = reinterpret_cast<uintptr_t>(a), y = reinterpret_cast<uintptr_t>(b);
        return x < y + n && y < x + n;
    };
    if (overlap(v0, u0) || overlap(v0, u1) || overlap(v1, u0) || overlap(v1, u1) || overlap(v0, v1))
        return fail(WFD_ERR_INVALID, "v0 and v1 must not overlap each other, u0 or u1");
    const cudaError_t e = launch_temporal_reg(u0, u1, v0, v1, wavespeed, dt, dx, dy, N, M, M_padded, false,
                                              static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(WFD_ERR_CUDA, "temporal step launch failed: %s", cudaGetErrorString(e));
    return WFD_OK;
}

int wfd_step2d_order2(const float* u0, const float* u1, float* u2, float wavespeed, float dt,
                      float dx, float dy, int N, int M, int M_padded, void* stream) {
    if (!u0 || !u1 || !u2) return fail(WFD_ERR_INVALID, "NULL field");
    if (N < 3 || M < 3 || M_padded < M || M_padded % 4)
        return fail(WFD_ERR_INVALID, "need N, M >= 3 and M_padded >= M, M_padded %% 4 == 0");
    if (!aligned16(u0) || !aligned16(u1) || !aligned16(u2))
        return fail(WFD_ERR_INVALID, "fields must be 16-byte aligned");
    if ((long long)N * M_padded >= (1ll << 31)) return fail(WFD_ERR_INVALID, "grid too large");
    // rows i (N) are the kernel's z axis with spacing dx, columns j (M) its x
    // axis with spacing dy; all of dt^2 c^2 / h^2 goes into the weights, m = 1.
    const float cz = float((double)dt * dt * wavespeed * wavespeed / ((double)dx * dx));
    const float cx = float((double)dt * dt * wavespeed * wavespeed / ((double)dy * dy));
    StepArgs a{};
    a.u_new = u2;
    a.m = nullptr;
    a.m_const = 1.f;
    a.nz = N; a.ny = 1; a.nx = M; a.ld = M_padded;
    a.plane = M_padded;
    a.shot_stride = (long long)N * M_padded;
    a.nshot = 1; a.shots_per_cta = 1;
    a.tiles_x = cdiv(M, T2_TX); a.tiles_y = 1; a.tiles_z = cdiv(N, T2_TZ);
    a.c0 = -2.f * (cz + cx);
    a.cz[0] = cz;
    a.cx[0] = cx;
    a.err = nullptr;
    CUtensorMap mc, mo;
    const cuuint32_t bc[3] = {T2_W, T2_TZ + 2, 1};
    const cuuint32_t bo[3] = {T2_TX, T2_TZ, 1};
    int rc;
    if ((rc = make_field_map(&mc, u1, false, 2, N, 1, M, M_padded, 1, bc))) return rc;
    if ((rc = make_field_map(&mo, u0, false, 2, N, 1, M, M_padded, 1, bo))) return rc;
    cudaError_t e = launch_step2d(1, MODE_PLAIN, T2_TZ, mc, mo, mc, a, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(WFD_ERR_CUDA, "step launch failed: %s", cudaGetErrorString(e));
    return WFD_OK;
}

}  // extern "C"
