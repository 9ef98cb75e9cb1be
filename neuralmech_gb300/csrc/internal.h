// Internal interface between the C-ABI layer (api.cu) and the kernels.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace wfd {

// Device error bits, OR-ed into the workspace's status word.
enum : unsigned {
    DEV_ERR_TMA_TIMEOUT = 1u << 0,   // an mbarrier wait for a TMA tile gave up
    DEV_ERR_BAD_POSITION = 1u << 1,  // a source/receiver outside the updated interior
};

// ---------------------------------------------------------------- 2D tiles
// One CTA = 256 threads = 8 warps. A lane owns 4 consecutive x cells (one
// float4); a warp owns RB consecutive rows; the CTA tile is TX x (8 RB) cells,
// RB = 4 (32 rows, the default) or 2 (16 rows).
// u_n is staged with a halo of R rows and XH = 4 columns (XH keeps every TMA
// x coordinate 16-byte aligned for any R <= 4).
constexpr int T2_THREADS = 256;
constexpr int T2_TX = 128;
constexpr int T2_XH = 4;
constexpr int T2_W = T2_TX + 2 * T2_XH;  // staged row length (floats)
constexpr int T2_TZ = 32;  // default tile rows; 16 is the other variant
constexpr int T2_STAGES = 2;
constexpr int T2_MAX_SPC = 64;  // shots one 2D CTA may walk through

// What a step kernel does besides the stencil update.
enum StepMode : int {
    MODE_PLAIN = 0,     // update only
    MODE_SAVE_LAP = 1,  // update + store L u_n (forward recompute)
    MODE_GRAD = 2,      // update + accumulate q_{k+1} * L u_k into the gradient (adjoint)
    MODE_GRAD_U = 3,    // as MODE_GRAD, with L u_k computed in the kernel from a staged u_k
                        // tile (2D one-step kernel; the map_lap box is then the u_n box)
    MODE_SUMMED = 4,    // update only, in the summed (increment) form (2D one-step and 3D kernels):
                        // the state is (u_n, d_n = u_n - u_{n-1}); map_old stages d_n,
                        // d_{n+1} goes to d_new in place and u_{n+1} = u_n + d_{n+1} to u_new
    MODE_GRAD_U16 = 5,  // as MODE_GRAD_U with u_k kept in block floating point: map_lap stages
                        // its int16 mantissas (box 144 x (tile_rows + 2R) x 1 at x0 - 8),
                        // map_lx its exponent bytes (box 64 x (tile_rows + 2R) x 1 at x0/4 - 16)
};

// Kept levels in block floating point (WFD_LEVEL_BFP16): a level is
// [nshot][nz][ld] int16 mantissas plus [nshot][nz][eld] exponent bytes, one per
// 4 cells along x (eld = ld / 4 rounded up to 16 bytes, the TMA row pitch).
inline int bfp_eld(int ld) { return (ld / 4 + 15) / 16 * 16; }

// A set of points (sources or receivers) bucketed by the tile that owns them.
// off[s * ntiles + t] .. off[s * ntiles + t + 1] index ent[], ent = {cell, p}
// with cell the in-shot linear index (z * plane + y * ld + x) and p the point
// number within the shot.
struct PointLists {
    const int* off = nullptr;
    const int2* ent = nullptr;
};

struct StepArgs {
    float* u_new;              // overwritten level, [nshot][cells] (aliases the u_{n-1} buffer)
    const float* m;            // (v dt / dx)^2, [cells]; null -> m_const
    float m_const;
    const float* gz;           // sponge profiles (null = no sponge on that axis)
    const float* gy;
    const float* gx;
    int nz, ny, nx, ld;        // ny = 1 in 2D
    long long plane;           // ny * ld (3D) or ld (2D): z stride
    long long shot_stride;     // cells per shot (nz * plane)
    int nshot, shots_per_cta;
    int tiles_x, tiles_y, tiles_z;
    float c0;                  // centre weight (all axes)
    float cz[4], cy[4], cx[4]; // axis weights for k = 1..R, already scaled by (dx/h)^2
    float2 c0p, czp[4], cyp[4], cxp[4]; // the same as duplicated pairs, operands of the
                                        // packed FP32x2 arithmetic (set by the launchers)
    // injection into u_new: u += g * scale * val (* m at the cell when inj_times_m)
    PointLists inj;
    const float* inj_val;      // [nshot][inj_nt][inj_np]
    int inj_np, inj_nt, inj_t;
    float inj_scale;
    int inj_times_m;
    // sampling of the staged level u_n: out[s][smp_t][p] = scale * u_n(cell) (/ m)
    PointLists smp;
    float* smp_out;            // [nshot][smp_nt][smp_np]
    int smp_np, smp_nt, smp_t;
    float smp_scale;
    int smp_div_m;
    // Laplacian store (MODE_SAVE_LAP writes, MODE_GRAD reads via TMA)
    void* lap;                 // [nshot][cells] FP32 or BF16
    int lap_bf16;
    float* grad;               // [cells], MODE_GRAD accumulation target
    // variable density (stencil2d_vd.cu): m holds k = kappa dt^2/dx^2
    float cs[4];               // staggered first-derivative weights c_1..c_R
    float2 csp[4];             // the same as duplicated pairs (set by the launchers)
    float vd_sz;               // (dx/dz)^2
    float *grad_bx, *grad_bz;  // MODE_GRAD_U accumulators at the half points (z, x+1/2), (z+1/2, x)
    int zero_ring;             // 2D one-step kernel: also write the fixed ring (and the row
                               // padding) of u_new, as 0; else leave those cells untouched
    float* d_new;              // MODE_SUMMED: the increment field d, [nshot][cells], updated
                               // in place (injections are added to it as well as to u_new)
    unsigned* err;
};

// Reduced-precision storage step (stencil2d_lp.cu): fields [shot][z][ld] of
// FP16 or int16 (fmt WFD_FIELD_FP16 / _I16), int16 with scales
// [shot][z][nblk] FP32 (one per 32 cells along x). a carries the geometry,
// weights, m, sponge and point lists (a.shot_stride in cells); a.inj_t is the
// step's source sample, a.smp_t the trace index of u_{n+1}.
struct LpArgs {
    StepArgs a;
    const void* cur;  // u_n (read-only in the launch)
    const float* scur;
    const void* old;  // u_{n-1}
    const float* sold;
    void* nw;         // u_{n+1} (may alias old)
    float* snw;
    int nblk;         // scale blocks per row: ceil(ld / 32) rounded up to 4
    long long sstride;  // scales per shot: nz * nblk
};
// map_cur: u_n (16-bit, box 144 x (32 + 2R) x 1 at x0 - 8); map_old: u_{n-1}
// (box 128 x 32 x 1); map_cs / map_os (int16 only): their scale rows (FP32,
// [shot][z][nblk] with nblk a multiple of 4; boxes 12 x (32 + 2R) x 1 at block
// x0/32 - 4 and 4 x 32 x 1 at block x0/32).
// The eight-step drop-in (dropin.cu): maps over u0 and u1 ([N][Mp], extent M)
// with the box temporal_box() gives.
void temporal_box(unsigned* cols, unsigned* rows);
cudaError_t launch_temporal(const CUtensorMap& m0, const CUtensorMap& m1, float* v0, float* v1, float wavespeed,
                            float dt, float dx, float dy, int N, int M, int Mp, cudaStream_t s);
// The eight-step drop-in with the window in registers (no TMA): exact = the
// reference expression in IEEE operations, else pre-divided weights and FMAs.
// Grid (ceil(M / 240), ceil(N / 32)) CTAs of 256 threads.
cudaError_t launch_temporal_reg(const float* u0, const float* u1, float* v0, float* v1, float wavespeed, float dt,
                                float dx, float dy, int N, int M, int Mp, bool exact, cudaStream_t s);
cudaError_t launch_step2d_lp(int R, int fmt, const CUtensorMap& map_cur, const CUtensorMap& map_old,
                             const CUtensorMap& map_cs, const CUtensorMap& map_os, const LpArgs& p,
                             cudaStream_t s);
// u_final[row][x] (FP32, nx per row) from a reduced-precision field.
cudaError_t launch_decode_field(int fmt, const void* f, const float* sc, float* out, long long nrows, int nx,
                                int ld, int nblk, cudaStream_t s);

// Variable-density step (stencil2d_vd.cu), mode MODE_PLAIN or MODE_GRAD_U on
// 128 x 16 tiles. map_f: the field (box 144 x (16 + 4R) x 1 at x0 - 8, z0 - 2R);
// map_o: u_{n-1} (box 128 x 16 x 1); map_u: u_k as map_f (MODE_GRAD_U); map_b:
// b = 1/rho ([nz][ld], box 144 x (16 + 2R + 1) at x0 - 8, z0 - R).
cudaError_t launch_step2d_vd(int R, int mode, const CUtensorMap& map_f, const CUtensorMap& map_o,
                             const CUtensorMap& map_u, const CUtensorMap& map_b, const StepArgs& a, cudaStream_t s);
cudaError_t launch_vd_params(const float* kappa, const float* rho, float* k, float* b, int nz, int nx, int ld,
                             float scale, cudaStream_t s);
cudaError_t launch_vd_finalize(const float* G, const float* Gbx, const float* Gbz, const float* k, const float* rho,
                               float* gkap, float* grho, int nz, int nx, int ld, int R, float scale, cudaStream_t s);

// Launches one time step of the 2D kernel of half-width R (1, 2, 4), mode and
// tile height tile_rows (16 or 32).
// map_cur: u_n (box T2_W x (tile_rows + 2R) x 1); map_old: u_{n-1} (box
// T2_TX x tile_rows x 1); map_lap: Laplacian store (box T2_TX x tile_rows x 1,
// MODE_GRAD), the level u_k (MODE_GRAD_U: the box of map_cur) or its mantissas
// (MODE_GRAD_U16).
// map_lx: MODE_GRAD_U16's exponent tiles (null otherwise).
cudaError_t launch_step2d(int R, int mode, int tile_rows, const CUtensorMap& map_cur,
                          const CUtensorMap& map_old, const CUtensorMap& map_lap, const StepArgs& a,
                          cudaStream_t s, const CUtensorMap* map_lx = nullptr);

// ---------------------------------------------------------------- 2D, two steps per launch
// Tile T = K2_TX x K2_TZ cells; u_n is staged on T plus 2R rows / 8 columns
// (K2_UW wide), u_{n-1} and m on E = T plus R rows / 4 columns (K2_EW wide).
constexpr int K2_TX = 120;
constexpr int K2_TZ = 24;  // (two stages and the m tile fit two CTAs per SM)
constexpr int K2_EW = K2_TX + 8;
constexpr int K2_UW = K2_TX + 16;
constexpr int K2_THREADS = 256;

struct Step2Args {
    StepArgs a;         // step 2: u_new = u_{n+2}, inj/inj_t (tile lists), smp/smp_t
                        // (samples u_{n+1}); a.smp also serves step 1
    float* u_mid;       // u_{n+1} output on the tile
    PointLists inj_e;   // step-1 injection: points inside the tile's extended region E
    int inj_t1;         // step-1 injection time index (-1: none)
    int smp_t1;         // step-1 sampling time index of u_n (-1: none)
    int two_steps;      // 0: step 1 only (u_{n+1} to u_mid)
    // summed form (the state is u_n and d_n = u_n - u_{n-1}): map_o stages d_n
    // on E; d_{n+2} goes to d_out, u_{n+2} to a.u_new; the intermediate level
    // (u_{n+1} to u_mid, d_{n+1} to d_mid) is written only with write_mid (a
    // checkpoint or a kept level needs it), or when two_steps is 0
    int summed;
    float* d_out;       // d_{n+2}, [nshot][cells]; may not alias the staged d_n
    float* d_mid;       // d_{n+1}, [nshot][cells] (write_mid or !two_steps)
    int write_mid;
    // summed form: block-floating-point copies of the kept levels u_{n+1}
    // (lq_mid, le_mid) and u_{n+2} (lq_out, le_out), null where not kept;
    // mantissas [nshot][cells], exponents [nshot][nz][eld]
    short* lq_mid;
    unsigned char* le_mid;
    short* lq_out;
    unsigned char* le_out;
    int eld;
};

// map_u: u_n (box K2_UW x (K2_TZ + 4R) x 1); map_o: u_{n-1}, or d_n in the summed form
// (box K2_EW x (K2_TZ + 2R) x 1); map_m: m ([nz][ld], box K2_EW x (K2_TZ + 2R)).
// Plain steps only (no L u store, no gradient term); a.shots_per_cta shots per CTA.
cudaError_t launch_step2d_k2(int R, const CUtensorMap& map_u, const CUtensorMap& map_o,
                             const CUtensorMap& map_m, const Step2Args& p, cudaStream_t s);

// ---------------------------------------------------------------- 2D, K steps per launch (orders 2, 4)
// A window of WR_W columns x WR_H rows per CTA, held in registers (a column
// per thread); K = WR_HALO / R steps per launch (8 at order 2, 4 at order 4),
// after which the inner WR_OX x WR_OZ tile is exact.
constexpr int WR_W = 256;
constexpr int WR_H = 40;
constexpr int WR_HALO = 8;
constexpr int WR_OX = WR_W - 2 * WR_HALO;  // 240 output columns per CTA
constexpr int WR_OZ = WR_H - 2 * WR_HALO;  // 24 output rows per CTA

struct RegArgs {
    const float* u0;  // u_{n-1}, [nshot][cells]
    const float* u1;  // u_n
    float* v0;        // u_{n+k-1} on the output tiles (neither input aliases an output)
    float* v1;        // u_{n+k}
    PointLists src;   // sources inside each tile's window (the tile plus WR_HALO on every side)
    int n0;           // absolute index of the launch's first step (u_{n0} -> u_{n0+1})
    int ksteps;       // steps of this launch, 1 .. WR_HALO / R
};

// Forward steps n0 .. n0 + ksteps - 1 of every shot (leapfrog, FP32, 2D, R = 1
// or 2): a.m, a.gz, a.gx, the weights and the tile geometry (a.tiles_x,
// a.tiles_z of WR_OX x WR_OZ tiles); sources from q.src, wavelet a.inj_val
// (a.inj_nt, a.inj_np, a.inj_scale); receivers a.smp (tile lists), sampled
// after every step into a.smp_out[shot][step][rec] (the level u_{step+1}).
cudaError_t launch_wave_reg(int R, const StepArgs& a, const RegArgs& q, cudaStream_t s);

// ---------------------------------------------------------------- 3D tiles
// One CTA (one shot) marches along z through a (TY x TX) column of the grid
// for T3_ZCHUNK output planes; a thread owns 4 x cells and keeps the 2R + 1
// z taps of each in registers.
constexpr int T3_TX = 64;
constexpr int T3_TY = 16;
constexpr int T3_XH = 4;
constexpr int T3_W = T3_TX + 2 * T3_XH;
constexpr int T3_ROWS = 1;                       // tile rows per thread
constexpr int T3_THREADS = (T3_TX / 4) * T3_TY / T3_ROWS;
constexpr int T3_ZCHUNK = 64;                    // planes per CTA (z blocking)

// map_cur: u_n planes (box T3_W x (T3_TY + 2R) x 1 x 1); map_old, map_lap:
// output-plane tiles (box T3_TX x T3_TY x 1 x 1); map_m: the model m
// ([z][y][ld], box T3_TX x T3_TY x 1).
cudaError_t launch_step3d(int R, int mode, const CUtensorMap& map_cur, const CUtensorMap& map_old,
                          const CUtensorMap& map_lap, const CUtensorMap& map_m, const StepArgs& a,
                          cudaStream_t s);
bool step3d_available();

// Counts kernel launches (wfd_kernel_launches); every launcher calls it.
void count_launch(int n = 1);

// Records `message` as the calling thread's wfd_last_error() and returns status.
int set_error(int status, const char* message);

// ---------------------------------------------------------------- helpers (aux.cu)
cudaError_t launch_vel_to_m(const float* vel, float* m, int nz, int ny, int nx, int ld,
                            float scale, cudaStream_t s);
// Per-(shot, tile) point lists. With halo_z / halo_x > 0 a point joins every
// tile whose region grown by that halo contains it (at most 4 in 2D); ent must
// then hold 4 entries per point.
cudaError_t launch_build_lists(const int32_t* pos, int nshot, int np, int nz, int ny, int nx,
                               int ld, int R, int tile_z, int tile_y, int tile_x, int tiles_z,
                               int tiles_y, int tiles_x, int* counts, int* off, int2* ent,
                               unsigned* err, cudaStream_t s, int halo_z = 0, int halo_x = 0);
// The damped frame of fields [z][ld]: rows [0, W), [nz - W, nz), and columns
// [0, cl), [cr, ld) of the other rows, saved to / restored from a compact store
// (band_cells per shot, shots contiguous).
long long band_cells(int nz, int ld, int W, int cl, int cr);
cudaError_t launch_band(float* field, float* store, long long shot_stride, int nshot, int nz, int ld, int W,
                        int cl, int cr, bool save, cudaStream_t s);
cudaError_t launch_gather(const float* u, long long shot_stride, PointLists lists, int ntiles,
                          int nshot, int np, const float* m, float scale, int div_m,
                          float* out, int out_nt, int out_t, cudaStream_t s);
// Checkpoint codec: format 0 FP32 copy, 1 BF16, 2 int16 + FP32 scale per 32
// values (scales stored after the n int16 values). n is a multiple of 4.
size_t ckpt_bytes(int format, long long n);
cudaError_t launch_pack(const float* src, void* dst, long long n, int format, cudaStream_t s);
cudaError_t launch_unpack(const void* src, float* dst, long long n, int format, cudaStream_t s);
// dst = from - (the unpacked src): u_{k0-1} = u_k0 - d_k0 from a summed-form checkpoint
cudaError_t launch_unpack_diff(const void* src, const float* from, float* dst, long long n, int format,
                               cudaStream_t s);
cudaError_t launch_residual_misfit(const float* d, const float* obs, float* res, long long n,
                                   double* misfit, cudaStream_t s);
cudaError_t launch_grad_finalize(const float* G, const float* vel, float* grad_vel, int nz,
                                 int ny, int nx, int ld, int R, cudaStream_t s);
cudaError_t launch_sum_sq(const float* x, long long n, double* out, cudaStream_t s);

// ---------------------------------------------------------------- imaging (imaging.cu)
cudaError_t launch_analytic(const float* traces, long long ntr, int nt, const float* g, float2* h,
                            cudaStream_t s);
cudaError_t launch_tfm(const float2* h, int E, const float* xe, const float* ye, int nt, float dt,
                       float t0, float c, const float* xp, const float* yp, int P, int reciprocity,
                       float* image, cudaStream_t s);

}  // namespace wfd
