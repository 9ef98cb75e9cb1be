// FP64 CPU oracle for the finite-difference acoustic wave path.
//
// TEST INFRASTRUCTURE ONLY. The parity tests, the smoke check and the CPU
// baseline of bench.py call it as their reference; the product library
// never links, loads or falls back to it.
//
// What it restates:
//  * the explicit 2nd-order-in-time update of projects/18_simple_wave_fd/
//    step2D_wave.cu:59-81 (padded_step) and 2D_wave_cupy.py:54-62 (fd_step):
//    u_new = 2 u - u_old + dt^2 c^2 Lap(u) on the interior, the outer ring held
//    fixed (homogeneous Dirichlet);
//  * generalised to space order 2R (R = 1, 2, 4) with the standard central
//    second-derivative weights, a per-cell velocity, 2D and 3D, and an
//    exponential (Cerjan) sponge applied as a per-cell factor g:
//        u_{n+1} = g (2 u_n + v^2 dt^2 L u_n + s w_n) - g^2 u_{n-1}
//    (damping both stored levels once per step, the classic sponge);
//  * point sources added at their cells (scaled by s and by g) and receivers
//    sampling u_{n+1} at their cells, traces laid out (shot, step, receiver)
//    as the reference's full matrix capture stacks them
//    (projects/18_fwi/plate.py:62-64);
//  * the L2 misfit J = 1/2 sum (d - d_obs)^2 and its exact discrete adjoint
//    gradient with respect to the velocity and to the wavelets, computed with
//    exact FP64 checkpoints and segment recomputation.
//
// All arrays are dense (no row padding), index (z, y, x) with x fastest; 2D
// problems have ny == 1 and no y stencil.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

extern "C" {

struct orc_problem {
    int32_t ndim;    // 2 or 3
    int32_t order;   // 2, 4 or 8
    int32_t nz, ny, nx;
    int32_t nshot, nt, nsrc, nrec;
    int32_t ckpt_every;  // 0: ceil(sqrt(nt))
    double dt, dz, dy, dx;
    double src_scale;
};

// Central second-derivative weights of order 2R on a unit grid:
// a_k = 2 (-1)^(k+1) (R!)^2 / (k^2 (R-k)! (R+k)!), a_0 = -2 sum_k a_k.
int orc_fd_coeffs(int order, double* a) {
    if (order != 2 && order != 4 && order != 6 && order != 8) return -1;
    const int R = order / 2;
    auto fact = [](int n) {
        double f = 1;
        for (int i = 2; i <= n; ++i) f *= i;
        return f;
    };
    double s = 0;
    for (int k = 1; k <= R; ++k) {
        a[k] = 2.0 * ((k % 2) ? 1.0 : -1.0) * fact(R) * fact(R) /
               (double(k) * k * fact(R - k) * fact(R + k));
        s += a[k];
    }
    a[0] = -2.0 * s;
    return 0;
}

}  // extern "C"

namespace {

struct Grid {
    int ndim, R, nz, ny, nx;
    long ncell;
    long sz, sy;  // strides of z and y
    double az[5], ay[5], ax[5];  // per-axis weights a_k / h^2
    double diag;                  // sum of the axis a_0 / h^2
};

Grid make_grid(const orc_problem& p) {
    Grid g{};
    g.ndim = p.ndim;
    g.R = p.order / 2;
    g.nz = p.nz;
    g.ny = p.ndim == 3 ? p.ny : 1;
    g.nx = p.nx;
    g.ncell = (long)g.nz * g.ny * g.nx;
    g.sy = g.nx;
    g.sz = (long)g.ny * g.nx;
    double a[5] = {0, 0, 0, 0, 0};
    orc_fd_coeffs(p.order, a);
    for (int k = 0; k <= g.R; ++k) {
        g.az[k] = a[k] / (p.dz * p.dz);
        g.ax[k] = a[k] / (p.dx * p.dx);
        g.ay[k] = p.ndim == 3 ? a[k] / (p.dy * p.dy) : 0.0;
    }
    g.diag = g.az[0] + g.ax[0] + (p.ndim == 3 ? g.ay[0] : 0.0);
    return g;
}

inline bool interior(const Grid& g, int z, int y, int x) {
    const int R = g.R;
    if (z < R || z >= g.nz - R || x < R || x >= g.nx - R) return false;
    if (g.ndim == 3 && (y < R || y >= g.ny - R)) return false;
    return true;
}

inline double laplacian(const Grid& g, const double* u, long c) {
    double s = g.diag * u[c];
    for (int k = 1; k <= g.R; ++k) {
        s += g.az[k] * (u[c - k * g.sz] + u[c + k * g.sz]);
        s += g.ax[k] * (u[c - k] + u[c + k]);
        if (g.ndim == 3) s += g.ay[k] * (u[c - k * g.sy] + u[c + k * g.sy]);
    }
    return s;
}

// Per-cell sponge factor from the 1D profiles (null profile = 1).
struct Sponge {
    const double *gz, *gy, *gx;
    double at(int z, int y, int x) const {
        double g = 1.0;
        if (gz) g *= gz[z];
        if (gy) g *= gy[y];
        if (gx) g *= gx[x];
        return g;
    }
};

// One interior update: un = g (2 uc + w Lap(uc)) - g^2 uo, w = v^2 dt^2.
// Writes only interior cells; lap_out (optional) receives Lap(uc) there.
void step(const Grid& g, const Sponge& sp, const double* w, const double* uo,
          const double* uc, double* un, double* lap_out) {
#pragma omp parallel for schedule(static)
    for (int z = 0; z < g.nz; ++z)
        for (int y = 0; y < g.ny; ++y)
            for (int x = 0; x < g.nx; ++x) {
                if (!interior(g, z, y, x)) continue;
                const long c = z * g.sz + y * g.sy + x;
                const double L = laplacian(g, uc, c);
                const double gg = sp.at(z, y, x);
                un[c] = gg * (2.0 * uc[c] + w[c] * L) - gg * gg * uo[c];
                if (lap_out) lap_out[c] = L;
            }
}

long cell_of(const Grid& g, const int32_t* pos) {
    return (long)pos[0] * g.sz + (long)pos[1] * g.sy + pos[2];
}

bool positions_ok(const Grid& g, const int32_t* pos, long n) {
    for (long i = 0; i < n; ++i) {
        const int32_t* q = pos + 3 * i;
        if (!interior(g, q[0], g.ndim == 3 ? q[1] : g.R, q[2])) return false;
        if (g.ndim == 2 && q[1] != 0) return false;
    }
    return true;
}

}  // namespace

extern "C" {

// One step of the generic update on dense arrays:
// un = g (2 uc + w Lap uc) - g^2 uo on the interior; the ring of un is left
// untouched. w is per cell (v^2 dt^2) when w_field is given, else w_const.
int orc_step(const orc_problem* p, const double* w_field, double w_const, const double* gz,
             const double* gy, const double* gx, const double* uo, const double* uc,
             double* un) {
    const Grid g = make_grid(*p);
    std::vector<double> wc;
    if (!w_field) {
        wc.assign(g.ncell, w_const);
        w_field = wc.data();
    }
    step(g, Sponge{gz, gy, gx}, w_field, uo, uc, un, nullptr);
    return 0;
}

// Forward modelling of nshot shots sharing one velocity model.
// vel[ncell], wavelet[nshot][nt][nsrc], src[nshot][nsrc][3], rec[nshot][nrec][3]
// (z, y, x; y = 0 in 2D) -> traces[nshot][nt][nrec], traces[s][n] = u_{n+1}(rec).
// u_final (optional) receives u_nt of every shot, [nshot][ncell].
int orc_forward(const orc_problem* p, const double* vel, const double* gz, const double* gy,
                const double* gx, const double* wavelet, const int32_t* src,
                const int32_t* rec, double* traces, double* u_final) {
    const Grid g = make_grid(*p);
    if (!positions_ok(g, src, (long)p->nshot * p->nsrc) ||
        !positions_ok(g, rec, (long)p->nshot * p->nrec))
        return -2;
    std::vector<double> w(g.ncell);
    for (long c = 0; c < g.ncell; ++c) w[c] = vel[c] * vel[c] * p->dt * p->dt;
    const Sponge sp{gz, gy, gx};
    std::vector<double> ua(g.ncell), ub(g.ncell);
    for (int s = 0; s < p->nshot; ++s) {
        std::fill(ua.begin(), ua.end(), 0.0);
        std::fill(ub.begin(), ub.end(), 0.0);
        double* uo = ua.data();  // u_{n-1}
        double* uc = ub.data();  // u_n
        const int32_t* sp_pos = src + 3L * s * p->nsrc;
        const int32_t* rp_pos = rec + 3L * s * p->nrec;
        for (int n = 0; n < p->nt; ++n) {
            step(g, sp, w.data(), uo, uc, uo, nullptr);  // uo now holds u_{n+1}
            for (int i = 0; i < p->nsrc; ++i) {
                const int32_t* q = sp_pos + 3 * i;
                const long c = cell_of(g, q);
                uo[c] += sp.at(q[0], q[1], q[2]) * p->src_scale *
                         wavelet[((long)s * p->nt + n) * p->nsrc + i];
            }
            for (int r = 0; r < p->nrec; ++r)
                traces[((long)s * p->nt + n) * p->nrec + r] = uo[cell_of(g, rp_pos + 3 * r)];
            std::swap(uo, uc);
        }
        if (u_final) std::memcpy(u_final + (long)s * g.ncell, uc, sizeof(double) * g.ncell);
    }
    return 0;
}

// Misfit J = 1/2 sum_{s,n,r} (d - d_obs)^2 and its exact discrete gradient.
//
// Adjoint, in the scaled variable q = w g mu (mu the Lagrange multiplier):
//   q_k = g (2 q_{k+1} + w L q_{k+1} + w P^T r_{k-1}) - g^2 q_{k+2},
//   k = nt .. 1, q_{nt+1} = q_{nt+2} = 0, r_n = d_n - d_obs_n,
// which is the forward update itself (L is symmetric on the interior).
//   dJ/dw      = sum_{n=0}^{nt-1} q_{n+1} L u_n / w
//   dJ/dv      = 2 v dt^2 dJ/dw
//   dJ/dwav_n  = s * q_{n+1}(src) / w(src)
// Forward states are recomputed per segment from exact FP64 checkpoints of
// (u_{k-1}, u_k) every ckpt_every steps.
// Outputs: grad_vel[ncell] (summed over shots), grad_wavelet[nshot][nt][nsrc]
// (optional), traces[nshot][nt][nrec] (optional), *misfit.
int orc_gradient(const orc_problem* p, const double* vel, const double* gz, const double* gy,
                 const double* gx, const double* wavelet, const int32_t* src,
                 const int32_t* rec, const double* observed, double* grad_vel,
                 double* grad_wavelet, double* traces, double* misfit) {
    const Grid g = make_grid(*p);
    if (!positions_ok(g, src, (long)p->nshot * p->nsrc) ||
        !positions_ok(g, rec, (long)p->nshot * p->nrec))
        return -2;
    const long N = g.ncell;
    const int nt = p->nt;
    const int K = p->ckpt_every > 0 ? p->ckpt_every : (int)std::ceil(std::sqrt((double)nt));
    const int nseg = (nt + K - 1) / K;
    std::vector<double> w(N);
    for (long c = 0; c < N; ++c) w[c] = vel[c] * vel[c] * p->dt * p->dt;
    const Sponge sp{gz, gy, gx};

    std::vector<double> G(N, 0.0);
    std::vector<double> ua(N), ub(N), qa(N), qb(N);
    std::vector<double> ckpt((size_t)nseg * 2 * N);
    std::vector<double> lap((size_t)K * N);
    std::vector<double> d((size_t)nt * p->nrec), res((size_t)nt * p->nrec);
    double J = 0.0;

    for (int s = 0; s < p->nshot; ++s) {
        const int32_t* sp_pos = src + 3L * s * p->nsrc;
        const int32_t* rp_pos = rec + 3L * s * p->nrec;
        const double* wav = wavelet + (long)s * nt * p->nsrc;
        auto inject = [&](double* u, int n) {
            for (int i = 0; i < p->nsrc; ++i) {
                const int32_t* q = sp_pos + 3 * i;
                u[cell_of(g, q)] += sp.at(q[0], q[1], q[2]) * p->src_scale * wav[n * p->nsrc + i];
            }
        };
        // forward pass with checkpoints of (u_{k-1}, u_k) at k = j K
        std::fill(ua.begin(), ua.end(), 0.0);
        std::fill(ub.begin(), ub.end(), 0.0);
        double* uo = ua.data();
        double* uc = ub.data();
        for (int n = 0; n < nt; ++n) {
            if (n % K == 0) {
                std::memcpy(&ckpt[(size_t)(n / K) * 2 * N], uo, sizeof(double) * N);
                std::memcpy(&ckpt[(size_t)(n / K) * 2 * N + N], uc, sizeof(double) * N);
            }
            step(g, sp, w.data(), uo, uc, uo, nullptr);
            inject(uo, n);
            for (int r = 0; r < p->nrec; ++r) d[(size_t)n * p->nrec + r] = uo[cell_of(g, rp_pos + 3 * r)];
            std::swap(uo, uc);
        }
        const double* obs = observed + (long)s * nt * p->nrec;
        for (size_t i = 0; i < d.size(); ++i) {
            res[i] = d[i] - obs[i];
            J += 0.5 * res[i] * res[i];
        }
        if (traces) std::memcpy(traces + (long)s * nt * p->nrec, d.data(), sizeof(double) * d.size());

        // adjoint pass, segment by segment from the last
        std::fill(qa.begin(), qa.end(), 0.0);
        std::fill(qb.begin(), qb.end(), 0.0);
        double* qo = qa.data();  // q_{k+2}
        double* qc = qb.data();  // q_{k+1}
        auto adjoint_step = [&](int k) {  // produces q_k into qo, then rotates
            step(g, sp, w.data(), qo, qc, qo, nullptr);
            for (int r = 0; r < p->nrec; ++r) {
                const int32_t* q = rp_pos + 3 * r;
                const long c = cell_of(g, q);
                qo[c] += sp.at(q[0], q[1], q[2]) * w[c] * res[(size_t)(k - 1) * p->nrec + r];
            }
            std::swap(qo, qc);  // qc = q_k
        };
        double* gw = grad_wavelet ? grad_wavelet + (long)s * nt * p->nsrc : nullptr;
        auto sample_wavelet_grad = [&](int n, const double* q_np1) {  // q_{n+1}
            if (!gw) return;
            for (int i = 0; i < p->nsrc; ++i) {
                const long c = cell_of(g, sp_pos + 3 * i);
                gw[n * p->nsrc + i] = p->src_scale * q_np1[c] / w[c];
            }
        };
        adjoint_step(nt);  // q_nt (its gradient term pairs q_{nt+1} = 0)
        for (int j = nseg - 1; j >= 0; --j) {
            const int k0 = j * K, k1 = std::min(nt, k0 + K);
            // recompute u_k and L u_k for k in [k0, k1)
            std::memcpy(ua.data(), &ckpt[(size_t)j * 2 * N], sizeof(double) * N);
            std::memcpy(ub.data(), &ckpt[(size_t)j * 2 * N + N], sizeof(double) * N);
            uo = ua.data();
            uc = ub.data();
            for (int k = k0; k < k1; ++k) {
                step(g, sp, w.data(), uo, uc, uo, &lap[(size_t)(k - k0) * N]);
                // lap of the ring is never read: gradient terms are interior only
                inject(uo, k);
                std::swap(uo, uc);
            }
            for (int k = k1 - 1; k >= std::max(k0, 1); --k) {
                // qc = q_{k+1}: gradient term q_{k+1} L u_k, wavelet term n = k
                const double* L = &lap[(size_t)(k - k0) * N];
#pragma omp parallel for schedule(static)
                for (long c = 0; c < N; ++c) G[c] += qc[c] * L[c];
                sample_wavelet_grad(k, qc);
                adjoint_step(k);  // qc = q_k
            }
        }
        sample_wavelet_grad(0, qc);  // qc = q_1
    }
    // G accumulates sum q L u on the interior (ring cells stay 0)
    for (int z = 0; z < g.nz; ++z)
        for (int y = 0; y < g.ny; ++y)
            for (int x = 0; x < g.nx; ++x) {
                const long c = z * g.sz + y * g.sy + x;
                grad_vel[c] = interior(g, z, y, x) ? 2.0 * vel[c] * p->dt * p->dt * G[c] / w[c] : 0.0;
            }
    *misfit = J;
    return 0;
}


}  // extern "C"

// ---------------------------------------------------------------------------
// Variable density (2D): the conservative acoustic operator
//     p_tt = kappa div(b grad p) + s,   b = 1 / rho,
// the two-phase medium of cuwave's AcousticWave (projects/8_physics_drivers/
// waveND.py:52-65; 1_benchmark_2D/README.md:141-144: 1/rho and 1/kappa are the
// interpolated quantities). Staggered differences of order 2R on a unit grid,
//     (D f)_j = sum_k c_k (f_{j+k} - f_{j-k+1})   at the half point j + 1/2,
// c_k = 1/(2k-1) prod_{m != k} (2m-1)^2 / ((2m-1)^2 - (2k-1)^2), fluxes
// F = b_half D u with b_half the mean of the two cells' b, and
//     Lb u = sum_k c_k (Fx_{x+k-1} - Fx_{x-k}) + sz sum_k c_k (Fz_{z+k-1} - Fz_{z-k}),
// sz = (dx/dz)^2. Fields and b are zero outside the grid. The update on the
// interior is u_{n+1} = g (2 u_n + k Lb u_n + s w_n) - g^2 u_{n-1}, k = kappa dt^2/dx^2;
// k b = (c dt / dx)^2 recovers the constant-density scaling.
//
// Lb = -Dx^T Bx Dx - sz Dz^T Bz Dz is symmetric, so the adjoint in q = k g mu is
// the same update with k-weighted residuals injected, and
//     dJ/dk_c      = sum_n q_{n+1,c} (Lb u_n)_c / k_c,
//     dJ/dbx_{z,j} = -sum_n (Dx q_{n+1})_{z,j} (Dx u_n)_{z,j},  dJ/dbz likewise times sz,
//     dJ/db_c      = (dJ/dbx_{x-1} + dJ/dbx_x + dJ/dbz_{z-1} + dJ/dbz_z) / 2,
//     dJ/dkappa = dJ/dk dt^2 / dx^2,  dJ/drho = -dJ/db / rho^2.
// The forward states are kept in full (FP64, small problems).
namespace {

void stag_coeffs(int R, double* c) {
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

struct VdGrid {
    int R, nz, nx;
    double c[5], sz;
};

// value of a zero-extended field
inline double at(const VdGrid& g, const double* f, int z, int x) {
    return (z < 0 || z >= g.nz || x < 0 || x >= g.nx) ? 0.0 : f[(long)z * g.nx + x];
}
inline double dx_half(const VdGrid& g, const double* f, int z, int j) {  // (Dx f) at (z, j + 1/2)
    double s = 0;
    for (int k = 1; k <= g.R; ++k) s += g.c[k] * (at(g, f, z, j + k) - at(g, f, z, j - k + 1));
    return s;
}
inline double dz_half(const VdGrid& g, const double* f, int i, int x) {  // (Dz f) at (i + 1/2, x)
    double s = 0;
    for (int k = 1; k <= g.R; ++k) s += g.c[k] * (at(g, f, i + k, x) - at(g, f, i - k + 1, x));
    return s;
}
inline double bx_half(const VdGrid& g, const double* b, int z, int j) {
    return 0.5 * (at(g, b, z, j) + at(g, b, z, j + 1));
}
inline double bz_half(const VdGrid& g, const double* b, int i, int x) {
    return 0.5 * (at(g, b, i, x) + at(g, b, i + 1, x));
}
inline double lb(const VdGrid& g, const double* b, const double* u, int z, int x) {
    double s = 0;
    for (int k = 1; k <= g.R; ++k) {
        const int j1 = x + k - 1, j0 = x - k;
        s += g.c[k] * (bx_half(g, b, z, j1) * dx_half(g, u, z, j1) - bx_half(g, b, z, j0) * dx_half(g, u, z, j0));
        const int i1 = z + k - 1, i0 = z - k;
        s += g.sz * g.c[k] *
             (bz_half(g, b, i1, x) * dz_half(g, u, i1, x) - bz_half(g, b, i0, x) * dz_half(g, u, i0, x));
    }
    return s;
}

void vd_step(const VdGrid& g, const Grid& gg, const Sponge& sp, const double* k, const double* b,
             const double* uo, const double* uc, double* un, double* lb_out) {
#pragma omp parallel for schedule(static)
    for (int z = 0; z < g.nz; ++z)
        for (int x = 0; x < g.nx; ++x) {
            if (!interior(gg, z, 0, x)) continue;
            const long c = (long)z * g.nx + x;
            const double L = lb(g, b, uc, z, x);
            const double s = sp.at(z, 0, x);
            un[c] = s * (2.0 * uc[c] + k[c] * L) - s * s * uo[c];
            if (lb_out) lb_out[c] = L;
        }
}

VdGrid make_vd(const orc_problem& p) {
    VdGrid g{};
    g.R = p.order / 2;
    g.nz = p.nz;
    g.nx = p.nx;
    stag_coeffs(g.R, g.c);
    g.sz = (p.dx * p.dx) / (p.dz * p.dz);
    return g;
}

}  // namespace

extern "C" {

int orc_stag_coeffs(int order, double* c) {
    if (order != 2 && order != 4 && order != 8) return -1;
    stag_coeffs(order / 2, c);
    return 0;
}

// Variable-density forward: traces[s][n][r] = u_{n+1}(rec); u_final optional.
int orc_vd_forward(const orc_problem* p, const double* kappa, const double* rho, const double* gz,
                   const double* gx, const double* wavelet, const int32_t* src, const int32_t* rec,
                   double* traces, double* u_final) {
    if (p->ndim != 2) return -1;
    const Grid gg = make_grid(*p);
    const VdGrid g = make_vd(*p);
    if (!positions_ok(gg, src, (long)p->nshot * p->nsrc) || !positions_ok(gg, rec, (long)p->nshot * p->nrec))
        return -2;
    const long N = gg.ncell;
    std::vector<double> k(N), b(N), ua(N), ub(N);
    for (long c = 0; c < N; ++c) {
        k[c] = kappa[c] * p->dt * p->dt / (p->dx * p->dx);
        b[c] = 1.0 / rho[c];
    }
    const Sponge sp{gz, nullptr, gx};
    for (int s = 0; s < p->nshot; ++s) {
        std::fill(ua.begin(), ua.end(), 0.0);
        std::fill(ub.begin(), ub.end(), 0.0);
        double *uo = ua.data(), *uc = ub.data();
        const int32_t* sp_pos = src + 3L * s * p->nsrc;
        const int32_t* rp_pos = rec + 3L * s * p->nrec;
        for (int n = 0; n < p->nt; ++n) {
            vd_step(g, gg, sp, k.data(), b.data(), uo, uc, uo, nullptr);
            for (int i = 0; i < p->nsrc; ++i) {
                const int32_t* q = sp_pos + 3 * i;
                uo[cell_of(gg, q)] += sp.at(q[0], 0, q[2]) * p->src_scale * wavelet[((long)s * p->nt + n) * p->nsrc + i];
            }
            for (int r = 0; r < p->nrec; ++r)
                traces[((long)s * p->nt + n) * p->nrec + r] = uo[cell_of(gg, rp_pos + 3 * r)];
            std::swap(uo, uc);
        }
        if (u_final) std::memcpy(u_final + (long)s * N, uc, sizeof(double) * N);
    }
    return 0;
}

// Misfit J = 1/2 sum (d - d_obs)^2 and its gradient w.r.t. kappa, rho (summed
// over shots) and the wavelets (optional), from the exact discrete adjoint.
int orc_vd_gradient(const orc_problem* p, const double* kappa, const double* rho, const double* gz,
                    const double* gx, const double* wavelet, const int32_t* src, const int32_t* rec,
                    const double* observed, double* grad_kappa, double* grad_rho, double* grad_wavelet,
                    double* traces, double* misfit) {
    if (p->ndim != 2) return -1;
    const Grid gg = make_grid(*p);
    const VdGrid g = make_vd(*p);
    if (!positions_ok(gg, src, (long)p->nshot * p->nsrc) || !positions_ok(gg, rec, (long)p->nshot * p->nrec))
        return -2;
    const long N = gg.ncell;
    const int nt = p->nt;
    std::vector<double> k(N), b(N);
    for (long c = 0; c < N; ++c) {
        k[c] = kappa[c] * p->dt * p->dt / (p->dx * p->dx);
        b[c] = 1.0 / rho[c];
    }
    const Sponge sp{gz, nullptr, gx};
    std::vector<double> GK(N, 0.0), GBX(N, 0.0), GBZ(N, 0.0);  // half points (z, x + 1/2), (z + 1/2, x)
    std::vector<double> U((size_t)(nt + 1) * N), qa(N), qb(N), L(N);
    std::vector<double> d((size_t)nt * p->nrec), res((size_t)nt * p->nrec);
    double J = 0.0;
    for (int s = 0; s < p->nshot; ++s) {
        const int32_t* sp_pos = src + 3L * s * p->nsrc;
        const int32_t* rp_pos = rec + 3L * s * p->nrec;
        const double* wav = wavelet + (long)s * nt * p->nsrc;
        // forward, every level kept: U[n] = u_n, n = 0 .. nt (u_0 = u_{-1} = 0)
        std::fill(U.begin(), U.begin() + N, 0.0);
        std::vector<double> um(N, 0.0);
        for (int n = 0; n < nt; ++n) {
            double* un = &U[(size_t)(n + 1) * N];
            const double* uc = &U[(size_t)n * N];
            const double* uo = n == 0 ? um.data() : &U[(size_t)(n - 1) * N];
            std::fill(un, un + N, 0.0);
            vd_step(g, gg, sp, k.data(), b.data(), uo, uc, un, nullptr);
            for (int i = 0; i < p->nsrc; ++i) {
                const int32_t* q = sp_pos + 3 * i;
                un[cell_of(gg, q)] += sp.at(q[0], 0, q[2]) * p->src_scale * wav[n * p->nsrc + i];
            }
            for (int r = 0; r < p->nrec; ++r) d[(size_t)n * p->nrec + r] = un[cell_of(gg, rp_pos + 3 * r)];
        }
        const double* obs = observed + (long)s * nt * p->nrec;
        for (size_t i = 0; i < d.size(); ++i) {
            res[i] = d[i] - obs[i];
            J += 0.5 * res[i] * res[i];
        }
        if (traces) std::memcpy(traces + (long)s * nt * p->nrec, d.data(), sizeof(double) * d.size());
        // adjoint: q_k = g (2 q_{k+1} + k Lb q_{k+1} + k P^T r_{k-1}) - g^2 q_{k+2}
        std::fill(qa.begin(), qa.end(), 0.0);
        std::fill(qb.begin(), qb.end(), 0.0);
        double *qo = qa.data(), *qc = qb.data();
        auto adjoint_step = [&](int kk) {
            vd_step(g, gg, sp, k.data(), b.data(), qo, qc, qo, nullptr);
            for (int r = 0; r < p->nrec; ++r) {
                const int32_t* q = rp_pos + 3 * r;
                const long c = cell_of(gg, q);
                qo[c] += sp.at(q[0], 0, q[2]) * k[c] * res[(size_t)(kk - 1) * p->nrec + r];
            }
            std::swap(qo, qc);
        };
        double* gw = grad_wavelet ? grad_wavelet + (long)s * nt * p->nsrc : nullptr;
        adjoint_step(nt);
        for (int n = nt - 1; n >= 0; --n) {
            // qc = q_{n+1}: the terms of u_n
            const double* u = &U[(size_t)n * N];
#pragma omp parallel for schedule(static)
            for (int z = 0; z < g.nz; ++z)
                for (int x = 0; x < g.nx; ++x) {
                    const long c = (long)z * g.nx + x;
                    if (interior(gg, z, 0, x)) GK[c] += qc[c] * lb(g, b.data(), u, z, x);
                    GBX[c] -= dx_half(g, qc, z, x) * dx_half(g, u, z, x);
                    GBZ[c] -= g.sz * dz_half(g, qc, z, x) * dz_half(g, u, z, x);
                }
            if (gw)
                for (int i = 0; i < p->nsrc; ++i) {
                    const long c = cell_of(gg, sp_pos + 3 * i);
                    gw[n * p->nsrc + i] = p->src_scale * qc[c] / k[c];
                }
            if (n >= 1) adjoint_step(n);
        }
    }
    for (int z = 0; z < g.nz; ++z)
        for (int x = 0; x < g.nx; ++x) {
            const long c = (long)z * g.nx + x;
            grad_kappa[c] = interior(gg, z, 0, x) ? GK[c] / k[c] * p->dt * p->dt / (p->dx * p->dx) : 0.0;
            const double db = 0.5 * ((x > 0 ? GBX[c - 1] : 0.0) + GBX[c] + (z > 0 ? GBZ[c - g.nx] : 0.0) + GBZ[c]);
            grad_rho[c] = -db / (rho[c] * rho[c]);
        }
    *misfit = J;
    return 0;
}

}  // extern "C"
