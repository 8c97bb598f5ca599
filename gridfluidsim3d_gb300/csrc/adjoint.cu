// adjoint.cu -- the differentiable FLIP rollout: forward with per-substep
// checkpoints, and the hand-written adjoint of every stage of the substep.
//
// Forward (gfs_diff_forward): particles start at the given positions with
// velocities sampled from a parameter MAC field (Catmull-Rom, as G2P samples),
// run `nsteps` substeps of the device-resident core (capi.cu sim_step), and the
// output is the cell-centred particle density (splat kernel of radius 1.5 dx).
// The particle state at the start of every substep and every substep's pressure
// are kept in HBM.
//
// Backward (gfs_diff_backward), substep by substep in reverse, with the
// discrete structure (fluid cells, splat set masks, fill contributors,
// extrapolation layers) of the substep held fixed:
//   1. recompute the substep's grids from its checkpoint (classify, splat with
//      weight sums, fill, layers, saved extrapolation, pressure set-up, apply of
//      the checkpointed pressure, extrapolation);
//   2. k_adj_g2p: per particle, the adjoint of the FLIP update and of RK4
//      through the Jacobians of the Catmull-Rom samples; the sample adjoints
//      scatter into the MAC / saved adjoint face grids.  The scatter is in
//      fixed point (64-bit integer atomics at a per-pass power-of-two scale
//      found by a first pass over the particles), so the grids, and every
//      gradient computed from them, are bitwise the same from run to run;
//   3. k_adj_extrap_layer: adjoint of each extrapolation layer pass, in reverse
//      layer order (a gather: a face receives from the layer faces it fed);
//   4. pressure: p_bar = -k G^T u_bar on the fluid cells (k_adj_pbar), then
//      A lambda = p_bar with the same MIC(0)-PCG on the same (symmetric)
//      matrix, then u_bar += D^T lambda / dx and the apply pass-through
//      (k_adj_div);
//   5. body force: identity; the filled field's adjoint is the MAC's plus the
//      saved field's;
//   6. k_fill_count + k_adj_fill: adjoint of the 26-neighbour fill;
//   7. k_adj_p2g: per particle, the adjoint of u = sum w v / sum w (a gather
//      over the faces within dx of the particle, quotient rule for the weights).
// Adjoints travel per particle id, since every substep re-sorts the particles.
// A solid collision is differentiated through its placement (the end point
// pulled back before the entry plane of the first solid voxel, with the voxel
// and the plane held fixed).  Removals (particles left in solid cells, the
// per-cell cap) are not differentiated: a particle removed during a substep has
// zero adjoint from then on.
#include <cmath>
#include <cstring>
#include <vector>

#include "gfs_internal.h"
#include "gfs_interp.cuh"

namespace gfs {

static constexpr double DIFF_DENSITY_RADIUS = 1.5;   // cells

__device__ __forceinline__ uint32_t pid(const float4 &P) { return __float_as_uint(P.w); }

// w(s) = (1-s)^2 (1 - 4s/9) and dw/ds, s = r^2 / R^2 < 1
__device__ __forceinline__ float kern_w(float s) {
    float a = 1.0f - s;
    return a * a * (1.0f - (4.0f / 9.0f) * s);
}
__device__ __forceinline__ float kern_dw(float s) {
    float a = 1.0f - s;
    return -2.0f * a * (1.0f - (4.0f / 9.0f) * s) - (4.0f / 9.0f) * a * a;
}

__device__ __forceinline__ float dist2_exact(float ax, float ay, float az) {
    return __fadd_rn(__fadd_rn(__fmul_rn(ax, ax), __fmul_rn(ay, ay)), __fmul_rn(az, az));
}

// --------------------------------------------------------- pad / unpad

__global__ void k_diff_pad(const float *__restrict__ src, GridDim f, float *__restrict__ dst) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y, k = blockIdx.z;
    if (i >= f.nx) return;
    dst[f.at(i, j, k)] = src[i + (long long)f.nx * (j + (long long)f.ny * k)];
}

__global__ void k_diff_unpad(const float *__restrict__ src, GridDim f, float *__restrict__ dst) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y, k = blockIdx.z;
    if (i >= f.nx) return;
    dst[i + (long long)f.nx * (j + (long long)f.ny * k)] = src[f.at(i, j, k)];
}

// ------------------------------------------------------- forward pieces

__global__ void k_diff_pack(const float *__restrict__ pts, long long n, float4 *__restrict__ pos,
                            float4 *__restrict__ vel) {
    long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= n) return;
    pos[q] = make_float4(pts[3 * q], pts[3 * q + 1], pts[3 * q + 2], __uint_as_float((uint32_t)q));
    vel[q] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// initial velocities: Catmull-Rom samples of the parameter field
__global__ void k_diff_sample(AdvArgs A, const float4 *__restrict__ pos, float4 *__restrict__ vel, long long n,
                              const float *__restrict__ u, const float *__restrict__ v, const float *__restrict__ w) {
    long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= n) return;
    float4 P = pos[q];
    float3 s = eval_velocity(A, u, v, w, P.x, P.y, P.z);
    vel[q] = make_float4(s.x, s.y, s.z, 0.f);
}

// cell-centred density, one thread per cell over the particles of the 27
// surrounding cells (particles sorted by cell: `offset` is the cell start list)
__global__ void k_diff_density(GridDim c, double dx, const float4 *__restrict__ pos,
                               const uint32_t *__restrict__ offset, float inv_r2, float *__restrict__ rho) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y, k = blockIdx.z;
    if (i >= c.nx) return;
    const float cx = (float)(((double)i + 0.5) * dx), cy = (float)(((double)j + 0.5) * dx),
                cz = (float)(((double)k + 0.5) * dx);
    float acc = 0.f;
    for (int kk = k - 1; kk <= k + 1; kk++) {
        if (kk < 0 || kk >= c.nz) continue;
        for (int jj = j - 1; jj <= j + 1; jj++) {
            if (jj < 0 || jj >= c.ny) continue;
            long long row = (long long)c.nx * (jj + (long long)c.ny * kk);
            int i0 = max(i - 1, 0), i1 = min(i + 1, c.nx - 1);
            for (uint32_t q = offset[row + i0]; q < offset[row + i1 + 1]; q++) {
                float4 P = pos[q];
                float s = dist2_exact(cx - P.x, cy - P.y, cz - P.z) * inv_r2;
                if (s < 1.0f) acc += kern_w(s);
            }
        }
    }
    rho[i + (long long)c.nx * (j + (long long)c.ny * k)] = acc;
}

// x_bar of the density: sum over the cells near the particle of rho_bar dw/dx
__global__ void k_adj_density(GridDim c, double dx, const float4 *__restrict__ pos, long long n,
                              const float *__restrict__ rho_bar, float inv_r2, float4 *__restrict__ ax,
                              float4 *__restrict__ av) {
    long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= n) return;
    float4 P = pos[q];
    int ci = (int)floor((double)P.x / dx - 0.5), cj = (int)floor((double)P.y / dx - 0.5),
        ck = (int)floor((double)P.z / dx - 0.5);
    float gx = 0.f, gy = 0.f, gz = 0.f;
    for (int kk = ck - 1; kk <= ck + 2; kk++)
        for (int jj = cj - 1; jj <= cj + 2; jj++)
            for (int ii = ci - 1; ii <= ci + 2; ii++) {
                if (ii < 0 || jj < 0 || kk < 0 || ii >= c.nx || jj >= c.ny || kk >= c.nz) continue;
                float ex = (float)(((double)ii + 0.5) * dx) - P.x, ey = (float)(((double)jj + 0.5) * dx) - P.y,
                      ez = (float)(((double)kk + 0.5) * dx) - P.z;
                float s = dist2_exact(ex, ey, ez) * inv_r2;
                if (!(s < 1.0f)) continue;
                float rb = rho_bar[ii + (long long)c.nx * (jj + (long long)c.ny * kk)];
                // d w / d x_p = w'(s) * (-2 (node - x_p)) / R^2
                float f = rb * kern_dw(s) * (-2.0f * inv_r2);
                gx += f * ex;
                gy += f * ey;
                gz += f * ez;
            }
    uint32_t id = pid(P);
    ax[id] = make_float4(gx, gy, gz, 0.f);
    av[id] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// ---------------------------------------------- 2. FLIP + RK4 adjoint

__device__ __forceinline__ float3 mtv(const float J[3][3], float3 c) {   // J^T c
    return make_float3(J[0][0] * c.x + J[1][0] * c.y + J[2][0] * c.z, J[0][1] * c.x + J[1][1] * c.y + J[2][1] * c.z,
                       J[0][2] * c.x + J[1][2] * c.y + J[2][2] * c.z);
}
__device__ __forceinline__ float3 f3add(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 f3scale(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }

// Fixed-point scale of one scatter pass: terms are rounded to multiples of inv = 2^-S.
struct FixScale {
    double scale, inv;   // 2^S, 2^-S (0 when there is nothing to scatter)
    unsigned maxbits;    // largest |scatter value| of the pass, as float bits
};

// S = 61 - e - lg with max |value| < 2^e and at most 2^lg terms per node: every
// term is below 2^(61 - lg) in magnitude, so no node sum leaves (-2^61, 2^61).
// A value that is not finite sets *status and leaves the pass without a scatter.
__global__ void k_fix_scale(FixScale *fs, int lg, unsigned *status) {
    const unsigned b = fs->maxbits;
    if (b == 0u || b >= 0x7f800000u) {
        fs->scale = 0.0;
        fs->inv = 0.0;
        if (b) *status = 1u;
        return;
    }
    const int e = (int)max(b >> 23, 1u) - 126;
    const int S = 61 - e - lg;
    fs->scale = __longlong_as_double((long long)(S + 1023) << 52);
    fs->inv = __longlong_as_double((long long)(1023 - S) << 52);
}

__global__ void k_fix_unpack(const unsigned long long *__restrict__ acc, long long n, const FixScale *__restrict__ fs,
                             float *__restrict__ out) {
    long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q < n) out[q] = (float)((double)(long long)acc[q] * fs->inv);
}

// One particle of the G2P / RK4 adjoint.  SCALE_PASS: only the largest |value| the
// particle scatters (float bits); otherwise the fixed-point scatter and the
// per-particle adjoints.
template <bool SCALE_PASS>
__device__ __forceinline__ unsigned adj_g2p_particle(const AdvArgs &A, long long q, const float4 *__restrict__ pos,
                                                     const float *__restrict__ mu, const float *__restrict__ mv,
                                                     const float *__restrict__ mw, const float *__restrict__ su,
                                                     const float *__restrict__ sv, const float *__restrict__ sw,
                                                     const float4 *__restrict__ ax_in,
                                                     const float4 *__restrict__ av_in, float4 *__restrict__ ax_out,
                                                     float4 *__restrict__ av_out, unsigned long long *__restrict__ gmu,
                                                     unsigned long long *__restrict__ gmv,
                                                     unsigned long long *__restrict__ gmw,
                                                     unsigned long long *__restrict__ gsu,
                                                     unsigned long long *__restrict__ gsv,
                                                     unsigned long long *__restrict__ gsw,
                                                     const uint8_t *__restrict__ mat, double scale) {
    unsigned mb = 0u;
    auto scatter_velocity = [&](unsigned long long *gu, unsigned long long *gv, unsigned long long *gw, float px,
                                float py, float pz, float3 c) {
        if (SCALE_PASS)
            mb = abs_bits_max(mb, c);
        else
            scatter_velocity_fixed(A, gu, gv, gw, px, py, pz, c, scale);
    };
    const float4 P = pos[q];
    const uint32_t id = pid(P);
    const float4 XB = ax_in[id], VB = av_in[id];
    const float3 x = make_float3(P.x, P.y, P.z);
    const float3 xb = make_float3(XB.x, XB.y, XB.z), vb = make_float3(VB.x, VB.y, VB.z);
    // forward recompute (k_g2p_advect): samples and the RK4 stage points
    float Ja[3][3], Js[3][3], J2[3][3], J3[3][3], J4[3][3];
    float3 k1 = eval_velocity_jac(A, mu, mv, mw, x.x, x.y, x.z, Ja);
    eval_velocity_jac(A, su, sv, sw, x.x, x.y, x.z, Js);
    float3 y2 = axpy3(x, A.h, k1);
    float3 k2 = eval_velocity_jac(A, mu, mv, mw, y2.x, y2.y, y2.z, J2);
    float3 y3 = axpy3(x, A.h, k2);
    float3 k3 = eval_velocity_jac(A, mu, mv, mw, y3.x, y3.y, y3.z, J3);
    float3 y4 = axpy3(x, A.f1, k3);
    float3 k4 = eval_velocity_jac(A, mu, mv, mw, y4.x, y4.y, y4.z, J4);
    // the step's end point and its collision, exactly as k_g2p_advect forms them
    float3 p1 = make_float3(rk4_comb(x.x, A.f6, k1.x, k2.x, k3.x, k4.x), rk4_comb(x.y, A.f6, k1.y, k2.y, k3.y, k4.y),
                            rk4_comb(x.z, A.f6, k1.z, k2.z, k3.z, k4.z));
    float3 xb_rk = xb, xb_direct = make_float3(0.f, 0.f, 0.f);
    {
        int ci, cj, ck;
        pos_cell(A, p1.x, p1.y, p1.z, ci, cj, ck);
        if (!(isfinite(p1.x) && isfinite(p1.y) && isfinite(p1.z)) || cell_solid(A, mat, ci, cj, ck)) {
            CollisionHit hit;
            resolve_collision(A, mat, x, p1, &hit);
            if (!hit.moved) {
                // the particle kept its position: p1' = p0
                xb_rk = make_float3(0.f, 0.f, 0.f);
                xb_direct = xb;
            } else {
                // p1' = p0 + ((b - p0_a) / u_a - back) u, u = (p1 - p0) / |p1 - p0|, entry plane x_a = b
                // (resolve_collision, collision.cpp:404-449), differentiated in p0 and p1
                const float q[3] = {p1.x - x.x, p1.y - x.y, p1.z - x.z};
                const float L = sqrtf(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
                const float u[3] = {q[0] / L, q[1] / L, q[2] / L};
                const float g[3] = {xb.x, xb.y, xb.z};
                const float p0a[3] = {x.x, x.y, x.z};
                const int a = hit.axis;
                const float ua = u[a];
                const float back = (float)(0.05 * A.dx);
                const float da = hit.plane - p0a[a];
                const float sv = da / ua - back;
                const float ug = u[0] * g[0] + u[1] * g[1] + u[2] * g[2];
                float qb[3], dr[3];
                for (int c = 0; c < 3; c++) {
                    float ea = c == a ? 1.f : 0.f;
                    qb[c] = -da / (ua * ua * L) * (ea - ua * u[c]) * ug + (sv / L) * (g[c] - u[c] * ug);
                    dr[c] = g[c] - ea * ug / ua - qb[c];
                }
                xb_rk = make_float3(qb[0], qb[1], qb[2]);
                xb_direct = make_float3(dr[0], dr[1], dr[2]);
            }
        }
    }
    // FLIP: v' = a_pic a + b_flip (v + a - s)
    const float3 abar = f3scale(vb, A.a_pic + A.b_flip);
    const float3 sbar = f3scale(vb, -A.b_flip);
    // RK4: x' = x + f6 (k1 + 2 k2 + 2 k3 + k4)
    float3 xbar = f3add(xb_rk, xb_direct);
    float3 kb1 = f3scale(xb_rk, A.f6), kb2 = f3scale(xb_rk, 2.0f * A.f6), kb3 = kb2, kb4 = kb1;
    {   // stage 4: k4 = u(y4), y4 = x + f1 k3
        float3 yb = mtv(J4, kb4);
        scatter_velocity(gmu, gmv, gmw, y4.x, y4.y, y4.z, kb4);
        xbar = f3add(xbar, yb);
        kb3 = f3add(kb3, f3scale(yb, A.f1));
    }
    {   // stage 3: k3 = u(y3), y3 = x + h k2
        float3 yb = mtv(J3, kb3);
        scatter_velocity(gmu, gmv, gmw, y3.x, y3.y, y3.z, kb3);
        xbar = f3add(xbar, yb);
        kb2 = f3add(kb2, f3scale(yb, A.h));
    }
    {   // stage 2: k2 = u(y2), y2 = x + h k1
        float3 yb = mtv(J2, kb2);
        scatter_velocity(gmu, gmv, gmw, y2.x, y2.y, y2.z, kb2);
        xbar = f3add(xbar, yb);
        kb1 = f3add(kb1, f3scale(yb, A.h));
    }
    {   // stage 1 and the FLIP sample: k1 = a = u(x)
        float3 c = f3add(kb1, abar);
        scatter_velocity(gmu, gmv, gmw, x.x, x.y, x.z, c);
        xbar = f3add(xbar, mtv(Ja, c));
    }
    scatter_velocity(gsu, gsv, gsw, x.x, x.y, x.z, sbar);
    if (SCALE_PASS) return mb;
    xbar = f3add(xbar, mtv(Js, sbar));
    ax_out[id] = make_float4(xbar.x, xbar.y, xbar.z, 0.f);
    float3 vbar = f3scale(vb, A.b_flip);
    av_out[id] = make_float4(vbar.x, vbar.y, vbar.z, 0.f);
    return 0u;
}

// The G2P / RK4 adjoint, run twice: the scale pass finds the largest value the
// launch scatters (k_fix_scale turns it into the fixed-point scale), the second
// pass scatters in fixed point and writes the per-particle adjoints.  The
// integer sums make the face-grid adjoints independent of particle order.
template <bool SCALE_PASS>
__global__ void __launch_bounds__(128) k_adj_g2p(AdvArgs A, const float4 *__restrict__ pos,
                                                 const float4 *__restrict__ vel, long long n,
                                                 const float *__restrict__ mu, const float *__restrict__ mv,
                                                 const float *__restrict__ mw, const float *__restrict__ su,
                                                 const float *__restrict__ sv, const float *__restrict__ sw,
                                                 const float4 *__restrict__ ax_in, const float4 *__restrict__ av_in,
                                                 float4 *__restrict__ ax_out, float4 *__restrict__ av_out,
                                                 unsigned long long *__restrict__ gmu,
                                                 unsigned long long *__restrict__ gmv,
                                                 unsigned long long *__restrict__ gmw,
                                                 unsigned long long *__restrict__ gsu,
                                                 unsigned long long *__restrict__ gsv,
                                                 unsigned long long *__restrict__ gsw,
                                                 const uint8_t *__restrict__ mat, FixScale *__restrict__ fs) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const double scale = SCALE_PASS ? 0.0 : fs->scale;
    unsigned mb = 0u;
    if (q < n)
        mb = adj_g2p_particle<SCALE_PASS>(A, q, pos, mu, mv, mw, su, sv, sw, ax_in, av_in, ax_out, av_out, gmu, gmv,
                                          gmw, gsu, gsv, gsw, mat, scale);
    if (SCALE_PASS) {
        mb = __reduce_max_sync(0xffffffffu, mb);
        if ((threadIdx.x & 31) == 0 && mb) atomicMax(&fs->maxbits, mb);
    }
}

// ---------------------------------------------- 3. extrapolation adjoint

__device__ __forceinline__ bool borders_layer(const int8_t *__restrict__ layer, const GridDim &c, int d, int i,
                                              int j, int k, int value) {
    int n = d == 0 ? c.nx : (d == 1 ? c.ny : c.nz);
    int t = d == 0 ? i : (d == 1 ? j : k);
    int pi = i - (d == 0), pj = j - (d == 1), pk = k - (d == 2);
    if (t == n) return layer[c.at(pi, pj, pk)] == value;
    if (t > 0) return layer[c.at(i, j, k)] == value || layer[c.at(pi, pj, pk)] == value;
    return layer[c.at(i, j, k)] == value;
}

__device__ __forceinline__ bool extrap_target(const uint8_t *__restrict__ mat, const int8_t *__restrict__ layer,
                                              const GridDim &c, int d, int i, int j, int k, int L) {
    return borders_layer(layer, c, d, i, j, k, L) && !borders_layer(layer, c, d, i, j, k, L - 1) &&
           !face_borders(mat, c, d, i, j, k, GFS_SOLID);
}

struct AdjExtrapArgs {
    GridDim c, f[3];
    int L;
};

// Layer pass L wrote f = mean over its 6 neighbours g that border layer L-1;
// its adjoint sends f_bar / n_f to each such g and drops f_bar.
__global__ void __launch_bounds__(128) k_adj_extrap_layer(AdjExtrapArgs A, const uint8_t *__restrict__ mat,
                                                          const int8_t *__restrict__ layer,
                                                          const float *__restrict__ gu, const float *__restrict__ gv,
                                                          const float *__restrict__ gw, float *__restrict__ ou,
                                                          float *__restrict__ ov, float *__restrict__ ow) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    int k = blockIdx.z * blockDim.z + threadIdx.z;
    const GridDim &c = A.c;
    if (i > c.nx || j > c.ny || k > c.nz) return;
    const float *gin[3] = {gu, gv, gw};
    float *gout[3] = {ou, ov, ow};
    const int L = A.L;
    const int nb[6][3] = {{-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const GridDim &f = A.f[d];
        if (!f.in(i, j, k)) continue;
        long long at = f.at(i, j, k);
        if (extrap_target(mat, layer, c, d, i, j, k, L)) {
            gout[d][at] = 0.0f;
            continue;
        }
        float acc = gin[d][at];
        if (borders_layer(layer, c, d, i, j, k, L - 1)) {
            for (int q = 0; q < 6; q++) {
                int a = i + nb[q][0], b = j + nb[q][1], e = k + nb[q][2];
                if (!f.in(a, b, e) || !extrap_target(mat, layer, c, d, a, b, e, L)) continue;
                int cnt = 0;
                for (int r = 0; r < 6; r++) {
                    int a2 = a + nb[r][0], b2 = b + nb[r][1], e2 = e + nb[r][2];
                    if (f.in(a2, b2, e2) && borders_layer(layer, c, d, a2, b2, e2, L - 1)) cnt++;
                }
                if (cnt > 0) acc += gin[d][f.at(a, b, e)] / (float)cnt;
            }
        }
        gout[d][at] = acc;
    }
}

// ------------------------------------------------- 4. pressure adjoint

struct AdjPArgs {
    GridDim c, f[3];
    double kscale;     // dt / (density dx)
    double sdiv;       // 1/dx of the divergence (pressuresolver.cpp:164, as k_ps_setup forms it)
    double fscale;     // the solid-face correction's float 1/dx
};

__device__ __forceinline__ bool apply_face(const uint8_t *__restrict__ mat, const GridDim &c, int d, int i, int j,
                                           int k) {
    return face_borders(mat, c, d, i, j, k, GFS_FLUID) && !face_borders(mat, c, d, i, j, k, GFS_SOLID);
}

// p_bar on the fluid cells: u' = u - k (p_hi - p_lo) on the apply faces
__global__ void k_adj_pbar(AdjPArgs A, const uint8_t *__restrict__ mat, const float *__restrict__ gu,
                           const float *__restrict__ gv, const float *__restrict__ gw, double *__restrict__ pbar) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y, k = blockIdx.z;
    const GridDim &c = A.c;
    if (i >= c.nx) return;
    long long e = c.at(i, j, k);
    double acc = 0.0;
    if (mat[e] == GFS_FLUID) {
        const float *g[3] = {gu, gv, gw};
        for (int d = 0; d < 3; d++) {
            // lower face (index = cell): this cell is its upper cell
            if (apply_face(mat, c, d, i, j, k)) acc -= A.kscale * (double)g[d][A.f[d].at(i, j, k)];
            int a = i + (d == 0), b = j + (d == 1), q = k + (d == 2);
            if (apply_face(mat, c, d, a, b, q)) acc += A.kscale * (double)g[d][A.f[d].at(a, b, q)];
        }
    }
    pbar[e] = acc;
}

// u_bar before the apply: the pass-through part plus D^T lambda (b = -div u / dx
// with the solid-face corrections of k_ps_setup)
__global__ void __launch_bounds__(128) k_adj_div(AdjPArgs A, const uint8_t *__restrict__ mat,
                                                 const double *__restrict__ lam, float *__restrict__ gu,
                                                 float *__restrict__ gv, float *__restrict__ gw) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    int k = blockIdx.z * blockDim.z + threadIdx.z;
    const GridDim &c = A.c;
    if (i > c.nx || j > c.ny || k > c.nz) return;
    float *g[3] = {gu, gv, gw};
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const GridDim &f = A.f[d];
        if (!f.in(i, j, k)) continue;
        long long at = f.at(i, j, k);
        double acc = (double)g[d][at];
        if (face_borders(mat, c, d, i, j, k, GFS_FLUID) && face_borders(mat, c, d, i, j, k, GFS_SOLID)) acc = 0.0;
        long long e0 = c.at(i - (d == 0), j - (d == 1), k - (d == 2)), e1 = c.at(i, j, k);
        // cells outside the grid read as solid through the padded material
        bool in1 = c.in(i, j, k), in0 = c.in(i - (d == 0), j - (d == 1), k - (d == 2));
        uint8_t m0 = in0 ? mat[e0] : (uint8_t)GFS_SOLID, m1 = in1 ? mat[e1] : (uint8_t)GFS_SOLID;
        if (m1 == GFS_FLUID) acc += lam[e1] * (A.sdiv - (m0 == GFS_SOLID ? A.fscale : 0.0));
        if (m0 == GFS_FLUID) acc += lam[e0] * (-A.sdiv + (m1 == GFS_SOLID ? A.fscale : 0.0));
        g[d][at] = (float)acc;
    }
}

// ------------------------------------------------------ 6. fill adjoint

struct AdjFillArgs {
    GridDim c, f[3];
};

__device__ __forceinline__ bool fill_qual(int d, const float *__restrict__ val, const uint8_t *__restrict__ mask,
                                          long long n) {
    return d == 0 ? (fabsf(val[n]) > 0.0f) : (mask[n] != 0);
}

// number of qualifying 26-neighbours of every face the fill averaged
__global__ void __launch_bounds__(128) k_fill_count(AdjFillArgs A, const uint8_t *__restrict__ mat,
                                                    const float *__restrict__ uval, const uint8_t *__restrict__ umask,
                                                    const float *__restrict__ vval, const uint8_t *__restrict__ vmask,
                                                    const float *__restrict__ wval, const uint8_t *__restrict__ wmask,
                                                    float *__restrict__ cu, float *__restrict__ cv,
                                                    float *__restrict__ cw) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    int k = blockIdx.z * blockDim.z + threadIdx.z;
    const GridDim &c = A.c;
    if (i > c.nx || j > c.ny || k > c.nz) return;
    const float *vals[3] = {uval, vval, wval};
    const uint8_t *masks[3] = {umask, vmask, wmask};
    float *cnt[3] = {cu, cv, cw};
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const GridDim &f = A.f[d];
        if (!f.in(i, j, k)) continue;
        long long at = f.at(i, j, k);
        float n = 0.f;
        if (face_borders(mat, c, d, i, j, k, GFS_FLUID) && !masks[d][at]) {
            for (int kk = k - 1; kk <= k + 1; kk++)
                for (int jj = j - 1; jj <= j + 1; jj++)
                    for (int ii = i - 1; ii <= i + 1; ii++) {
                        if ((ii == i && jj == j && kk == k) || !f.in(ii, jj, kk)) continue;
                        if (fill_qual(d, vals[d], masks[d], f.at(ii, jj, kk))) n += 1.f;
                    }
        }
        cnt[d][at] = n;
    }
}

// splat-field adjoint from the filled field's: set faces bordering fluid pass
// through; a qualifying face receives f_bar / n_f from every averaged neighbour f
__global__ void __launch_bounds__(128) k_adj_fill(AdjFillArgs A, const uint8_t *__restrict__ mat,
                                                  const float *__restrict__ uval, const uint8_t *__restrict__ umask,
                                                  const float *__restrict__ vval, const uint8_t *__restrict__ vmask,
                                                  const float *__restrict__ wval, const uint8_t *__restrict__ wmask,
                                                  const float *__restrict__ cu, const float *__restrict__ cv,
                                                  const float *__restrict__ cw, const float *__restrict__ fu,
                                                  const float *__restrict__ fv, const float *__restrict__ fw,
                                                  float *__restrict__ ou, float *__restrict__ ov,
                                                  float *__restrict__ ow) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    int k = blockIdx.z * blockDim.z + threadIdx.z;
    const GridDim &c = A.c;
    if (i > c.nx || j > c.ny || k > c.nz) return;
    const float *vals[3] = {uval, vval, wval};
    const uint8_t *masks[3] = {umask, vmask, wmask};
    const float *cnt[3] = {cu, cv, cw};
    const float *fb[3] = {fu, fv, fw};
    float *out[3] = {ou, ov, ow};
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const GridDim &f = A.f[d];
        if (!f.in(i, j, k)) continue;
        long long at = f.at(i, j, k);
        float acc = 0.f;
        if (masks[d][at] && face_borders(mat, c, d, i, j, k, GFS_FLUID)) acc = fb[d][at];
        if (fill_qual(d, vals[d], masks[d], at)) {
            for (int kk = k - 1; kk <= k + 1; kk++)
                for (int jj = j - 1; jj <= j + 1; jj++)
                    for (int ii = i - 1; ii <= i + 1; ii++) {
                        if ((ii == i && jj == j && kk == k) || !f.in(ii, jj, kk)) continue;
                        long long n = f.at(ii, jj, kk);
                        float cn = cnt[d][n];
                        if (cn > 0.f) acc += fb[d][n] / cn;   // cnt > 0 only on averaged faces
                    }
        }
        out[d][at] = acc;
    }
}

// ------------------------------------------------------- 7. P2G adjoint

struct AdjSplatArgs {
    GridDim f[3];
    double dx;
    float half, r2_thresh, inv_r2;
};

__global__ void __launch_bounds__(128) k_adj_p2g(AdjSplatArgs A, const float4 *__restrict__ pos,
                                                 const float4 *__restrict__ vel, long long n,
                                                 const float *__restrict__ uval, const float *__restrict__ vval,
                                                 const float *__restrict__ wval, const uint8_t *__restrict__ umask,
                                                 const uint8_t *__restrict__ vmask, const uint8_t *__restrict__ wmask,
                                                 const float *__restrict__ usum, const float *__restrict__ vsum,
                                                 const float *__restrict__ wsum, const float *__restrict__ gu,
                                                 const float *__restrict__ gv, const float *__restrict__ gw,
                                                 float4 *__restrict__ ax, float4 *__restrict__ av) {
    long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= n) return;
    const float4 P = pos[q], V = vel[q];
    const uint32_t id = pid(P);
    const float *vals[3] = {uval, vval, wval};
    const uint8_t *masks[3] = {umask, vmask, wmask};
    const float *sums[3] = {usum, vsum, wsum};
    const float *gb[3] = {gu, gv, gw};
    const float vp[3] = {V.x, V.y, V.z};
    float xb[3] = {0.f, 0.f, 0.f}, vb[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const GridDim &f = A.f[d];
        // p - offset of component d (fluidsimulation.cpp:2537-2545), in float
        float px = d == 0 ? P.x : __fsub_rn(P.x, A.half);
        float py = d == 1 ? P.y : __fsub_rn(P.y, A.half);
        float pz = d == 2 ? P.z : __fsub_rn(P.z, A.half);
        int ci = (int)floor((double)px / A.dx), cj = (int)floor((double)py / A.dx), ck = (int)floor((double)pz / A.dx);
        for (int kk = ck; kk <= ck + 1; kk++)
            for (int jj = cj; jj <= cj + 1; jj++)
                for (int ii = ci; ii <= ci + 1; ii++) {
                    if (!f.in(ii, jj, kk)) continue;
                    long long at = f.at(ii, jj, kk);
                    if (!masks[d][at]) continue;
                    float gx = (float)((double)(float)ii * A.dx), gy = (float)((double)(float)jj * A.dx),
                          gz = (float)((double)(float)kk * A.dx);
                    float ex = __fsub_rn(gx, px), ey = __fsub_rn(gy, py), ez = __fsub_rn(gz, pz);
                    float d2 = dist2_exact(ex, ey, ez);
                    if (!(d2 < A.r2_thresh)) continue;
                    float s = d2 * A.inv_r2;
                    float w = kern_w(s);
                    float W = sums[d][at];
                    float g = gb[d][at];
                    vb[d] += g * w / W;
                    float h = g * (vp[d] - vals[d][at]) / W * kern_dw(s) * (-2.0f * A.inv_r2);
                    xb[0] += h * ex;
                    xb[1] += h * ey;
                    xb[2] += h * ez;
                }
    }
    float4 X = ax[id], Vv = av[id];
    ax[id] = make_float4(X.x + xb[0], X.y + xb[1], X.z + xb[2], 0.f);
    av[id] = make_float4(Vv.x + vb[0], Vv.y + vb[1], Vv.z + vb[2], 0.f);
}

// initial velocities: u0_bar = scatter of v_bar at the starting positions, in
// the same two passes as k_adj_g2p (scale, then fixed-point scatter)
template <bool SCALE_PASS>
__global__ void k_adj_sample(AdvArgs A, const float4 *__restrict__ pos, long long n, const float4 *__restrict__ av,
                             unsigned long long *__restrict__ gu, unsigned long long *__restrict__ gv,
                             unsigned long long *__restrict__ gw, FixScale *__restrict__ fs) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    unsigned mb = 0u;
    if (q < n) {
        const float4 P = pos[q];
        const float4 B = av[pid(P)];
        const float3 c = make_float3(B.x, B.y, B.z);
        if (SCALE_PASS)
            mb = abs_bits_max(mb, c);
        else
            scatter_velocity_fixed(A, gu, gv, gw, P.x, P.y, P.z, c, fs->scale);
    }
    if (SCALE_PASS) {
        mb = __reduce_max_sync(0xffffffffu, mb);
        if ((threadIdx.x & 31) == 0 && mb) atomicMax(&fs->maxbits, mb);
    }
}

// Per-block sums of the particle positions (FP64) into part[3 * block + 0..2]:
// a fixed grid, a fixed grid-stride split and fixed shuffle / shared-memory trees,
// so the sums do not depend on scheduling.
static constexpr int CENTROID_BLOCKS = 64, CENTROID_THREADS = 256;
__global__ void __launch_bounds__(CENTROID_THREADS) k_diff_centroid(const float4 *__restrict__ pos, long long n,
                                                                   double *__restrict__ part) {
    __shared__ double sh[CENTROID_THREADS / 32][3];
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        float4 P = pos[q];
        sx += P.x;
        sy += P.y;
        sz += P.z;
    }
    for (int o = 16; o > 0; o >>= 1) {
        sx += __shfl_down_sync(0xffffffffu, sx, o);
        sy += __shfl_down_sync(0xffffffffu, sy, o);
        sz += __shfl_down_sync(0xffffffffu, sz, o);
    }
    const int warp = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        sh[warp][0] = sx;
        sh[warp][1] = sy;
        sh[warp][2] = sz;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double t = 0.0;
        for (int w = 0; w < CENTROID_THREADS / 32; w++) t += sh[w][threadIdx.x];
        part[3 * blockIdx.x + threadIdx.x] = t;
    }
}

// the centroid from the per-block sums, added in block order
__global__ void k_diff_centroid_out(const double *__restrict__ part, int nblocks, double inv_n,
                                    float *__restrict__ out) {
    const int c = threadIdx.x;
    if (c >= 3) return;
    double t = 0.0;
    for (int b = 0; b < nblocks; b++) t += part[3 * b + c];
    out[c] = (float)(t * inv_n);
}

// x_bar += g_c / n for every particle present at one substep boundary (the
// centroid's adjoint there); pos lists those particles, ax is indexed by id
__global__ void k_adj_centroid(const float4 *__restrict__ pos, float4 *__restrict__ ax, long long n,
                               const float *__restrict__ gc, float inv_n) {
    long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= n) return;
    uint32_t id = pid(pos[q]);
    float4 X = ax[id];
    ax[id] = make_float4(X.x + gc[0] * inv_n, X.y + gc[1] * inv_n, X.z + gc[2] * inv_n, 0.f);
}

// id-ordered xyz of a by-id float4 array
__global__ void k_diff_export(const float4 *__restrict__ a, long long n, float *__restrict__ out) {
    long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= n) return;
    float4 A = a[q];
    out[3 * q] = A.x;
    out[3 * q + 1] = A.y;
    out[3 * q + 2] = A.z;
}

// initial velocities given per particle (by id = input order)
__global__ void k_diff_set_vel(const float4 *__restrict__ pos, long long n, const float *__restrict__ v0,
                               float4 *__restrict__ vel) {
    long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= n) return;
    uint32_t id = pid(pos[q]);
    vel[q] = make_float4(v0[3 * id], v0[3 * id + 1], v0[3 * id + 2], 0.f);
}

__global__ void k_diff_add(float *__restrict__ a, const float *__restrict__ b, long long n) {
    long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q < n) a[q] += b[q];
}

// -------------------------------------------------------------- driver

struct DiffRun {
    Sim *s = nullptr;
    int nsteps = 0;
    long long n = 0;
    double dt = 0.0;
    bool have_forward = false;
    DevMem ck;                       // (nsteps + 1) x [pos n | vel n] float4
    DevMem ax, av, bx, bv;           // adjoints by particle id
    DevMem g0[3], g1[3], g2[3], wsum[3], cnt[3], par[3];   // padded face grids
    DevMem pbar;                     // padded cells, double
    DevMem cen;                      // per-block position sums of one centroid, double
    DevMem acc[6];                   // fixed-point face adjoints: MAC u v w, saved u v w
    DevMem fix;                      // FixScale of the current scatter pass
    DevMem status;                   // non-finite scatter values seen (unsigned)
    DevMem ckp;                      // nsteps x padded-cell pressure of every substep (double)
    bool sampled = true;             // initial velocities sampled from the parameter field
    std::vector<long long> count;    // particles at the start of every substep (and at the end)
    double fwd_ms = 0.0, bwd_ms = 0.0;
    size_t peak_bytes = 0;
};

static float4 *ck_pos(DiffRun *d, int step) { return d->ck.as<float4>() + (size_t)step * 2 * d->n; }
static float4 *ck_vel(DiffRun *d, int step) { return d->ck.as<float4>() + ((size_t)step * 2 + 1) * d->n; }

static float *const *fptr(DevMem m[3], float *out[3]) {
    for (int q = 0; q < 3; q++) out[q] = m[q].as<float>();
    return out;
}

static int diff_alloc(DiffRun *d) {
    Sim *s = d->s;
    const Grids &g = s->g;
    if (d->ck.alloc((size_t)(d->nsteps + 1) * 2 * d->n * sizeof(float4))) return GFS_ERR_NOMEM;
    for (DevMem *m : {&d->ax, &d->av, &d->bx, &d->bv})
        if (m->alloc((size_t)d->n * sizeof(float4))) return GFS_ERR_NOMEM;
    for (int q = 0; q < 3; q++) {
        size_t fb = (size_t)g.f[q].size * sizeof(float);
        for (DevMem *m : {&d->g0[q], &d->g1[q], &d->g2[q], &d->wsum[q], &d->cnt[q], &d->par[q]})
            if (m->alloc(fb)) return GFS_ERR_NOMEM;
    }
    if (d->pbar.alloc((size_t)g.c.size * sizeof(double))) return GFS_ERR_NOMEM;
    for (int q = 0; q < 6; q++)
        if (d->acc[q].alloc((size_t)g.f[q % 3].size * sizeof(unsigned long long))) return GFS_ERR_NOMEM;
    if (d->fix.alloc(sizeof(FixScale)) || d->status.alloc(sizeof(unsigned))) return GFS_ERR_NOMEM;
    if (d->cen.alloc((size_t)CENTROID_BLOCKS * 3 * sizeof(double))) return GFS_ERR_NOMEM;
    if (d->ckp.alloc((size_t)d->nsteps * g.c.size * sizeof(double))) return GFS_ERR_NOMEM;
    GFS_CUDA_CHECK(cudaMemsetAsync(d->pbar.p, 0, d->pbar.bytes, s->ctx->stream));
    return GFS_OK;
}

static dim3 face_block() { return dim3(32, 2, 2); }
static dim3 face_grid(const GridDim &c) {
    return dim3(grid_blocks(c.nx + 1, 32), grid_blocks(c.ny + 1, 2), grid_blocks(c.nz + 1, 2));
}

// the grids of one substep from its checkpoint (stages of sim_step up to G2P)
static int recompute(DiffRun *d, int step, float *const wsum[3]) {
    Sim *s = d->s;
    Ctx *ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    const long long m = d->count[step];
    GFS_CUDA_CHECK(cudaMemcpyAsync(s->pos.p, ck_pos(d, step), m * sizeof(float4), cudaMemcpyDeviceToDevice, st));
    GFS_CUDA_CHECK(cudaMemcpyAsync(s->vel.p, ck_vel(d, step), m * sizeof(float4), cudaMemcpyDeviceToDevice, st));
    uint32_t num[4] = {(uint32_t)m, 0, 0, 0};
    GFS_CUDA_CHECK(cudaMemcpyAsync(s->num.p, num, sizeof(num), cudaMemcpyHostToDevice, st));
    s->n_bound = m;
    int rc;
    if ((rc = sort_particles(s, false))) return rc;   // already in (cell, id) order: rebuilds the cell lists
    if ((long long)s->n_bound != m) {
        set_error(GFS_ERR_STATE, "checkpoint %d lost particles on re-sort", step);
        return GFS_ERR_STATE;
    }
    if ((rc = classify_cells(s))) return rc;
    if ((rc = splat_velocity(s, wsum))) return rc;
    if ((rc = face_fill(s, d->dt))) return rc;
    int layers = (int)std::ceil(s->params.cfl + 2.0);
    if (layers > 120) layers = 120;
    if ((rc = build_layers(s, layers))) return rc;
    float *saved[3] = {s->saved[0].as<float>(), s->saved[1].as<float>(), s->saved[2].as<float>()};
    if ((rc = extrapolate_field(s, saved, layers, false))) return rc;
    float *mac[3] = {s->mac[0].as<float>(), s->mac[1].as<float>(), s->mac[2].as<float>()};
    // the system's set-up for the adjoint solve; the pressure itself is the forward's
    if ((rc = pressure_setup(ctx, s->ps, s->g, s->mat.as<uint8_t>(), mac))) return rc;
    GFS_CUDA_CHECK(cudaMemcpyAsync(s->ps.p.p, d->ckp.as<double>() + (size_t)step * s->g.c.size,
                                   (size_t)s->g.c.size * sizeof(double), cudaMemcpyDeviceToDevice, st));
    if ((rc = pressure_apply(s, d->dt))) return rc;
    return extrapolate_field(s, mac, layers, false);
}

// adjoint of the extrapolation of one field, in place in g (tmp: scratch)
static int adj_extrapolate(DiffRun *d, DevMem g[3], DevMem tmp[3], int layers) {
    Sim *s = d->s;
    Ctx *ctx = s->ctx;
    AdjExtrapArgs A;
    A.c = s->g.c;
    for (int q = 0; q < 3; q++) A.f[q] = s->g.f[q];
    DevMem *in = g, *out = tmp;
    for (int L = layers; L >= 1; L--) {
        A.L = L;
        k_adj_extrap_layer<<<face_grid(A.c), face_block(), 0, ctx->stream>>>(
            A, s->mat.as<uint8_t>(), s->layer.as<int8_t>(), in[0].as<float>(), in[1].as<float>(), in[2].as<float>(),
            out[0].as<float>(), out[1].as<float>(), out[2].as<float>());
        ctx->launches++;
        std::swap(in, out);
    }
    GFS_LAUNCH_CHECK();
    if (in != g)
        for (int q = 0; q < 3; q++)
            GFS_CUDA_CHECK(cudaMemcpyAsync(g[q].p, in[q].p, g[q].bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    return GFS_OK;
}

int diff_create(Sim *s, int nsteps, long long n, double dt, DiffRun **out) {
    if (nsteps < 1 || n < 1 || n > s->capacity || !(dt > 0.0) || !std::isfinite(dt)) {
        set_error(GFS_ERR_INVALID, "invalid rollout (steps %d, particles %lld of capacity %lld, dt %g)", nsteps, n,
                  (long long)s->capacity, dt);
        return GFS_ERR_INVALID;
    }
    DiffRun *d = new DiffRun();
    d->s = s;
    d->nsteps = nsteps;
    d->n = n;
    d->dt = dt;
    int rc = diff_alloc(d);
    if (rc) {
        delete d;
        return rc;
    }
    *out = d;
    return GFS_OK;
}

void diff_destroy(DiffRun *d) { delete d; }

void diff_info(DiffRun *d, double *fwd_ms, double *bwd_ms, long long *bytes) {
    if (fwd_ms) *fwd_ms = d->fwd_ms;
    if (bwd_ms) *bwd_ms = d->bwd_ms;
    if (bytes) {
        size_t b = d->ck.bytes + d->ckp.bytes + d->cen.bytes + d->ax.bytes + d->av.bytes + d->bx.bytes +
                   d->bv.bytes + d->pbar.bytes + d->fix.bytes + d->status.bytes;
        for (int q = 0; q < 6; q++) b += d->acc[q].bytes;
        for (int q = 0; q < 3; q++)
            b += d->g0[q].bytes + d->g1[q].bytes + d->g2[q].bytes + d->wsum[q].bytes + d->cnt[q].bytes +
                 d->par[q].bytes;
        *bytes = (long long)b;
    }
}

int diff_forward(DiffRun *d, const float *d_pos, const float *d_vel0, const float *const d_u0[3], float *d_density,
                 float *d_centroids) {
    Sim *s = d->s;
    Ctx *ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    const Grids &g = s->g;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    const int T = 128;
    k_diff_pack<<<grid_blocks(d->n, T), T, 0, st>>>(d_pos, d->n, s->pos.as<float4>(), s->vel.as<float4>());
    uint32_t num[4] = {(uint32_t)d->n, 0, 0, 0};
    GFS_CUDA_CHECK(cudaMemcpyAsync(s->num.p, num, sizeof(num), cudaMemcpyHostToDevice, st));
    s->n_bound = d->n;
    int rc = sort_particles(s, false);
    if (rc) return rc;
    d->sampled = d_vel0 == nullptr;
    if (d->sampled) {
        // parameter field into the (padded) MAC buffers, then the initial velocities
        for (int q = 0; q < 3; q++) {
            GFS_CUDA_CHECK(cudaMemsetAsync(s->mac[q].p, 0, s->mac[q].bytes, st));
            dim3 grid(grid_blocks(g.f[q].nx, 128), g.f[q].ny, g.f[q].nz);
            k_diff_pad<<<grid, 128, 0, st>>>(d_u0[q], g.f[q], s->mac[q].as<float>());
        }
        AdvArgs A = make_adv(g, d->dt, s->params.ratio_pic);
        k_diff_sample<<<grid_blocks(d->n, T), T, 0, st>>>(A, s->pos.as<float4>(), s->vel.as<float4>(), d->n,
                                                          s->mac[0].as<float>(), s->mac[1].as<float>(),
                                                          s->mac[2].as<float>());
        ctx->launches += 4;
    } else {
        k_diff_set_vel<<<grid_blocks(d->n, T), T, 0, st>>>(s->pos.as<float4>(), d->n, d_vel0, s->vel.as<float4>());
        ctx->launches++;
    }
    ctx->launches++;
    GFS_LAUNCH_CHECK();
    if ((long long)s->n_bound != d->n) {
        set_error(GFS_ERR_INVALID, "%lld of the %lld starting particles lie in solid cells or over the per-cell cap",
                  d->n - (long long)s->n_bound, d->n);
        return GFS_ERR_INVALID;
    }
    d->count.assign(d->nsteps + 1, 0);
    long long m = d->n;
    for (int step = 0; step < d->nsteps; step++) {
        d->count[step] = m;
        GFS_CUDA_CHECK(cudaMemcpyAsync(ck_pos(d, step), s->pos.p, m * sizeof(float4), cudaMemcpyDeviceToDevice, st));
        GFS_CUDA_CHECK(cudaMemcpyAsync(ck_vel(d, step), s->vel.p, m * sizeof(float4), cudaMemcpyDeviceToDevice, st));
        gfs_step_stats stats{};
        if ((rc = sim_step(s, d->dt, &stats))) return rc;
        GFS_CUDA_CHECK(cudaMemcpyAsync(d->ckp.as<double>() + (size_t)step * g.c.size, s->ps.p.p,
                                       (size_t)g.c.size * sizeof(double), cudaMemcpyDeviceToDevice, st));
        m = stats.num_particles;
    }
    d->count[d->nsteps] = m;
    GFS_CUDA_CHECK(cudaMemcpyAsync(ck_pos(d, d->nsteps), s->pos.p, m * sizeof(float4), cudaMemcpyDeviceToDevice, st));
    GFS_CUDA_CHECK(cudaMemcpyAsync(ck_vel(d, d->nsteps), s->vel.p, m * sizeof(float4), cudaMemcpyDeviceToDevice, st));
    const double R = DIFF_DENSITY_RADIUS * g.dx;
    dim3 cgrid(grid_blocks(g.c.nx, 128), g.c.ny, g.c.nz);
    if (d_density) {
        k_diff_density<<<cgrid, 128, 0, st>>>(g.c, g.dx, s->pos.as<float4>(), s->offset.as<uint32_t>(),
                                              (float)(1.0 / (R * R)), d_density);
        ctx->launches++;
    }
    if (d_centroids) {
        for (int step = 0; step <= d->nsteps; step++) {
            k_diff_centroid<<<CENTROID_BLOCKS, CENTROID_THREADS, 0, st>>>(ck_pos(d, step), d->count[step],
                                                                         d->cen.as<double>());
            k_diff_centroid_out<<<1, 32, 0, st>>>(d->cen.as<double>(), CENTROID_BLOCKS, 1.0 / (double)d->count[step],
                                                  d_centroids + 3 * step);
        }
        ctx->launches += 2 * (d->nsteps + 1);
    }
    GFS_LAUNCH_CHECK();
    cudaEventRecord(e1, st);
    GFS_CUDA_CHECK(cudaEventSynchronize(e1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    d->fwd_ms = ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    d->have_forward = true;
    return GFS_OK;
}

static int ceil_log2(long long v) {
    int l = 0;
    while ((1LL << l) < v) l++;
    return l;
}

// fixed-point sums acc[first .. first+count) -> float face grids out[0 .. count)
static int fix_unpack(DiffRun *d, int first, int count, DevMem *out) {
    cudaStream_t st = d->s->ctx->stream;
    for (int q = 0; q < count; q++) {
        const long long cnt = d->s->g.f[(first + q) % 3].size;
        k_fix_unpack<<<grid_blocks(cnt, 256), 256, 0, st>>>(d->acc[first + q].as<unsigned long long>(), cnt,
                                                            d->fix.as<FixScale>(), out[q].as<float>());
    }
    d->s->ctx->launches += count;
    GFS_LAUNCH_CHECK();
    return GFS_OK;
}

static int fix_begin(DiffRun *d, int count) {
    cudaStream_t st = d->s->ctx->stream;
    for (int q = 0; q < count; q++) GFS_CUDA_CHECK(cudaMemsetAsync(d->acc[q].p, 0, d->acc[q].bytes, st));
    GFS_CUDA_CHECK(cudaMemsetAsync(d->fix.p, 0, d->fix.bytes, st));
    return GFS_OK;
}

// k_adj_g2p's two passes over the m particles of a substep, then g0 / g1 from the sums
static int adj_g2p(DiffRun *d, const AdvArgs &A, long long m, int lg) {
    Sim *s = d->s;
    cudaStream_t st = s->ctx->stream;
    const int T = 128;
    int rc;
    if ((rc = fix_begin(d, 6))) return rc;
    unsigned long long *a[6];
    for (int q = 0; q < 6; q++) a[q] = d->acc[q].as<unsigned long long>();
    FixScale *fs = d->fix.as<FixScale>();
    const float *mac[3] = {s->mac[0].as<float>(), s->mac[1].as<float>(), s->mac[2].as<float>()};
    const float *sav[3] = {s->saved[0].as<float>(), s->saved[1].as<float>(), s->saved[2].as<float>()};
    if (m > 0) {
        k_adj_g2p<true><<<grid_blocks(m, T), T, 0, st>>>(A, s->pos.as<float4>(), s->vel.as<float4>(), m, mac[0],
                                                         mac[1], mac[2], sav[0], sav[1], sav[2], d->ax.as<float4>(),
                                                         d->av.as<float4>(), d->bx.as<float4>(), d->bv.as<float4>(),
                                                         a[0], a[1], a[2], a[3], a[4], a[5], s->mat.as<uint8_t>(), fs);
        k_fix_scale<<<1, 1, 0, st>>>(fs, lg, d->status.as<unsigned>());
        k_adj_g2p<false><<<grid_blocks(m, T), T, 0, st>>>(A, s->pos.as<float4>(), s->vel.as<float4>(), m, mac[0],
                                                          mac[1], mac[2], sav[0], sav[1], sav[2], d->ax.as<float4>(),
                                                          d->av.as<float4>(), d->bx.as<float4>(), d->bv.as<float4>(),
                                                          a[0], a[1], a[2], a[3], a[4], a[5], s->mat.as<uint8_t>(), fs);
        s->ctx->launches += 3;
        GFS_LAUNCH_CHECK();
    }
    if ((rc = fix_unpack(d, 0, 3, d->g0))) return rc;
    return fix_unpack(d, 3, 3, d->g1);
}

// k_adj_sample's two passes over the starting particles, then par from the sums
static int adj_sample(DiffRun *d, const AdvArgs &A) {
    Sim *s = d->s;
    cudaStream_t st = s->ctx->stream;
    const int T = 128;
    int rc;
    if ((rc = fix_begin(d, 3))) return rc;
    unsigned long long *a[3];
    for (int q = 0; q < 3; q++) a[q] = d->acc[q].as<unsigned long long>();
    FixScale *fs = d->fix.as<FixScale>();
    if (d->n > 0) {
        k_adj_sample<true><<<grid_blocks(d->n, T), T, 0, st>>>(A, ck_pos(d, 0), d->n, d->av.as<float4>(), a[0],
                                                               a[1], a[2], fs);
        k_fix_scale<<<1, 1, 0, st>>>(fs, ceil_log2(d->n), d->status.as<unsigned>());
        k_adj_sample<false><<<grid_blocks(d->n, T), T, 0, st>>>(A, ck_pos(d, 0), d->n, d->av.as<float4>(), a[0],
                                                                a[1], a[2], fs);
        s->ctx->launches += 3;
        GFS_LAUNCH_CHECK();
    }
    return fix_unpack(d, 0, 3, d->par);
}

int diff_backward(DiffRun *d, const float *d_rho_bar, const float *d_grad_centroids, float *const d_grad[3],
                  float *d_grad_vel0, float *d_grad_pos0) {
    if (!d->have_forward) {
        set_error(GFS_ERR_STATE, "backward needs a forward run first");
        return GFS_ERR_STATE;
    }
    Sim *s = d->s;
    Ctx *ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    const Grids &g = s->g;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    const int T = 128;
    const double R = DIFF_DENSITY_RADIUS * g.dx;
    // density adjoint at the final positions (ids removed earlier keep zero adjoints)
    GFS_CUDA_CHECK(cudaMemsetAsync(d->status.p, 0, d->status.bytes, st));
    GFS_CUDA_CHECK(cudaMemsetAsync(d->ax.p, 0, d->ax.bytes, st));
    GFS_CUDA_CHECK(cudaMemsetAsync(d->av.p, 0, d->av.bytes, st));
    const long long mN = d->count[d->nsteps];
    if (d_rho_bar) {
        k_adj_density<<<grid_blocks(mN, T), T, 0, st>>>(g.c, g.dx, ck_pos(d, d->nsteps), mN, d_rho_bar,
                                                        (float)(1.0 / (R * R)), d->ax.as<float4>(),
                                                        d->av.as<float4>());
        ctx->launches++;
    }
    if (d_grad_centroids) {
        k_adj_centroid<<<grid_blocks(mN, T), T, 0, st>>>(ck_pos(d, d->nsteps), d->ax.as<float4>(), mN,
                                                         d_grad_centroids + 3 * d->nsteps,
                                                         (float)(1.0 / (double)mN));
        ctx->launches++;
    }
    GFS_LAUNCH_CHECK();
    int layers = (int)std::ceil(s->params.cfl + 2.0);
    if (layers > 120) layers = 120;
    AdvArgs A = make_adv(g, d->dt, s->params.ratio_pic);
    AdjPArgs P;
    P.c = g.c;
    for (int q = 0; q < 3; q++) P.f[q] = g.f[q];
    P.kscale = d->dt / (s->params.density * g.dx);
    P.sdiv = (double)(1.0f / (float)g.dx);
    P.fscale = (double)(1.0f / (float)g.dx);
    AdjFillArgs F;
    F.c = g.c;
    for (int q = 0; q < 3; q++) F.f[q] = g.f[q];
    AdjSplatArgs SA;
    for (int q = 0; q < 3; q++) SA.f[q] = g.f[q];
    SA.dx = g.dx;
    SA.half = (float)(0.5 * g.dx);
    {
        float f = (float)(g.dx * g.dx);
        if ((double)f < g.dx * g.dx) f = nextafterf(f, INFINITY);
        SA.r2_thresh = f;
    }
    SA.inv_r2 = (float)(1.0 / (g.dx * g.dx));
    int rc;
    float *wp[3];
    for (int step = d->nsteps - 1; step >= 0; step--) {
        if ((rc = recompute(d, step, fptr(d->wsum, wp)))) return rc;
        const long long m = d->count[step];
        // 2. G2P / RK4: g0 = MAC adjoint, g1 = saved adjoint (from the fixed-point sums);
        // (bx, bv) by id, zero for ids not present in this substep
        GFS_CUDA_CHECK(cudaMemsetAsync(d->bx.p, 0, d->bx.bytes, st));
        GFS_CUDA_CHECK(cudaMemsetAsync(d->bv.p, 0, d->bv.bytes, st));
        // a MAC node takes at most 4 terms per particle (the RK4 stages), a saved node 1
        if ((rc = adj_g2p(d, A, m, ceil_log2(4 * m)))) return rc;
        // 3. extrapolations
        if ((rc = adj_extrapolate(d, d->g0, d->g2, layers))) return rc;
        if ((rc = adj_extrapolate(d, d->g1, d->g2, layers))) return rc;
        // 4. pressure: p_bar, A lambda = p_bar, u_bar += D^T lambda / dx (+ pass-through)
        dim3 cgrid(grid_blocks(g.c.nx, 128), g.c.ny, g.c.nz);
        k_adj_pbar<<<cgrid, 128, 0, st>>>(P, s->mat.as<uint8_t>(), d->g0[0].as<float>(), d->g0[1].as<float>(),
                                          d->g0[2].as<float>(), d->pbar.as<double>());
        ctx->launches++;
        GFS_LAUNCH_CHECK();
        gfs_step_stats ps{};
        // the adjoint system has the forward's matrix; it is solved in the forward's precision form
        // (MIXED: FP32 inner PCG with FP64 residual updates) to the same FP64 residual rule
        if ((rc = pressure_solve_rhs(ctx, s->ps, g, d->pbar.as<double>(), s->params.density, d->dt, 1e-7, 2000, &ps,
                                     s->params.precision == GFS_PRECISION_MIXED)))
            return rc;
        k_adj_div<<<face_grid(g.c), face_block(), 0, st>>>(P, s->mat.as<uint8_t>(), s->ps.p.as<double>(),
                                                          d->g0[0].as<float>(), d->g0[1].as<float>(),
                                                          d->g0[2].as<float>());
        ctx->launches++;
        GFS_LAUNCH_CHECK();
        // 5. filled-field adjoint = MAC adjoint + saved adjoint (into g0)
        for (int q = 0; q < 3; q++) {
            long long cnt = g.f[q].size;
            k_diff_add<<<grid_blocks(cnt, 256), 256, 0, st>>>(d->g0[q].as<float>(), d->g1[q].as<float>(), cnt);
        }
        ctx->launches += 3;
        // 6. fill
        k_fill_count<<<face_grid(g.c), face_block(), 0, st>>>(
            F, s->mat.as<uint8_t>(), s->sval[0].as<float>(), s->smask[0].as<uint8_t>(), s->sval[1].as<float>(),
            s->smask[1].as<uint8_t>(), s->sval[2].as<float>(), s->smask[2].as<uint8_t>(), d->cnt[0].as<float>(),
            d->cnt[1].as<float>(), d->cnt[2].as<float>());
        k_adj_fill<<<face_grid(g.c), face_block(), 0, st>>>(
            F, s->mat.as<uint8_t>(), s->sval[0].as<float>(), s->smask[0].as<uint8_t>(), s->sval[1].as<float>(),
            s->smask[1].as<uint8_t>(), s->sval[2].as<float>(), s->smask[2].as<uint8_t>(), d->cnt[0].as<float>(),
            d->cnt[1].as<float>(), d->cnt[2].as<float>(), d->g0[0].as<float>(), d->g0[1].as<float>(),
            d->g0[2].as<float>(), d->g2[0].as<float>(), d->g2[1].as<float>(), d->g2[2].as<float>());
        ctx->launches += 2;
        GFS_LAUNCH_CHECK();
        // 7. P2G into (bx, bv), then they become the adjoints of this substep's start
        k_adj_p2g<<<grid_blocks(m, T), T, 0, st>>>(
            SA, s->pos.as<float4>(), s->vel.as<float4>(), m, s->sval[0].as<float>(), s->sval[1].as<float>(),
            s->sval[2].as<float>(), s->smask[0].as<uint8_t>(), s->smask[1].as<uint8_t>(), s->smask[2].as<uint8_t>(),
            d->wsum[0].as<float>(), d->wsum[1].as<float>(), d->wsum[2].as<float>(), d->g2[0].as<float>(),
            d->g2[1].as<float>(), d->g2[2].as<float>(), d->bx.as<float4>(), d->bv.as<float4>());
        ctx->launches++;
        GFS_LAUNCH_CHECK();
        std::swap(d->ax.p, d->bx.p);
        std::swap(d->av.p, d->bv.p);
        if (d_grad_centroids) {   // the centroid at the start of this substep
            k_adj_centroid<<<grid_blocks(m, T), T, 0, st>>>(ck_pos(d, step), d->ax.as<float4>(), m,
                                                            d_grad_centroids + 3 * step, (float)(1.0 / (double)m));
            ctx->launches++;
        }
    }
    if (d_grad_vel0) {
        k_diff_export<<<grid_blocks(d->n, T), T, 0, st>>>(d->av.as<float4>(), d->n, d_grad_vel0);
        ctx->launches++;
    }
    if (d_grad[0] && d->sampled) {
        // the parameter field: u0_bar = scatter of v_bar at the starting positions
        if ((rc = adj_sample(d, A))) return rc;
        for (int q = 0; q < 3; q++) {
            dim3 grid(grid_blocks(g.f[q].nx, 128), g.f[q].ny, g.f[q].nz);
            k_diff_unpad<<<grid, 128, 0, st>>>(d->par[q].as<float>(), g.f[q], d_grad[q]);
        }
        ctx->launches += 3;
    }
    if (d_grad_pos0) {
        // with the initial velocities held fixed (their dependence on the
        // starting positions through the parameter field is not included)
        k_diff_export<<<grid_blocks(d->n, T), T, 0, st>>>(d->ax.as<float4>(), d->n, d_grad_pos0);
        ctx->launches++;
    }
    GFS_LAUNCH_CHECK();
    cudaEventRecord(e1, st);
    GFS_CUDA_CHECK(cudaEventSynchronize(e1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    d->bwd_ms = ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    unsigned bad = 0;
    GFS_CUDA_CHECK(cudaMemcpy(&bad, d->status.p, sizeof(bad), cudaMemcpyDeviceToHost));
    if (bad) {
        set_error(GFS_ERR_INVALID, "backward: an adjoint value is not finite (check the loss gradients)");
        return GFS_ERR_INVALID;
    }
    return GFS_OK;
}

}  // namespace gfs
