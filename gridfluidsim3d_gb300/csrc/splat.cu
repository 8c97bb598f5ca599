// splat.cu -- particle -> MAC-grid velocity splat (P2G) and the face fill.
//
// k_splat_gather computes, for every face node of U, V and W at once, the
// weighted average of the particles within radius dx, the quantity
// FluidSimulation::_computeVelocityScalarField forms with ScalarField
// (fluidsimulation.cpp:2526-2595, scalarfield.cpp:90-106,167-201) and the
// reference's GPU path forms with compute_scalar_field_weight_point_values
// (kernels/scalarfield.cl:202-268).
//
// Design: particles are sorted by cell, so the candidates of one node are nine
// contiguous runs (one per (j,k) row of the 3x3x3 cell neighbourhood, three
// consecutive cells each).  One thread owns the corner (i,j,k) and the three
// faces U(i, j+1/2, k+1/2), V(i+1/2, j, k+1/2), W(i+1/2, j+1/2, k): a particle
// in cell (ci,cj,ck) can reach U only if ci <= i, V only if cj <= j, W only if
// ck <= k.  Each thread sums in a fixed order (rows k-major, particles in
// (cell, id) order), so the splat is deterministic and uses no atomics.
//
// Distances are formed exactly as the reference does (float node position
// (float)i*dx, float offset subtraction, float dot product without FMA), so
// the set of (particle, node) pairs is the reference's.  The weight
// 1 - 4/9 s^3 + 17/9 s^2 - 22/9 s (s = r^2/R^2) is evaluated in float in the
// factored form (1-s)^2 (1 - 4s/9), which is the same polynomial and keeps
// full relative precision near s = 1.
#include "gfs_internal.h"

namespace gfs {

struct SplatArgs {
    GridDim c, f[3];
    double dx;
    float half;        // (float)(0.5*dx): the face offsets (fluidsimulation.cpp:2537-2545)
    float r2_thresh;   // (double)d2 < dx*dx  <=>  d2 < r2_thresh
    float inv_r2;
    float set_thresh;  // (double)w > 1e-9   <=>  w > set_thresh
};

__device__ __forceinline__ float dist2_exact(float ax, float ay, float az) {
    // vmath::dot (vmath.h:71-73): x*x + y*y + z*z in float, left to right, no FMA.
    return __fadd_rn(__fadd_rn(__fmul_rn(ax, ax), __fmul_rn(ay, ay)), __fmul_rn(az, az));
}

__device__ __forceinline__ float splat_weight(float d2, float inv_r2) {
    float s = d2 * inv_r2;
    float a = 1.0f - s;
    return a * a * (1.0f - (4.0f / 9.0f) * s);
}

__global__ void __launch_bounds__(128) k_splat_gather(SplatArgs A, const float4 *__restrict__ pos,
                                                      const float4 *__restrict__ vel,
                                                      const uint32_t *__restrict__ offset,
                                                      float *__restrict__ uval, uint8_t *__restrict__ umask,
                                                      float *__restrict__ vval, uint8_t *__restrict__ vmask,
                                                      float *__restrict__ wval, uint8_t *__restrict__ wmask,
                                                      float *__restrict__ usum, float *__restrict__ vsum,
                                                      float *__restrict__ wsum) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    int k = blockIdx.z * blockDim.z + threadIdx.z;
    const GridDim &c = A.c;
    if (i > c.nx || j > c.ny || k > c.nz) return;
    bool vu = j < c.ny && k < c.nz;
    bool vv = i < c.nx && k < c.nz;
    bool vw = i < c.nx && j < c.ny;
    // node positions: Grid3d::GridIndexToPosition (grid3d.h:79-81) -> float
    float gx = (float)((double)(float)i * A.dx);
    float gy = (float)((double)(float)j * A.dx);
    float gz = (float)((double)(float)k * A.dx);
    float su = 0.f, wu = 0.f, sv = 0.f, wv = 0.f, sw = 0.f, ww = 0.f;
    int i0 = max(i - 1, 0), i1 = min(i + 1, c.nx - 1);
    for (int ck = k - 1; ck <= k + 1; ck++) {
        if (ck < 0 || ck >= c.nz) continue;
        bool nw = vw && ck <= k;
        for (int cj = j - 1; cj <= j + 1; cj++) {
            if (cj < 0 || cj >= c.ny) continue;
            bool nv = vv && cj <= j;
            long long row = (long long)c.nx * (cj + (long long)c.ny * ck);
            uint32_t b = __ldg(offset + row + i0);
            uint32_t e = __ldg(offset + row + i1 + 1);
            // particles before `mid` are in cells <= i (they can reach U)
            uint32_t mid = (i + 1 <= i1) ? __ldg(offset + row + i + 1) : e;
            for (uint32_t q = b; q < e; q++) {
                float4 p = __ldg(pos + q);
                bool nu = vu && q < mid;
                float dU = 0.f, dV = 0.f, dW = 0.f;
                bool hu = false, hv = false, hw = false;
                if (nu) {
                    // p - offset(0, h, h), then gpos - p'
                    float ax = gx - p.x, ay = gy - __fsub_rn(p.y, A.half), az = gz - __fsub_rn(p.z, A.half);
                    dU = dist2_exact(ax, ay, az);
                    hu = dU < A.r2_thresh;
                }
                if (nv) {
                    float ax = gx - __fsub_rn(p.x, A.half), ay = gy - p.y, az = gz - __fsub_rn(p.z, A.half);
                    dV = dist2_exact(ax, ay, az);
                    hv = dV < A.r2_thresh;
                }
                if (nw) {
                    float ax = gx - __fsub_rn(p.x, A.half), ay = gy - __fsub_rn(p.y, A.half), az = gz - p.z;
                    dW = dist2_exact(ax, ay, az);
                    hw = dW < A.r2_thresh;
                }
                if (hu | hv | hw) {
                    float4 v = __ldg(vel + q);
                    if (hu) { float w = splat_weight(dU, A.inv_r2); su += w * v.x; wu += w; }
                    if (hv) { float w = splat_weight(dV, A.inv_r2); sv += w * v.y; wv += w; }
                    if (hw) { float w = splat_weight(dW, A.inv_r2); sw += w * v.z; ww += w; }
                }
            }
        }
    }
    // ScalarField::applyWeightField (scalarfield.cpp:90-106) and the 1e-9 mask
    // (weight sums on request: the adjoint of the division needs them)
    if (vu) {
        long long f = A.f[0].at(i, j, k);
        uval[f] = wu > 0.f ? su / wu : su;
        umask[f] = wu > A.set_thresh;
        if (usum) usum[f] = wu;
    }
    if (vv) {
        long long f = A.f[1].at(i, j, k);
        vval[f] = wv > 0.f ? sv / wv : sv;
        vmask[f] = wv > A.set_thresh;
        if (vsum) vsum[f] = wv;
    }
    if (vw) {
        long long f = A.f[2].at(i, j, k);
        wval[f] = ww > 0.f ? sw / ww : sw;
        wmask[f] = ww > A.set_thresh;
        if (wsum) wsum[f] = ww;
    }
}

static float float_ceil_of(double x) {
    float f = (float)x;
    if ((double)f < x) f = nextafterf(f, INFINITY);
    return f;
}

static float float_floor_of(double x) {
    float f = (float)x;
    if ((double)f > x) f = nextafterf(f, -INFINITY);
    return f;
}

int splat_velocity(Sim *s, float *const wsum[3]) {
    Ctx *ctx = s->ctx;
    ProfScope prof(ctx, KC_SPLAT);
    SplatArgs A;
    A.c = s->g.c;
    for (int d = 0; d < 3; d++) A.f[d] = s->g.f[d];
    A.dx = s->g.dx;
    A.half = (float)(0.5 * s->g.dx);
    A.r2_thresh = float_ceil_of(s->g.dx * s->g.dx);
    A.inv_r2 = (float)(1.0 / (s->g.dx * s->g.dx));
    A.set_thresh = float_floor_of(1e-9);
    dim3 block(32, 2, 2);
    dim3 grid(grid_blocks(A.c.nx + 1, 32), grid_blocks(A.c.ny + 1, 2), grid_blocks(A.c.nz + 1, 2));
    k_splat_gather<<<grid, block, 0, ctx->stream>>>(
        A, s->pos.as<float4>(), s->vel.as<float4>(), s->offset.as<uint32_t>(), s->sval[0].as<float>(),
        s->smask[0].as<uint8_t>(), s->sval[1].as<float>(), s->smask[1].as<uint8_t>(),
        s->sval[2].as<float>(), s->smask[2].as<uint8_t>(), wsum ? wsum[0] : nullptr, wsum ? wsum[1] : nullptr,
        wsum ? wsum[2] : nullptr);
    ctx->launches++;
    GFS_LAUNCH_CHECK();
    return GFS_OK;
}

// -------------------------------------------------------------- face fill

struct FillArgs {
    GridDim c, f[3];
    float add[3];      // (float)(g*dt) where |g| > 0, else 0 (fluidsimulation.cpp:2766-2805)
    int has_add[3];
};

// 26-neighbour average of unset faces (fluidsimulation.cpp:2618-2639 and the V/W
// twins): neighbours in k, j, i order; U counts a neighbour when its value is
// nonzero, V and W when it is set (the reference's asymmetry, :2630 vs :2675).
__device__ __forceinline__ float fill_average(const float *__restrict__ val,
                                              const uint8_t *__restrict__ mask, const GridDim &f,
                                              int d, int i, int j, int k) {
    double avg = 0.0, wsum = 0.0;
    for (int kk = k - 1; kk <= k + 1; kk++)
        for (int jj = j - 1; jj <= j + 1; jj++)
            for (int ii = i - 1; ii <= i + 1; ii++) {
                if (ii == i && jj == j && kk == k) continue;
                if (!f.in(ii, jj, kk)) continue;
                long long n = f.at(ii, jj, kk);
                float v = val[n];
                bool ok = d == 0 ? (fabsf(v) > 0.0f) : (mask[n] != 0);
                if (ok) {
                    avg += (double)v;
                    wsum += 1.0;
                }
            }
    return wsum > 0.0 ? (float)(avg / wsum) : 0.0f;
}

// One thread per corner node; writes the advected MAC face (with body force) and
// the saved copy of the pre-force field (fluidsimulation.cpp:3306).
__global__ void __launch_bounds__(128) k_face_fill(FillArgs A, const uint8_t *__restrict__ mat,
                                                   const float *__restrict__ uval, const uint8_t *__restrict__ umask,
                                                   const float *__restrict__ vval, const uint8_t *__restrict__ vmask,
                                                   const float *__restrict__ wval, const uint8_t *__restrict__ wmask,
                                                   float *__restrict__ mu, float *__restrict__ mv, float *__restrict__ mw,
                                                   float *__restrict__ su, float *__restrict__ sv, float *__restrict__ sw) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    int k = blockIdx.z * blockDim.z + threadIdx.z;
    const GridDim &c = A.c;
    if (i > c.nx || j > c.ny || k > c.nz) return;
    const float *vals[3] = {uval, vval, wval};
    const uint8_t *masks[3] = {umask, vmask, wmask};
    float *macs[3] = {mu, mv, mw};
    float *saves[3] = {su, sv, sw};
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const GridDim &f = A.f[d];
        if (!f.in(i, j, k)) continue;
        long long at = f.at(i, j, k);
        float out = 0.0f;
        bool fluid = face_borders(mat, c, d, i, j, k, GFS_FLUID);
        if (fluid) {
            if (masks[d][at]) out = vals[d][at];
            else out = fill_average(vals[d], masks[d], f, d, i, j, k);
        }
        saves[d][at] = out;
        macs[d][at] = (fluid && A.has_add[d]) ? out + A.add[d] : out;
    }
}

int face_fill(Sim *s, double dt) {
    Ctx *ctx = s->ctx;
    ProfScope prof(ctx, KC_FILL);
    FillArgs A;
    A.c = s->g.c;
    for (int d = 0; d < 3; d++) {
        A.f[d] = s->g.f[d];
        float gd = s->params.gravity[d];
        A.has_add[d] = fabs((double)gd) > 0.0;
        A.add[d] = (float)((double)gd * dt);
    }
    dim3 block(32, 2, 2);
    dim3 grid(grid_blocks(A.c.nx + 1, 32), grid_blocks(A.c.ny + 1, 2), grid_blocks(A.c.nz + 1, 2));
    k_face_fill<<<grid, block, 0, ctx->stream>>>(
        A, s->mat.as<uint8_t>(), s->sval[0].as<float>(), s->smask[0].as<uint8_t>(), s->sval[1].as<float>(),
        s->smask[1].as<uint8_t>(), s->sval[2].as<float>(), s->smask[2].as<uint8_t>(), s->mac[0].as<float>(),
        s->mac[1].as<float>(), s->mac[2].as<float>(), s->saved[0].as<float>(), s->saved[1].as<float>(),
        s->saved[2].as<float>());
    ctx->launches++;
    GFS_LAUNCH_CHECK();
    return GFS_OK;
}

}  // namespace gfs
