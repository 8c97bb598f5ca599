// gfs_interp.cuh -- MAC-grid sampling shared by the G2P / advection kernels
// (advect.cu) and their adjoints (adjoint.cu).
//
// The sample is MACVelocityField::evaluateVelocityAtPosition
// (macvelocityfield.cpp:350-559): Catmull-Rom over a 4x4x4 stencil per
// component (Interpolation::tricubicInterpolate, interpolation.cpp:26-46),
// evaluated in FP32 in separable form on the padded face grids (the zero halo is
// the reference's out-of-range value).  The gradient and the transposed
// (scatter) forms below differentiate exactly that separable sum.
#pragma once

#include "gfs_internal.h"

namespace gfs {

struct AdvArgs {
    GridDim f[3], c;
    float inv_dx;      // (float)(1/dx)
    float bound[3];    // x < dx*n  <=>  x < bound (bound = smallest float >= dx*n)
    double dx, inv_dx_d;
    int pow2;
    float h, f1, f6;   // RK4: (float)(0.5*dt), (float)dt, (float)(dt/6.0f)
    float a_pic, b_flip;
};

// The four x taps g[at .. at+3] of one stencil row: four 4-byte loads from a face
// grid, or one aligned 16-byte load from its row quads (k_row_quads in advect.cu:
// quad x holds the grid's values at storage indices x .. x+3).
__device__ __forceinline__ float4 row_taps(const float *__restrict__ g, long long at) {
    return make_float4(__ldg(g + at), __ldg(g + at + 1), __ldg(g + at + 2), __ldg(g + at + 3));
}
__device__ __forceinline__ float4 row_taps(const float4 *__restrict__ q, long long at) { return __ldg(q + at); }

// One Catmull-Rom row w0 v0 + w1 v1 + w2 v2 + w3 v3: the product w1 v1 rounded,
// then w0 v0, w2 v2 and w3 v3 fused into the running sum in that order.  The order
// is spelled out so that every sampler below (the scalar and the row-quad forms,
// and the gradient form the adjoint recomputes the forward with) rounds the same
// way; it is the order the substep parity tests against the oracle hold with.
__device__ __forceinline__ float cr_row(const float w[4], float4 t) {
    return __fmaf_rn(w[3], t.w, __fmaf_rn(w[2], t.z, __fmaf_rn(w[0], t.x, __fmul_rn(w[1], t.y))));
}
// a += w r, fused
#define CR_ACC(a, w, r) ((a) = __fmaf_rn((w), (r), (a)))

template <class G>
__device__ __forceinline__ float interp_component(const G *__restrict__ g, const GridDim &f, float X, float Y,
                                                  float Z) {
    float fi = floorf(X), fj = floorf(Y), fk = floorf(Z);
    int i = (int)fi, j = (int)fj, k = (int)fk;
    float wx[4], wy[4], wz[4];
    catmull_rom_weights(X - fi, wx);
    catmull_rom_weights(Y - fj, wy);
    catmull_rom_weights(Z - fk, wz);
    const long long sy = f.sx, sz = (long long)f.sx * f.sy;
    const long long base = f.at(i - 1, j - 1, k - 1);
    float acc = 0.0f;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        float accb = 0.0f;
#pragma unroll
        for (int b = 0; b < 4; b++) CR_ACC(accb, wy[b], cr_row(wx, row_taps(g, base + b * sy + c * sz)));
        CR_ACC(acc, wz[c], accb);
    }
    return acc;
}

// MACVelocityField::evaluateVelocityAtPosition: zero outside [0, n*dx).  G is
// float (the face grids) or float4 (their row quads).
template <class G>
__device__ __forceinline__ float3 eval_velocity(const AdvArgs &A, const G *__restrict__ u, const G *__restrict__ v,
                                                const G *__restrict__ w, float x, float y, float z) {
    if (!(x >= 0.f && y >= 0.f && z >= 0.f && x < A.bound[0] && y < A.bound[1] && z < A.bound[2]))
        return make_float3(0.f, 0.f, 0.f);
    float X, Y, Z;
    if (A.pow2) {
        X = x * A.inv_dx;
        Y = y * A.inv_dx;
        Z = z * A.inv_dx;
    } else {
        X = (float)((double)x * A.inv_dx_d);
        Y = (float)((double)y * A.inv_dx_d);
        Z = (float)((double)z * A.inv_dx_d);
    }
    // U samples at (i, j+1/2, k+1/2): shift y and z by half a cell, etc.
    float vx = interp_component(u, A.f[0], X, Y - 0.5f, Z - 0.5f);
    float vy = interp_component(v, A.f[1], X - 0.5f, Y, Z - 0.5f);
    float vz = interp_component(w, A.f[2], X - 0.5f, Y - 0.5f, Z);
    return make_float3(vx, vy, vz);
}

__device__ __forceinline__ bool finite3(float3 a) { return isfinite(a.x) && isfinite(a.y) && isfinite(a.z); }

__device__ __forceinline__ void pos_cell(const AdvArgs &A, float x, float y, float z, int &i, int &j, int &k) {
    if (A.pow2) {
        i = (int)floorf(x * A.inv_dx);
        j = (int)floorf(y * A.inv_dx);
        k = (int)floorf(z * A.inv_dx);
    } else {
        i = (int)floor((double)x * A.inv_dx_d);
        j = (int)floor((double)y * A.inv_dx_d);
        k = (int)floor((double)z * A.inv_dx_d);
    }
}

__device__ __forceinline__ bool cell_solid(const AdvArgs &A, const uint8_t *__restrict__ mat, int i, int j, int k) {
    if (!A.c.in(i, j, k)) return true;   // out of range reads as solid
    return mat[A.c.at(i, j, k)] == GFS_SOLID;
}


__device__ __forceinline__ float3 axpy3(float3 p, float h, float3 k) {
    return make_float3(__fadd_rn(p.x, __fmul_rn(h, k.x)), __fadd_rn(p.y, __fmul_rn(h, k.y)),
                       __fadd_rn(p.z, __fmul_rn(h, k.z)));
}

// p0 + f6 * (k1 + 2 k2 + 2 k3 + k4), float, left to right (particleadvector.cpp:1051)
__device__ __forceinline__ float rk4_comb(float p, float f6, float k1, float k2, float k3, float k4) {
    float sum = __fadd_rn(__fadd_rn(__fadd_rn(k1, __fmul_rn(2.0f, k2)), __fmul_rn(2.0f, k3)), k4);
    return __fadd_rn(p, __fmul_rn(f6, sum));
}


AdvArgs make_adv(const Grids &g, double dt, double ratio_pic);

// Collision::getLineSegmentVoxelIntersection (collision.cpp:303-402)
static __device__ bool segment_voxel(const AdvArgs &A, const uint8_t *__restrict__ mat, float3 p0in, float3 p1in,
                              int &vi, int &vj, int &vk) {
    float s = (float)(1.0 / A.dx);
    float p0x = __fmul_rn(p0in.x, s), p0y = __fmul_rn(p0in.y, s), p0z = __fmul_rn(p0in.z, s);
    float p1x = __fmul_rn(p1in.x, s), p1y = __fmul_rn(p1in.y, s), p1z = __fmul_rn(p1in.z, s);
    int gx0 = (int)floorf(p0x), gy0 = (int)floorf(p0y), gz0 = (int)floorf(p0z);
    int gx1 = (int)floorf(p1x), gy1 = (int)floorf(p1y), gz1 = (int)floorf(p1z);
    int sx = gx1 > gx0 ? 1 : gx1 < gx0 ? -1 : 0;
    int sy = gy1 > gy0 ? 1 : gy1 < gy0 ? -1 : 0;
    int sz = gz1 > gz0 ? 1 : gz1 < gz0 ? -1 : 0;
    int gx = gx0, gy = gy0, gz = gz0;
    double gxp = gx0 + (gx1 > gx0 ? 1 : 0), gyp = gy0 + (gy1 > gy0 ? 1 : 0), gzp = gz0 + (gz1 > gz0 ? 1 : 0);
    double vx = p1x == p0x ? 1.0 : (double)__fsub_rn(p1x, p0x);
    double vy = p1y == p0y ? 1.0 : (double)__fsub_rn(p1y, p0y);
    double vz = p1z == p0z ? 1.0 : (double)__fsub_rn(p1z, p0z);
    double vxvy = vx * vy, vxvz = vx * vz, vyvz = vy * vz;
    double errx = (gxp - (double)p0x) * vyvz, erry = (gyp - (double)p0y) * vxvz, errz = (gzp - (double)p0z) * vxvy;
    double derrx = sx * vyvz, derry = sy * vxvz, derrz = sz * vxvy;
    int limit = abs(gx1 - gx0) + abs(gy1 - gy0) + abs(gz1 - gz0) + 3;
    for (int it = 0; it < limit; it++) {
        if (A.c.in(gx, gy, gz) && mat[A.c.at(gx, gy, gz)] == GFS_SOLID) {
            vi = gx; vj = gy; vk = gz;
            return true;
        }
        if (gx == gx1 && gy == gy1 && gz == gz1) break;
        double xr = fabs(errx), yr = fabs(erry), zr = fabs(errz);
        if (sx != 0 && (sy == 0 || xr < yr) && (sz == 0 || xr < zr)) { gx += sx; errx += derrx; }
        else if (sy != 0 && (sz == 0 || yr < zr)) { gy += sy; erry += derry; }
        else if (sz != 0) { gz += sz; errz += derrz; }
    }
    return false;
}

// FluidSimulation::_resolveParticleSolidCellCollision (fluidsimulation.cpp:3145-3179)
// with Collision::rayIntersectsAABB (collision.cpp:404-449, including its use of
// dir.x to guard dir.z).
// What a collision did, for its adjoint: moved = p1 was placed before the entry
// plane x_axis = plane of the first solid voxel along p0 -> p1 (else p0 was kept).
struct CollisionHit {
    bool moved = false;
    int axis = 0;
    float plane = 0.f;
};

static __device__ float3 resolve_collision(const AdvArgs &A, const uint8_t *__restrict__ mat, float3 p0, float3 p1,
                                    CollisionHit *hit = nullptr) {
    int vi, vj, vk;
    if (!segment_voxel(A, mat, p0, p1, vi, vj, vk)) return p0;
    float dxr = __fsub_rn(p1.x, p0.x), dyr = __fsub_rn(p1.y, p0.y), dzr = __fsub_rn(p1.z, p0.z);
    float len = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dxr, dxr), __fmul_rn(dyr, dyr)), __fmul_rn(dzr, dzr)));
    float linv = (float)(1.0 / (double)len);
    float3 rn = make_float3(__fmul_rn(dxr, linv), __fmul_rn(dyr, linv), __fmul_rn(dzr, linv));
    float bmin[3], bmax[3];
    int vv[3] = {vi, vj, vk};
    for (int q = 0; q < 3; q++) {
        bmin[q] = (float)((double)(float)vv[q] * A.dx);
        bmax[q] = __fadd_rn(bmin[q], (float)A.dx);
    }
    float dir[3] = {rn.x, rn.y, rn.z};
    const double eps = 1e-10;
    if (fabs((double)dir[0]) < eps) dir[0] = dir[0] < 0 ? (float)-eps : (float)eps;
    if (fabs((double)dir[1]) < eps) dir[1] = dir[1] < 0 ? (float)-eps : (float)eps;
    if (fabs((double)dir[0]) < eps) dir[2] = dir[2] < 0 ? (float)-eps : (float)eps;
    float inv[3] = {(float)(1.0 / (double)dir[0]), (float)(1.0 / (double)dir[1]), (float)(1.0 / (double)dir[2])};
    float p0a[3] = {p0.x, p0.y, p0.z};
    double tmin = 0, tmax = 0;
    int axis = 0;
    float plane = bmin[0];
    for (int q = 0; q < 3; q++) {
        double t1 = (double)__fmul_rn(__fsub_rn(bmin[q], p0a[q]), inv[q]);
        double t2 = (double)__fmul_rn(__fsub_rn(bmax[q], p0a[q]), inv[q]);
        double tn = fmin(t1, t2);
        if (q == 0 || tn > tmin) {
            axis = q;
            plane = t1 <= t2 ? bmin[q] : bmax[q];
        }
        if (q == 0) { tmin = tn; tmax = fmax(t1, t2); }
        else { tmin = fmax(tmin, tn); tmax = fmin(tmax, fmax(t1, t2)); }
    }
    if (!(tmax > fmax(tmin, 0.0))) return p0;
    float ft = (float)tmin;
    float cp[3];
    for (int q = 0; q < 3; q++) cp[q] = __fadd_rn(p0a[q], __fmul_rn(ft, dir[q]));
    float back = (float)(0.05 * A.dx);
    float3 res = make_float3(__fsub_rn(cp[0], __fmul_rn(back, rn.x)), __fsub_rn(cp[1], __fmul_rn(back, rn.y)),
                             __fsub_rn(cp[2], __fmul_rn(back, rn.z)));
    int ri, rj, rk;
    pos_cell(A, res.x, res.y, res.z, ri, rj, rk);
    if (cell_solid(A, mat, ri, rj, rk)) return p0;
    if (hit) {
        hit->moved = true;
        hit->axis = axis;
        hit->plane = plane;
    }
    return res;
}



// d/dx of the Catmull-Rom basis weights of catmull_rom_weights
__device__ __forceinline__ void catmull_rom_dweights(float x, float d[4]) {
    float x2 = x * x;
    d[0] = 0.5f * (-1.0f + 4.0f * x - 3.0f * x2);
    d[1] = 0.5f * (-10.0f * x + 9.0f * x2);
    d[2] = 0.5f * (1.0f + 8.0f * x - 9.0f * x2);
    d[3] = 0.5f * (3.0f * x2 - 2.0f * x);
}

// Sample and gradient (in index units) of one component at index-space (X, Y, Z).
__device__ __forceinline__ float interp_component_grad(const float *__restrict__ g, const GridDim &f, float X,
                                                       float Y, float Z, float grad[3]) {
    float fi = floorf(X), fj = floorf(Y), fk = floorf(Z);
    int i = (int)fi, j = (int)fj, k = (int)fk;
    float wx[4], wy[4], wz[4], dx_[4], dy_[4], dz_[4];
    catmull_rom_weights(X - fi, wx);
    catmull_rom_weights(Y - fj, wy);
    catmull_rom_weights(Z - fk, wz);
    catmull_rom_dweights(X - fi, dx_);
    catmull_rom_dweights(Y - fj, dy_);
    catmull_rom_dweights(Z - fk, dz_);
    const long long sy = f.sx, sz = (long long)f.sx * f.sy;
    const float *base = g + f.at(i - 1, j - 1, k - 1);
    float acc = 0.f, gx = 0.f, gy = 0.f, gz = 0.f;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        float ab = 0.f, abx = 0.f, aby = 0.f;
#pragma unroll
        for (int b = 0; b < 4; b++) {
            const float4 t = row_taps(base, (long long)(b * sy + c * sz));
            const float r = cr_row(wx, t);
            const float rx = cr_row(dx_, t);
            CR_ACC(ab, wy[b], r);
            CR_ACC(abx, wy[b], rx);
            CR_ACC(aby, dy_[b], r);
        }
        CR_ACC(acc, wz[c], ab);
        CR_ACC(gx, wz[c], abx);
        CR_ACC(gy, wz[c], aby);
        CR_ACC(gz, dz_[c], ab);
    }
    grad[0] = gx;
    grad[1] = gy;
    grad[2] = gz;
    return acc;
}

// Index-space coordinates of a world position (as eval_velocity forms them).
__device__ __forceinline__ void to_index(const AdvArgs &A, float x, float y, float z, float &X, float &Y, float &Z) {
    if (A.pow2) {
        X = x * A.inv_dx;
        Y = y * A.inv_dx;
        Z = z * A.inv_dx;
    } else {
        X = (float)((double)x * A.inv_dx_d);
        Y = (float)((double)y * A.inv_dx_d);
        Z = (float)((double)z * A.inv_dx_d);
    }
}

__device__ __forceinline__ bool inside(const AdvArgs &A, float x, float y, float z) {
    return x >= 0.f && y >= 0.f && z >= 0.f && x < A.bound[0] && y < A.bound[1] && z < A.bound[2];
}

// Velocity and its Jacobian J[r][c] = d v_r / d x_c (world units) at a position.
__device__ __forceinline__ float3 eval_velocity_jac(const AdvArgs &A, const float *__restrict__ u,
                                                    const float *__restrict__ v, const float *__restrict__ w,
                                                    float x, float y, float z, float J[3][3]) {
#pragma unroll
    for (int r = 0; r < 3; r++) J[r][0] = J[r][1] = J[r][2] = 0.f;
    if (!inside(A, x, y, z)) return make_float3(0.f, 0.f, 0.f);
    float X, Y, Z;
    to_index(A, x, y, z, X, Y, Z);
    const float s = (float)A.inv_dx_d;
    float vx = interp_component_grad(u, A.f[0], X, Y - 0.5f, Z - 0.5f, J[0]);
    float vy = interp_component_grad(v, A.f[1], X - 0.5f, Y, Z - 0.5f, J[1]);
    float vz = interp_component_grad(w, A.f[2], X - 0.5f, Y - 0.5f, Z, J[2]);
#pragma unroll
    for (int r = 0; r < 3; r++) {
        J[r][0] *= s;
        J[r][1] *= s;
        J[r][2] *= s;
    }
    return make_float3(vx, vy, vz);
}

// Transpose of interp_component in fixed point: g[node] += round(weight(node) * c * scale)
// by 64-bit integer atomics.  Integer addition is associative, so the node sums do
// not depend on the order in which the particles arrive.  |weight| <= 1 for
// Catmull-Rom, so |term| <= |c| * scale; the caller picks scale (a power of two)
// so that no node sum can leave the int64 range.
// round(w) to the nearest int64, ties to even, in FP32 and integer arithmetic (|w| < 2^62):
// below 2^23 the 32-bit conversion, above it w is an integer whose 24-bit significand
// is shifted into place.
__device__ __forceinline__ long long fix_round(float w) {
    if (fabsf(w) < 8388608.0f) return (long long)__float2int_rn(w);
    const unsigned bits = __float_as_uint(w);
    const long long mag = (long long)((bits & 0x7FFFFFu) | 0x800000u) << (int)(((bits >> 23) & 0xFFu) - 150u);
    return (bits >> 31) ? -mag : mag;
}

__device__ __forceinline__ void scatter_component_fixed(unsigned long long *__restrict__ g, const GridDim &f, float X,
                                                        float Y, float Z, float c, double scale) {
    if (c == 0.0f || scale == 0.0) return;
    // The term is round((double)(weight * c) * scale) with scale a power of two.  Within
    // float range the scaling is exact in FP32 too (a result below the normal range rounds
    // to 0 either way), so the term is formed without FP64, whose rate on GB300 is a
    // small fraction of FP32's; outside that range the FP64 form runs.
    const float scalef = (scale >= 0x1p-126 && scale <= 0x1p126) ? (float)scale : 0.0f;
    float fi = floorf(X), fj = floorf(Y), fk = floorf(Z);
    int i = (int)fi, j = (int)fj, k = (int)fk;
    float wx[4], wy[4], wz[4];
    catmull_rom_weights(X - fi, wx);
    catmull_rom_weights(Y - fj, wy);
    catmull_rom_weights(Z - fk, wz);
    const long long sy = f.sx, sz = (long long)f.sx * f.sy;
    unsigned long long *base = g + f.at(i - 1, j - 1, k - 1);
#pragma unroll
    for (int cc = 0; cc < 4; cc++)
#pragma unroll
        for (int b = 0; b < 4; b++) {
            float wbc = wz[cc] * wy[b] * c;
            unsigned long long *row = base + b * sy + cc * sz;
#pragma unroll
            for (int a = 0; a < 4; a++) {
                const float w = wx[a] * wbc;
                const long long t = scalef != 0.0f ? fix_round(w * scalef) : __double2ll_rn((double)w * scale);
                if (t) atomicAdd(row + a, (unsigned long long)t);
            }
        }
}

// Transpose of eval_velocity: adds c (a velocity adjoint) into fixed-point face grids.
__device__ __forceinline__ void scatter_velocity_fixed(const AdvArgs &A, unsigned long long *__restrict__ u,
                                                       unsigned long long *__restrict__ v,
                                                       unsigned long long *__restrict__ w, float x, float y, float z,
                                                       float3 c, double scale) {
    if (!inside(A, x, y, z)) return;
    float X, Y, Z;
    to_index(A, x, y, z, X, Y, Z);
    scatter_component_fixed(u, A.f[0], X, Y - 0.5f, Z - 0.5f, c.x, scale);
    scatter_component_fixed(v, A.f[1], X - 0.5f, Y, Z - 0.5f, c.y, scale);
    scatter_component_fixed(w, A.f[2], X - 0.5f, Y - 0.5f, Z, c.z, scale);
}

// The largest |component| of a scatter value, as float bits: for |x| the bit
// patterns order like the values, and a NaN sorts above +inf.
__device__ __forceinline__ unsigned abs_bits_max(unsigned m, float3 c) {
    m = max(m, __float_as_uint(fabsf(c.x)));
    m = max(m, __float_as_uint(fabsf(c.y)));
    return max(m, __float_as_uint(fabsf(c.z)));
}

}  // namespace gfs
