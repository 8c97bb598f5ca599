// advect.cu -- grid -> particle: PIC/FLIP velocity update and RK advection.
//
// k_g2p_advect fuses stages 11 and 12 of FluidSimulation::_stepFluid
// (fluidsimulation.cpp:3104-3209) for one particle per thread, in the
// particles' (cell, id) order so that a warp touches a compact set of faces:
//   vnew = tricubic(MAC, p), vold = tricubic(saved, p)
//   v    = 0.05 vnew + 0.95 (v + vnew - vold)                (:3118-3128)
//   p1   = RK4 through MAC (k1 = vnew: the same sample)       (particleadvector.cpp:1045-1054)
//   if cell(p1) is solid: pull p1 back along p0->p1           (:3145-3179, collision.cpp:303-449)
// The tricubic sample is MACVelocityField::evaluateVelocityAtPosition
// (macvelocityfield.cpp:350-559): Catmull-Rom over a 4x4x4 stencil per
// component, evaluated here in FP32 in separable form, reading the padded face
// grids (the four MAC samples: their row quads, one 16-byte load per stencil row)
// through the read-only path with no bounds checks (the zero halo is the
// reference's out-of-range value).  With a power-of-two dx the stencil index
// and the fractional offsets are formed exactly as the reference's doubles.
#include <mutex>

#include "gfs_internal.h"
#include "gfs_interp.cuh"

namespace gfs {

// Row quads of a face grid: q[x] = (g[x], g[x+1], g[x+2], g[x+3]) at every
// storage index x, 0 past the grid's end.  A Catmull-Rom stencil row of four x
// taps is then one aligned 16-byte load (row_taps) where the grid itself needs
// four 4-byte loads.  The four MAC samples of G2P (vnew and the RK4 stages) read
// the quads of the MAC field; the one sample of the saved field reads its taps
// directly (quads of both fields measured slower: their build costs more than the
// one sample saves).  blockIdx.y picks the grid.
struct QuadJob {
    const float *src[3];
    float4 *dst[3];
    long long n[3];
};

__global__ void __launch_bounds__(256) k_row_quads(QuadJob J) {
    const float *__restrict__ g = J.src[blockIdx.y];
    float4 *__restrict__ q = J.dst[blockIdx.y];
    const long long n = J.n[blockIdx.y];
    for (long long x = blockIdx.x * 256ll + threadIdx.x; x < n; x += (long long)gridDim.x * 256) {
        float4 t;
        t.x = g[x];
        t.y = x + 1 < n ? g[x + 1] : 0.f;
        t.z = x + 2 < n ? g[x + 2] : 0.f;
        t.w = x + 3 < n ? g[x + 3] : 0.f;
        q[x] = t;
    }
}

__global__ void __launch_bounds__(128) k_g2p_advect(AdvArgs A, float4 *__restrict__ pos, float4 *__restrict__ vel,
                                                    const uint32_t *__restrict__ num, long long nbound,
                                                    const float4 *__restrict__ mu, const float4 *__restrict__ mv,
                                                    const float4 *__restrict__ mw, const float *__restrict__ su,
                                                    const float *__restrict__ sv, const float *__restrict__ sw,
                                                    const uint8_t *__restrict__ mat) {
    long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (p >= nbound || p >= (long long)num[0]) return;
    float4 P = pos[p];
    float4 V = vel[p];
    float3 vnew = eval_velocity(A, mu, mv, mw, P.x, P.y, P.z);
    float3 vold = eval_velocity(A, su, sv, sw, P.x, P.y, P.z);
    // ParticleAdvector::_validateOutput on both samples (particleadvector.cpp:1139-1149)
    float3 vn = finite3(vnew) ? vnew : make_float3(0.f, 0.f, 0.f);
    float3 vo = finite3(vold) ? vold : make_float3(0.f, 0.f, 0.f);
    float4 Vn;
    Vn.x = __fadd_rn(__fmul_rn(A.a_pic, vn.x), __fmul_rn(A.b_flip, __fsub_rn(__fadd_rn(V.x, vn.x), vo.x)));
    Vn.y = __fadd_rn(__fmul_rn(A.a_pic, vn.y), __fmul_rn(A.b_flip, __fsub_rn(__fadd_rn(V.y, vn.y), vo.y)));
    Vn.z = __fadd_rn(__fmul_rn(A.a_pic, vn.z), __fmul_rn(A.b_flip, __fsub_rn(__fadd_rn(V.z, vn.z), vo.z)));
    Vn.w = 0.f;
    // RK4 through the MAC field; k1 is the vnew sample
    float3 p0 = make_float3(P.x, P.y, P.z);
    float3 k1 = vnew;
    float3 t = axpy3(p0, A.h, k1);
    float3 k2 = eval_velocity(A, mu, mv, mw, t.x, t.y, t.z);
    t = axpy3(p0, A.h, k2);
    float3 k3 = eval_velocity(A, mu, mv, mw, t.x, t.y, t.z);
    t = axpy3(p0, A.f1, k3);
    float3 k4 = eval_velocity(A, mu, mv, mw, t.x, t.y, t.z);
    float3 p1 = make_float3(rk4_comb(p0.x, A.f6, k1.x, k2.x, k3.x, k4.x),
                            rk4_comb(p0.y, A.f6, k1.y, k2.y, k3.y, k4.y),
                            rk4_comb(p0.z, A.f6, k1.z, k2.z, k3.z, k4.z));
    int ci, cj, ck;
    pos_cell(A, p1.x, p1.y, p1.z, ci, cj, ck);
    if (!(isfinite(p1.x) && isfinite(p1.y) && isfinite(p1.z)) || cell_solid(A, mat, ci, cj, ck))
        p1 = resolve_collision(A, mat, p0, p1);
    pos[p] = make_float4(p1.x, p1.y, p1.z, P.w);
    vel[p] = Vn;
}

static float float_ceil_of(double x) {
    float f = (float)x;
    if ((double)f < x) f = nextafterf(f, INFINITY);
    return f;
}

AdvArgs make_adv(const Grids &g, double dt, double ratio_pic) {
    AdvArgs A;
    for (int d = 0; d < 3; d++) A.f[d] = g.f[d];
    A.c = g.c;
    A.dx = g.dx;
    A.inv_dx_d = 1.0 / g.dx;
    A.inv_dx = (float)(1.0 / g.dx);
    int e;
    double m = frexp(g.dx, &e);
    A.pow2 = (m == 0.5) ? 1 : 0;
    A.bound[0] = float_ceil_of(g.dx * g.ni);
    A.bound[1] = float_ceil_of(g.dx * g.nj);
    A.bound[2] = float_ceil_of(g.dx * g.nk);
    A.h = (float)(0.5 * dt);
    A.f1 = (float)dt;
    A.f6 = (float)(dt / 6.0f);
    A.a_pic = (float)ratio_pic;
    A.b_flip = (float)(1 - ratio_pic);
    return A;
}

int g2p_advect(Sim *s, double dt) {
    Ctx *ctx = s->ctx;
    ProfScope prof(ctx, KC_G2P);
    AdvArgs A = make_adv(s->g, dt, s->params.ratio_pic);
    long long nb = s->n_bound;
    if (nb == 0) return GFS_OK;
    QuadJob J;
    for (int d = 0; d < 3; d++) {
        J.src[d] = s->mac[d].as<float>();
        J.dst[d] = s->quad[d].as<float4>();
        J.n[d] = s->g.f[d].size;
    }
    k_row_quads<<<dim3((unsigned)ctx->num_sms * 4, 3), 256, 0, ctx->stream>>>(J);
    ctx->launches++;
    GFS_LAUNCH_CHECK();
    k_g2p_advect<<<grid_blocks(nb, 128), 128, 0, ctx->stream>>>(
        A, s->pos.as<float4>(), s->vel.as<float4>(), s->num.as<uint32_t>(), nb, s->quad[0].as<float4>(),
        s->quad[1].as<float4>(), s->quad[2].as<float4>(), s->saved[0].as<float>(), s->saved[1].as<float>(),
        s->saved[2].as<float>(), s->mat.as<uint8_t>());
    ctx->launches++;
    GFS_LAUNCH_CHECK();
    return GFS_OK;
}

// -------------------------------------------- standalone point evaluation

// order 0: tricubic sample (validated); 1..4: RK of that order
// (ParticleAdvector::_RK1.._RK4, particleadvector.cpp:1045-1078).
__global__ void __launch_bounds__(128) k_points(AdvArgs A, const float *__restrict__ pts, long long n,
                                                const float *__restrict__ u, const float *__restrict__ v,
                                                const float *__restrict__ w, float *__restrict__ out, int order,
                                                int validate, float dtf, float h05, float h075, float f9) {
    long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= n) return;
    float3 p0 = make_float3(pts[3 * q], pts[3 * q + 1], pts[3 * q + 2]);
    float3 r;
    float3 k1 = eval_velocity(A, u, v, w, p0.x, p0.y, p0.z);
    if (order == 0) {
        r = (validate && !finite3(k1)) ? make_float3(0.f, 0.f, 0.f) : k1;
    } else if (order == 1) {
        r = axpy3(p0, dtf, k1);
    } else if (order == 2) {
        float3 t = axpy3(p0, h05, k1);
        float3 k2 = eval_velocity(A, u, v, w, t.x, t.y, t.z);
        r = axpy3(p0, dtf, k2);
    } else if (order == 3) {
        float3 t = axpy3(p0, h05, k1);
        float3 k2 = eval_velocity(A, u, v, w, t.x, t.y, t.z);
        t = axpy3(p0, h075, k2);
        float3 k3 = eval_velocity(A, u, v, w, t.x, t.y, t.z);
        // p0 + (float)(dt/9.0f)*(2k1 + 3k2 + 4k3)
        float sx = __fadd_rn(__fadd_rn(__fmul_rn(2.f, k1.x), __fmul_rn(3.f, k2.x)), __fmul_rn(4.f, k3.x));
        float sy = __fadd_rn(__fadd_rn(__fmul_rn(2.f, k1.y), __fmul_rn(3.f, k2.y)), __fmul_rn(4.f, k3.y));
        float sz = __fadd_rn(__fadd_rn(__fmul_rn(2.f, k1.z), __fmul_rn(3.f, k2.z)), __fmul_rn(4.f, k3.z));
        r = make_float3(__fadd_rn(p0.x, __fmul_rn(f9, sx)), __fadd_rn(p0.y, __fmul_rn(f9, sy)),
                        __fadd_rn(p0.z, __fmul_rn(f9, sz)));
    } else {
        float3 t = axpy3(p0, A.h, k1);
        float3 k2 = eval_velocity(A, u, v, w, t.x, t.y, t.z);
        t = axpy3(p0, A.h, k2);
        float3 k3 = eval_velocity(A, u, v, w, t.x, t.y, t.z);
        t = axpy3(p0, A.f1, k3);
        float3 k4 = eval_velocity(A, u, v, w, t.x, t.y, t.z);
        r = make_float3(rk4_comb(p0.x, A.f6, k1.x, k2.x, k3.x, k4.x), rk4_comb(p0.y, A.f6, k1.y, k2.y, k3.y, k4.y),
                        rk4_comb(p0.z, A.f6, k1.z, k2.z, k3.z, k4.z));
    }
    out[3 * q] = r.x;
    out[3 * q + 1] = r.y;
    out[3 * q + 2] = r.z;
}

int interpolate_points(Ctx *ctx, const Grids &g, float *const mac[3], const float *d_points, int64_t n,
                       float *d_out, int rk_order, double dt, bool validate) {
    if (n == 0) return GFS_OK;
    AdvArgs A = make_adv(g, dt, 0.0);
    k_points<<<grid_blocks(n, 128), 128, 0, ctx->stream>>>(A, d_points, n, mac[0], mac[1], mac[2], d_out, rk_order,
                                                           validate ? 1 : 0, (float)dt, (float)(0.5 * dt),
                                                           (float)(0.75 * dt), (float)(dt / 9.0f));
    ctx->launches++;
    GFS_LAUNCH_CHECK();
    return GFS_OK;
}


// ------------------------------------------------ no-allocation variant
//
// gfs_tricubic_interpolate_noalloc: the tricubic sampler of
// gfs_tricubic_interpolate for callers that cannot allocate device memory
// (hosts whose device memory all comes from their own allocator or arena,
// real-time or callback code where cudaMalloc / cudaFree are not allowed).
// The caller passes device-accessible inputs and outputs and a stream; the
// padded copies of U, V and W that the sampler reads live in the fixed scratch
// array below, which every GPU that loads this library keeps until the process
// exits.  All calls share that array: two calls that overlap on the GPU race on
// it, and each call first clears the part it uses (the halo must read as zero).

#define GFS_NOALLOC_SCRATCH_FLOATS (12u << 20)   // 48 MiB: padded U+V+W of up to ~150^3 cells

static __device__ __align__(256) float g_noalloc_scratch[GFS_NOALLOC_SCRATCH_FLOATS];

namespace {
std::mutex g_noalloc_mu;
float *g_noalloc_base[256] = {nullptr};   // device address of the scratch, per device

__global__ void k_pad_face(const float *__restrict__ src, GridDim g, float *__restrict__ dst) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y, k = blockIdx.z;
    if (i >= g.nx) return;
    dst[g.at(i, j, k)] = src[i + (long long)g.nx * (j + (long long)g.ny * k)];
}
}  // namespace

}  // namespace gfs

extern "C" int gfs_tricubic_interpolate_noalloc(int ni, int nj, int nk, double dx, const float *d_u,
                                                const float *d_v, const float *d_w, const float *d_points,
                                                int64_t n, float *d_out, void *stream) {
    using namespace gfs;
    if (ni <= 0 || nj <= 0 || nk <= 0 || !(dx > 0.0) || n < 0 || !d_u || !d_v || !d_w ||
        (n > 0 && (!d_points || !d_out))) {
        set_error(GFS_ERR_INVALID, "gfs_tricubic_interpolate_noalloc: invalid arguments");
        return GFS_ERR_INVALID;
    }
    // the padded extents below are int sums: reject dimensions that could overflow
    // them before forming any (the scratch bound rejects everything near this anyway)
    if (ni > (1 << 20) || nj > (1 << 20) || nk > (1 << 20) || (long long)ni * nj * nk >= (1LL << 31)) {
        set_error(GFS_ERR_INVALID, "gfs_tricubic_interpolate_noalloc: a %d x %d x %d grid is too large", ni, nj, nk);
        return GFS_ERR_INVALID;
    }
    Grids g = make_grids(ni, nj, nk, dx);
    unsigned long long need = (unsigned long long)g.f[0].size + g.f[1].size + g.f[2].size;
    if (need > GFS_NOALLOC_SCRATCH_FLOATS) {
        set_error(GFS_ERR_INVALID,
                  "gfs_tricubic_interpolate_noalloc: a %d x %d x %d grid needs %llu scratch floats, the fixed "
                  "scratch holds %u",
                  ni, nj, nk, need, (unsigned)GFS_NOALLOC_SCRATCH_FLOATS);
        return GFS_ERR_INVALID;
    }
    int dev = 0;
    GFS_CUDA_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 256) {
        set_error(GFS_ERR_INVALID, "gfs_tricubic_interpolate_noalloc: device %d out of range", dev);
        return GFS_ERR_INVALID;
    }
    float *base = nullptr;
    {
        // first call on this device (the current one): look up the scratch's device
        // address.  A cached address that the runtime no longer knows as device
        // memory of this device (the device was reset since, and the library's
        // module loaded again) is looked up again.
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (g_noalloc_base[dev]) {
            cudaPointerAttributes at{};
            if (cudaPointerGetAttributes(&at, g_noalloc_base[dev]) != cudaSuccess ||
                at.type != cudaMemoryTypeDevice || at.device != dev) {
                cudaGetLastError();
                g_noalloc_base[dev] = nullptr;
            }
        }
        if (!g_noalloc_base[dev]) {
            void *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) {
                set_error(GFS_ERR_CUDA, "gfs_tricubic_interpolate_noalloc: cudaGetSymbolAddress: %s",
                          cudaGetErrorString(e));
                return GFS_ERR_CUDA;
            }
            g_noalloc_base[dev] = static_cast<float *>(p);
        }
        base = g_noalloc_base[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    float *pad[3] = {base, base + g.f[0].size, base + g.f[0].size + g.f[1].size};
    const float *src[3] = {d_u, d_v, d_w};
    GFS_CUDA_CHECK(cudaMemsetAsync(base, 0, (size_t)need * sizeof(float), st));
    for (int d = 0; d < 3; d++) {
        dim3 grid(grid_blocks(g.f[d].nx, 128), g.f[d].ny, g.f[d].nz);
        k_pad_face<<<grid, 128, 0, st>>>(src[d], g.f[d], pad[d]);
    }
    GFS_LAUNCH_CHECK();
    if (n > 0) {
        AdvArgs A = make_adv(g, 0.0, 0.0);
        k_points<<<grid_blocks(n, 128), 128, 0, st>>>(A, d_points, n, pad[0], pad[1], pad[2], d_out, 0, 1, 0.f, 0.f,
                                                      0.f, 0.f);
        GFS_LAUNCH_CHECK();
    }
    return GFS_OK;
}
