// gfs_common.cuh -- shared device/host definitions of the GB300 FLIP core.
//
// Grid storage.  Every grid (cell grids ni x nj x nk and the three MAC face
// grids) is stored dense with a halo of GFS_PAD cells on every side, x fastest:
//     storage index = (i+P) + SX*((j+P) + SY*(k+P)),  SX = nx+2P, SY = ny+2P.
// The halo of a face grid holds 0 (the reference's out-of-range value for
// MACVelocityField, macvelocityfield.cpp:37-45); the halo of the material grid
// holds SOLID (fluidmaterialgrid.cpp:26).  Stencils therefore never branch on
// bounds.  Particles live in SoA float4: pos4 = (x, y, z, id bits),
// vel4 = (vx, vy, vz, 0), sorted by (cell, id).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#define GFS_PAD 2

#define GFS_AIR 0
#define GFS_FLUID 1
#define GFS_SOLID 2

// Per-cell pressure flags: bit0 = fluid, bits1..3 = number of non-solid
// 6-neighbours (the MatrixCell::diag of pressuresolver.h:81-88).
#define GFS_PF_FLUID 1u

struct GridDim {
    int nx, ny, nz;      // logical extent
    int sx, sy;          // storage strides: sx = nx + 2P, sy = ny + 2P
    long long size;      // total storage elements

    __host__ __device__ inline long long at(int i, int j, int k) const {
        return (long long)(i + GFS_PAD) + (long long)sx * ((long long)(j + GFS_PAD) + (long long)sy * (k + GFS_PAD));
    }
    __host__ __device__ inline bool in(int i, int j, int k) const {
        return i >= 0 && j >= 0 && k >= 0 && i < nx && j < ny && k < nz;
    }
};

static inline GridDim make_grid(int nx, int ny, int nz) {
    GridDim g;
    g.nx = nx; g.ny = ny; g.nz = nz;
    g.sx = nx + 2 * GFS_PAD;
    g.sy = ny + 2 * GFS_PAD;
    g.size = (long long)g.sx * g.sy * (long long)(nz + 2 * GFS_PAD);
    return g;
}

// The four grids of one simulation: cells and U/V/W faces.
struct Grids {
    GridDim c, f[3];
    int ni, nj, nk;
    double dx;
};

static inline Grids make_grids(int ni, int nj, int nk, double dx) {
    Grids g;
    g.ni = ni; g.nj = nj; g.nk = nk; g.dx = dx;
    g.c = make_grid(ni, nj, nk);
    g.f[0] = make_grid(ni + 1, nj, nk);
    g.f[1] = make_grid(ni, nj + 1, nk);
    g.f[2] = make_grid(ni, nj, nk + 1);
    return g;
}

// FluidMaterialGrid::isFaceBorderingMaterialU/V/W (fluidmaterialgrid.cpp:119-143)
// over a padded material grid.  Face (i,j,k) of direction d separates cell
// (i,j,k) - e_d from cell (i,j,k); at the faces on the domain boundary only the
// inside cell counts.
__device__ __forceinline__ bool face_borders(const uint8_t *mat, const GridDim &c, int d, int i,
                                             int j, int k, uint8_t m) {
    int n = d == 0 ? c.nx : (d == 1 ? c.ny : c.nz);
    int t = d == 0 ? i : (d == 1 ? j : k);
    int pi = i - (d == 0), pj = j - (d == 1), pk = k - (d == 2);
    if (t == n) return mat[c.at(pi, pj, pk)] == m;
    if (t > 0) return mat[c.at(i, j, k)] == m || mat[c.at(pi, pj, pk)] == m;
    return mat[c.at(i, j, k)] == m;
}

// Catmull-Rom weights of Interpolation::cubicInterpolate (interpolation.cpp:44-46)
// written in separable form: cubic(p, x) = sum_a w_a(x) p[a].
__device__ __forceinline__ void catmull_rom_weights(float x, float w[4]) {
    float x2 = x * x, x3 = x2 * x;
    w[0] = 0.5f * (-x + 2.0f * x2 - x3);
    w[1] = 0.5f * (2.0f - 5.0f * x2 + 3.0f * x3);
    w[2] = 0.5f * (x + 4.0f * x2 - 3.0f * x3);
    w[3] = 0.5f * (x3 - x2);
}

// Bounded spin for wavefront progress flags: after this many polls a kernel
// records GFS_DEV_ERR_TIMEOUT and stops waiting.
#define GFS_SPIN_LIMIT (1 << 22)
#define GFS_DEV_ERR_TIMEOUT 1u

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_u32(unsigned *p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

#define GFS_CUDA_CHECK(expr)                                                       \
    do {                                                                           \
        cudaError_t _e = (expr);                                                   \
        if (_e != cudaSuccess) {                                                   \
            gfs::set_error(GFS_ERR_CUDA, "%s:%d: %s: %s", __FILE__, __LINE__, #expr, \
                           cudaGetErrorString(_e));                                \
            return GFS_ERR_CUDA;                                                   \
        }                                                                          \
    } while (0)

#define GFS_LAUNCH_CHECK()                                                          \
    do {                                                                            \
        cudaError_t _e = cudaGetLastError();                                        \
        if (_e != cudaSuccess) {                                                    \
            gfs::set_error(GFS_ERR_CUDA, "%s:%d: kernel launch: %s", __FILE__, __LINE__, \
                           cudaGetErrorString(_e));                                 \
            return GFS_ERR_CUDA;                                                    \
        }                                                                           \
    } while (0)

static inline unsigned grid_blocks(long long n, int threads) {
    long long b = (n + threads - 1) / threads;
    return (unsigned)(b < 1 ? 1 : b);
}
