// sources.cu -- fluid sources on the device-resident particles:
// FluidSimulation::_updateFluidSources (fluidsimulation.cpp:1854-1879), which
// the reference calls at the start of _updateFluidCells (:1990-1994), after the
// particles in solid cells are removed and before the cells are classified.
//
// Each inflow source, in order (_updateInflowFluidSource, :1836-1852):
//   1. its overlapping air cells (FluidSource::getAirCells, fluidsource.cpp;
//      sphere: cell centres strictly within the radius,
//      SphericalFluidSource::_getOverlappingCells; cuboid: every cell of its index
//      bounds, CuboidFluidSource::_getOverlappingCells) each get 8 marker
//      particles at the 2x2x2 sub-cell centres plus jitter, with the source's
//      velocity, and become fluid (_addNewFluidCells :1749-1759,
//      _addMarkerParticlesToCell :1223-1246);
//   2. within the source's AABB fitted to the grid, every sub-cell of an
//      overlapping fluid-or-air cell that holds no marker particle gets one, at
//      the sub-cell centre plus jitter, and its cell becomes fluid
//      (_getNewFluidParticles :1769-1834, _addNewFluidParticles :1761-1768).
// Then the particles in the overlapping fluid cells of the outflow sources are
// removed (_removeMarkerParticlesFromCells :1717-1730).
//
// Geometry follows the reference's types step by step: positions are
// vmath::vec3 (float), radii, extents and dx double, index bounds from
// Grid3d::getGridIndexBounds / fitAABBtoGrid (grid3d.h:350-371, 426-439, 485-502), the overlap
// test a float dot product compared with a double radius squared.  The box
// bounds are computed on the host; the per-cell tests run on the device with
// non-contracted float arithmetic.
//
// Jitter: the reference draws each component from rand() in [-j, j], j = 0.25 *
// jitter factor * dx (:1219-1221, factor 0.1 by default, fluidsimulation.h:1111).
// The rand() stream is not reproducible outside that process, so here each
// component is a counter-based hash of (seed, particle id, axis) mapped to
// [-j, j]; with a jitter factor of 0 the positions are the reference's exactly.
// New particles take ids from the simulation's next unused id, in the order
// the reference creates them (cells, then sub-cells, each i fastest).
#include <cmath>
#include <cstdint>
#include <unordered_set>
#include <vector>

#include "gfs_internal.h"

namespace gfs {

#define GFS_REMOVE_FLAG 0x80   // material bit: remove the cell's particles at the next sort

namespace {

// ---- vmath / Grid3d steps on the host (grid3d.h) ------------------------------
struct I3 {
    int i, j, k;
};
I3 pos_to_index(float x, float y, float z, double dx) {   // positionToGridIndex (:58-63)
    double inv = 1.0 / dx;
    return {(int)floor(x * inv), (int)floor(y * inv), (int)floor(z * inv)};
}
float index_to_pos(int i, double dx) { return (float)((float)i * dx); }   // GridIndexToPosition
bool in_range(I3 g, int ni, int nj, int nk) {
    return g.i >= 0 && g.j >= 0 && g.k >= 0 && g.i < ni && g.j < nj && g.k < nk;
}

// Grid3d::getGridIndexBounds(vec3 p, double r, ...) (:350-371)
void bounds_sphere(const float p[3], double r, double dx, int ni, int nj, int nk, I3 &g1, I3 &g2) {
    I3 c = pos_to_index(p[0], p[1], p[2], dx);
    float t[3] = {p[0] - index_to_pos(c.i, dx), p[1] - index_to_pos(c.j, dx), p[2] - index_to_pos(c.k, dx)};
    double inv = 1.0 / dx;
    int cc[3] = {c.i, c.j, c.k}, lo[3], hi[3], mx[3] = {ni, nj, nk};
    for (int a = 0; a < 3; a++) {
        lo[a] = cc[a] - (int)fmax(0.0, ceil((r - t[a]) * inv));
        hi[a] = cc[a] + (int)fmax(0.0, ceil((r - dx + t[a]) * inv));
        lo[a] = (int)fmax(lo[a], 0);
        hi[a] = (int)fmin(hi[a], mx[a] - 1);
    }
    g1 = {lo[0], lo[1], lo[2]};
    g2 = {hi[0], hi[1], hi[2]};
}

// An AABB: float position, double extents (aabb.h)
struct Box {
    float p[3];
    double w[3];
};

// Grid3d::getGridIndexBounds(AABB, ...) (:426-439)
void bounds_box(const Box &b, double dx, int ni, int nj, int nk, I3 &g1, I3 &g2) {
    float q[3] = {b.p[0] + (float)b.w[0], b.p[1] + (float)b.w[1], b.p[2] + (float)b.w[2]};
    g1 = pos_to_index(b.p[0], b.p[1], b.p[2], dx);
    g2 = pos_to_index(q[0], q[1], q[2], dx);
    g1 = {(int)fmax(g1.i, 0), (int)fmax(g1.j, 0), (int)fmax(g1.k, 0)};
    g2 = {(int)fmin(g2.i, ni - 1), (int)fmin(g2.j, nj - 1), (int)fmin(g2.k, nk - 1)};
}

// Grid3d::fitAABBtoGrid (:485-502) and AABB(vec3 p1, vec3 p2) (aabb.cpp:33-45)
Box fit_box(const Box &b, double dx, int ni, int nj, int nk) {
    float pmin[3] = {b.p[0], b.p[1], b.p[2]};
    float pmax[3] = {b.p[0] + (float)b.w[0], b.p[1] + (float)b.w[1], b.p[2] + (float)b.w[2]};
    I3 gmin = pos_to_index(pmin[0], pmin[1], pmin[2], dx);
    I3 gmax = pos_to_index(pmax[0], pmax[1], pmax[2], dx);
    if (!in_range(gmin, ni, nj, nk)) pmin[0] = pmin[1] = pmin[2] = 0.0f;
    const float eps = 10e-9f;
    if (!in_range(gmax, ni, nj, nk)) {
        float dxf = (float)dx;
        pmax[0] = index_to_pos(gmax.i, dx) + dxf - eps;
        pmax[1] = index_to_pos(gmax.j, dx) + dxf - eps;
        pmax[2] = index_to_pos(gmax.k, dx) + dxf - eps;
    }
    Box o;
    for (int a = 0; a < 3; a++) {
        double mn = fmin(pmin[a], pmax[a]), mx = fmax(pmin[a], pmax[a]);
        o.p[a] = (float)mn;
        o.w[a] = mx - mn;
    }
    return o;
}

}  // namespace

// Geometry of one source for the kernels.
struct SrcGeom {
    int sphere;
    float c[3];          // sphere centre
    double rsq;          // radius^2
    int g1[3], n1[3];    // overlapping-cell index bounds: first cell, extent
    int f1[3], nf[3];    // fitted-AABB index bounds (the sub-cell grid covers 2 nf)
    float fp[3];         // fitted AABB position
    double fw[3];        // fitted AABB extents
    float off[3];        // GridIndexToPosition(f1)
    float vel[3];
};

__host__ SrcGeom source_geometry(const gfs_fluid_source &src, double dx, int ni, int nj, int nk) {
    SrcGeom G{};
    G.sphere = src.shape == GFS_SOURCE_SPHERE;
    I3 g1, g2;
    Box aabb;
    if (G.sphere) {
        double r = src.radius > 0.0 ? src.radius : 0.0;   // SphericalFluidSource(pos, r) (:25-29)
        for (int a = 0; a < 3; a++) G.c[a] = src.position[a];
        G.rsq = r * r;
        bounds_sphere(src.position, r, dx, ni, nj, nk, g1, g2);
        // SphericalFluidSource::getAABB (:48-52)
        float rf = (float)r;
        for (int a = 0; a < 3; a++) {
            aabb.p[a] = src.position[a] - rf;
            aabb.w[a] = 2.0 * r;
        }
    } else {
        for (int a = 0; a < 3; a++) {
            aabb.p[a] = src.position[a];
            aabb.w[a] = src.size[a];
        }
        bounds_box(aabb, dx, ni, nj, nk, g1, g2);
    }
    int lo[3] = {g1.i, g1.j, g1.k}, hi[3] = {g2.i, g2.j, g2.k};
    for (int a = 0; a < 3; a++) {
        G.g1[a] = lo[a];
        G.n1[a] = hi[a] >= lo[a] ? hi[a] - lo[a] + 1 : 0;
    }
    Box fit = fit_box(aabb, dx, ni, nj, nk);
    I3 f1, f2;
    bounds_box(fit, dx, ni, nj, nk, f1, f2);
    int flo[3] = {f1.i, f1.j, f1.k}, fhi[3] = {f2.i, f2.j, f2.k};
    for (int a = 0; a < 3; a++) {
        G.f1[a] = flo[a];
        G.nf[a] = fhi[a] >= flo[a] ? fhi[a] - flo[a] + 1 : 0;
        G.fp[a] = fit.p[a];
        G.fw[a] = fit.w[a];
        G.off[a] = index_to_pos(flo[a], dx);
        G.vel[a] = src.velocity[a];
    }
    return G;
}

// ---- device side ---------------------------------------------------------------

// jitter component in [-j, j] for (seed, particle id, axis): splitmix64 of the counter
__device__ __forceinline__ float jitter_component(unsigned long long seed, uint32_t id, int axis, double j) {
    unsigned long long z = seed + 0x9E3779B97F4A7C15ull * ((unsigned long long)id * 3ull + (unsigned long long)axis + 1ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    double u = (double)(z >> 11) * (1.0 / 9007199254740992.0);
    return (float)(-j + 2.0 * j * u);
}

// GridIndexToCellCenter (grid3d.h:103-106): (float)i*dx + 0.5*dx in double, stored as float
__device__ __forceinline__ float cell_center(int i, double dx) { return (float)((double)(float)i * dx + 0.5 * dx); }

__device__ __forceinline__ void box_index(long long li, const int n[3], int &x, int &y, int &z) {
    x = (int)(li % n[0]);
    long long r = li / n[0];
    y = (int)(r % n[1]);
    z = (int)(r / n[1]);
}

// 1. overlapping cells: 1 air (gets 8 particles), 2 fluid, 0 other
__global__ void k_src_cells(SrcGeom G, GridDim c, double dx, const uint8_t *__restrict__ mat,
                            uint8_t *__restrict__ mark, uint32_t *__restrict__ is_air, long long n) {
    long long li = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (li >= n) return;
    int x, y, z;
    box_index(li, G.n1, x, y, z);
    int i = G.g1[0] + x, j = G.g1[1] + y, k = G.g1[2] + z;
    bool overlap = true;
    if (G.sphere) {
        // SphericalFluidSource::_getOverlappingCells: float v = centre - position, dot in float
        float vx = __fsub_rn(cell_center(i, dx), G.c[0]), vy = __fsub_rn(cell_center(j, dx), G.c[1]),
              vz = __fsub_rn(cell_center(k, dx), G.c[2]);
        float d2 = __fadd_rn(__fadd_rn(__fmul_rn(vx, vx), __fmul_rn(vy, vy)), __fmul_rn(vz, vz));
        overlap = (double)d2 < G.rsq;
    }
    uint8_t m = mat[c.at(i, j, k)];
    uint8_t t = overlap ? (m == GFS_AIR ? 1 : (m == GFS_FLUID ? 2 : 0)) : 0;
    mark[li] = t;
    is_air[li] = t == 1;
}

// _addMarkerParticlesToCell (:1223-1246): 8 particles at the cell's 2x2x2
// sub-cell centres plus jitter, written to slots slot0.. with ids id0..
__device__ __forceinline__ void add_cell_particles(int i, int j, int k, double dx, const float v[3],
                                                   float4 *__restrict__ pos, float4 *__restrict__ vel,
                                                   long long slot0, uint32_t id0, unsigned long long seed,
                                                   double jit) {
    const double q = 0.25 * dx;
    const float cx = cell_center(i, dx), cy = cell_center(j, dx), cz = cell_center(k, dx);
    // (-,-,-) (+,-,-) (+,-,+) (-,-,+) (-,+,-) (+,+,-) (+,+,+) (-,+,+)
    const int sx[8] = {-1, 1, 1, -1, -1, 1, 1, -1}, sy[8] = {-1, -1, -1, -1, 1, 1, 1, 1},
              sz[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
    for (int idx = 0; idx < 8; idx++) {
        uint32_t id = id0 + (uint32_t)idx;
        float px = (float)((double)cx + sx[idx] * q), py = (float)((double)cy + sy[idx] * q),
              pz = (float)((double)cz + sz[idx] * q);
        px = __fadd_rn(px, jitter_component(seed, id, 0, jit));
        py = __fadd_rn(py, jitter_component(seed, id, 1, jit));
        pz = __fadd_rn(pz, jitter_component(seed, id, 2, jit));
        pos[slot0 + idx] = make_float4(px, py, pz, __uint_as_float(id));
        vel[slot0 + idx] = make_float4(v[0], v[1], v[2], 0.f);
    }
}

// 1'. 8 particles per air cell, the cell becomes fluid
__global__ void k_src_fill_cells(SrcGeom G, GridDim c, double dx, uint8_t *__restrict__ mat,
                                 const uint8_t *__restrict__ mark, const uint32_t *__restrict__ scan, long long n,
                                 float4 *__restrict__ pos, float4 *__restrict__ vel, long long base,
                                 uint32_t id0, unsigned long long seed, double jit) {
    long long li = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (li >= n || mark[li] != 1) return;
    int x, y, z;
    box_index(li, G.n1, x, y, z);
    int i = G.g1[0] + x, j = G.g1[1] + y, k = G.g1[2] + z;
    mat[c.at(i, j, k)] = GFS_FLUID;
    long long q8 = (long long)scan[li] * 8;
    add_cell_particles(i, j, k, dx, G.vel, pos, vel, base + q8, id0 + (uint32_t)q8, seed, jit);
}

// 2. sub-cell grid of the fitted AABB: 1 for the sub-cells of overlapping fluid-or-air cells
__global__ void k_src_subgrid(SrcGeom G, const uint8_t *__restrict__ mark, uint32_t *__restrict__ sub, long long n) {
    long long li = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (li >= n) return;
    const int ns[3] = {2 * G.nf[0], 2 * G.nf[1], 2 * G.nf[2]};
    int x, y, z;
    box_index(li, ns, x, y, z);
    int i = G.f1[0] + x / 2 - G.g1[0], j = G.f1[1] + y / 2 - G.g1[1], k = G.f1[2] + z / 2 - G.g1[2];
    bool valid = false;
    if (i >= 0 && j >= 0 && k >= 0 && i < G.n1[0] && j < G.n1[1] && k < G.n1[2])
        valid = mark[i + (long long)G.n1[0] * (j + (long long)G.n1[1] * k)] != 0;
    sub[li] = valid ? 1u : 0u;
}

// 2'. sub-cells holding a particle inside the fitted AABB are not refilled
__global__ void k_src_occupy(SrcGeom G, double dx, const float4 *__restrict__ pos, long long n,
                             uint32_t *__restrict__ sub) {
    long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= n) return;
    float4 p = pos[q];
    // AABB::isPointInside (aabb.cpp:123-126)
    if (!((double)p.x >= (double)G.fp[0] && (double)p.y >= (double)G.fp[1] && (double)p.z >= (double)G.fp[2] &&
          (double)p.x < (double)G.fp[0] + G.fw[0] && (double)p.y < (double)G.fp[1] + G.fw[1] &&
          (double)p.z < (double)G.fp[2] + G.fw[2]))
        return;
    const double inv = 1.0 / (0.5 * dx);
    int x = (int)floor((double)__fsub_rn(p.x, G.off[0]) * inv), y = (int)floor((double)__fsub_rn(p.y, G.off[1]) * inv),
        z = (int)floor((double)__fsub_rn(p.z, G.off[2]) * inv);
    if (x < 0 || y < 0 || z < 0 || x >= 2 * G.nf[0] || y >= 2 * G.nf[1] || z >= 2 * G.nf[2]) return;
    sub[x + 2LL * G.nf[0] * (y + 2LL * G.nf[1] * z)] = 0u;
}

// 2''. one particle per empty sub-cell: its centre + offset + jitter; its cell becomes fluid
__global__ void k_src_new_particles(SrcGeom G, GridDim c, double dx, uint8_t *__restrict__ mat,
                                    const uint32_t *__restrict__ sub, const uint32_t *__restrict__ scan,
                                    long long n, float4 *__restrict__ pos, float4 *__restrict__ vel, long long base,
                                    uint32_t id0, unsigned long long seed, double jit) {
    long long li = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (li >= n || !sub[li]) return;
    const int ns[3] = {2 * G.nf[0], 2 * G.nf[1], 2 * G.nf[2]};
    int x, y, z;
    box_index(li, ns, x, y, z);
    const double hdx = 0.5 * dx;
    long long q = scan[li];
    uint32_t id = id0 + (uint32_t)q;
    float px = __fadd_rn(__fadd_rn(cell_center(x, hdx), G.off[0]), jitter_component(seed, id, 0, jit));
    float py = __fadd_rn(__fadd_rn(cell_center(y, hdx), G.off[1]), jitter_component(seed, id, 1, jit));
    float pz = __fadd_rn(__fadd_rn(cell_center(z, hdx), G.off[2]), jitter_component(seed, id, 2, jit));
    pos[base + q] = make_float4(px, py, pz, __uint_as_float(id));
    vel[base + q] = make_float4(G.vel[0], G.vel[1], G.vel[2], 0.f);
    const double inv = 1.0 / dx;
    int i = (int)floor((double)px * inv), j = (int)floor((double)py * inv), k = (int)floor((double)pz * inv);
    if (c.in(i, j, k)) mat[c.at(i, j, k)] = GFS_FLUID;
}

// largest particle id + 1 (ids ride in pos.w)
__global__ void k_src_max_id(const float4 *__restrict__ pos, long long n, uint32_t *__restrict__ out) {
    long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    uint32_t v = q < n ? __float_as_uint(pos[q].w) + 1u : 0u;
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_down_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0 && v) atomicMax(out, v);
}

// outflow: the overlapping fluid cells are flagged for removal
__global__ void k_src_outflow(SrcGeom G, GridDim c, double dx, uint8_t *__restrict__ mat, long long n) {
    long long li = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (li >= n) return;
    int x, y, z;
    box_index(li, G.n1, x, y, z);
    int i = G.g1[0] + x, j = G.g1[1] + y, k = G.g1[2] + z;
    if (G.sphere) {
        float vx = __fsub_rn(cell_center(i, dx), G.c[0]), vy = __fsub_rn(cell_center(j, dx), G.c[1]),
              vz = __fsub_rn(cell_center(k, dx), G.c[2]);
        float d2 = __fadd_rn(__fadd_rn(__fmul_rn(vx, vx), __fmul_rn(vy, vy)), __fmul_rn(vz, vz));
        if (!((double)d2 < G.rsq)) return;
    }
    long long at = c.at(i, j, k);
    if ((mat[at] & 0x7F) == GFS_FLUID) mat[at] |= GFS_REMOVE_FLAG;
}

__global__ void k_src_clear_flags(uint8_t *__restrict__ mat, long long n) {
    long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q < n) mat[q] &= (uint8_t)~GFS_REMOVE_FLAG;
}

// ---- fluid-cell queues (FluidSimulation::addFluidCells / removeFluidCells) ----

// One queued cell of _addedFluidCellQueue with its group's velocity.
struct CellEntry {
    int i, j, k;
    float v[3];
};

// addFluidCells keeps only the cells that are air when it is called (:900-902)
__global__ void k_cells_material(GridDim c, const uint8_t *__restrict__ mat, const int32_t *__restrict__ ijk,
                                 long long n, uint8_t *__restrict__ out) {
    long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q < n) out[q] = mat[c.at(ijk[3 * q], ijk[3 * q + 1], ijk[3 * q + 2])];
}

// _addNewFluidCells (:1749-1759): the entries whose cell is still air
__global__ void k_cells_air(GridDim c, const uint8_t *__restrict__ mat, const CellEntry *__restrict__ e,
                            long long n, uint32_t *__restrict__ is_air) {
    long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q < n) is_air[q] = mat[c.at(e[q].i, e[q].j, e[q].k)] == GFS_AIR;
}

// ... get 8 particles each and become fluid
__global__ void k_cells_fill(GridDim c, double dx, uint8_t *__restrict__ mat, const CellEntry *__restrict__ e,
                             const uint32_t *__restrict__ is_air, const uint32_t *__restrict__ scan, long long n,
                             float4 *__restrict__ pos, float4 *__restrict__ vel, long long base, uint32_t id0,
                             unsigned long long seed, double jit) {
    long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= n || !is_air[q]) return;
    const CellEntry E = e[q];
    mat[c.at(E.i, E.j, E.k)] = GFS_FLUID;
    long long q8 = (long long)scan[q] * 8;
    add_cell_particles(E.i, E.j, E.k, dx, E.v, pos, vel, base + q8, id0 + (uint32_t)q8, seed, jit);
}

// _updateRemovedFluidCellQueue (:1895-1930): the listed cells lose their particles at a sort
__global__ void k_cells_mark_removal(GridDim c, uint8_t *__restrict__ mat, const int32_t *__restrict__ ijk,
                                     long long n) {
    long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q < n) mat[c.at(ijk[3 * q], ijk[3 * q + 1], ijk[3 * q + 2])] |= GFS_REMOVE_FLAG;
}

// ---- driver ------------------------------------------------------------------

namespace {
int scan_into(Ctx *ctx, Sim *s, uint32_t *in, uint32_t *out, long long n, uint32_t *total) {
    // exclusive scan of n flags (the entry n is the total)
    cudaStream_t st = ctx->stream;
    if (s->src_tmp.ensure(scan_temp_elems(n + 1) * sizeof(uint32_t))) return GFS_ERR_NOMEM;
    GFS_CUDA_CHECK(cudaMemsetAsync(in + n, 0, sizeof(uint32_t), st));
    int rc = exclusive_scan_u32(ctx, in, out, n + 1, s->src_tmp.as<uint32_t>(), st);
    if (rc) return rc;
    GFS_CUDA_CHECK(cudaMemcpyAsync(total, out + n, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    GFS_CUDA_CHECK(cudaStreamSynchronize(st));
    return GFS_OK;
}

// New particles take ids after every id given so far; after caller-chosen ids
// that is the largest id + 1, found on the device once.
int ensure_next_id(Sim *s, long long n) {
    if (s->next_id_valid) return GFS_OK;
    Ctx *ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    const int T = 256;
    if (s->src_a.ensure(sizeof(uint32_t))) return GFS_ERR_NOMEM;
    GFS_CUDA_CHECK(cudaMemsetAsync(s->src_a.p, 0, sizeof(uint32_t), st));
    if (n > 0) {
        k_src_max_id<<<grid_blocks(n, T), T, 0, st>>>(s->pos.as<float4>(), n, s->src_a.as<uint32_t>());
        ctx->launches++;
        GFS_LAUNCH_CHECK();
    }
    uint32_t mx = 0;
    GFS_CUDA_CHECK(cudaMemcpyAsync(&mx, s->src_a.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    GFS_CUDA_CHECK(cudaStreamSynchronize(st));
    s->next_id = mx > s->next_id ? mx : s->next_id;
    s->next_id_valid = true;
    return GFS_OK;
}

int capacity_check(Sim *s, long long n, long long add, const char *what = "fluid sources") {
    if (n + add > s->capacity) {
        set_error(GFS_ERR_INVALID, "%s: %lld particles exceed the simulation's capacity %lld", what,
                  n + add, (long long)s->capacity);
        return GFS_ERR_INVALID;
    }
    return GFS_OK;
}
}  // namespace

// _updateFluidSources on the device state (particles sorted, those in solid
// cells removed).  Leaves the particles unsorted (need_sort) when any were added.
int update_fluid_sources(Sim *s, int64_t *added, int64_t *removed) {
    Ctx *ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    const Grids &g = s->g;
    const double dx = g.dx;
    const int T = 256;
    if (added) *added = 0;
    if (removed) *removed = 0;
    if (s->sources.empty()) return GFS_OK;
    int rc = GFS_OK;
    if (s->need_sort && (rc = sort_particles(s, true))) return rc;
    uint32_t hn = 0;
    GFS_CUDA_CHECK(cudaMemcpyAsync(&hn, s->num.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    GFS_CUDA_CHECK(cudaStreamSynchronize(st));
    long long n = hn, n0 = hn;
    if ((rc = ensure_next_id(s, n))) return rc;
    const double jit = 0.25 * s->jitter_factor * dx;
    uint8_t *mat = s->mat.as<uint8_t>();
    bool any_outflow = false;
    for (const gfs_fluid_source &src : s->sources) {
        if (!src.active) continue;
        if (src.outflow) {
            any_outflow = true;
            continue;
        }
        SrcGeom G = source_geometry(src, dx, g.ni, g.nj, g.nk);
        long long n1 = (long long)G.n1[0] * G.n1[1] * G.n1[2];
        long long ns = 8LL * G.nf[0] * G.nf[1] * G.nf[2];
        if (s->src_mark.ensure((size_t)(n1 > 0 ? n1 : 1)) ||
            s->src_a.ensure((size_t)(std::max(n1, ns) + 1) * sizeof(uint32_t)) ||
            s->src_b.ensure((size_t)(std::max(n1, ns) + 1) * sizeof(uint32_t)))
            return GFS_ERR_NOMEM;
        uint8_t *mark = s->src_mark.as<uint8_t>();
        uint32_t *a = s->src_a.as<uint32_t>(), *b = s->src_b.as<uint32_t>();
        // 1. air cells: 8 particles each
        if (n1 > 0) {
            k_src_cells<<<grid_blocks(n1, T), T, 0, st>>>(G, g.c, dx, mat, mark, a, n1);
            ctx->launches++;
            GFS_LAUNCH_CHECK();
            uint32_t nair = 0;
            if ((rc = scan_into(ctx, s, a, b, n1, &nair))) return rc;
            if ((rc = capacity_check(s, n, 8LL * nair))) return rc;
            k_src_fill_cells<<<grid_blocks(n1, T), T, 0, st>>>(G, g.c, dx, mat, mark, b, n1, s->pos.as<float4>(),
                                                               s->vel.as<float4>(), n, s->next_id,
                                                               s->jitter_seed, jit);
            ctx->launches++;
            GFS_LAUNCH_CHECK();
            n += 8LL * nair;
            s->next_id += 8u * nair;
        }
        // 2. empty sub-cells of the overlapping fluid-or-air cells: one particle each
        if (ns > 0 && n1 > 0) {
            k_src_subgrid<<<grid_blocks(ns, T), T, 0, st>>>(G, mark, a, ns);
            ctx->launches++;
            GFS_LAUNCH_CHECK();
            if (n > 0) {
                k_src_occupy<<<grid_blocks(n, T), T, 0, st>>>(G, dx, s->pos.as<float4>(), n, a);
                ctx->launches++;
                GFS_LAUNCH_CHECK();
            }
            uint32_t nnew = 0;
            if ((rc = scan_into(ctx, s, a, b, ns, &nnew))) return rc;
            if ((rc = capacity_check(s, n, nnew))) return rc;
            k_src_new_particles<<<grid_blocks(ns, T), T, 0, st>>>(G, g.c, dx, mat, a, b, ns, s->pos.as<float4>(),
                                                                  s->vel.as<float4>(), n, s->next_id,
                                                                  s->jitter_seed, jit);
            ctx->launches++;
            GFS_LAUNCH_CHECK();
            n += nnew;
            s->next_id += nnew;
        }
    }
    if (n != n0) {
        uint32_t hn2 = (uint32_t)n;
        GFS_CUDA_CHECK(cudaMemcpyAsync(s->num.p, &hn2, sizeof(uint32_t), cudaMemcpyHostToDevice, st));
        s->n_bound = n;
        s->need_sort = true;
    }
    if (added) *added = n - n0;
    if (any_outflow) {
        // the outflow sources' fluid cells (after the inflows) lose their particles at a sort
        for (const gfs_fluid_source &src : s->sources) {
            if (!src.active || !src.outflow) continue;
            SrcGeom G = source_geometry(src, dx, g.ni, g.nj, g.nk);
            long long n1 = (long long)G.n1[0] * G.n1[1] * G.n1[2];
            if (n1 <= 0) continue;
            k_src_outflow<<<grid_blocks(n1, T), T, 0, st>>>(G, g.c, dx, mat, n1);
            ctx->launches++;
            GFS_LAUNCH_CHECK();
        }
        if ((rc = sort_particles(s, true))) return rc;
        k_src_clear_flags<<<grid_blocks(g.c.size, T), T, 0, st>>>(mat, g.c.size);
        ctx->launches++;
        GFS_LAUNCH_CHECK();
        if (removed) *removed = n - s->n_bound;
    }
    return GFS_OK;
}

// The fluid-cell queues on the device state, as _updateFluidCells applies them
// before the sources (fluidsimulation.cpp:1990-1993): every queued added cell
// that is still air gets 8 particles with its group's velocity and becomes
// fluid, groups and cells in the order they were queued (a cell queued twice
// is fluid the second time); then the particles in the queued removed cells,
// new ones included, are removed (the material is left as it is).  On an
// error nothing is added and the queues are kept.
int update_fluid_cell_queues(Sim *s, int64_t *added, int64_t *removed) {
    Ctx *ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    const Grids &g = s->g;
    const int T = 256;
    if (added) *added = 0;
    if (removed) *removed = 0;
    if (s->added_cells.empty() && s->removed_cells.empty()) return GFS_OK;
    int rc = GFS_OK;
    uint32_t hn = 0;
    GFS_CUDA_CHECK(cudaMemcpyAsync(&hn, s->num.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    GFS_CUDA_CHECK(cudaStreamSynchronize(st));
    long long n = hn, n0 = hn;
    uint8_t *mat = s->mat.as<uint8_t>();
    if (!s->added_cells.empty()) {
        std::vector<CellEntry> ent;
        std::unordered_set<long long> seen;
        for (const Sim::CellGroup &grp : s->added_cells)
            for (size_t q = 0; q + 2 < grp.ijk.size(); q += 3) {
                CellEntry e{grp.ijk[q], grp.ijk[q + 1], grp.ijk[q + 2], {grp.vel[0], grp.vel[1], grp.vel[2]}};
                if (seen.insert(g.c.at(e.i, e.j, e.k)).second) ent.push_back(e);
            }
        long long m = (long long)ent.size();
        if ((rc = ensure_next_id(s, n))) return rc;
        if (s->src_mark.ensure((size_t)m * sizeof(CellEntry)) || s->src_a.ensure((size_t)(m + 1) * sizeof(uint32_t)) ||
            s->src_b.ensure((size_t)(m + 1) * sizeof(uint32_t)))
            return GFS_ERR_NOMEM;
        const CellEntry *E = s->src_mark.as<CellEntry>();
        uint32_t *a = s->src_a.as<uint32_t>(), *b = s->src_b.as<uint32_t>();
        GFS_CUDA_CHECK(cudaMemcpyAsync(s->src_mark.p, ent.data(), (size_t)m * sizeof(CellEntry),
                                       cudaMemcpyHostToDevice, st));
        k_cells_air<<<grid_blocks(m, T), T, 0, st>>>(g.c, mat, E, m, a);
        ctx->launches++;
        GFS_LAUNCH_CHECK();
        uint32_t nair = 0;
        if ((rc = scan_into(ctx, s, a, b, m, &nair))) return rc;
        if ((rc = capacity_check(s, n, 8LL * nair, "added fluid cells"))) return rc;
        if (nair > 0) {
            k_cells_fill<<<grid_blocks(m, T), T, 0, st>>>(g.c, g.dx, mat, E, a, b, m, s->pos.as<float4>(),
                                                          s->vel.as<float4>(), n, s->next_id, s->jitter_seed,
                                                          0.25 * s->jitter_factor * g.dx);
            ctx->launches++;
            GFS_LAUNCH_CHECK();
            n += 8LL * nair;
            s->next_id += 8u * nair;
            uint32_t hn2 = (uint32_t)n;
            GFS_CUDA_CHECK(cudaMemcpyAsync(s->num.p, &hn2, sizeof(uint32_t), cudaMemcpyHostToDevice, st));
            GFS_CUDA_CHECK(cudaStreamSynchronize(st));
            s->n_bound = n;
            s->need_sort = true;
        }
        s->added_cells.clear();
        s->added_cells.shrink_to_fit();
    }
    if (added) *added = n - n0;
    if (!s->removed_cells.empty()) {
        long long m = (long long)s->removed_cells.size() / 3;
        if (s->src_mark.ensure((size_t)m * 3 * sizeof(int32_t))) return GFS_ERR_NOMEM;
        GFS_CUDA_CHECK(cudaMemcpyAsync(s->src_mark.p, s->removed_cells.data(), (size_t)m * 3 * sizeof(int32_t),
                                       cudaMemcpyHostToDevice, st));
        k_cells_mark_removal<<<grid_blocks(m, T), T, 0, st>>>(g.c, mat, s->src_mark.as<int32_t>(), m);
        ctx->launches++;
        GFS_LAUNCH_CHECK();
        if ((rc = sort_particles(s, true))) return rc;
        k_src_clear_flags<<<grid_blocks(g.c.size, T), T, 0, st>>>(mat, g.c.size);
        ctx->launches++;
        GFS_LAUNCH_CHECK();
        GFS_CUDA_CHECK(cudaStreamSynchronize(st));
        if (removed) *removed = n - s->n_bound;
        s->removed_cells.clear();
        s->removed_cells.shrink_to_fit();
    }
    return GFS_OK;
}

}  // namespace gfs

using namespace gfs;

extern "C" {

int gfs_sim_set_fluid_sources(gfs_sim *sim, const gfs_fluid_source *sources, int n) {
    if (!sim || n < 0 || (n > 0 && !sources)) {
        set_error(GFS_ERR_INVALID, "gfs_sim_set_fluid_sources: invalid arguments");
        return GFS_ERR_INVALID;
    }
    for (int q = 0; q < n; q++) {
        const gfs_fluid_source &src = sources[q];
        bool ok = src.shape == GFS_SOURCE_SPHERE || src.shape == GFS_SOURCE_CUBOID;
        for (int a = 0; a < 3; a++) ok = ok && std::isfinite(src.position[a]) && std::isfinite(src.velocity[a]);
        if (src.shape == GFS_SOURCE_SPHERE) ok = ok && std::isfinite(src.radius);
        else
            for (int a = 0; a < 3; a++) ok = ok && std::isfinite(src.size[a]) && src.size[a] >= 0.0;
        if (!ok) {
            set_error(GFS_ERR_INVALID, "gfs_sim_set_fluid_sources: source %d has an unknown shape or non-finite "
                      "geometry", q);
            return GFS_ERR_INVALID;
        }
    }
    sim->s.sources.assign(sources, sources + n);
    return GFS_OK;
}

int gfs_sim_set_marker_particle_jitter(gfs_sim *sim, double factor, uint64_t seed) {
    if (!sim || !(factor >= 0.0 && factor <= 1.0)) {
        set_error(GFS_ERR_INVALID, "gfs_sim_set_marker_particle_jitter: factor must be in [0, 1]");
        return GFS_ERR_INVALID;
    }
    sim->s.jitter_factor = factor;
    sim->s.jitter_seed = seed;
    return GFS_OK;
}

int gfs_sim_update_fluid_sources(gfs_sim *sim, int64_t *num_added, int64_t *num_removed) {
    if (!sim) {
        set_error(GFS_ERR_INVALID, "sim must not be NULL");
        return GFS_ERR_INVALID;
    }
    Sim *s = &sim->s;
    int64_t qa = 0, qr = 0, sa = 0, sr = 0;
    int rc = GFS_OK;
    if (s->need_sort && (rc = sort_particles(s, true))) return rc;
    if ((rc = update_fluid_cell_queues(s, &qa, &qr))) return rc;
    if ((rc = update_fluid_sources(s, &sa, &sr))) return rc;
    if (num_added) *num_added = qa + sa;
    if (num_removed) *num_removed = qr + sr;
    if (s->need_sort) return sort_particles(s, true);
    return GFS_OK;
}

namespace {
int check_cells(const char *fn, const gfs_sim *sim, const int32_t *ijk, int n) {
    if (!sim || n < 0 || (n > 0 && !ijk)) {
        set_error(GFS_ERR_INVALID, "%s: invalid arguments", fn);
        return GFS_ERR_INVALID;
    }
    const Grids &g = sim->s.g;
    for (int q = 0; q < n; q++) {
        // FluidSimulation::addFluidCells / removeFluidCells throw std::out_of_range
        if (!g.c.in(ijk[3 * q], ijk[3 * q + 1], ijk[3 * q + 2])) {
            set_error(GFS_ERR_INVALID, "%s: fluid cell index out of range (i: %d j: %d k: %d)", fn, ijk[3 * q],
                      ijk[3 * q + 1], ijk[3 * q + 2]);
            return GFS_ERR_INVALID;
        }
    }
    return GFS_OK;
}
}  // namespace

int gfs_sim_add_fluid_cells(gfs_sim *sim, const int32_t *ijk, int n, const float *velocity) {
    int rc = check_cells("gfs_sim_add_fluid_cells", sim, ijk, n);
    if (rc || n == 0) return rc;
    Sim *s = &sim->s;
    Ctx *ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    const int T = 256;
    // the cells that are air now (fluidsimulation.cpp:900-902)
    if (s->src_a.ensure((size_t)n * 3 * sizeof(int32_t)) || s->src_b.ensure((size_t)n)) return GFS_ERR_NOMEM;
    GFS_CUDA_CHECK(cudaMemcpyAsync(s->src_a.p, ijk, (size_t)n * 3 * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    k_cells_material<<<grid_blocks(n, T), T, 0, st>>>(s->g.c, s->mat.as<uint8_t>(), s->src_a.as<int32_t>(), n,
                                                      s->src_b.as<uint8_t>());
    ctx->launches++;
    GFS_LAUNCH_CHECK();
    std::vector<uint8_t> m((size_t)n);
    GFS_CUDA_CHECK(cudaMemcpyAsync(m.data(), s->src_b.p, (size_t)n, cudaMemcpyDeviceToHost, st));
    GFS_CUDA_CHECK(cudaStreamSynchronize(st));
    Sim::CellGroup grp;
    for (int a = 0; a < 3; a++) grp.vel[a] = velocity ? velocity[a] : 0.0f;
    for (int q = 0; q < n; q++)
        if (m[q] == GFS_AIR) grp.ijk.insert(grp.ijk.end(), ijk + 3 * q, ijk + 3 * q + 3);
    if (!grp.ijk.empty()) s->added_cells.push_back(std::move(grp));
    return GFS_OK;
}

int gfs_sim_remove_fluid_cells(gfs_sim *sim, const int32_t *ijk, int n) {
    int rc = check_cells("gfs_sim_remove_fluid_cells", sim, ijk, n);
    if (rc || n == 0) return rc;
    sim->s.removed_cells.insert(sim->s.removed_cells.end(), ijk, ijk + 3 * (size_t)n);
    return GFS_OK;
}

}  // extern "C"
