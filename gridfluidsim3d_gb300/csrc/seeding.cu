// seeding.cu -- FluidSimulation::initialize's fluid seeding, on the host.
//
// FluidSimulation::_initializeFluidMaterial (fluidsimulation.cpp:1383-1399) turns
// the implicit fluid points (addImplicitFluidPoint, :703-724) and fluid cuboids
// (addFluidCuboid, :726-765) into marker particles:
//   1. a scalar field on the (ni+1) x (nj+1) x (nk+1) cell corners: every point
//      adds the splat kernel 1 - 4/9 s^3 + 17/9 s^2 - 22/9 s (s = d^2 / r^2, within
//      r; ScalarField::addPoint, scalarfield.cpp:121-166), every cuboid adds
//      threshold + 1e-5 on the corners inside it (ScalarField::addCuboid, :203-230);
//      corners of solid cells are clamped to the threshold 0.5 when read
//      (setMaterialGrid / getScalarFieldValue, :337-408);
//   2. fluid cells: non-solid cells whose corner average exceeds 0.5
//      (_getInitialFluidCellsFromScalarField, :1265-1281);
//   3. fluid cells without an air cell among their 26 neighbours are full and get
//      8 particles on the 2 x 2 x 2 sub-lattice, centre +-dx/4
//      (_addMarkerParticlesToCell, :1223-1246); the other fluid cells and the air
//      cells next to fluid are partial: each of their 8 half-size sub-cells whose
//      centre lies inside the field (tricubic sample > 0.5, ScalarField::
//      isPointInside / tricubicInterpolation, :497-550) gets one particle
//      (_getFullAndPartiallyFullFluidCells / _getPartiallyFullFluidCellParticles,
//      :1283-1352), kept when its cell is in range and not solid (_addMarkerParticle).
// The float / double steps of the reference are kept operation by operation: the
// particle positions are the reference's exactly when the jitter factor is 0.
//
// Deviation: the reference jitters each particle by _randomDouble(-j, j) per axis
// (rand(), j = 0.25 * jitter factor * dx); here the jitter is the counter-based
// hash the fluid sources use (splitmix64 of seed, particle number and axis), so a
// seeding is reproducible.  The reference's sample points of the field are
// indexed [i][j][k] where its interpolant expects [k][j][i]
// (Interpolation::tricubicInterpolate, interpolation.cpp:26-33): the cubic over
// the innermost (k) index takes the x weight and the outermost (i) the z
// weight.  That is kept, since it decides which sub-cells receive particles.
#include <cmath>
#include <cstring>
#include <vector>

#include "gfs_internal.h"

namespace gfs {

namespace {

constexpr double kThreshold = 0.5;   // ScalarField::_surfaceThreshold (scalarfield.h:114)

struct V3 {
    float x, y, z;
};

inline V3 v3(double x, double y, double z) { return V3{(float)x, (float)y, (float)z}; }

// Grid3d::GridIndexToPosition as a vec3 (grid3d.h:79-81): (float)i * dx, stored as float
inline V3 corner(int i, int j, int k, double dx) {
    return v3((double)(float)i * dx, (double)(float)j * dx, (double)(float)k * dx);
}

inline double seed_jitter(unsigned long long seed, unsigned long long counter, int axis, double j) {
    unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (counter * 3ull + (unsigned long long)axis + 1ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    double u = (double)(z >> 11) * (1.0 / 9007199254740992.0);
    return -j + 2.0 * j * u;
}

// Interpolation::cubicInterpolate (interpolation.cpp:44-46), Catmull-Rom
inline double cubic(const double p[4], double x) {
    return p[1] + 0.5 * x * (p[2] - p[0] + x * (2.0 * p[0] - 5.0 * p[1] + 4.0 * p[2] - p[3] +
                                               x * (3.0 * (p[1] - p[2]) + p[3] - p[0])));
}

struct Field {
    int W, H, D;
    double dx;
    std::vector<float> v;
    std::vector<uint8_t> solid_vertex;
    long long at(int i, int j, int k) const { return (long long)i + (long long)W * (j + (long long)H * k); }
    bool in(int i, int j, int k) const { return i >= 0 && j >= 0 && k >= 0 && i < W && j < H && k < D; }

    // ScalarField::addPoint(p, r) (scalarfield.cpp:121-166), bounds of
    // Grid3d::getGridIndexBounds(p, r, dx, ...) (grid3d.h:350-371)
    void add_point(V3 p, double r) {
        const double c1 = (4.0 / 9.0) * (1.0 / (r * r * r * r * r * r));
        const double c2 = (17.0 / 9.0) * (1.0 / (r * r * r * r));
        const double c3 = (22.0 / 9.0) * (1.0 / (r * r));
        const double invdx = 1.0 / dx;
        const int ci = (int)floor(p.x * invdx), cj = (int)floor(p.y * invdx), ck = (int)floor(p.z * invdx);
        const V3 cp = corner(ci, cj, ck, dx);
        const V3 tr{p.x - cp.x, p.y - cp.y, p.z - cp.z};
        const double inv = 1.0 / dx;
        int i0 = ci - (int)fmax(0, ceil((r - tr.x) * inv)), j0 = cj - (int)fmax(0, ceil((r - tr.y) * inv)),
            k0 = ck - (int)fmax(0, ceil((r - tr.z) * inv));
        int i1 = ci + (int)fmax(0, ceil((r - dx + tr.x) * inv)), j1 = cj + (int)fmax(0, ceil((r - dx + tr.y) * inv)),
            k1 = ck + (int)fmax(0, ceil((r - dx + tr.z) * inv));
        i0 = (int)fmax(i0, 0); j0 = (int)fmax(j0, 0); k0 = (int)fmax(k0, 0);
        i1 = (int)fmin(i1, W - 1); j1 = (int)fmin(j1, H - 1); k1 = (int)fmin(k1, D - 1);
        const double rsq = r * r;
        for (int k = k0; k <= k1; k++)
            for (int j = j0; j <= j1; j++)
                for (int i = i0; i <= i1; i++) {
                    const V3 g = corner(i, j, k, dx);
                    const V3 d{g.x - p.x, g.y - p.y, g.z - p.z};
                    const double s = (double)(d.x * d.x + d.y * d.y + d.z * d.z);   // vmath::dot, in float
                    if (s < rsq) {
                        const double w = 1.0 - c1 * s * s * s + c2 * s * s - c3 * s;
                        v[at(i, j, k)] += (float)w;
                    }
                }
    }

    // ScalarField::addCuboid(pos, w, h, d) (scalarfield.cpp:203-230), bounds of
    // Grid3d::getGridIndexBounds(AABB, ...) (grid3d.h:426-439), AABB::isPointInside
    // (aabb.cpp:123-126)
    void add_cuboid(V3 p, double w, double h, double d) {
        const double invdx = 1.0 / dx;
        const V3 q{p.x + (float)w, p.y + (float)h, p.z + (float)d};
        int i0 = (int)floor(p.x * invdx), j0 = (int)floor(p.y * invdx), k0 = (int)floor(p.z * invdx);
        int i1 = (int)floor(q.x * invdx), j1 = (int)floor(q.y * invdx), k1 = (int)floor(q.z * invdx);
        i0 = (int)fmax(i0, 0); j0 = (int)fmax(j0, 0); k0 = (int)fmax(k0, 0);
        i1 = (int)fmin(i1, W - 1); j1 = (int)fmin(j1, H - 1); k1 = (int)fmin(k1, D - 1);
        const double add = kThreshold + 10e-6;
        for (int k = k0; k <= k1; k++)
            for (int j = j0; j <= j1; j++)
                for (int i = i0; i <= i1; i++) {
                    const V3 g = corner(i, j, k, dx);
                    if (g.x >= p.x && g.y >= p.y && g.z >= p.z && g.x < p.x + w && g.y < p.y + h && g.z < p.z + d)
                        v[at(i, j, k)] += (float)add;
                }
    }

    // ScalarField::getScalarFieldValue: corners of solid cells read at most the threshold
    double value(int i, int j, int k) const {
        double x = v[at(i, j, k)];
        if (solid_vertex[at(i, j, k)] && x > kThreshold) x = kThreshold;
        return x;
    }

    // ScalarField::getScalarFieldValueAtCellCenter (scalarfield.cpp:414-428)
    double cell_center_value(int i, int j, int k) const {
        double s = 0.0;
        s += value(i, j, k);
        s += value(i + 1, j, k);
        s += value(i, j + 1, k);
        s += value(i + 1, j + 1, k);
        s += value(i, j, k + 1);
        s += value(i + 1, j, k + 1);
        s += value(i, j + 1, k + 1);
        s += value(i + 1, j + 1, k + 1);
        return 0.125 * s;
    }

    // ScalarField::tricubicInterpolation (scalarfield.cpp:497-545) on the raw values
    double sample(V3 p) const {
        if (!(p.x >= 0 && p.y >= 0 && p.z >= 0 && p.x < dx * W && p.y < dx * H && p.z < dx * D)) return 0.0;
        const double invdx = 1.0 / dx;
        const int i = (int)floor(p.x * invdx), j = (int)floor(p.y * invdx), k = (int)floor(p.z * invdx);
        const double gx = (double)i * dx, gy = (double)j * dx, gz = (double)k * dx;
        const double inv = 1 / dx;
        const double ix = (p.x - gx) * inv, iy = (p.y - gy) * inv, iz = (p.z - gz) * inv;
        double lo = INFINITY, hi = -INFINITY;
        double pts[4][4][4];
        // pts[a][b][c]: a the i offset, b the j offset, c the k offset, visited k-outer
        // like the reference, whose running min / max depends on the visiting order
        for (int c = 0; c < 4; c++)
            for (int b = 0; b < 4; b++)
                for (int a = 0; a < 4; a++) {
                    const int ii = i - 1 + a, jj = j - 1 + b, kk = k - 1 + c;
                    double x = in(ii, jj, kk) ? (double)v[at(ii, jj, kk)] : 0.0;
                    if (in(ii, jj, kk)) {
                        if (x < lo) lo = x;
                        else if (x > hi) hi = x;
                    }
                    pts[a][b][c] = x;
                }
        double outer[4];
        for (int a = 0; a < 4; a++) {
            double mid[4];
            for (int b = 0; b < 4; b++) mid[b] = cubic(pts[a][b], ix);
            outer[a] = cubic(mid, iy);
        }
        double val = cubic(outer, iz);
        if (val < lo) val = lo;
        else if (val > hi) val = hi;
        return val;
    }
};

}  // namespace

int seed_fluid_particles(int ni, int nj, int nk, double dx, const uint8_t *mat_in, const double *points,
                         int npoints, const double *cuboids, int ncuboids, double jitter_factor,
                         unsigned long long seed, std::vector<float> &out, std::vector<uint8_t> *mat_out) {
    const long long nc = (long long)ni * nj * nk;
    std::vector<uint8_t> mat(mat_in, mat_in + nc);
    auto cell = [&](int i, int j, int k) -> long long { return (long long)i + (long long)ni * (j + (long long)nj * k); };
    auto in_grid = [&](int i, int j, int k) { return i >= 0 && j >= 0 && k >= 0 && i < ni && j < nj && k < nk; };
    // _initializeSolidCells (fluidsimulation.cpp:1191-1213): the border is solid
    for (int k = 0; k < nk; k++)
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++)
                if (i == 0 || j == 0 || k == 0 || i == ni - 1 || j == nj - 1 || k == nk - 1) mat[cell(i, j, k)] = GFS_SOLID;
    Field F;
    F.W = ni + 1; F.H = nj + 1; F.D = nk + 1; F.dx = dx;
    F.v.assign((size_t)F.W * F.H * F.D, 0.0f);
    F.solid_vertex.assign(F.v.size(), 0);
    for (int q = 0; q < npoints; q++) {
        const double *pt = points + 4 * q;
        if (!(pt[3] >= 0.0)) {
            set_error(GFS_ERR_INVALID, "implicit fluid point %d: radius must be >= 0 (got %g)", q, pt[3]);
            return GFS_ERR_INVALID;
        }
        F.add_point(v3(pt[0], pt[1], pt[2]), pt[3]);
    }
    for (int q = 0; q < ncuboids; q++) {
        const double *c = cuboids + 6 * q;
        if (!(c[3] >= 0.0 && c[4] >= 0.0 && c[5] >= 0.0)) {
            set_error(GFS_ERR_INVALID, "fluid cuboid %d: dimensions must be >= 0", q);
            return GFS_ERR_INVALID;
        }
        F.add_cuboid(v3(c[0], c[1], c[2]), c[3], c[4], c[5]);
    }
    for (int k = 0; k < nk; k++)
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++)
                if (mat[cell(i, j, k)] == GFS_SOLID)
                    for (int c = 0; c < 8; c++) F.solid_vertex[F.at(i + (c & 1), j + ((c >> 1) & 1), k + (c >> 2))] = 1;
    // fluid cells, in k -> j -> i order
    std::vector<long long> fluid;
    for (int k = 0; k < nk; k++)
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++)
                if (mat[cell(i, j, k)] != GFS_SOLID && F.cell_center_value(i, j, k) > kThreshold) fluid.push_back(cell(i, j, k));
    std::vector<uint8_t> m2 = mat;
    for (long long c : fluid) m2[c] = GFS_FLUID;
    // out-of-range cells read as solid (fluidmaterialgrid.cpp:28)
    auto neighbours = [&](int i, int j, int k, uint8_t what) {
        for (int c = k - 1; c <= k + 1; c++)
            for (int b = j - 1; b <= j + 1; b++)
                for (int a = i - 1; a <= i + 1; a++) {
                    if (a == i && b == j && c == k) continue;
                    const uint8_t m = in_grid(a, b, c) ? m2[cell(a, b, c)] : (uint8_t)GFS_SOLID;
                    if (m == what) return true;
                }
        return false;
    };
    std::vector<long long> full;
    std::vector<uint8_t> partial((size_t)nc, 0);
    for (long long c : fluid) {
        const int i = (int)(c % ni), j = (int)((c / ni) % nj), k = (int)(c / ((long long)ni * nj));
        if (neighbours(i, j, k, GFS_AIR)) partial[c] = 1;
        else full.push_back(c);
    }
    for (int k = 0; k < nk; k++)
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++)
                if (m2[cell(i, j, k)] == GFS_AIR && neighbours(i, j, k, GFS_FLUID)) partial[cell(i, j, k)] = 1;
    const double jit = 0.25 * jitter_factor * dx;   // _getMarkerParticleJitter (fluidsimulation.cpp:1219-1221)
    unsigned long long counter = 0;
    auto jitter3 = [&](float &x, float &y, float &z) {
        const unsigned long long c = counter++;
        x = x + (float)seed_jitter(seed, c, 0, jit);
        y = y + (float)seed_jitter(seed, c, 1, jit);
        z = z + (float)seed_jitter(seed, c, 2, jit);
    };
    // partial cells' sub-cell particles (_getPartiallyFullFluidCellParticles): sub-cells
    // of half size in k -> j -> i order over the doubled grid
    std::vector<float> part;
    const double sdx = 0.5 * dx, hs = 0.5 * sdx;
    for (int k = 0; k < 2 * nk; k++)
        for (int j = 0; j < 2 * nj; j++)
            for (int i = 0; i < 2 * ni; i++) {
                if (!partial[cell(i / 2, j / 2, k / 2)]) continue;
                V3 c = v3((double)(float)i * sdx + hs, (double)(float)j * sdx + hs, (double)(float)k * sdx + hs);
                if (F.sample(c) > kThreshold) {
                    jitter3(c.x, c.y, c.z);
                    part.push_back(c.x);
                    part.push_back(c.y);
                    part.push_back(c.z);
                }
            }
    // full cells: 8 particles each (_addMarkerParticlesToCell), then the partial ones
    // that land in a non-solid cell of the grid (_addMarkerParticle)
    out.clear();
    out.reserve(full.size() * 24 + part.size());
    const double qd = 0.25 * dx;
    static const int corner_sign[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, -1, 1}, {-1, -1, 1},
                                          {-1, 1, -1}, {1, 1, -1}, {1, 1, 1}, {-1, 1, 1}};
    for (long long c : full) {
        const int i = (int)(c % ni), j = (int)((c / ni) % nj), k = (int)(c / ((long long)ni * nj));
        const double h = 0.5 * dx;
        const V3 ctr = v3((double)(float)i * dx + h, (double)(float)j * dx + h, (double)(float)k * dx + h);
        for (int q = 0; q < 8; q++) {
            V3 p = v3(ctr.x + corner_sign[q][0] * qd, ctr.y + corner_sign[q][1] * qd, ctr.z + corner_sign[q][2] * qd);
            jitter3(p.x, p.y, p.z);
            out.push_back(p.x);
            out.push_back(p.y);
            out.push_back(p.z);
        }
    }
    const double invdx = 1.0 / dx;
    for (size_t q = 0; q < part.size(); q += 3) {
        const int i = (int)floor(part[q] * invdx), j = (int)floor(part[q + 1] * invdx), k = (int)floor(part[q + 2] * invdx);
        if (in_grid(i, j, k) && mat[cell(i, j, k)] != GFS_SOLID) {
            out.push_back(part[q]);
            out.push_back(part[q + 1]);
            out.push_back(part[q + 2]);
        }
    }
    if (mat_out) *mat_out = mat;
    return GFS_OK;
}

}  // namespace gfs

using namespace gfs;

extern "C" int gfs_seed_fluid_particles(int ni, int nj, int nk, double dx, const uint8_t *h_material,
                                        const double *points, int npoints, const double *cuboids, int ncuboids,
                                        double jitter_factor, uint64_t seed, float *h_positions, int64_t capacity,
                                        int64_t *n) {
    if (!h_material || !n || ni < 3 || nj < 3 || nk < 3 || (long long)ni * nj * nk >= (1LL << 31) || !(dx > 0) ||
        npoints < 0 || ncuboids < 0 || (npoints > 0 && !points) || (ncuboids > 0 && !cuboids) ||
        !(jitter_factor >= 0.0 && jitter_factor <= 1.0)) {
        set_error(GFS_ERR_INVALID, "gfs_seed_fluid_particles: invalid arguments");
        return GFS_ERR_INVALID;
    }
    std::vector<float> out;
    int rc = seed_fluid_particles(ni, nj, nk, dx, h_material, points, npoints, cuboids, ncuboids, jitter_factor,
                                  (unsigned long long)seed, out, nullptr);
    if (rc) return rc;
    const int64_t count = (int64_t)(out.size() / 3);
    *n = count;
    if (!h_positions) return GFS_OK;
    if (capacity < count) {
        set_error(GFS_ERR_INVALID, "gfs_seed_fluid_particles: %lld particles, room for %lld", (long long)count,
                  (long long)capacity);
        return GFS_ERR_INVALID;
    }
    if (count) memcpy(h_positions, out.data(), out.size() * sizeof(float));
    return GFS_OK;
}
