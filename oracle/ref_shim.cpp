// ref_shim.cpp -- extern "C" entry points into the reference's own CPU classes.
//
// TEST INFRASTRUCTURE ONLY.  Compiled (by oracle/Makefile, target `ref`) together
// with the reference's unmodified CL-free sources, where they lie, into
// oracle/_ref/libgfsref.so.  It is used to pin the C restatement in
// gfs_oracle.c against the reference itself and to generate the golden
// fixtures under tests/golden/.  Nothing in the product path links it.
//
// Each function builds the reference's own data structures from flat arrays
// (Array3d index i + W*(j + H*k)), calls one reference routine, and copies the
// result out:
//   gfsref_velocity_scalar_field -> ScalarField::addPointValue + applyWeightField
//                                   (scalarfield.cpp:90-106,167-201), configured
//                                   like FluidSimulation::_computeVelocityScalarField
//                                   (fluidsimulation.cpp:2526-2595)
//   gfsref_add_point_values      -> ScalarField::addPoint / addPointValue
//                                   (scalarfield.cpp:126-201) onto a field that
//                                   starts from the caller's values, optional
//                                   weight field and max threshold
//   gfsref_pressure_solve        -> PressureSolver::solve (pressuresolver.cpp:116)
//   gfsref_evaluate_velocity     -> MACVelocityField::evaluateVelocityAtPosition
//                                   (macvelocityfield.cpp:549)
//   gfsref_extrapolate           -> MACVelocityField::extrapolateVelocityField
//                                   (macvelocityfield.cpp:786)
//   gfsref_segment_voxel / gfsref_ray_aabb -> Collision (collision.cpp:303,404)
#include <cstdint>
#include <cstring>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "aabb.h"
#include "array3d.h"
#include "collision.h"
#include "fluidmaterialgrid.h"
#include "gridindexvector.h"
#include "logfile.h"
#include "macvelocityfield.h"
#include "pressuresolver.h"
#include "scalarfield.h"
#include "vmath.h"

namespace {

void fill_material(FluidMaterialGrid &g, const uint8_t *mat, int ni, int nj, int nk) {
    for (int k = 0; k < nk; k++)
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++) {
                uint8_t m = mat[i + ni * (j + nj * k)];
                if (m == 1) g.setFluid(i, j, k);
                else if (m == 2) g.setSolid(i, j, k);
                else g.setAir(i, j, k);
            }
}

void fill_array(Array3d<float> &a, const float *src) {
    for (int k = 0; k < a.depth; k++)
        for (int j = 0; j < a.height; j++)
            for (int i = 0; i < a.width; i++)
                a.set(i, j, k, src[i + a.width * (j + a.height * k)]);
}

void read_array(Array3d<float> &a, float *dst) {
    for (int k = 0; k < a.depth; k++)
        for (int j = 0; j < a.height; j++)
            for (int i = 0; i < a.width; i++)
                dst[i + a.width * (j + a.height * k)] = a(i, j, k);
}

void fill_mac(MACVelocityField &m, int ni, int nj, int nk, const float *u, const float *v,
              const float *w) {
    Array3d<float> au(ni + 1, nj, nk, 0.0f), av(ni, nj + 1, nk, 0.0f), aw(ni, nj, nk + 1, 0.0f);
    fill_array(au, u);
    fill_array(av, v);
    fill_array(aw, w);
    m.setU(au);
    m.setV(av);
    m.setW(aw);
}

}  // namespace

extern "C" {

void gfsref_add_point_values(const float *pos, const float *val, int64_t n, double r, const float *offset,
                             double dx, int W, int H, int D, float *field, float *weight, int thr_set,
                             double thr) {
    ScalarField sf(W, H, D, dx);
    if (weight) sf.enableWeightField();
    sf.setPointRadius(r);
    sf.setOffset(vmath::vec3(offset[0], offset[1], offset[2]));
    if (thr_set) sf.setMaxScalarFieldThreshold(thr);
    Array3d<float> *fp = sf.getPointerToScalarField();
    Array3d<float> *wp = weight ? sf.getPointerToWeightField() : nullptr;
    for (int k = 0; k < D; k++)
        for (int j = 0; j < H; j++)
            for (int i = 0; i < W; i++) {
                fp->set(i, j, k, field[i + W * (j + H * k)]);
                if (wp) wp->set(i, j, k, weight[i + W * (j + H * k)]);
            }
    for (int64_t q = 0; q < n; q++) {
        vmath::vec3 p(pos[3 * q], pos[3 * q + 1], pos[3 * q + 2]);
        if (val) sf.addPointValue(p, (double)val[q]);
        else sf.addPoint(p);
    }
    for (int k = 0; k < D; k++)
        for (int j = 0; j < H; j++)
            for (int i = 0; i < W; i++) {
                field[i + W * (j + H * k)] = fp->get(i, j, k);
                if (wp) weight[i + W * (j + H * k)] = wp->get(i, j, k);
            }
}

void gfsref_velocity_scalar_field(int dir, int ni, int nj, int nk, double dx, const float *pos,
                                  const float *vel, int64_t n, float *field, float *weight) {
    int W = ni + (dir == 0), H = nj + (dir == 1), D = nk + (dir == 2);
    ScalarField grid(W, H, D, dx);
    grid.enableWeightField();
    grid.setPointRadius(dx);
    vmath::vec3 offset;
    if (dir == 0) offset = vmath::vec3(0.0, 0.5 * dx, 0.5 * dx);
    else if (dir == 1) offset = vmath::vec3(0.5 * dx, 0.0, 0.5 * dx);
    else offset = vmath::vec3(0.5 * dx, 0.5 * dx, 0.0);
    grid.setOffset(offset);
    for (int64_t p = 0; p < n; p++) {
        vmath::vec3 pp(pos[3 * p], pos[3 * p + 1], pos[3 * p + 2]);
        grid.addPointValue(pp, vel[3 * p + dir]);
    }
    grid.applyWeightField();
    read_array(*grid.getPointerToScalarField(), field);
    read_array(*grid.getPointerToWeightField(), weight);
}

// Returns the CG iteration number the reference logs ("CG Iterations: N"),
// 200 when it logs "Iterations limit reached", -1 when CG never ran.
int gfsref_pressure_solve(int ni, int nj, int nk, double dx, double density, double dt,
                          const uint8_t *mat, const float *u, const float *v, const float *w,
                          double *pressure_out) {
    FluidMaterialGrid mgrid(ni, nj, nk);
    fill_material(mgrid, mat, ni, nj, nk);
    GridIndexVector cells(ni, nj, nk);
    for (int k = 0; k < nk; k++)
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++)
                if (mgrid.isCellFluid(i, j, k)) cells.push_back(i, j, k);
    MACVelocityField mac(ni, nj, nk, dx);
    fill_mac(mac, ni, nj, nk, u, v, w);
    LogFile log;
    log.setPath("/nonexistent-gfsref-log-dir");

    PressureSolverParameters params;
    params.cellwidth = dx;
    params.density = density;
    params.deltaTime = dt;
    params.fluidCells = &cells;
    params.materialGrid = &mgrid;
    params.velocityField = &mac;
    params.logfile = &log;

    VectorXd pressure((int)cells.size());
    std::ostringstream captured;
    std::streambuf *old = std::cout.rdbuf(captured.rdbuf());
    PressureSolver solver;
    solver.solve(params, pressure);
    std::cout.rdbuf(old);

    for (size_t i = 0; i < cells.size(); i++) pressure_out[i] = pressure[(int)i];
    std::string s = captured.str();
    size_t at = s.find("CG Iterations: ");
    if (at != std::string::npos) return std::stoi(s.substr(at + 15));
    if (s.find("Iterations limit reached") != std::string::npos) return 200;
    return -1;
}

void gfsref_evaluate_velocity(int ni, int nj, int nk, double dx, const float *u, const float *v,
                              const float *w, const float *pos, int64_t n, float *out) {
    MACVelocityField mac(ni, nj, nk, dx);
    fill_mac(mac, ni, nj, nk, u, v, w);
    for (int64_t p = 0; p < n; p++) {
        vmath::vec3 r = mac.evaluateVelocityAtPosition(
            vmath::vec3(pos[3 * p], pos[3 * p + 1], pos[3 * p + 2]));
        out[3 * p] = r.x;
        out[3 * p + 1] = r.y;
        out[3 * p + 2] = r.z;
    }
}

void gfsref_extrapolate(int ni, int nj, int nk, double dx, const uint8_t *mat, int layers,
                        float *u, float *v, float *w) {
    FluidMaterialGrid mgrid(ni, nj, nk);
    fill_material(mgrid, mat, ni, nj, nk);
    MACVelocityField mac(ni, nj, nk, dx);
    fill_mac(mac, ni, nj, nk, u, v, w);
    mac.extrapolateVelocityField(mgrid, layers);
    read_array(*mac.getArray3dU(), u);
    read_array(*mac.getArray3dV(), v);
    read_array(*mac.getArray3dW(), w);
}

int gfsref_segment_voxel(const float *p0, const float *p1, double dx, int ni, int nj, int nk,
                         const uint8_t *mat, int *voxel) {
    FluidMaterialGrid mgrid(ni, nj, nk);
    fill_material(mgrid, mat, ni, nj, nk);
    GridIndex g;
    bool ok = Collision::getLineSegmentVoxelIntersection(vmath::vec3(p0[0], p0[1], p0[2]),
                                                         vmath::vec3(p1[0], p1[1], p1[2]), dx,
                                                         mgrid, &g);
    voxel[0] = g.i;
    voxel[1] = g.j;
    voxel[2] = g.k;
    return ok ? 1 : 0;
}

int gfsref_ray_aabb(const float *p0, const float *dir, const float *bpos, double w, double h,
                    double d, float *out) {
    AABB box(vmath::vec3(bpos[0], bpos[1], bpos[2]), w, h, d);
    vmath::vec3 c;
    bool ok = Collision::rayIntersectsAABB(vmath::vec3(p0[0], p0[1], p0[2]),
                                           vmath::vec3(dir[0], dir[1], dir[2]), box, &c);
    out[0] = c.x;
    out[1] = c.y;
    out[2] = c.z;
    return ok ? 1 : 0;
}

}  // extern "C"
