// fluidsim_c.cu -- the reference's FluidSimulation C exports (c_bindings/
// fluidsimulation_c.cpp) for the per-substep core, over the device-resident
// simulation of capi.cu.  A FluidSimulation here is a gfs_sim on the process's
// shared context plus what FluidSimulation keeps on the host until initialize():
// the implicit fluid points and fluid cuboids (fluidsimulation.h:1112-1113), the
// frame counter and the sum of the constant body forces.  Every export reports
// through `int *err` (1 success, 0 failure) and CBindings_get_error_message(),
// the reference's convention (c_bindings/cbindings.cpp:11-13, 77-79).
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "gfs.h"
#include "gfs_fluidsimulation_c.h"

struct FluidSimulation {
    gfs_sim *sim = nullptr;
    int isize = 0, jsize = 0, ksize = 0;
    double dx = 0.0;
    bool initialized = false;
    int frame = 0;
    std::vector<double> points;    // x y z r
    std::vector<double> cuboids;   // x y z width height depth
    float force[3] = {0.f, 0.f, 0.f};
};

namespace {

thread_local char g_cb_err[4096] = "";

void cb_fail(int *err, const char *msg) {
    snprintf(g_cb_err, sizeof(g_cb_err), "%s", msg);
    if (err) *err = 0;
}

// a failed library call: its message becomes the binding's
bool cb_check(int rc, int *err) {
    if (rc == GFS_OK) return true;
    cb_fail(err, gfs_last_error());
    return false;
}

bool cb_ok(int *err) {
    if (err) *err = 1;
    return true;
}

// one context per process, on GFS_DEVICE (default 0), as the drop-in classes use
gfs_ctx *shared_ctx() {
    static std::mutex mu;
    static gfs_ctx *ctx = nullptr;
    static bool tried = false;
    std::lock_guard<std::mutex> lock(mu);
    if (!tried) {
        tried = true;
        const char *dev = std::getenv("GFS_DEVICE");
        if (gfs_ctx_create(dev ? std::atoi(dev) : 0, &ctx) != GFS_OK) ctx = nullptr;
    }
    return ctx;
}

bool with_grid(FluidSimulation *obj, int *err) {
    if (!obj) {
        cb_fail(err, "FluidSimulation is NULL");
        return false;
    }
    if (!obj->sim) {
        cb_fail(err, "FluidSimulation has no grid (created empty)");
        return false;
    }
    return true;
}

int push_force(FluidSimulation *obj) {
    gfs_sim_params p;
    int rc = gfs_sim_get_params(obj->sim, &p);
    if (rc) return rc;
    for (int d = 0; d < 3; d++) p.gravity[d] = obj->force[d];
    return gfs_sim_set_params(obj->sim, &p);
}

// particles [start, end) as xyz triples of positions and velocities
bool particle_range(FluidSimulation *obj, int start, int end, std::vector<float> &pos, std::vector<float> &vel,
                    int *err) {
    int64_t n = 0;
    if (!cb_check(gfs_sim_num_particles(obj->sim, &n), err)) return false;
    if (start < 0 || end < start || end > n) {
        cb_fail(err, "marker particle range out of bounds");
        return false;
    }
    pos.resize((size_t)std::max<int64_t>(n, 1) * 3);
    vel.resize((size_t)std::max<int64_t>(n, 1) * 3);
    int64_t got = n;
    return cb_check(gfs_sim_get_particles(obj->sim, pos.data(), vel.data(), nullptr, &got), err);
}

}  // namespace

extern "C" {

FluidSimulation *FluidSimulation_new_from_empty(int *err) {
    cb_ok(err);
    return new FluidSimulation();
}

FluidSimulation *FluidSimulation_new_from_dimensions(int isize, int jsize, int ksize, double dx, int *err) {
    if (isize <= 0 || jsize <= 0 || ksize <= 0 || !(dx > 0.0)) {
        cb_fail(err, "grid dimensions and cell size must be positive");
        return nullptr;
    }
    gfs_ctx *ctx = shared_ctx();
    if (!ctx) {
        cb_fail(err, "no CUDA device could be initialised");
        return nullptr;
    }
    FluidSimulation *obj = new FluidSimulation();
    obj->isize = isize;
    obj->jsize = jsize;
    obj->ksize = ksize;
    obj->dx = dx;
    // capacity: 8 particles per cell, the most initialize() seeds
    const int64_t cap = (int64_t)8 * isize * jsize * ksize;
    if (!cb_check(gfs_sim_create(ctx, isize, jsize, ksize, dx, cap, &obj->sim), err) ||
        !cb_check(push_force(obj), err)) {   // no body force until one is added
        if (obj->sim) gfs_sim_destroy(obj->sim);
        delete obj;
        return nullptr;
    }
    cb_ok(err);
    return obj;
}

void FluidSimulation_destroy(FluidSimulation *obj) {
    if (!obj) return;
    if (obj->sim) gfs_sim_destroy(obj->sim);
    delete obj;
}

void FluidSimulation_initialize(FluidSimulation *obj, int *err) {
    if (!with_grid(obj, err)) return;
    if (obj->initialized) {
        cb_ok(err);
        return;
    }
    int64_t n = 0;
    if (!cb_check(gfs_sim_initialize(obj->sim, obj->points.data(), (int)(obj->points.size() / 4),
                                     obj->cuboids.data(), (int)(obj->cuboids.size() / 6), &n),
                  err))
        return;
    obj->initialized = true;
    cb_ok(err);
}

int FluidSimulation_is_initialized(FluidSimulation *obj, int *err) {
    if (!obj) {
        cb_fail(err, "FluidSimulation is NULL");
        return 0;
    }
    cb_ok(err);
    return obj->initialized ? 1 : 0;
}

void FluidSimulation_update(FluidSimulation *obj, double dt, int *err) {
    if (!with_grid(obj, err)) return;
    if (!obj->initialized) {
        cb_fail(err, "FluidSimulation must be initialized before update");
        return;
    }
    if (!(dt >= 0.0)) {
        cb_fail(err, "delta time must be >= 0");
        return;
    }
    gfs_step_stats st;
    if (!cb_check(gfs_sim_step(obj->sim, dt, &st), err)) return;
    obj->frame++;
    cb_ok(err);
}

int FluidSimulation_get_current_frame(FluidSimulation *obj, int *err) {
    if (!obj) {
        cb_fail(err, "FluidSimulation is NULL");
        return 0;
    }
    cb_ok(err);
    return obj->frame;
}

double FluidSimulation_get_cell_size(FluidSimulation *obj, int *err) {
    if (!obj) {
        cb_fail(err, "FluidSimulation is NULL");
        return 0.0;
    }
    cb_ok(err);
    return obj->dx;
}

void FluidSimulation_get_grid_dimensions(FluidSimulation *obj, int *i, int *j, int *k, int *err) {
    if (!obj || !i || !j || !k) {
        cb_fail(err, "NULL argument");
        return;
    }
    *i = obj->isize;
    *j = obj->jsize;
    *k = obj->ksize;
    cb_ok(err);
}

int FluidSimulation_get_grid_width(FluidSimulation *obj, int *err) {
    int i = 0, j = 0, k = 0;
    FluidSimulation_get_grid_dimensions(obj, &i, &j, &k, err);
    return i;
}

int FluidSimulation_get_grid_height(FluidSimulation *obj, int *err) {
    int i = 0, j = 0, k = 0;
    FluidSimulation_get_grid_dimensions(obj, &i, &j, &k, err);
    return j;
}

int FluidSimulation_get_grid_depth(FluidSimulation *obj, int *err) {
    int i = 0, j = 0, k = 0;
    FluidSimulation_get_grid_dimensions(obj, &i, &j, &k, err);
    return k;
}

// FluidSimulation::getSimulationDimensions: cells x cell width (fluidsimulation.cpp:95-111)
void FluidSimulation_get_simulation_dimensions(FluidSimulation *obj, double *width, double *height, double *depth,
                                               int *err) {
    if (!obj || !width || !height || !depth) {
        cb_fail(err, "NULL argument");
        return;
    }
    *width = (double)obj->isize * obj->dx;
    *height = (double)obj->jsize * obj->dx;
    *depth = (double)obj->ksize * obj->dx;
    cb_ok(err);
}

double FluidSimulation_get_simulation_width(FluidSimulation *obj, int *err) {
    double w = 0, h = 0, d = 0;
    FluidSimulation_get_simulation_dimensions(obj, &w, &h, &d, err);
    return w;
}

double FluidSimulation_get_simulation_height(FluidSimulation *obj, int *err) {
    double w = 0, h = 0, d = 0;
    FluidSimulation_get_simulation_dimensions(obj, &w, &h, &d, err);
    return h;
}

double FluidSimulation_get_simulation_depth(FluidSimulation *obj, int *err) {
    double w = 0, h = 0, d = 0;
    FluidSimulation_get_simulation_dimensions(obj, &w, &h, &d, err);
    return d;
}

double FluidSimulation_get_density(FluidSimulation *obj, int *err) {
    if (!with_grid(obj, err)) return 0.0;
    gfs_sim_params p;
    if (!cb_check(gfs_sim_get_params(obj->sim, &p), err)) return 0.0;
    cb_ok(err);
    return p.density;
}

void FluidSimulation_set_density(FluidSimulation *obj, double density, int *err) {
    if (!with_grid(obj, err)) return;
    if (!(density > 0.0)) {   // FluidSimulation::setDensity requires a positive density
        cb_fail(err, "density must be greater than 0");
        return;
    }
    gfs_sim_params p;
    if (!cb_check(gfs_sim_get_params(obj->sim, &p), err)) return;
    p.density = density;
    if (cb_check(gfs_sim_set_params(obj->sim, &p), err)) cb_ok(err);
}

void FluidSimulation_add_body_force(FluidSimulation *obj, double fx, double fy, double fz, int *err) {
    if (!with_grid(obj, err)) return;
    obj->force[0] += (float)fx;   // vec3 sums in float (fluidsimulation.cpp:2758)
    obj->force[1] += (float)fy;
    obj->force[2] += (float)fz;
    if (cb_check(push_force(obj), err)) cb_ok(err);
}

Vector3_t FluidSimulation_get_constant_body_force(FluidSimulation *obj, int *err) {
    Vector3_t f = {0.f, 0.f, 0.f};
    if (!obj) {
        cb_fail(err, "FluidSimulation is NULL");
        return f;
    }
    f.x = obj->force[0];
    f.y = obj->force[1];
    f.z = obj->force[2];
    cb_ok(err);
    return f;
}

void FluidSimulation_reset_body_force(FluidSimulation *obj, int *err) {
    if (!with_grid(obj, err)) return;
    obj->force[0] = obj->force[1] = obj->force[2] = 0.f;
    if (cb_check(push_force(obj), err)) cb_ok(err);
}

void FluidSimulation_add_implicit_fluid_point(FluidSimulation *obj, double x, double y, double z, double r, int *err) {
    if (!with_grid(obj, err)) return;
    // FluidSimulation::addImplicitFluidPoint (fluidsimulation.cpp:707-724)
    if (r < 0.0) {
        cb_fail(err, "implicit fluid point radius must be greater than or equal to 0");
        return;
    }
    if (obj->initialized) {
        cb_fail(err, "implicit fluid point must be added before the simulation is initialized");
        return;
    }
    obj->points.insert(obj->points.end(), {x, y, z, r});
    cb_ok(err);
}

void FluidSimulation_add_fluid_cuboid(FluidSimulation *obj, AABB_t b, int *err) {
    if (!with_grid(obj, err)) return;
    if (obj->initialized) {   // FluidSimulation::addFluidCuboid (fluidsimulation.cpp:726-765)
        cb_fail(err, "fluid cuboid must be added before the simulation is initialized");
        return;
    }
    obj->cuboids.insert(obj->cuboids.end(), {(double)b.position.x, (double)b.position.y, (double)b.position.z,
                                             (double)b.width, (double)b.height, (double)b.depth});
    cb_ok(err);
}

static void solid_cells(FluidSimulation *obj, GridIndex_t *cells, int n, bool add, int *err) {
    if (!with_grid(obj, err)) return;
    if (n < 0 || (n > 0 && !cells)) {
        cb_fail(err, "invalid cell list");
        return;
    }
    std::vector<int32_t> ijk((size_t)3 * std::max(n, 1));
    for (int q = 0; q < n; q++) {
        ijk[3 * q] = cells[q].i;
        ijk[3 * q + 1] = cells[q].j;
        ijk[3 * q + 2] = cells[q].k;
    }
    const int rc = add ? gfs_sim_add_solid_cells(obj->sim, ijk.data(), n)
                       : gfs_sim_remove_solid_cells(obj->sim, ijk.data(), n);
    if (cb_check(rc, err)) cb_ok(err);
}

void FluidSimulation_add_solid_cells(FluidSimulation *obj, GridIndex_t *cells, int n, int *err) {
    solid_cells(obj, cells, n, true, err);
}

void FluidSimulation_remove_solid_cells(FluidSimulation *obj, GridIndex_t *cells, int n, int *err) {
    solid_cells(obj, cells, n, false, err);
}

int FluidSimulation_get_num_marker_particles(FluidSimulation *obj, int *err) {
    if (!with_grid(obj, err)) return 0;
    int64_t n = 0;
    if (!cb_check(gfs_sim_num_particles(obj->sim, &n), err)) return 0;
    cb_ok(err);
    return (int)n;
}

void FluidSimulation_get_marker_particles(FluidSimulation *obj, int startidx, int endidx, MarkerParticle_t *out,
                                          int *err) {
    if (!with_grid(obj, err)) return;
    std::vector<float> pos, vel;
    if (!particle_range(obj, startidx, endidx, pos, vel, err)) return;
    if (endidx > startidx && !out) {
        cb_fail(err, "output pointer is NULL");
        return;
    }
    for (int q = startidx; q < endidx; q++) {
        MarkerParticle_t &m = out[q - startidx];
        m.position = {pos[3 * (size_t)q], pos[3 * (size_t)q + 1], pos[3 * (size_t)q + 2]};
        m.velocity = {vel[3 * (size_t)q], vel[3 * (size_t)q + 1], vel[3 * (size_t)q + 2]};
    }
    cb_ok(err);
}

static void particle_vectors(FluidSimulation *obj, int startidx, int endidx, Vector3_t *out, bool velocities,
                             int *err) {
    if (!with_grid(obj, err)) return;
    std::vector<float> pos, vel;
    if (!particle_range(obj, startidx, endidx, pos, vel, err)) return;
    if (endidx > startidx && !out) {
        cb_fail(err, "output pointer is NULL");
        return;
    }
    const std::vector<float> &src = velocities ? vel : pos;
    for (int q = startidx; q < endidx; q++)
        out[q - startidx] = {src[3 * (size_t)q], src[3 * (size_t)q + 1], src[3 * (size_t)q + 2]};
    cb_ok(err);
}

void FluidSimulation_get_marker_particle_positions(FluidSimulation *obj, int startidx, int endidx, Vector3_t *out,
                                                   int *err) {
    particle_vectors(obj, startidx, endidx, out, false, err);
}

void FluidSimulation_get_marker_particle_velocities(FluidSimulation *obj, int startidx, int endidx, Vector3_t *out,
                                                    int *err) {
    particle_vectors(obj, startidx, endidx, out, true, err);
}

char *CBindings_get_error_message(void) { return g_cb_err; }

}  // extern "C"
