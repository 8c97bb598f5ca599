/* gfs_fluidsimulation_c.h -- GridFluidSim3D's FluidSimulation C exports for the
 * per-substep core, over libgfs's device-resident simulation (gfs_sim_*).
 *
 * Same names, argument lists and error convention as the reference's
 * c_bindings/fluidsimulation_c.cpp, so a caller of those exports (pyfluid's
 * ctypes layer, pyfluid/fluidsimulation.py and pyfluid/pybindings.py) reaches
 * the CUDA core without change for the calls below:
 *   - every export takes `int *err` last and sets it to 1 (success) or 0
 *     (failure); CBindings_get_error_message() then holds the message
 *     (c_bindings/cbindings.cpp:11-13, 77-79);
 *   - the structs have the reference's layouts (c_bindings/vector3_c.h:4-8,
 *     aabb_c.h:6-11, gridindex_c.h:4-8, markerparticle_c.h:6-9).
 *
 * FluidSimulation_update(obj, dt) runs one substep of the core (gfs_sim_step:
 * classification, velocity splat, fill, extrapolation, body force, MICCG(0)
 * pressure, PIC/FLIP and RK4 advection with collisions, per-cell cap) with the
 * particles resident on the device.  Meshing, diffuse particles and CFL-driven
 * substepping are not part of this core; the exports for them are not provided.
 * Marker particles come back in the device's (cell, id) order.
 */
#ifndef GFS_FLUIDSIMULATION_C_H
#define GFS_FLUIDSIMULATION_C_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct Vector3_t {
    float x;
    float y;
    float z;
} Vector3_t;

typedef struct AABB_t {
    Vector3_t position;
    float width;
    float height;
    float depth;
} AABB_t;

typedef struct GridIndex_t {
    int i;
    int j;
    int k;
} GridIndex_t;

typedef struct MarkerParticle_t {
    Vector3_t position;
    Vector3_t velocity;
} MarkerParticle_t;

typedef struct FluidSimulation FluidSimulation;

/* fluidsimulation_c.cpp:16-42: an empty simulation (no grid: only destroy and
   the dimension queries succeed) and one of isize x jsize x ksize cells of width
   dx on the current CUDA device (GFS_DEVICE, default 0, as the drop-in classes). */
FluidSimulation *FluidSimulation_new_from_empty(int *err);
FluidSimulation *FluidSimulation_new_from_dimensions(int isize, int jsize, int ksize, double dx, int *err);
void FluidSimulation_destroy(FluidSimulation *obj);                       /* :59-61 */
/* :63-71: the solid border and the fluid seeded from the implicit points and
   cuboids added so far (gfs_sim_initialize); a second call does nothing. */
void FluidSimulation_initialize(FluidSimulation *obj, int *err);
int FluidSimulation_is_initialized(FluidSimulation *obj, int *err);
/* :73-77: one substep of length dt (the simulation must be initialized). */
void FluidSimulation_update(FluidSimulation *obj, double dt, int *err);
int FluidSimulation_get_current_frame(FluidSimulation *obj, int *err);    /* :90-94 */
double FluidSimulation_get_cell_size(FluidSimulation *obj, int *err);     /* :103-107 */
void FluidSimulation_get_grid_dimensions(FluidSimulation *obj, int *i, int *j, int *k, int *err);  /* :109-114 */
int FluidSimulation_get_grid_width(FluidSimulation *obj, int *err);       /* :116-120 */
int FluidSimulation_get_grid_height(FluidSimulation *obj, int *err);      /* :122-126 */
int FluidSimulation_get_grid_depth(FluidSimulation *obj, int *err);       /* :128-132 */
void FluidSimulation_get_simulation_dimensions(FluidSimulation *obj, double *width, double *height, double *depth,
                                               int *err);                  /* :134-140 */
double FluidSimulation_get_simulation_width(FluidSimulation *obj, int *err);   /* :142-147 */
double FluidSimulation_get_simulation_height(FluidSimulation *obj, int *err);  /* :149-154 */
double FluidSimulation_get_simulation_depth(FluidSimulation *obj, int *err);   /* :156-161 */
double FluidSimulation_get_density(FluidSimulation *obj, int *err);       /* :163-167 */
void FluidSimulation_set_density(FluidSimulation *obj, double density, int *err);  /* :169-175 */
/* :638-679: the constant body force is the sum of the forces added (none at
   creation, as in the reference). */
void FluidSimulation_add_body_force(FluidSimulation *obj, double fx, double fy, double fz, int *err);
Vector3_t FluidSimulation_get_constant_body_force(FluidSimulation *obj, int *err);
void FluidSimulation_reset_body_force(FluidSimulation *obj, int *err);
/* :680-700: scene set-up for initialize (fluidsimulation.cpp:703-765). */
void FluidSimulation_add_implicit_fluid_point(FluidSimulation *obj, double x, double y, double z, double r, int *err);
void FluidSimulation_add_fluid_cuboid(FluidSimulation *obj, AABB_t cbbox, int *err);
/* :732-770: cells become solid / solid cells become air (gfs_sim_add_solid_cells). */
void FluidSimulation_add_solid_cells(FluidSimulation *obj, GridIndex_t *cells, int n, int *err);
void FluidSimulation_remove_solid_cells(FluidSimulation *obj, GridIndex_t *cells, int n, int *err);
/* :829-878: particles [startidx, endidx) of the current set. */
int FluidSimulation_get_num_marker_particles(FluidSimulation *obj, int *err);
void FluidSimulation_get_marker_particles(FluidSimulation *obj, int startidx, int endidx, MarkerParticle_t *out,
                                          int *err);
void FluidSimulation_get_marker_particle_positions(FluidSimulation *obj, int startidx, int endidx, Vector3_t *out,
                                                   int *err);
void FluidSimulation_get_marker_particle_velocities(FluidSimulation *obj, int startidx, int endidx, Vector3_t *out,
                                                    int *err);
/* c_bindings/cbindings.cpp:77-79: the message of the last failed export. */
char *CBindings_get_error_message(void);

#ifdef __cplusplus
}
#endif

#endif
