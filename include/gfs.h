/*
 * gfs.h -- C ABI of libgfs, the GB300 (sm_103a) per-substep FLIP core of
 * GridFluidSim3D: marker-particle -> MAC-grid velocity splat, MICCG(0)
 * pressure projection, PIC/FLIP grid -> particle update with RK4 advection.
 *
 * Conventions (all entry points):
 *   - every call returns int status: GFS_OK (0) or a GFS_ERR_* code; the message
 *     of the last failure on the calling thread is gfs_last_error().  This is
 *     the reference's c_bindings convention (cbindings.h:20-135: a status plus a
 *     global error string) without exceptions crossing the ABI;
 *   - grids are flat float/uint8 arrays in the reference's Array3d order,
 *     index i + W*(j + H*k) (array3d.h:394-402); U is (ni+1) x nj x nk,
 *     V is ni x (nj+1) x nk, W is ni x nj x (nk+1); material is uint8,
 *     0 air, 1 fluid, 2 solid (fluidmaterialgrid.h:29-33);
 *   - particle positions / velocities are float xyz triples (vmath::vec3,
 *     vmath.h:33-56); ids are uint32 and travel with their particle;
 *   - pointers named h_* are host memory, borrowed for the duration of the call
 *     (pinned memory makes the copies asynchronous-capable and faster);
 *   - a gfs_ctx owns one CUDA stream and its device buffers; calls on one
 *     context must come from one thread at a time (the reference is
 *     single-threaded).
 */
#ifndef GFS_H
#define GFS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GFS_OK 0
#define GFS_ERR_INVALID 1   /* bad argument (sizes, null pointers, dt < 0 ...) */
#define GFS_ERR_CUDA 2      /* CUDA runtime error (message names the call)     */
#define GFS_ERR_NOMEM 3     /* device allocation failed                        */
#define GFS_ERR_TIMEOUT 4   /* a wavefront wait hit its bound (device status)  */
#define GFS_ERR_STATE 5     /* call out of order (e.g. step before particles)  */

/* Pressure-solve precision. PLAIN: FP64 vectors, stencil, preconditioner and
   dots, the reference's arithmetic (pressuresolver.cpp).  MIXED: FP32 vectors,
   stencil and MIC(0) apply, FP64 dots/norms and an FP64 iterative-refinement
   residual r = b - A p; the stopping rule (max|r| < tol, evaluated in FP64) is
   the reference's. */
#define GFS_PRECISION_PLAIN 0
#define GFS_PRECISION_MIXED 1

typedef struct gfs_ctx gfs_ctx;
typedef struct gfs_sim gfs_sim;

/* ------------------------------------------------------------- library */

/* Message of the last failed call on this thread ("" if none). */
const char *gfs_last_error(void);
/* Library version string. */
const char *gfs_version(void);

/* ------------------------------------------------------------- context */

/* Create a context on CUDA device `device` (its own non-blocking stream).
   Replaces the OpenCL context set-up of CLScalarField::initialize
   (clscalarfield.cpp:33-66) and ParticleAdvector::initialize
   (particleadvector.cpp:33-63). */
int gfs_ctx_create(int device, gfs_ctx **out);
/* Closes the context.  Simulations created on it stay usable until they are
   destroyed; the last of them frees the context (so the two may be destroyed in
   either order, as a garbage collector may do). */
int gfs_ctx_destroy(gfs_ctx *ctx);
/* Wait for all work queued on the context's stream. */
int gfs_ctx_synchronize(gfs_ctx *ctx);
/* The context's cudaStream_t, for callers that time or order work on it. */
int gfs_ctx_stream(gfs_ctx *ctx, void **stream);
/* Device name (cf. getDeviceInfo, clscalarfield.h:112 / particleadvector.h:72). */
int gfs_ctx_device_name(gfs_ctx *ctx, char *buf, int buflen);

/* ------------------------------------------- splat (CLScalarField drop-in) */

/* Weighted point splat: for every point p with value v and every grid node x
   (node (i,j,k) sits at (i,j,k)*dx) inside the index bounds of p - offset
   (Grid3d::getGridIndexBounds, grid3d.h:350-371) and strictly within `radius`:
       field += w*v,  weight += w,   w = 1 - 4/9 s^3 + 17/9 s^2 - 22/9 s,
       s = |x - (p - offset)|^2 / radius^2
   (ScalarField::addPoint / addPointValue, scalarfield.cpp:121-201).
   Replaces CLScalarField::addPointValues(points, values, radius, offset, dx,
   scalarfield[, weightfield]) (clscalarfield.h:83-95, clscalarfield.cpp:144-267)
   and, with h_values = NULL (v = 1), CLScalarField::addPoints(points, radius,
   offset, dx, field) (clscalarfield.h:70-74, clscalarfield.cpp:68-122), and
   their kernels (kernels/scalarfield.cl:79-268).  Adds into the caller's
   arrays (the accelerated path's semantics, clscalarfield.cpp:1413,1448);
   h_weightfield may be NULL (no weight field).  Field dims W x H x D, x fastest.
   threshold_set != 0 applies CLScalarField::setMaxScalarFieldValueThreshold
   (clscalarfield.cpp:303-318) per node: a node whose incoming value exceeds
   `threshold` receives nothing.  Each node sums its contributions in a fixed
   order, so the result does not depend on scheduling. */
int gfs_scalar_field_add_point_values(gfs_ctx *ctx, const float *h_points, const float *h_values,
                                      int64_t n, double radius, const float offset[3], double dx,
                                      int W, int H, int D, float *h_scalarfield,
                                      float *h_weightfield, int threshold_set, double threshold);

/* Velocity splat of one MAC component: FluidSimulation::_computeVelocityScalarField
   (fluidsimulation.cpp:2526-2595): weighted splat of velocity[dir] with radius dx
   and the face offset of `dir`, then field /= weight where weight > 0
   (ScalarField::applyWeightField, scalarfield.cpp:90-106) and
   is_set = weight > 1e-9.  Outputs are the face grid of `dir` (fully written). */
int gfs_velocity_scalar_field(gfs_ctx *ctx, int dir, int ni, int nj, int nk, double dx,
                              const float *h_positions, const float *h_velocities, int64_t n,
                              float *h_field, uint8_t *h_is_set);

/* ------------------------------------- G2P / RK (ParticleAdvector drop-in) */

/* Catmull-Rom tricubic velocity at each point from a MAC field.
   Replaces ParticleAdvector::tricubicInterpolate(particles, vfield, output)
   (particleadvector.h:101-103, particleadvector.cpp:401-455) and its kernel
   tricubic_interpolate_kernel (kernels/tricubicinterpolate.cl:279-328);
   the arithmetic follows MACVelocityField::evaluateVelocityAtPosition
   (macvelocityfield.cpp:549-559).  Non-finite results become 0
   (ParticleAdvector::_validateOutput, particleadvector.cpp:1139-1149). */
int gfs_tricubic_interpolate(gfs_ctx *ctx, int ni, int nj, int nk, double dx, const float *h_u,
                             const float *h_v, const float *h_w, const float *h_points,
                             int64_t n, float *h_out);

/* Runge-Kutta advection of order 1..4 through a MAC field.
   Replaces ParticleAdvector::advectParticlesRK4/3/2/1
   (particleadvector.h:80-98, particleadvector.cpp:209-399; formulas of
   _RK4/_RK3/_RK2/_RK1 :1045-1078). */
int gfs_advect_particles(gfs_ctx *ctx, int order, int ni, int nj, int nk, double dx,
                         const float *h_u, const float *h_v, const float *h_w, double dt,
                         const float *h_points, int64_t n, float *h_out);

/* No counterpart in the reference: the tricubic sampler of gfs_tricubic_interpolate
   for callers that cannot allocate device memory -- hosts whose device memory all
   comes from their own allocator or arena, and real-time or callback code where
   cudaMalloc / cudaFree are not allowed.  It allocates nothing: d_u, d_v, d_w
   (face grids as in gfs_tricubic_interpolate), d_points (n xyz) and d_out (n xyz)
   are device-accessible memory the caller owns, and the kernels run on the
   caller's `stream` (a cudaStream_t; NULL = the legacy default stream).  The
   padded copies of U, V, W it needs live in a fixed 48 MiB scratch array that
   every GPU loading libgfs holds until the process exits; grids whose padded
   faces need more than 12,582,912 floats (about 150^3 cells) are rejected with
   GFS_ERR_INVALID.  The first call on a device (the current device) looks up the
   scratch's device address; make that first call before any stream capture.
   Every call checks the cached address with cudaPointerGetAttributes; after a
   cudaDeviceReset, which unloads the scratch, the first call looks it up again
   (make that call before any stream capture too).
   All calls share the scratch: calls that overlap on the GPU race on it.  The
   call is asynchronous; results are ready when `stream` has been synchronised. */
int gfs_tricubic_interpolate_noalloc(int ni, int nj, int nk, double dx, const float *d_u,
                                     const float *d_v, const float *d_w, const float *d_points,
                                     int64_t n, float *d_out, void *stream);

/* -------------------------------------- pressure (PressureSolver drop-in) */

/* MICCG(0) pressure solve.  Replaces PressureSolver::solve(params, pressure)
   (pressuresolver.h:117, pressuresolver.cpp:116-498).  Fluid cells are the
   material's fluid cells in lexicographic k->j->i order, the order
   FluidSimulation::_updateFluidCells builds (fluidsimulation.cpp:2031-2039);
   h_pressure receives one double per fluid cell in that order and must hold
   *num_fluid_cells entries (call with h_pressure = NULL to query the count).
   tol <= 0 / max_iters <= 0 select the reference's 1e-6 / 200
   (pressuresolver.h:159-160).  *iterations is the CG iteration number the
   reference logs (pressuresolver.cpp:477, 200 when the cap is hit, -1 when
   max|b| < tol); for MIXED it counts inner FP32 iterations. */
int gfs_pressure_solve(gfs_ctx *ctx, int ni, int nj, int nk, double dx, double density,
                       double dt, const uint8_t *h_material, const float *h_u,
                       const float *h_v, const float *h_w, int precision, double tol,
                       int max_iters, double *h_pressure, int64_t *num_fluid_cells,
                       int *iterations, double *max_residual);

/* ------------------------------ device-resident substep (FluidSimulation) */

typedef struct gfs_sim_params {
    double density;          /* _density = 20 (fluidsimulation.h:1154)                  */
    double ratio_pic;        /* _ratioPICFLIP = 0.05f (fluidsimulation.h:1161)          */
    double cfl;              /* _CFLConditionNumber = 5 -> ceil(cfl+2) extrapolation layers */
    float gravity[3];        /* sum of constant body forces (fluidsimulation.cpp:2758)  */
    int max_particles_per_cell; /* _maxMarkerParticlesPerCell = 100 (fluidsimulation.h:1167) */
    int precision;           /* GFS_PRECISION_PLAIN / GFS_PRECISION_MIXED               */
    double tol;              /* pressure tolerance, max|r| (pressuresolver.h:159)       */
    int max_cg_iterations;   /* 200 (pressuresolver.h:160)                              */
} gfs_sim_params;

typedef struct gfs_step_stats {
    int64_t num_particles;
    int64_t num_fluid_cells;
    int cg_iterations;       /* as gfs_pressure_solve                                   */
    int refinements;         /* MIXED: outer FP64 refinement steps                      */
    int sweeps;              /* forward (= backward) MIC(0) solves that did work        */
    double cg_max_residual;  /* FP64 max|b - A p| at exit                               */
    double pressure_ms;      /* device time of the pressure solve                       */
    double step_ms;          /* device time of the whole substep                        */
} gfs_step_stats;

/* Fill p with the reference's defaults. */
int gfs_sim_default_params(gfs_sim_params *p);

/* A simulation of ni x nj x nk cells of width dx holding up to max_particles
   particles on the device (the state FluidSimulation keeps in _markerParticles,
   _materialGrid and _MACVelocity, fluidsimulation.h:1047-1171). */
int gfs_sim_create(gfs_ctx *ctx, int ni, int nj, int nk, double dx, int64_t max_particles,
                   gfs_sim **out);
int gfs_sim_destroy(gfs_sim *sim);
int gfs_sim_set_params(gfs_sim *sim, const gfs_sim_params *p);
int gfs_sim_get_params(gfs_sim *sim, gfs_sim_params *p);
/* Material grid in (ni*nj*nk uint8).  Particles in solid cells are removed
   at the next step, as FluidSimulation::_removeMarkerParticlesInSolidCells does
   (fluidsimulation.cpp:1933-1958). */
int gfs_sim_set_material(gfs_sim *sim, const uint8_t *h_material);
int gfs_sim_get_material(gfs_sim *sim, uint8_t *h_material);
/* FluidSimulation::addSolidCells / removeSolidCells (fluidsimulation.cpp:845-885,
   c_bindings/fluidsimulation_c.cpp FluidSimulation_add_solid_cells /
   _remove_solid_cells): n cells (int32 triples i, j, k) become solid / a solid
   cell becomes air.  An index out of range fails with GFS_ERR_INVALID and changes
   nothing (the reference throws std::out_of_range).  Particles in new solid cells
   are removed at the next step. */
int gfs_sim_add_solid_cells(gfs_sim *sim, const int32_t *ijk, int n);
int gfs_sim_remove_solid_cells(gfs_sim *sim, const int32_t *ijk, int n);

/* FluidSimulation::initialize (fluidsimulation.cpp:48-55, 1407-1434) with the
   implicit fluid points (addImplicitFluidPoint, :703-724; `points` holds npoints
   rows x y z r) and fluid cuboids (addFluidCuboid, :726-765; `cuboids` holds
   ncuboids rows x y z width height depth): the domain border becomes solid
   (_initializeSolidCells) and the fluid is seeded from the scalar field of the
   points and cuboids (_initializeFluidMaterial, :1383-1399; see
   gfs_seed_fluid_particles): 8 particles on the 2x2x2 sub-lattice of every full
   fluid cell, sub-cell particles inside the surface for the cells at the surface.
   The particles replace the simulation's, at rest, ids 0..n-1; their jitter is
   gfs_sim_set_marker_particle_jitter's (factor 0.1 by default; 0 reproduces the
   reference's positions exactly).  *num_particles (may be NULL) receives the
   count; more than the simulation's capacity fails with GFS_ERR_INVALID. */
int gfs_sim_initialize(gfs_sim *sim, const double *points, int npoints, const double *cuboids, int ncuboids,
                       int64_t *num_particles);

/* The seeding of gfs_sim_initialize on the host alone (no device needed): the
   marker-particle positions (xyz triples, in the reference's creation order: the
   full cells' 8 particles cell by cell in k -> j -> i order, then the sub-cell
   particles) of ni x nj x nk cells of width dx whose material is h_material (its
   border is taken as solid).  h_positions = NULL queries the count into *n;
   otherwise it must hold `capacity` >= *n triples.  jitter_factor in [0, 1]:
   each component moves by a value in +-0.25 * jitter_factor * dx from a
   counter-based hash of `seed` (the reference draws it from rand()). */
int gfs_seed_fluid_particles(int ni, int nj, int nk, double dx, const uint8_t *h_material,
                             const double *points, int npoints, const double *cuboids, int ncuboids,
                             double jitter_factor, uint64_t seed, float *h_positions, int64_t capacity,
                             int64_t *n);

/* Replace the particle set (host -> device). ids may be NULL (0..n-1). */
int gfs_sim_set_particles(gfs_sim *sim, const float *h_positions, const float *h_velocities,
                          const uint32_t *h_ids, int64_t n);
/* Current particle count (may sync the stream). */
int gfs_sim_num_particles(gfs_sim *sim, int64_t *n);
/* Particles device -> host, in the device's (cell, id) order.  Arrays must hold
   gfs_sim_num_particles entries; any pointer may be NULL. */
int gfs_sim_get_particles(gfs_sim *sim, float *h_positions, float *h_velocities,
                          uint32_t *h_ids, int64_t *n);
/* The MAC velocity field after the last step (post-extrapolation). */
int gfs_sim_get_velocity_field(gfs_sim *sim, float *h_u, float *h_v, float *h_w);
/* The float pressure grid of the last step (0 outside fluid). */
int gfs_sim_get_pressure_grid(gfs_sim *sim, float *h_pressure);

/* One FLIP substep of length dt on the device-resident state: stages 1, 5-9,
   11, 12 of FluidSimulation::_stepFluid (fluidsimulation.cpp:3262-3390), i.e.
   _updateFluidCells, _advectVelocityField (+ saved field, extrapolation),
   _applyBodyForcesToVelocityField, _updatePressureGrid,
   _applyPressureToVelocityField, _extrapolateFluidVelocities,
   _updateMarkerParticleVelocities and _advanceMarkerParticles.  Meshing, level
   set, diffuse material and fluid sources are not part of it.  stats may be
   NULL; filling it synchronises the stream. */
int gfs_sim_step(gfs_sim *sim, double dt, gfs_step_stats *stats);

/* The same substep called the way the reference's host code would call it:
   particles arrive in host arrays, are copied to the device, stepped, and copied
   back (h_ids may be NULL).  On return *n holds the surviving count and the
   arrays hold the new state in (cell, id) order.  Arrays must have room for the
   input count. */
int gfs_sim_step_host(gfs_sim *sim, double dt, float *h_positions, float *h_velocities,
                      uint32_t *h_ids, int64_t *n, gfs_step_stats *stats);

/* The substep of gfs_sim_step run only up to the end of one of its stages,
   numbered as FluidSimulation::_stepFluid numbers them (fluidsimulation.cpp:
   3262-3390), so that each stage's grids can be read and compared with the
   reference's:
     GFS_STAGE_UPDATE_FLUID_CELLS (1)  _updateFluidCells
     GFS_STAGE_BODY_FORCES        (6)  + _advectVelocityField, the saved field
                                         and its extrapolation, body forces
                                         (the splat/fill and the body force are
                                         one kernel here, so 5 alone is not a stop)
     GFS_STAGE_PRESSURE           (7)  + _updatePressureGrid
     GFS_STAGE_APPLY_PRESSURE     (8)  + _applyPressureToVelocityField
     GFS_STAGE_EXTRAPOLATE        (9)  + _extrapolateFluidVelocities
     GFS_STAGE_ALL               (12)  the whole substep (= gfs_sim_step)
   Before GFS_STAGE_ALL the particles are not advanced: a later gfs_sim_step
   runs the whole substep from the same particles.  Other values fail with
   GFS_ERR_INVALID. */
#define GFS_STAGE_UPDATE_FLUID_CELLS 1
#define GFS_STAGE_BODY_FORCES 6
#define GFS_STAGE_PRESSURE 7
#define GFS_STAGE_APPLY_PRESSURE 8
#define GFS_STAGE_EXTRAPOLATE 9
#define GFS_STAGE_ALL 12
int gfs_sim_step_stages(gfs_sim *sim, double dt, int last_stage, gfs_step_stats *stats);
/* CLScalarField::addPoints (clscalarfield.cpp:68-122, kernels/scalarfield.cl:
   79-138) of the simulation's own marker particles, which never leave the
   device: every particle adds w(|x - (p - offset)|^2 / radius^2) to each node x
   of a W x H x D grid of spacing dx within `radius` (the splat of
   gfs_scalar_field_add_point_values with every value 1), into h_field (host,
   added to).  This is the scalar field IsotropicParticleMesher builds from the
   marker positions inside every substep (isotropicparticlemesher.cpp:309-390);
   the call replaces the host copy of 40M positions that the host-array entry
   point needs.  threshold_set / threshold: as gfs_scalar_field_add_point_values. */
int gfs_sim_add_marker_particle_points(gfs_sim *sim, double radius, const float offset[3], double dx, int W,
                                       int H, int D, float *h_field, int threshold_set, double threshold);

/* The saved field of the last (partial) step: the velocity field after
   _advectVelocityField, extrapolated (FluidSimulation::_savedVelocityField,
   fluidsimulation.cpp:3306-3307), which the PIC/FLIP update reads. */
int gfs_sim_get_saved_velocity_field(gfs_sim *sim, float *h_u, float *h_v, float *h_w);

/* Accuracy of the last step's pressure solve against FP64: the same system
   (matrix and right-hand side of that step, dt its step length) is solved again
   by FP64 MIC(0)-PCG to max|r| < rel_tol * max|b|; reports the FP64 residual
   max|b - A p| of the step's solution p and max|p - p_ref| / max|p_ref|.  The
   simulation's state is unchanged. */
int gfs_sim_pressure_check(gfs_sim *sim, double dt, double rel_tol, double *fp64_residual,
                           double *rel_error, int *ref_iterations);

/* ---------------------------------------------------------- fluid sources */

/* A fluid source (FluidSource, fluidsource.h; SphericalFluidSource(vec3 position,
   double radius), sphericalfluidsource.cpp:25-29; CuboidFluidSource(vec3 position,
   double width, height, depth), cuboidfluidsource.cpp:25-41) as
   FluidSimulation::addSphericalFluidSource / addCuboidFluidSource register it
   (fluidsimulation.cpp:767-795). */
#define GFS_SOURCE_SPHERE 0
#define GFS_SOURCE_CUBOID 1
typedef struct gfs_fluid_source {
    int shape;             /* GFS_SOURCE_SPHERE or GFS_SOURCE_CUBOID                  */
    int outflow;           /* 0: inflow (setAsInFlow, the default); 1: outflow        */
    int active;            /* activate() / deactivate()                               */
    float position[3];     /* sphere centre; cuboid minimum corner (vmath::vec3)      */
    double radius;         /* sphere radius                                           */
    double size[3];        /* cuboid width, height, depth                             */
    float velocity[3];     /* setVelocity: velocity of the particles an inflow adds   */
} gfs_fluid_source;

/* Replace the simulation's fluid sources (copied; n = 0 removes them all).
   While any is set, every gfs_sim_step applies them where the reference does, at
   the start of _updateFluidCells (fluidsimulation.cpp:1990-1994), after the
   particles in solid cells are removed: _updateFluidSources (:1854-1879). */
int gfs_sim_set_fluid_sources(gfs_sim *sim, const gfs_fluid_source *sources, int n);

/* Jitter of the particles sources add: each component in [-j, j],
   j = 0.25 * factor * dx (FluidSimulation::_getMarkerParticleJitter,
   fluidsimulation.cpp:1219-1221; factor 0.1 by default, fluidsimulation.h:1111).
   The reference draws the jitter from rand(); here it is a counter-based hash of
   (seed, particle id, axis), so runs are reproducible.  factor in [0, 1]; with 0
   the positions are the reference's exactly. */
int gfs_sim_set_marker_particle_jitter(gfs_sim *sim, double factor, uint64_t seed);

/* Queue n cells (int32 triples i, j, k) to become fluid at the next step, each
   with 8 marker particles of the given velocity (float[3]; NULL: zero).
   Replaces FluidSimulation::addFluidCells (fluidsimulation.cpp:887-918) and the
   C exports FluidSimulation_add_fluid_cells / _add_fluid_cells_velocity
   (c_bindings/fluidsimulation_c.cpp:770-808): only the cells that are air when
   called are queued; an index out of range fails with GFS_ERR_INVALID and
   queues nothing.  The next step applies the queue where the reference does
   (_updateAddedFluidCellQueue, :1881-1892): a queued cell that is still air
   gets its particles (the jitter of gfs_sim_set_marker_particle_jitter) and
   becomes fluid. */
int gfs_sim_add_fluid_cells(gfs_sim *sim, const int32_t *ijk, int n, const float *velocity);

/* Queue n cells whose marker particles the next step removes, after the added
   cells and before the fluid sources (_updateRemovedFluidCellQueue,
   :1895-1930).  Replaces FluidSimulation::removeFluidCells (:920-940) and
   FluidSimulation_remove_fluid_cells (c_bindings/fluidsimulation_c.cpp:810-828). */
int gfs_sim_remove_fluid_cells(gfs_sim *sim, const int32_t *ijk, int n);

/* Apply the queued fluid cells and the fluid sources once, outside a step (the
   part of _updateFluidCells before the cells are classified, :1990-1994), and
   sort the particles.  Outputs (totals of both) may be NULL. */
int gfs_sim_update_fluid_sources(gfs_sim *sim, int64_t *num_added, int64_t *num_removed);

/* ------------------------------------------------------------- savestates */

/* The header of a FluidSimulationSaveState file
   (FluidSimulationSaveState::loadState, fluidsimulationsavestate.cpp:101-117, and
   its getters getGridDimensions / getCellSize / getCurrentFrame /
   getNumMarkerParticles / getNumDiffuseParticles / getNumSolidCells /
   isFluidBrickGridEnabled, fluidsimulationsavestate.h:47-67).  Any output
   pointer may be NULL. */
int gfs_savestate_read_header(const char *path, int *ni, int *nj, int *nk, double *dx,
                              int *current_frame, int64_t *num_marker_particles,
                              int64_t *num_diffuse_particles, int64_t *num_solid_cells,
                              int *brick_grid);

/* FluidSimulation::saveState (fluidsimulation.cpp:60-65 ->
   FluidSimulationSaveState::saveState, fluidsimulationsavestate.cpp:31-99): the
   simulation's marker particles (in the device's (cell, id) order) and solid
   cells (i fastest) in the reference's file format, with current_frame in the
   header, no diffuse particles and no brick grid.  The particles go from the
   device to the file through pinned chunks; the call synchronises the stream. */
int gfs_sim_save_state(gfs_sim *sim, const char *path, int current_frame);

/* FluidSimulation(FluidSimulationSaveState&) (fluidsimulation.cpp:35-39,
   _initializeSimulationFromSaveState :1638-1663): replace the simulation's
   material grid by the file's solid cells (all other cells air) and its particles
   by the file's marker particles (ids 0..n-1 in file order; particles in solid
   cells are removed, as gfs_sim_set_particles does).  The grid dimensions and dx
   must equal the simulation's; diffuse particles and brick grid data are skipped.
   *current_frame (may be NULL) receives the header's frame.  Fails with
   GFS_ERR_INVALID on a missing, truncated or mismatching file. */
int gfs_sim_load_state(gfs_sim *sim, const char *path, int *current_frame);

/* ------------------------------------------------ differentiable rollout */

/* A differentiable rollout of `nsteps` substeps of length dt over n particles
   on a simulation's grid, material and parameters (no counterpart in the
   reference; the forward model is the substep of gfs_sim_step).  Particles
   start at d_positions (n x 3) with the velocities d_velocities (n x 3) or, if
   that is NULL, velocities sampled (Catmull-Rom, as G2P samples) from the
   parameter MAC field d_u0 / d_v0 / d_w0.  Outputs (each may be NULL): the
   cell-centred particle density after the last substep (ni*nj*nk floats, splat
   kernel 1 - 4/9 s^3 + 17/9 s^2 - 22/9 s of radius 1.5 dx at cell centres) and
   the particle centroid at the start of every substep and at the end
   ((nsteps + 1) x 3 floats).  The forward keeps every substep's particle state on
   the device; the backward recomputes each substep's grids from it and runs the
   adjoint of every stage with the substep's discrete structure (fluid cells,
   splat set masks, fill and extrapolation structure) held fixed; the pressure
   adjoint is a second MIC(0)-PCG solve with the same matrix.  Collisions and
   the per-cell cap are not differentiated: a forward in which particles are
   removed fails with GFS_ERR_STATE.  All pointers are DEVICE pointers on the
   simulation's GPU; face fields are unpadded, x fastest; per-particle arrays
   are in the input order.  The calls synchronise the context's stream. */
typedef struct gfs_diff gfs_diff;
int gfs_diff_create(gfs_sim *sim, int nsteps, int64_t n, double dt, gfs_diff **out);
int gfs_diff_destroy(gfs_diff *d);
int gfs_diff_forward(gfs_diff *d, const float *d_positions, const float *d_velocities, const float *d_u0,
                     const float *d_v0, const float *d_w0, float *d_density, float *d_centroids);
/* Gradients of a loss from its gradients with respect to the forward's outputs
   (d_grad_density, d_grad_centroids; NULL = not part of the loss).  Outputs
   (each may be NULL): the parameter field's gradient (when the velocities were
   sampled from it), the initial velocities' gradient, and the starting
   positions' gradient with the initial velocities held fixed. */
int gfs_diff_backward(gfs_diff *d, const float *d_grad_density, const float *d_grad_centroids,
                      float *d_grad_u0, float *d_grad_v0, float *d_grad_w0, float *d_grad_velocities,
                      float *d_grad_positions);
/* Device time of the last forward / backward and the rollout's own device bytes. */
int gfs_diff_info(gfs_diff *d, double *forward_ms, double *backward_ms, int64_t *device_bytes);

/* Number of kernel launches the library has issued on this context (for
   accounting in benchmarks). */
int gfs_ctx_launch_count(gfs_ctx *ctx, int64_t *count);

/* ------------------------------------------ wavefront kernels of the solve */

/* The MIC(0) triangular solves (PressureSolver::_applyPreconditioner,
   pressuresolver.cpp:304-386) run as i+j+k hyperplane wavefronts over blocks
   of 16 x 16 pencils.  BLOCK, CLUSTER_4X2 and CLUSTER_2X2 compute the same values
   in the same order: BLOCK hands block-edge values over through L2 words (four
   receiver warps per block poll them into shared memory); CLUSTER_4X2 / _2X2
   group 4 x 2 or 2 x 2 blocks into a thread-block cluster whose blocks hand over
   through distributed shared memory.  WARP (FP32 solves only) runs each block
   with one compute warp and no per-plane barrier, the same per-cell arithmetic
   and its own (deterministic) summation order of the backward solve's dot
   product; an FP64 solve asked to run WARP runs BLOCK.  AUTO (the default) runs
   WARP for FP32 solves and BLOCK for FP64 solves, the fastest on GB300 at 128^3
   and 256^3.
   A cluster shape set explicitly that cannot run on a grid makes the solve fail
   with GFS_ERR_INVALID.  The preconditioner build always runs its own kernel.
   No counterpart in the reference (its solves are sequential loops). */
#define GFS_SWEEP_AUTO 0
#define GFS_SWEEP_BLOCK 1
#define GFS_SWEEP_CLUSTER_4X2 2
#define GFS_SWEEP_CLUSTER_2X2 3
#define GFS_SWEEP_WARP 4
int gfs_ctx_set_sweep_kernel(gfs_ctx *ctx, int kind);
/* The kernel the context's last triangular solve ran (GFS_SWEEP_BLOCK /
   _CLUSTER_4X2 / _CLUSTER_2X2 / _WARP; GFS_SWEEP_AUTO before the first solve). */
int gfs_ctx_last_sweep_kernel(gfs_ctx *ctx, int *kind);

/* Bound of every wait of the wavefront kernels, in polls of the awaited word
   (default 4,194,304).  A wait that reaches it sets a device error bit, stops
   waiting and lets its kernel run to the end; the solve then fails with
   GFS_ERR_TIMEOUT and the context stays usable (the next solve starts clean).
   polls <= 0 restores the default.  The reference has no device waits; its
   failure path is the int *err + message of its C bindings (cbindings.h:25-135),
   which GFS_ERR_TIMEOUT and gfs_last_error() keep. */
int gfs_ctx_set_wait_limit(gfs_ctx *ctx, int64_t polls);
/* Fault injection for tests of that path: the next `sweeps` wavefront launches
   on this context wait for an exchange tag that no producer writes, so every
   waiting thread runs into the wait limit (set a small one first).  Nothing
   faults or hangs: each wait ends at its bound. */
int gfs_ctx_inject_wait_timeout(gfs_ctx *ctx, int sweeps);

/* Optional per-kernel-class timing with CUDA events recorded on the context's
   stream around every launch (the reference logs stage times with StopWatch,
   fluidsimulation.cpp:3273-3389).  Classes are numbered 0..GFS_NUM_KERNEL_CLASSES-1;
   gfs_ctx_profile_read returns a class's name, accumulated device time and
   launch count (it synchronises the stream). */
#define GFS_NUM_KERNEL_CLASSES 16
int gfs_ctx_profile_enable(gfs_ctx *ctx, int on);
int gfs_ctx_profile_reset(gfs_ctx *ctx);
int gfs_ctx_profile_read(gfs_ctx *ctx, int index, const char **name, double *total_ms,
                         int64_t *count);

#ifdef __cplusplus
}
#endif

#endif /* GFS_H */
