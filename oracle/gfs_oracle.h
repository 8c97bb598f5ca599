/*
 * gfs_oracle.h -- CPU restatement of GridFluidSim3D's per-substep FLIP core.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load
 * it.  The product path (libgfs) never links or calls it.
 *
 * Every function restates one piece of the reference's NoCL (CPU) code, with the
 * same float/double casts and the same loop order, and cites the file:line it
 * follows (paths relative to the reference's src/ directory).  Built with
 * -ffp-contract=off so that x86 and aarch64 give the same bits.
 *
 * Layout conventions (identical to the reference's Array3d):
 *   - every grid is a flat array with index  i + W*(j + H*k);
 *   - cell grids are ni x nj x nk, U is (ni+1) x nj x nk, V is ni x (nj+1) x nk,
 *     W is ni x nj x (nk+1);
 *   - material: 0 = air, 1 = fluid, 2 = solid (fluidmaterialgrid.h:29-33); a cell
 *     outside the grid reads as solid (fluidmaterialgrid.cpp:26);
 *   - particles: positions / velocities as float xyz triples, plus a uint32 id
 *     carried through removals so that results can be matched per particle.
 */
#ifndef GFS_ORACLE_H
#define GFS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GFO_AIR 0
#define GFO_FLUID 1
#define GFO_SOLID 2

/* ScalarField::addPointValue over a point list, weight field enabled
   (scalarfield.cpp:167-201; CLScalarField::_addPointValuesNoCL
   clscalarfield.cpp:1521-1541 but with "add into field" semantics). */
void gfo_splat_add(const float *pos, const float *val, int64_t n, double radius,
                   const float offset[3], double dx, int W, int H, int D,
                   float *field, float *weight);

/* CLScalarField::addPoints / addPointValues with add semantics: val NULL gives
   v = 1 (ScalarField::addPoint, scalarfield.cpp:126-160), weight may be NULL
   (no weight field).  thr_set != 0: a node whose value before the call exceeds
   thr receives nothing (ScalarField's per-node threshold test,
   scalarfield.cpp:141-143, applied to the incoming field). */
void gfo_splat_points(const float *pos, const float *val, int64_t n, double radius,
                      const float offset[3], double dx, int W, int H, int D,
                      float *field, float *weight, int thr_set, double thr);

/* ScalarField::applyWeightField (scalarfield.cpp:90-106). */
void gfo_apply_weight(int64_t count, float *field, const float *weight);

/* FluidSimulation::_computeVelocityScalarField (fluidsimulation.cpp:2526-2595):
   splat velocity component `dir` (0=U,1=V,2=W) of every particle onto the face
   grid of that component; writes the normalised field and the isValueSet mask
   (weight > 1e-9). */
void gfo_velocity_scalar_field(int dir, int ni, int nj, int nk, double dx,
                               const float *pos, const float *vel, int64_t n,
                               float *field, uint8_t *is_set);

/* FluidSimulation::_advectVelocityFieldU/V/W (fluidsimulation.cpp:2597-2736):
   splat + copy into fluid-bordering faces + 26-neighbour fill of unset faces. */
void gfo_advect_velocity_field(int ni, int nj, int nk, double dx, const uint8_t *mat,
                               const float *pos, const float *vel, int64_t n,
                               float *u, float *v, float *w);

/* The copy into fluid-bordering faces and the 26-neighbour fill of one component
   (out cleared first), from its splatted field and is-set mask. */
void gfo_face_fill(int dir, int ni, int nj, int nk, const uint8_t *mat, const float *grid,
                   const uint8_t *is_set, float *out);

/* Component `dir` of _advectVelocityField from a splat already accumulated into
   value / weight (gfo_splat_add, possibly in pieces): value /= weight, is-set
   mask weight > 1e-9, then gfo_face_fill into out. */
void gfo_velocity_from_splat(int dir, int ni, int nj, int nk, const uint8_t *mat, float *value,
                             const float *weight, float *out);

/* MACVelocityField::extrapolateVelocityField (macvelocityfield.cpp:754-797). */
void gfo_extrapolate(int ni, int nj, int nk, const uint8_t *mat, int num_layers,
                     float *u, float *v, float *w);

/* FluidSimulation::_applyConstantBodyForces (fluidsimulation.cpp:2766-2805). */
void gfo_body_force(int ni, int nj, int nk, const uint8_t *mat, const float g[3],
                    double dt, float *u, float *v, float *w);

/* PressureSolver::solve (pressuresolver.cpp:116-498).  Fluid cells are taken from
   `mat` in lexicographic k->j->i order (fluidsimulation.cpp:2031-2039).
   pressure_out has one double per fluid cell in that order.  Returns the number
   of fluid cells.  *iters = CG iteration count in the reference's numbering
   (the value its log prints; -1 if the solve exited before CG),
   *max_resid = max|r| at exit. tol / max_iters are the reference's
   1e-6 / 200 unless the caller overrides them. */
int64_t gfo_pressure_solve(int ni, int nj, int nk, double dx, double density, double dt,
                           const uint8_t *mat, const float *u, const float *v,
                           const float *w, double tol, int max_iters,
                           double *pressure_out, int *iters, double *max_resid);

/* max|b - A p| (double) for a compact pressure vector p, with the reference's b
   (pressuresolver.cpp:162-208) and stencil (:388-426). */
double gfo_pressure_residual(int ni, int nj, int nk, double dx, double density, double dt,
                             const uint8_t *mat, const float *u, const float *v, const float *w,
                             const double *p);

/* Scatter a compact pressure vector into a float cell grid
   (fluidsimulation.cpp:2884-2888). */
void gfo_pressure_to_grid(int ni, int nj, int nk, const uint8_t *mat,
                          const double *pressure, float *pgrid);

/* FluidSimulation::_applyPressureToVelocityField (fluidsimulation.cpp:2895-3061). */
void gfo_apply_pressure(int ni, int nj, int nk, double dx, double density, double dt,
                        const uint8_t *mat, const float *pgrid,
                        float *u, float *v, float *w);

/* MACVelocityField::evaluateVelocityAtPosition (macvelocityfield.cpp:549-559,
   _interpolateU/V/W :350-450, Interpolation::tricubicInterpolate
   interpolation.cpp:26-46) for each position. */
void gfo_evaluate_velocity(int ni, int nj, int nk, double dx, const float *u,
                           const float *v, const float *w, const float *pos,
                           int64_t n, float *out);

/* FluidSimulation::_updateRangeOfMarkerParticleVelocities
   (fluidsimulation.cpp:3104-3129): PIC/FLIP blend, in place on vel. */
void gfo_flip_update(int ni, int nj, int nk, double dx, double ratio_pic,
                     const float *u_new, const float *v_new, const float *w_new,
                     const float *u_old, const float *v_old, const float *w_old,
                     const float *pos, int64_t n, float *vel);

/* ParticleAdvector::_RK4 (particleadvector.cpp:1045-1054) per position. */
void gfo_advect_rk4(int ni, int nj, int nk, double dx, const float *u, const float *v,
                    const float *w, double dt, const float *pos, int64_t n, float *out);

/* FluidSimulation::_advanceRangeOfMarkerParticles collision step
   (fluidsimulation.cpp:3198-3207 -> _resolveParticleSolidCellCollision :3145-3179,
   Collision::getLineSegmentVoxelIntersection collision.cpp:303-402,
   Collision::rayIntersectsAABB :404-449).  p0 = old positions, p1 = advected
   positions, rewritten in place where p1 lands in a solid cell. */
void gfo_resolve_collisions(int ni, int nj, int nk, double dx, const uint8_t *mat,
                            const float *p0, int64_t n, float *p1);

/* Collision::getLineSegmentVoxelIntersection (collision.cpp:303-402): 1 and the
   first solid voxel on the segment p0 -> p1, or 0. */
int gfo_segment_voxel(const float *p0, const float *p1, double dx, int ni, int nj, int nk,
                      const uint8_t *mat, int *voxel);

/* Collision::rayIntersectsAABB (collision.cpp:404-449) for the box [bmin, bmax]. */
int gfo_ray_aabb(const float *p0, const float *dir, const float *bmin, const float *bmax, float *out);

/* FluidSimulation::_removeMarkerParticlesInSolidCells (fluidsimulation.cpp:1933-1958)
   followed by _updateFluidCells' reclassification (:1990-2041).  Compacts the
   particle arrays in place (order kept) and returns the surviving count. */
int64_t gfo_update_fluid_cells(int ni, int nj, int nk, double dx, uint8_t *mat,
                               float *pos, float *vel, uint32_t *ids, int64_t n);

/* FluidSimulation::_removeMarkerParticles (fluidsimulation.cpp:3221-3243) with a
   deterministic selection: in each cell the particles with the smallest ids are
   kept (the reference keeps a random subset after a rand() shuffle).  Order kept.
   Returns the surviving count. */
int64_t gfo_cap_particles_per_cell(int ni, int nj, int nk, double dx, int max_per_cell,
                                   float *pos, float *vel, uint32_t *ids, int64_t n);

/* Per-stage outputs of one substep, for stage-level comparisons. */
typedef struct gfo_substep_stats {
    int64_t num_fluid_cells;
    int64_t num_particles;
    int cg_iterations;
    double cg_max_resid;
} gfo_substep_stats;

/* FluidSimulation::_stepFluid stages 1, 5-9, 11, 12 (fluidsimulation.cpp:3262-3390)
   with meshing, level set, diffuse material and fluid sources off.
   Particles are updated in place; returns the surviving particle count.
   u/v/w receive the final (post-extrapolation) MAC field. pressure_grid (optional,
   ni*nj*nk floats) receives the pressure grid. */
int64_t gfo_substep(int ni, int nj, int nk, double dx, double dt, const float g[3],
                    double density, double ratio_pic, int num_layers, int max_per_cell,
                    uint8_t *mat, float *pos, float *vel, uint32_t *ids, int64_t n,
                    float *u, float *v, float *w, float *pressure_grid,
                    gfo_substep_stats *stats);

#ifdef __cplusplus
}
#endif

#endif
