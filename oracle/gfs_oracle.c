/*
 * gfs_oracle.c -- CPU restatement of GridFluidSim3D's per-substep FLIP core.
 *
 * TEST INFRASTRUCTURE ONLY (see gfs_oracle.h).  Single-threaded, like the
 * reference (which has no threads at all).  Compiled with -ffp-contract=off.
 *
 * Arithmetic types follow the reference exactly: vmath::vec3 is float
 * (vmath.h:33-56) and every vec3 operator works in float with a float scalar
 * (vmath.cpp:71-99); grid/interpolation math is double; Array3d<float> stores
 * float.  Comments name the reference line each block restates.
 */
#include "gfs_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ---------------------------------------------------------------- helpers */

static inline int64_t idx3(int i, int j, int k, int W, int H) {
    return (int64_t)i + (int64_t)W * ((int64_t)j + (int64_t)H * (int64_t)k);
}

static inline int in_range(int i, int j, int k, int W, int H, int D) {
    return i >= 0 && j >= 0 && k >= 0 && i < W && j < H && k < D;
}

/* FluidMaterialGrid: out-of-range cells are solid (fluidmaterialgrid.cpp:26). */
static inline uint8_t mat_at(const uint8_t *mat, int i, int j, int k, int ni, int nj, int nk) {
    if (!in_range(i, j, k, ni, nj, nk)) return GFO_SOLID;
    return mat[idx3(i, j, k, ni, nj)];
}

/* FluidMaterialGrid::isFaceBorderingMaterialU/V/W (fluidmaterialgrid.cpp:119-143). */
static inline int face_borders(const uint8_t *mat, int dir, int i, int j, int k,
                               int ni, int nj, int nk, uint8_t m) {
    if (dir == 0) {
        if (i == ni) return mat_at(mat, i - 1, j, k, ni, nj, nk) == m;
        if (i > 0) return mat_at(mat, i, j, k, ni, nj, nk) == m || mat_at(mat, i - 1, j, k, ni, nj, nk) == m;
        return mat_at(mat, i, j, k, ni, nj, nk) == m;
    } else if (dir == 1) {
        if (j == nj) return mat_at(mat, i, j - 1, k, ni, nj, nk) == m;
        if (j > 0) return mat_at(mat, i, j, k, ni, nj, nk) == m || mat_at(mat, i, j - 1, k, ni, nj, nk) == m;
        return mat_at(mat, i, j, k, ni, nj, nk) == m;
    } else {
        if (k == nk) return mat_at(mat, i, j, k - 1, ni, nj, nk) == m;
        if (k > 0) return mat_at(mat, i, j, k, ni, nj, nk) == m || mat_at(mat, i, j, k - 1, ni, nj, nk) == m;
        return mat_at(mat, i, j, k, ni, nj, nk) == m;
    }
}

static inline void face_dims(int dir, int ni, int nj, int nk, int *W, int *H, int *D) {
    *W = ni + (dir == 0);
    *H = nj + (dir == 1);
    *D = nk + (dir == 2);
}

/* Grid3d::positionToGridIndex (grid3d.h:58-63): floor(p * (1/dx)) in double. */
static inline void pos_to_cell(const float *p, double dx, int *i, int *j, int *k) {
    double invdx = 1.0 / dx;
    *i = (int)floor((double)p[0] * invdx);
    *j = (int)floor((double)p[1] * invdx);
    *k = (int)floor((double)p[2] * invdx);
}

/* --------------------------------------------------------------- a2: splat */

void gfo_splat_points(const float *pos, const float *val, int64_t n, double r,
                      const float offset[3], double dx, int W, int H, int D,
                      float *field, float *weight, int thr_set, double thr) {
    /* ScalarField::setPointRadius (scalarfield.cpp:38-44) */
    double coef1 = (4.0 / 9.0) * (1.0 / (r * r * r * r * r * r));
    double coef2 = (17.0 / 9.0) * (1.0 / (r * r * r * r));
    double coef3 = (22.0 / 9.0) * (1.0 / (r * r));
    double rsq = r * r;
    double inv = 1.0 / dx;
    float *before = NULL;
    float fthr = (float)thr;
    if (thr_set) {
        before = (float *)malloc((size_t)W * H * D * sizeof(float));
        memcpy(before, field, (size_t)W * H * D * sizeof(float));
    }
    for (int64_t pi = 0; pi < n; pi++) {
        /* p -= _gridOffset (float) */
        float p[3] = {pos[3 * pi] - offset[0], pos[3 * pi + 1] - offset[1], pos[3 * pi + 2] - offset[2]};
        double scale = val ? (double)val[pi] : 1.0;
        int ci, cj, ck;
        pos_to_cell(p, dx, &ci, &cj, &ck);
        /* cpos = vec3((float)c.i*dx, ...) -> float; trans = p - cpos (float) */
        float cpos[3] = {(float)((double)(float)ci * dx), (float)((double)(float)cj * dx),
                         (float)((double)(float)ck * dx)};
        float trans[3] = {p[0] - cpos[0], p[1] - cpos[1], p[2] - cpos[2]};
        int gimin = ci - (int)fmax(0, ceil((r - trans[0]) * inv));
        int gjmin = cj - (int)fmax(0, ceil((r - trans[1]) * inv));
        int gkmin = ck - (int)fmax(0, ceil((r - trans[2]) * inv));
        int gimax = ci + (int)fmax(0, ceil((r - dx + trans[0]) * inv));
        int gjmax = cj + (int)fmax(0, ceil((r - dx + trans[1]) * inv));
        int gkmax = ck + (int)fmax(0, ceil((r - dx + trans[2]) * inv));
        int i0 = (int)fmax(gimin, 0), j0 = (int)fmax(gjmin, 0), k0 = (int)fmax(gkmin, 0);
        int i1 = (int)fmin(gimax, W - 1), j1 = (int)fmin(gjmax, H - 1), k1 = (int)fmin(gkmax, D - 1);
        for (int k = k0; k <= k1; k++) {
            for (int j = j0; j <= j1; j++) {
                for (int i = i0; i <= i1; i++) {
                    int64_t f = idx3(i, j, k, W, H);
                    if (thr_set && before[f] > fthr) continue;
                    /* gpos = Grid3d::GridIndexToPosition(i,j,k,dx) (grid3d.h:79-81) */
                    float gx = (float)((double)(float)i * dx);
                    float gy = (float)((double)(float)j * dx);
                    float gz = (float)((double)(float)k * dx);
                    float vx = gx - p[0], vy = gy - p[1], vz = gz - p[2];
                    /* vmath::dot is float (vmath.h:71-73) */
                    float d2f = vx * vx + vy * vy + vz * vz;
                    double distsq = (double)d2f;
                    if (distsq < rsq) {
                        double wgt = 1.0 - coef1 * distsq * distsq * distsq + coef2 * distsq * distsq - coef3 * distsq;
                        field[f] += (float)(wgt * scale);
                        if (weight) weight[f] += (float)wgt;
                    }
                }
            }
        }
    }
    free(before);
}

/* ScalarField::addPointValue (scalarfield.cpp:167-201) with the bounds of
   Grid3d::getGridIndexBounds (grid3d.h:350-371) and the kernel of
   ScalarField::_evaluateTricubicFieldFunctionForRadiusSquared (:569-571),
   weight field enabled. */
void gfo_splat_add(const float *pos, const float *val, int64_t n, double r,
                   const float offset[3], double dx, int W, int H, int D,
                   float *field, float *weight) {
    gfo_splat_points(pos, val, n, r, offset, dx, W, H, D, field, weight, 0, 0.0);
}

void gfo_apply_weight(int64_t count, float *field, const float *weight) {
    for (int64_t f = 0; f < count; f++) {
        float wgt = weight[f];
        if (wgt > 0.0) {
            field[f] = field[f] / wgt;
        }
    }
}

void gfo_velocity_scalar_field(int dir, int ni, int nj, int nk, double dx,
                               const float *pos, const float *vel, int64_t n,
                               float *field, uint8_t *is_set) {
    int W, H, D;
    face_dims(dir, ni, nj, nk, &W, &H, &D);
    int64_t count = (int64_t)W * H * D;
    /* offset (fluidsimulation.cpp:2537-2545): vec3(0.0, 0.5*dx, 0.5*dx) etc. -> float */
    float half = (float)(0.5 * dx);
    float offset[3] = {half, half, half};
    offset[dir] = 0.0f;
    float *weight = (float *)calloc((size_t)count, sizeof(float));
    float *vals = (float *)malloc((size_t)(n > 0 ? n : 1) * sizeof(float));
    memset(field, 0, (size_t)count * sizeof(float));
    for (int64_t p = 0; p < n; p++) vals[p] = vel[3 * p + dir];
    gfo_splat_add(pos, vals, n, dx, offset, dx, W, H, D, field, weight);
    gfo_apply_weight(count, field, weight);
    /* eps = 1e-9 mask (fluidsimulation.cpp:2575-2586) */
    for (int64_t f = 0; f < count; f++) is_set[f] = ((double)weight[f] > 1e-9) ? 1 : 0;
    free(weight);
    free(vals);
}

/* -------------------------------------------------- a3: face copy and fill */

/* The face copy and 26-neighbour fill of one component (fluidsimulation.cpp:
   2597-2736) from the splatted field `grid` (after applyWeightField) and its
   is-set mask, into `out` (cleared first: _MACVelocity.clearU()). */
void gfo_face_fill(int dir, int ni, int nj, int nk, const uint8_t *mat, const float *grid,
                   const uint8_t *is_set, float *out) {
    int W, H, D;
    face_dims(dir, ni, nj, nk, &W, &H, &D);
    int64_t count = (int64_t)W * H * D;
    memset(out, 0, (size_t)count * sizeof(float));
    /* extrapolationIndices: fluid-bordering faces without a value, in
       k->j->i order (fluidsimulation.cpp:2604-2616) */
    int64_t *queue = (int64_t *)malloc((size_t)count * sizeof(int64_t));
    int64_t nq = 0;
    for (int k = 0; k < D; k++)
        for (int j = 0; j < H; j++)
            for (int i = 0; i < W; i++) {
                if (face_borders(mat, dir, i, j, k, ni, nj, nk, GFO_FLUID)) {
                    int64_t f = idx3(i, j, k, W, H);
                    if (!is_set[f]) queue[nq++] = f;
                    else out[f] = grid[f];
                }
            }
    /* 26-neighbour average (fluidsimulation.cpp:2618-2639); Grid3d::
       getNeighbourGridIndices26 order is k, j, i ascending (grid3d.h:224-236).
       U uses fabs(value) > 0, V and W use isValueSet (the reference's
       asymmetry, :2630 vs :2675/:2720). */
    for (int64_t q = 0; q < nq; q++) {
        int64_t f = queue[q];
        int gi = (int)(f % W), gj = (int)((f / W) % H), gk = (int)(f / ((int64_t)W * H));
        double avg = 0.0, wsum = 0.0;
        for (int kk = gk - 1; kk <= gk + 1; kk++)
            for (int jj = gj - 1; jj <= gj + 1; jj++)
                for (int ii = gi - 1; ii <= gi + 1; ii++) {
                    if (ii == gi && jj == gj && kk == gk) continue;
                    if (!in_range(ii, jj, kk, W, H, D)) continue;
                    int64_t nf = idx3(ii, jj, kk, W, H);
                    int ok = (dir == 0) ? (fabs((double)grid[nf]) > 0.0) : (is_set[nf] != 0);
                    if (ok) {
                        avg += (double)grid[nf];
                        wsum += 1.0;
                    }
                }
        if (wsum > 0.0) out[f] = (float)(avg / wsum);
    }
    free(queue);
}

/* _computeVelocityScalarField's tail (fluidsimulation.cpp:2567-2586) and the
   fill, from a splat already accumulated into value / weight (value is divided
   in place): the velocity component `dir` of _advectVelocityField. */
void gfo_velocity_from_splat(int dir, int ni, int nj, int nk, const uint8_t *mat, float *value,
                             const float *weight, float *out) {
    int W, H, D;
    face_dims(dir, ni, nj, nk, &W, &H, &D);
    int64_t count = (int64_t)W * H * D;
    uint8_t *is_set = (uint8_t *)malloc((size_t)count);
    gfo_apply_weight(count, value, weight);
    for (int64_t f = 0; f < count; f++) is_set[f] = ((double)weight[f] > 1e-9) ? 1 : 0;
    gfo_face_fill(dir, ni, nj, nk, mat, value, is_set, out);
    free(is_set);
}

void gfo_advect_velocity_field(int ni, int nj, int nk, double dx, const uint8_t *mat,
                               const float *pos, const float *vel, int64_t n,
                               float *u, float *v, float *w) {
    float *mac[3] = {u, v, w};
    for (int dir = 0; dir < 3; dir++) {
        int W, H, D;
        face_dims(dir, ni, nj, nk, &W, &H, &D);
        int64_t count = (int64_t)W * H * D;
        float *grid = (float *)malloc((size_t)count * sizeof(float));
        uint8_t *is_set = (uint8_t *)malloc((size_t)count);
        gfo_velocity_scalar_field(dir, ni, nj, nk, dx, pos, vel, n, grid, is_set);
        gfo_face_fill(dir, ni, nj, nk, mat, grid, is_set, mac[dir]);
        free(grid);
        free(is_set);
    }
}

/* ------------------------------------------------------ a4: extrapolation */

static inline int face_borders_layer(const int *layer, int dir, int i, int j, int k,
                                     int ni, int nj, int value) {
    /* MACVelocityField::_isFaceBorderingGridValueU/V/W (macvelocityfield.h:159-173) */
    if (dir == 0) {
        if (i == ni) return layer[idx3(i - 1, j, k, ni, nj)] == value;
        if (i > 0) return layer[idx3(i, j, k, ni, nj)] == value || layer[idx3(i - 1, j, k, ni, nj)] == value;
        return layer[idx3(i, j, k, ni, nj)] == value;
    } else if (dir == 1) {
        if (j == nj) return layer[idx3(i, j - 1, k, ni, nj)] == value;
        if (j > 0) return layer[idx3(i, j, k, ni, nj)] == value || layer[idx3(i, j - 1, k, ni, nj)] == value;
        return layer[idx3(i, j, k, ni, nj)] == value;
    } else {
        /* depth check uses grid.depth == nk */
        return -1; /* replaced below (needs nk) */
    }
}

static inline int face_borders_layer_w(const int *layer, int i, int j, int k, int ni, int nj,
                                       int nk, int value) {
    if (k == nk) return layer[idx3(i, j, k - 1, ni, nj)] == value;
    if (k > 0) return layer[idx3(i, j, k, ni, nj)] == value || layer[idx3(i, j, k - 1, ni, nj)] == value;
    return layer[idx3(i, j, k, ni, nj)] == value;
}

static inline int borders_layer(const int *layer, int dir, int i, int j, int k, int ni, int nj,
                                int nk, int value) {
    if (dir == 2) return face_borders_layer_w(layer, i, j, k, ni, nj, nk, value);
    return face_borders_layer(layer, dir, i, j, k, ni, nj, value);
}

void gfo_extrapolate(int ni, int nj, int nk, const uint8_t *mat, int num_layers,
                     float *u, float *v, float *w) {
    float *mac[3] = {u, v, w};
    int64_t ncell = (int64_t)ni * nj * nk;
    int *layer = (int *)malloc((size_t)ncell * sizeof(int));
    for (int64_t c = 0; c < ncell; c++) layer[c] = -1;

    /* _resetExtrapolatedFluidVelocities (macvelocityfield.cpp:720-752) */
    for (int dir = 0; dir < 3; dir++) {
        int W, H, D;
        face_dims(dir, ni, nj, nk, &W, &H, &D);
        for (int k = 0; k < D; k++)
            for (int j = 0; j < H; j++)
                for (int i = 0; i < W; i++)
                    if (!face_borders(mat, dir, i, j, k, ni, nj, nk, GFO_FLUID))
                        mac[dir][idx3(i, j, k, W, H)] = 0.0f;
    }

    /* _updateExtrapolationLayers / _updateExtrapolationLayer (:560-599) */
    for (int64_t c = 0; c < ncell; c++)
        if (mat[c] == GFO_FLUID) layer[c] = 0;
    for (int L = 1; L <= num_layers; L++) {
        for (int k = 0; k < nk; k++)
            for (int j = 0; j < nj; j++)
                for (int i = 0; i < ni; i++) {
                    if (layer[idx3(i, j, k, ni, nj)] == L - 1 && mat[idx3(i, j, k, ni, nj)] != GFO_SOLID) {
                        int nb[6][3] = {{i - 1, j, k}, {i + 1, j, k}, {i, j - 1, k},
                                        {i, j + 1, k}, {i, j, k - 1}, {i, j, k + 1}};
                        for (int q = 0; q < 6; q++) {
                            int a = nb[q][0], b = nb[q][1], c2 = nb[q][2];
                            if (in_range(a, b, c2, ni, nj, nk)) {
                                int64_t nc = idx3(a, b, c2, ni, nj);
                                if (layer[nc] == -1 && mat[nc] != GFO_SOLID) layer[nc] = L;
                            }
                        }
                    }
                }
    }

    /* _extrapolateVelocitiesForLayerIndexU/V/W (:665-718) with
       _getExtrapolatedVelocityForFaceU/V/W (:602-663) */
    for (int L = 1; L <= num_layers; L++) {
        for (int dir = 0; dir < 3; dir++) {
            int W, H, D;
            face_dims(dir, ni, nj, nk, &W, &H, &D);
            float *g = mac[dir];
            for (int k = 0; k < D; k++)
                for (int j = 0; j < H; j++)
                    for (int i = 0; i < W; i++) {
                        int ext = borders_layer(layer, dir, i, j, k, ni, nj, nk, L) &&
                                  !borders_layer(layer, dir, i, j, k, ni, nj, nk, L - 1) &&
                                  !face_borders(mat, dir, i, j, k, ni, nj, nk, GFO_SOLID);
                        if (!ext) continue;
                        int nb[6][3] = {{i - 1, j, k}, {i + 1, j, k}, {i, j - 1, k},
                                        {i, j + 1, k}, {i, j, k - 1}, {i, j, k + 1}};
                        double sum = 0.0, wsum = 0.0;
                        for (int q = 0; q < 6; q++) {
                            int a = nb[q][0], b = nb[q][1], c2 = nb[q][2];
                            if (in_range(a, b, c2, W, H, D) &&
                                borders_layer(layer, dir, a, b, c2, ni, nj, nk, L - 1)) {
                                sum += (double)g[idx3(a, b, c2, W, H)];
                                wsum++;
                            }
                        }
                        double val = (sum == 0.0) ? 0.0 : sum / wsum;
                        g[idx3(i, j, k, W, H)] = (float)val;
                    }
        }
    }
    free(layer);
}

/* ------------------------------------------------------- a5: body forces */

void gfo_body_force(int ni, int nj, int nk, const uint8_t *mat, const float g[3],
                    double dt, float *u, float *v, float *w) {
    float *mac[3] = {u, v, w};
    for (int dir = 0; dir < 3; dir++) {
        if (!(fabs((double)g[dir]) > 0.0)) continue;
        int W, H, D;
        face_dims(dir, ni, nj, nk, &W, &H, &D);
        /* MACVelocityField::addU: _u.add(i,j,k,(float)val) (macvelocityfield.cpp:204-210) */
        float add = (float)((double)g[dir] * dt);
        for (int k = 0; k < D; k++)
            for (int j = 0; j < H; j++)
                for (int i = 0; i < W; i++)
                    if (face_borders(mat, dir, i, j, k, ni, nj, nk, GFO_FLUID))
                        mac[dir][idx3(i, j, k, W, H)] += add;
    }
}

/* ----------------------------------------------------- a6-a11: pressure */

typedef struct {
    int ni, nj, nk;
    int64_t F;
    int32_t *cells;   /* flat cell index per fluid row, lexicographic */
    int32_t *keymap;  /* GridIndexKeyMap: cell -> row or -1 (gridindexkeymap.cpp:20-62) */
    uint8_t *diag, *pi, *pj, *pk; /* MatrixCell (pressuresolver.h:81-88) */
    double scale, negscale;
} gfo_ps;

static inline int32_t ps_find(const gfo_ps *s, int i, int j, int k) {
    if (!in_range(i, j, k, s->ni, s->nj, s->nk)) return -1;
    return s->keymap[idx3(i, j, k, s->ni, s->nj)];
}

static double vec_absmax(const double *x, int64_t n) {
    /* VectorXd::absMaxCoeff (pressuresolver.cpp:72-81) */
    double m = -INFINITY;
    for (int64_t i = 0; i < n; i++)
        if (fabs(x[i]) > m) m = fabs(x[i]);
    return m;
}

static double vec_dot(const double *a, const double *b, int64_t n) {
    double s = 0.0;
    for (int64_t i = 0; i < n; i++) s += a[i] * b[i];
    return s;
}

/* PressureSolver::_applyPreconditioner (pressuresolver.cpp:304-386) */
static void ps_apply_precon(const gfo_ps *s, const double *precon, const double *res,
                            double *vect, double *q) {
    int ni = s->ni, nj = s->nj;
    double negscale = s->negscale;
    for (int64_t idx = 0; idx < s->F; idx++) q[idx] = 0.0;
    for (int64_t idx = 0; idx < s->F; idx++) {
        int32_t c = s->cells[idx];
        int i = c % ni, j = (c / ni) % nj, k = c / (ni * nj);
        int32_t vim1 = ps_find(s, i - 1, j, k), vjm1 = ps_find(s, i, j - 1, k), vkm1 = ps_find(s, i, j, k - 1);
        double plusi_im1 = 0.0, precon_im1 = 0.0, q_im1 = 0.0;
        if (vim1 != -1) { plusi_im1 = (double)s->pi[vim1] * negscale; precon_im1 = precon[vim1]; q_im1 = q[vim1]; }
        double plusj_jm1 = 0.0, precon_jm1 = 0.0, q_jm1 = 0.0;
        if (vjm1 != -1) { plusj_jm1 = (double)s->pj[vjm1] * negscale; precon_jm1 = precon[vjm1]; q_jm1 = q[vjm1]; }
        double plusk_km1 = 0.0, precon_km1 = 0.0, q_km1 = 0.0;
        if (vkm1 != -1) { plusk_km1 = (double)s->pk[vkm1] * negscale; precon_km1 = precon[vkm1]; q_km1 = q[vkm1]; }
        double t = res[idx] - plusi_im1 * precon_im1 * q_im1 -
                   plusj_jm1 * precon_jm1 * q_jm1 -
                   plusk_km1 * precon_km1 * q_km1;
        t = t * precon[idx];
        q[idx] = t;
    }
    for (int64_t idx = s->F - 1; idx >= 0; idx--) {
        int32_t c = s->cells[idx];
        int i = c % ni, j = (c / ni) % nj, k = c / (ni * nj);
        int32_t vip1 = ps_find(s, i + 1, j, k), vjp1 = ps_find(s, i, j + 1, k), vkp1 = ps_find(s, i, j, k + 1);
        double vect_ip1 = vip1 != -1 ? vect[vip1] : 0.0;
        double vect_jp1 = vjp1 != -1 ? vect[vjp1] : 0.0;
        double vect_kp1 = vkp1 != -1 ? vect[vkp1] : 0.0;
        double plusi = (double)s->pi[idx] * negscale;
        double plusj = (double)s->pj[idx] * negscale;
        double plusk = (double)s->pk[idx] * negscale;
        double preconval = precon[idx];
        double t = q[idx] - plusi * preconval * vect_ip1 -
                   plusj * preconval * vect_jp1 -
                   plusk * preconval * vect_kp1;
        t = t * preconval;
        vect[idx] = t;
    }
}

/* PressureSolver::_applyMatrix (pressuresolver.cpp:388-426) */
static void ps_apply_matrix(const gfo_ps *s, const double *x, double *result) {
    int ni = s->ni, nj = s->nj;
    for (int64_t idx = 0; idx < s->F; idx++) {
        int32_t c = s->cells[idx];
        int i = c % ni, j = (c / ni) % nj, k = c / (ni * nj);
        double val = 0.0;
        int32_t v;
        v = ps_find(s, i - 1, j, k); if (v != -1) val += x[v];
        v = ps_find(s, i + 1, j, k); if (v != -1) val += x[v];
        v = ps_find(s, i, j - 1, k); if (v != -1) val += x[v];
        v = ps_find(s, i, j + 1, k); if (v != -1) val += x[v];
        v = ps_find(s, i, j, k - 1); if (v != -1) val += x[v];
        v = ps_find(s, i, j, k + 1); if (v != -1) val += x[v];
        val *= s->negscale;
        v = ps_find(s, i, j, k);
        val += (double)s->diag[v] * s->scale * x[v];
        result[v] = val;
    }
}

int64_t gfo_pressure_solve(int ni, int nj, int nk, double dx, double density, double dt,
                           const uint8_t *mat, const float *u, const float *v,
                           const float *w, double tol, int max_iters,
                           double *pressure_out, int *iters, double *max_resid) {
    gfo_ps s;
    memset(&s, 0, sizeof(s));
    s.ni = ni; s.nj = nj; s.nk = nk;
    int64_t ncell = (int64_t)ni * nj * nk;
    int64_t F = 0;
    for (int64_t c = 0; c < ncell; c++) F += (mat[c] == GFO_FLUID);
    s.F = F;
    *iters = -1;
    *max_resid = 0.0;
    if (F == 0) return 0;
    s.cells = (int32_t *)malloc((size_t)F * sizeof(int32_t));
    s.keymap = (int32_t *)malloc((size_t)ncell * sizeof(int32_t));
    {
        int64_t r = 0;
        for (int64_t c = 0; c < ncell; c++) {
            s.keymap[c] = -1;
            if (mat[c] == GFO_FLUID) { s.cells[r] = (int32_t)c; s.keymap[c] = (int32_t)r; r++; }
        }
    }
    for (int64_t i = 0; i < F; i++) pressure_out[i] = 0.0; /* pressure.fill(0.0) */

    int UW = ni + 1, VH = nj + 1;
    #define U_(i, j, k) (in_range(i, j, k, ni + 1, nj, nk) ? u[idx3(i, j, k, UW, nj)] : 0.0f)
    #define V_(i, j, k) (in_range(i, j, k, ni, nj + 1, nk) ? v[idx3(i, j, k, ni, VH)] : 0.0f)
    #define W_(i, j, k) (in_range(i, j, k, ni, nj, nk + 1) ? w[idx3(i, j, k, ni, nj)] : 0.0f)
    #define SOLID_(i, j, k) (mat_at(mat, i, j, k, ni, nj, nk) == GFO_SOLID)
    #define FLUID_(i, j, k) (mat_at(mat, i, j, k, ni, nj, nk) == GFO_FLUID)

    /* _calculateNegativeDivergenceVector (pressuresolver.cpp:162-208) */
    double *b = (double *)calloc((size_t)F, sizeof(double));
    double scale_div = 1.0f / (float)dx;
    for (int64_t idx = 0; idx < F; idx++) {
        int32_t c = s.cells[idx];
        int i = c % ni, j = (c / ni) % nj, k = c / (ni * nj);
        /* float sum of the six face terms, then promoted (:168-171) */
        float div = U_(i + 1, j, k) - U_(i, j, k) + V_(i, j + 1, k) - V_(i, j, k) +
                    W_(i, j, k + 1) - W_(i, j, k);
        b[idx] = -scale_div * (double)div;
    }
    {
        float usolid = 0.0f, vsolid = 0.0f, wsolid = 0.0f;
        float fscale = (float)scale_div;
        for (int64_t idx = 0; idx < F; idx++) {
            int32_t c = s.cells[idx];
            int i = c % ni, j = (c / ni) % nj, k = c / (ni * nj);
            if (SOLID_(i - 1, j, k)) b[idx] -= fscale * (U_(i, j, k) - usolid);
            if (SOLID_(i + 1, j, k)) b[idx] += fscale * (U_(i + 1, j, k) - usolid);
            if (SOLID_(i, j - 1, k)) b[idx] -= fscale * (V_(i, j, k) - vsolid);
            if (SOLID_(i, j + 1, k)) b[idx] += fscale * (V_(i, j + 1, k) - vsolid);
            if (SOLID_(i, j, k - 1)) b[idx] -= fscale * (W_(i, j, k) - wsolid);
            if (SOLID_(i, j, k + 1)) b[idx] += fscale * (W_(i, j, k + 1) - wsolid);
        }
    }
    if (vec_absmax(b, F) < tol) {
        *max_resid = vec_absmax(b, F);
        free(b); free(s.cells); free(s.keymap);
        return F;
    }

    /* _calculateMatrixCoefficients (pressuresolver.cpp:222-244) */
    s.diag = (uint8_t *)calloc((size_t)F, 1);
    s.pi = (uint8_t *)calloc((size_t)F, 1);
    s.pj = (uint8_t *)calloc((size_t)F, 1);
    s.pk = (uint8_t *)calloc((size_t)F, 1);
    for (int64_t idx = 0; idx < F; idx++) {
        int32_t c = s.cells[idx];
        int i = c % ni, j = (c / ni) % nj, k = c / (ni * nj);
        int nn = 0;
        if (!SOLID_(i - 1, j, k)) nn++;
        if (!SOLID_(i + 1, j, k)) nn++;
        if (!SOLID_(i, j - 1, k)) nn++;
        if (!SOLID_(i, j + 1, k)) nn++;
        if (!SOLID_(i, j, k - 1)) nn++;
        if (!SOLID_(i, j, k + 1)) nn++;
        s.diag[idx] = (uint8_t)nn;
        if (FLUID_(i + 1, j, k)) s.pi[idx] = 1;
        if (FLUID_(i, j + 1, k)) s.pj[idx] = 1;
        if (FLUID_(i, j, k + 1)) s.pk[idx] = 1;
    }
    s.scale = dt / (density * dx * dx);
    s.negscale = -s.scale;

    /* _calculatePreconditionerVector (pressuresolver.cpp:246-302) */
    double *precon = (double *)calloc((size_t)F, sizeof(double));
    {
        double scale = s.scale, negscale = s.negscale;
        double tau = 0.97, sigma = 0.25;
        for (int64_t idx = 0; idx < F; idx++) {
            int32_t c = s.cells[idx];
            int i = c % ni, j = (c / ni) % nj, k = c / (ni * nj);
            int32_t vim1 = ps_find(&s, i - 1, j, k), vjm1 = ps_find(&s, i, j - 1, k), vkm1 = ps_find(&s, i, j, k - 1);
            double diag = (double)s.diag[idx] * scale;
            double plusi_im1 = vim1 != -1 ? (double)s.pi[vim1] * negscale : 0.0;
            double plusi_jm1 = vjm1 != -1 ? (double)s.pi[vjm1] * negscale : 0.0;
            double plusi_km1 = vkm1 != -1 ? (double)s.pi[vkm1] * negscale : 0.0;
            double plusj_im1 = vim1 != -1 ? (double)s.pj[vim1] * negscale : 0.0;
            double plusj_jm1 = vjm1 != -1 ? (double)s.pj[vjm1] * negscale : 0.0;
            double plusj_km1 = vkm1 != -1 ? (double)s.pj[vkm1] * negscale : 0.0;
            double plusk_im1 = vim1 != -1 ? (double)s.pk[vim1] * negscale : 0.0;
            double plusk_jm1 = vjm1 != -1 ? (double)s.pk[vjm1] * negscale : 0.0;
            double plusk_km1 = vkm1 != -1 ? (double)s.pk[vkm1] * negscale : 0.0;
            double precon_im1 = vim1 != -1 ? precon[vim1] : 0.0;
            double precon_jm1 = vjm1 != -1 ? precon[vjm1] : 0.0;
            double precon_km1 = vkm1 != -1 ? precon[vkm1] : 0.0;
            double v1 = plusi_im1 * precon_im1;
            double v2 = plusj_jm1 * precon_jm1;
            double v3 = plusk_km1 * precon_km1;
            double v4 = precon_im1 * precon_im1;
            double v5 = precon_jm1 * precon_jm1;
            double v6 = precon_km1 * precon_km1;
            double e = diag - v1 * v1 - v2 * v2 - v3 * v3 -
                       tau * (plusi_im1 * (plusj_im1 + plusk_im1) * v4 +
                              plusj_jm1 * (plusi_jm1 + plusk_jm1) * v5 +
                              plusk_km1 * (plusi_km1 + plusj_km1) * v6);
            if (e < sigma * diag) e = diag;
            if (fabs(e) > 10e-9) precon[idx] = 1.0 / sqrt(e);
        }
    }

    /* _solvePressureSystem (pressuresolver.cpp:448-498) */
    double *residual = (double *)malloc((size_t)F * sizeof(double));
    double *aux = (double *)calloc((size_t)F, sizeof(double));
    double *search = (double *)malloc((size_t)F * sizeof(double));
    double *qtmp = (double *)malloc((size_t)F * sizeof(double));
    memcpy(residual, b, (size_t)F * sizeof(double));
    ps_apply_precon(&s, precon, residual, aux, qtmp);
    memcpy(search, aux, (size_t)F * sizeof(double));
    double sigma = vec_dot(aux, residual, F);
    int it = 0;
    int converged = 0;
    while (it < max_iters) {
        ps_apply_matrix(&s, search, aux);
        double alpha = sigma / vec_dot(aux, search, F);
        for (int64_t i = 0; i < F; i++) pressure_out[i] += search[i] * alpha;
        for (int64_t i = 0; i < F; i++) residual[i] += aux[i] * -alpha;
        if (vec_absmax(residual, F) < tol) { converged = 1; break; }
        ps_apply_precon(&s, precon, residual, aux, qtmp);
        double sigma_new = vec_dot(aux, residual, F);
        double beta = sigma_new / sigma;
        for (int64_t i = 0; i < F; i++) search[i] = aux[i] * 1.0 + search[i] * beta;
        sigma = sigma_new;
        it++;
    }
    (void)converged;
    *iters = it;
    *max_resid = vec_absmax(residual, F);

    free(residual); free(aux); free(search); free(qtmp); free(precon); free(b);
    free(s.diag); free(s.pi); free(s.pj); free(s.pk); free(s.cells); free(s.keymap);
    #undef U_
    #undef V_
    #undef W_
    #undef SOLID_
    #undef FLUID_
    return F;
}

void gfo_pressure_to_grid(int ni, int nj, int nk, const uint8_t *mat,
                          const double *pressure, float *pgrid) {
    int64_t ncell = (int64_t)ni * nj * nk, r = 0;
    for (int64_t c = 0; c < ncell; c++) {
        pgrid[c] = 0.0f;
        if (mat[c] == GFO_FLUID) pgrid[c] = (float)pressure[r++];
    }
}

/* ----------------------------------------------------- a12: apply pressure */

void gfo_apply_pressure(int ni, int nj, int nk, double dx, double density, double dt,
                        const uint8_t *mat, const float *pgrid,
                        float *u, float *v, float *w) {
    float *mac[3] = {u, v, w};
    double scale = dt / (density * dx);
    double invscale = 1.0 / scale;
    double usolid = 0.0;
    for (int dir = 0; dir < 3; dir++) {
        int W, H, D;
        face_dims(dir, ni, nj, nk, &W, &H, &D);
        int64_t count = (int64_t)W * H * D;
        float *g = mac[dir];
        float *tmp = (float *)calloc((size_t)count, sizeof(float));
        for (int k = 0; k < D; k++)
            for (int j = 0; j < H; j++)
                for (int i = 0; i < W; i++) {
                    int64_t f = idx3(i, j, k, W, H);
                    int bsolid = face_borders(mat, dir, i, j, k, ni, nj, nk, GFO_SOLID);
                    if (bsolid) tmp[f] = 0.0f;
                    if (face_borders(mat, dir, i, j, k, ni, nj, nk, GFO_FLUID) && !bsolid) {
                        /* _applyPressureToFaceU/V/W (fluidsimulation.cpp:2895-2987) */
                        int ci = i - (dir == 0), cj = j - (dir == 1), ck = k - (dir == 2);
                        int di = (dir == 0), dj = (dir == 1), dk = (dir == 2);
                        double p0, p1;
                        int s0 = mat_at(mat, ci, cj, ck, ni, nj, nk) == GFO_SOLID;
                        int s1 = mat_at(mat, ci + di, cj + dj, ck + dk, ni, nj, nk) == GFO_SOLID;
                        double face = (double)g[f];
                        if (!s0 && !s1) {
                            p0 = (double)pgrid[idx3(ci, cj, ck, ni, nj)];
                            p1 = (double)pgrid[idx3(ci + di, cj + dj, ck + dk, ni, nj)];
                        } else if (s0) {
                            p0 = (double)pgrid[idx3(ci + di, cj + dj, ck + dk, ni, nj)] - invscale * (face - usolid);
                            p1 = (double)pgrid[idx3(ci + di, cj + dj, ck + dk, ni, nj)];
                        } else {
                            p0 = (double)pgrid[idx3(ci, cj, ck, ni, nj)];
                            p1 = (double)pgrid[idx3(ci, cj, ck, ni, nj)] + invscale * (face - usolid);
                        }
                        double next = face - scale * (p1 - p0);
                        tmp[f] = (float)next;
                    }
                }
        /* _commitTemporaryVelocityFieldValues (fluidsimulation.cpp:2989-3019) */
        for (int k = 0; k < D; k++)
            for (int j = 0; j < H; j++)
                for (int i = 0; i < W; i++)
                    if (face_borders(mat, dir, i, j, k, ni, nj, nk, GFO_FLUID)) {
                        int64_t f = idx3(i, j, k, W, H);
                        g[f] = tmp[f];
                    }
        free(tmp);
    }
}

/* -------------------------------------------------- a13: tricubic sample */

/* Interpolation::cubicInterpolate (interpolation.cpp:44-46) */
static inline double cubic(const double p[4], double x) {
    return p[1] + 0.5 * x * (p[2] - p[0] + x * (2.0 * p[0] - 5.0 * p[1] + 4.0 * p[2] - p[3] +
                                                 x * (3.0 * (p[1] - p[2]) + p[3] - p[0])));
}

/* MACVelocityField::_interpolateU/V/W (macvelocityfield.cpp:350-450) */
static double interp_component(int dir, int ni, int nj, int nk, double dx, const float *g,
                               double x, double y, double z) {
    if (!(x >= 0 && y >= 0 && z >= 0 && x < dx * ni && y < dx * nj && z < dx * nk)) return 0.0;
    if (dir != 0) x -= 0.5 * dx;
    if (dir != 1) y -= 0.5 * dx;
    if (dir != 2) z -= 0.5 * dx;
    double invdx = 1.0 / dx;
    int i = (int)floor(x * invdx), j = (int)floor(y * invdx), k = (int)floor(z * invdx);
    double gx = (double)i * dx, gy = (double)j * dx, gz = (double)k * dx;
    double inv_dx = 1 / dx;
    double ix = (x - gx) * inv_dx, iy = (y - gy) * inv_dx, iz = (z - gz) * inv_dx;
    int W, H, D;
    face_dims(dir, ni, nj, nk, &W, &H, &D);
    double pts[4][4][4];
    for (int pk = 0; pk < 4; pk++)
        for (int pj = 0; pj < 4; pj++)
            for (int pi = 0; pi < 4; pi++) {
                int a = pi + i - 1, b = pj + j - 1, c = pk + k - 1;
                pts[pk][pj][pi] = in_range(a, b, c, W, H, D) ? (double)g[idx3(a, b, c, W, H)] : 0.0;
            }
    /* Interpolation::tricubicInterpolate / bicubicInterpolate (interpolation.cpp:26-42) */
    double arr[4];
    for (int pk = 0; pk < 4; pk++) {
        double row[4];
        for (int pj = 0; pj < 4; pj++) row[pj] = cubic(pts[pk][pj], ix);
        arr[pk] = cubic(row, iy);
    }
    return cubic(arr, iz);
}

static void eval_velocity(int ni, int nj, int nk, double dx, const float *u, const float *v,
                          const float *w, const float p[3], float out[3]) {
    double x = p[0], y = p[1], z = p[2];
    if (!(x >= 0 && y >= 0 && z >= 0 && x < dx * ni && y < dx * nj && z < dx * nk)) {
        out[0] = out[1] = out[2] = 0.0f;
        return;
    }
    out[0] = (float)interp_component(0, ni, nj, nk, dx, u, x, y, z);
    out[1] = (float)interp_component(1, ni, nj, nk, dx, v, x, y, z);
    out[2] = (float)interp_component(2, ni, nj, nk, dx, w, x, y, z);
}

void gfo_evaluate_velocity(int ni, int nj, int nk, double dx, const float *u,
                           const float *v, const float *w, const float *pos,
                           int64_t n, float *out) {
    for (int64_t p = 0; p < n; p++) eval_velocity(ni, nj, nk, dx, u, v, w, pos + 3 * p, out + 3 * p);
}

void gfo_flip_update(int ni, int nj, int nk, double dx, double ratio_pic,
                     const float *u_new, const float *v_new, const float *w_new,
                     const float *u_old, const float *v_old, const float *w_old,
                     const float *pos, int64_t n, float *vel) {
    float a = (float)ratio_pic, b = (float)(1 - ratio_pic);
    for (int64_t p = 0; p < n; p++) {
        float vn[3], vo[3];
        eval_velocity(ni, nj, nk, dx, u_new, v_new, w_new, pos + 3 * p, vn);
        eval_velocity(ni, nj, nk, dx, u_old, v_old, w_old, pos + 3 * p, vo);
        for (int c = 0; c < 3; c++) {
            float flip = vel[3 * p + c] + vn[c] - vo[c];
            vel[3 * p + c] = a * vn[c] + b * flip;
        }
    }
}

/* ------------------------------------------------------------ a14: RK4 */

void gfo_advect_rk4(int ni, int nj, int nk, double dx, const float *u, const float *v,
                    const float *w, double dt, const float *pos, int64_t n, float *out) {
    float h = (float)(0.5 * dt), f1 = (float)dt, f6 = (float)(dt / 6.0f);
    for (int64_t p = 0; p < n; p++) {
        const float *p0 = pos + 3 * p;
        float k1[3], k2[3], k3[3], k4[3], t[3];
        eval_velocity(ni, nj, nk, dx, u, v, w, p0, k1);
        for (int c = 0; c < 3; c++) t[c] = p0[c] + h * k1[c];
        eval_velocity(ni, nj, nk, dx, u, v, w, t, k2);
        for (int c = 0; c < 3; c++) t[c] = p0[c] + h * k2[c];
        eval_velocity(ni, nj, nk, dx, u, v, w, t, k3);
        for (int c = 0; c < 3; c++) t[c] = p0[c] + f1 * k3[c];
        eval_velocity(ni, nj, nk, dx, u, v, w, t, k4);
        for (int c = 0; c < 3; c++) {
            float sum = k1[c] + 2.0f * k2[c] + 2.0f * k3[c] + k4[c];
            out[3 * p + c] = p0[c] + f6 * sum;
        }
    }
}

/* ------------------------------------------------------- a15: collision */

/* Collision::getLineSegmentVoxelIntersection (collision.cpp:303-402) */
static int segment_voxel(const float p0in[3], const float p1in[3], double dx, const uint8_t *mat,
                         int ni, int nj, int nk, int vox[3]) {
    float s = (float)(1.0 / dx);
    float p0[3] = {p0in[0] * s, p0in[1] * s, p0in[2] * s};
    float p1[3] = {p1in[0] * s, p1in[1] * s, p1in[2] * s};
    int gx0 = (int)floor(p0[0]), gy0 = (int)floor(p0[1]), gz0 = (int)floor(p0[2]);
    int gx1 = (int)floor(p1[0]), gy1 = (int)floor(p1[1]), gz1 = (int)floor(p1[2]);
    int sx = gx1 > gx0 ? 1 : gx1 < gx0 ? -1 : 0;
    int sy = gy1 > gy0 ? 1 : gy1 < gy0 ? -1 : 0;
    int sz = gz1 > gz0 ? 1 : gz1 < gz0 ? -1 : 0;
    int gx = gx0, gy = gy0, gz = gz0;
    double gxp = gx0 + (gx1 > gx0 ? 1 : 0);
    double gyp = gy0 + (gy1 > gy0 ? 1 : 0);
    double gzp = gz0 + (gz1 > gz0 ? 1 : 0);
    double vx = p1[0] == p0[0] ? 1 : (double)(float)(p1[0] - p0[0]);
    double vy = p1[1] == p0[1] ? 1 : (double)(float)(p1[1] - p0[1]);
    double vz = p1[2] == p0[2] ? 1 : (double)(float)(p1[2] - p0[2]);
    double vxvy = vx * vy, vxvz = vx * vz, vyvz = vy * vz;
    double errx = (gxp - p0[0]) * vyvz;
    double erry = (gyp - p0[1]) * vxvz;
    double errz = (gzp - p0[2]) * vxvy;
    double derrx = sx * vyvz, derry = sy * vxvz, derrz = sz * vxvy;
    for (int iter = 0; iter < 1000000; iter++) {
        if (in_range(gx, gy, gz, ni, nj, nk) && mat[idx3(gx, gy, gz, ni, nj)] == GFO_SOLID) {
            vox[0] = gx; vox[1] = gy; vox[2] = gz;
            return 1;
        }
        if (gx == gx1 && gy == gy1 && gz == gz1) break;
        double xr = fabs(errx), yr = fabs(erry), zr = fabs(errz);
        if (sx != 0 && (sy == 0 || xr < yr) && (sz == 0 || xr < zr)) { gx += sx; errx += derrx; }
        else if (sy != 0 && (sz == 0 || yr < zr)) { gy += sy; erry += derry; }
        else if (sz != 0) { gz += sz; errz += derrz; }
    }
    return 0;
}

/* Collision::rayIntersectsAABB (collision.cpp:404-449), including its dir.x
   test guarding dir.z (:418-420). */
static int ray_aabb(const float p0[3], const float dirin[3], const float bmin[3],
                    const float bmax[3], float out[3]) {
    float dir[3] = {dirin[0], dirin[1], dirin[2]};
    double eps = 1e-10;
    if (fabs((double)dir[0]) < eps) dir[0] = dir[0] < 0 ? (float)-eps : (float)eps;
    if (fabs((double)dir[1]) < eps) dir[1] = dir[1] < 0 ? (float)-eps : (float)eps;
    if (fabs((double)dir[0]) < eps) dir[2] = dir[2] < 0 ? (float)-eps : (float)eps;
    float inv[3] = {(float)(1.0 / dir[0]), (float)(1.0 / dir[1]), (float)(1.0 / dir[2])};
    double t1 = (double)((bmin[0] - p0[0]) * inv[0]);
    double t2 = (double)((bmax[0] - p0[0]) * inv[0]);
    double tmin = fmin(t1, t2), tmax = fmax(t1, t2);
    t1 = (double)((bmin[1] - p0[1]) * inv[1]);
    t2 = (double)((bmax[1] - p0[1]) * inv[1]);
    tmin = fmax(tmin, fmin(t1, t2));
    tmax = fmin(tmax, fmax(t1, t2));
    t1 = (double)((bmin[2] - p0[2]) * inv[2]);
    t2 = (double)((bmax[2] - p0[2]) * inv[2]);
    tmin = fmax(tmin, fmin(t1, t2));
    tmax = fmin(tmax, fmax(t1, t2));
    if (tmax > fmax(tmin, 0.0)) {
        float ft = (float)tmin;
        for (int c = 0; c < 3; c++) out[c] = p0[c] + ft * dir[c];
        return 1;
    }
    return 0;
}

static void resolve_one(int ni, int nj, int nk, double dx, const uint8_t *mat,
                        const float p0[3], float p1[3]) {
    int vox[3];
    if (!segment_voxel(p0, p1, dx, mat, ni, nj, nk, vox)) { memcpy(p1, p0, 3 * sizeof(float)); return; }
    /* raynorm = vmath::normalize(p1 - p0) (vmath.h:89-92, operator/ vmath.cpp:90-93) */
    float d[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
    float len = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    float linv = (float)(1.0 / len);
    float rn[3] = {d[0] * linv, d[1] * linv, d[2] * linv};
    float bmin[3], bmax[3];
    for (int c = 0; c < 3; c++) {
        bmin[c] = (float)((double)(float)vox[c] * dx);
        bmax[c] = bmin[c] + (float)dx;
    }
    float cp[3];
    if (!ray_aabb(p0, rn, bmin, bmax, cp)) { memcpy(p1, p0, 3 * sizeof(float)); return; }
    float back = (float)(0.05 * dx);
    float res[3] = {cp[0] - back * rn[0], cp[1] - back * rn[1], cp[2] - back * rn[2]};
    int ri, rj, rk;
    pos_to_cell(res, dx, &ri, &rj, &rk);
    if (mat_at(mat, ri, rj, rk, ni, nj, nk) == GFO_SOLID) { memcpy(p1, p0, 3 * sizeof(float)); return; }
    memcpy(p1, res, 3 * sizeof(float));
}

int gfo_segment_voxel(const float *p0, const float *p1, double dx, int ni, int nj, int nk,
                      const uint8_t *mat, int *voxel) {
    return segment_voxel(p0, p1, dx, mat, ni, nj, nk, voxel);
}

int gfo_ray_aabb(const float *p0, const float *dir, const float *bmin, const float *bmax, float *out) {
    return ray_aabb(p0, dir, bmin, bmax, out);
}

void gfo_resolve_collisions(int ni, int nj, int nk, double dx, const uint8_t *mat,
                            const float *p0, int64_t n, float *p1) {
    for (int64_t p = 0; p < n; p++) {
        int i, j, k;
        pos_to_cell(p1 + 3 * p, dx, &i, &j, &k);
        if (mat_at(mat, i, j, k, ni, nj, nk) == GFO_SOLID)
            resolve_one(ni, nj, nk, dx, mat, p0 + 3 * p, p1 + 3 * p);
    }
}

/* --------------------------------------------------- a1 / a16: particles */

int64_t gfo_update_fluid_cells(int ni, int nj, int nk, double dx, uint8_t *mat,
                               float *pos, float *vel, uint32_t *ids, int64_t n) {
    /* _removeMarkerParticlesInSolidCells (fluidsimulation.cpp:1933-1958) */
    int64_t m = 0;
    for (int64_t p = 0; p < n; p++) {
        int i, j, k;
        pos_to_cell(pos + 3 * p, dx, &i, &j, &k);
        if (mat_at(mat, i, j, k, ni, nj, nk) == GFO_SOLID) continue;
        if (m != p) {
            memmove(pos + 3 * m, pos + 3 * p, 3 * sizeof(float));
            memmove(vel + 3 * m, vel + 3 * p, 3 * sizeof(float));
            ids[m] = ids[p];
        }
        m++;
    }
    /* interior fluid -> air (fluidsimulation.cpp:1998-2006) */
    for (int k = 1; k < nk - 1; k++)
        for (int j = 1; j < nj - 1; j++)
            for (int i = 1; i < ni - 1; i++)
                if (mat[idx3(i, j, k, ni, nj)] == GFO_FLUID) mat[idx3(i, j, k, ni, nj)] = GFO_AIR;
    /* particles mark their cell fluid (:2010-2016) */
    for (int64_t p = 0; p < m; p++) {
        int i, j, k;
        pos_to_cell(pos + 3 * p, dx, &i, &j, &k);
        if (in_range(i, j, k, ni, nj, nk)) mat[idx3(i, j, k, ni, nj)] = GFO_FLUID;
    }
    return m;
}

static int cmp_u64(const void *a, const void *b) {
    uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return (x > y) - (x < y);
}

int64_t gfo_cap_particles_per_cell(int ni, int nj, int nk, double dx, int max_per_cell,
                                   float *pos, float *vel, uint32_t *ids, int64_t n) {
    if (n == 0) return 0;
    /* keep the max_per_cell smallest ids of every cell */
    uint64_t *keys = (uint64_t *)malloc((size_t)n * sizeof(uint64_t));
    for (int64_t p = 0; p < n; p++) {
        int i, j, k;
        pos_to_cell(pos + 3 * p, dx, &i, &j, &k);
        uint64_t cell = in_range(i, j, k, ni, nj, nk) ? (uint64_t)idx3(i, j, k, ni, nj) : 0xFFFFFFFFull;
        keys[p] = (cell << 32) | ids[p];
    }
    qsort(keys, (size_t)n, sizeof(uint64_t), cmp_u64);
    /* ids are unique: mark removed ids through a sorted id list */
    uint64_t *removed = (uint64_t *)malloc((size_t)n * sizeof(uint64_t));
    int64_t nr = 0, run = 0;
    for (int64_t q = 0; q < n; q++) {
        if (q > 0 && (keys[q] >> 32) == (keys[q - 1] >> 32)) run++;
        else run = 0;
        if ((keys[q] >> 32) != 0xFFFFFFFFull && run >= max_per_cell) removed[nr++] = keys[q] & 0xFFFFFFFFull;
    }
    qsort(removed, (size_t)nr, sizeof(uint64_t), cmp_u64);
    int64_t m = 0;
    for (int64_t p = 0; p < n; p++) {
        uint64_t id = ids[p];
        int gone = 0;
        if (nr > 0) {
            int64_t lo = 0, hi = nr - 1;
            while (lo <= hi) {
                int64_t mid = (lo + hi) / 2;
                if (removed[mid] == id) { gone = 1; break; }
                if (removed[mid] < id) lo = mid + 1; else hi = mid - 1;
            }
        }
        if (gone) continue;
        if (m != p) {
            memmove(pos + 3 * m, pos + 3 * p, 3 * sizeof(float));
            memmove(vel + 3 * m, vel + 3 * p, 3 * sizeof(float));
            ids[m] = ids[p];
        }
        m++;
    }
    free(keys);
    free(removed);
    return m;
}

/* ------------------------------------------------------------- substep */

int64_t gfo_substep(int ni, int nj, int nk, double dx, double dt, const float g[3],
                    double density, double ratio_pic, int num_layers, int max_per_cell,
                    uint8_t *mat, float *pos, float *vel, uint32_t *ids, int64_t n,
                    float *u, float *v, float *w, float *pressure_grid,
                    gfo_substep_stats *stats) {
    int64_t ncell = (int64_t)ni * nj * nk;
    int64_t nu = (int64_t)(ni + 1) * nj * nk, nv = (int64_t)ni * (nj + 1) * nk, nw = (int64_t)ni * nj * (nk + 1);

    /* 1. _updateFluidCells */
    n = gfo_update_fluid_cells(ni, nj, nk, dx, mat, pos, vel, ids, n);
    int64_t F = 0;
    for (int64_t c = 0; c < ncell; c++) F += (mat[c] == GFO_FLUID);

    /* 5. _advectVelocityField, saved = MAC, extrapolate(saved) */
    gfo_advect_velocity_field(ni, nj, nk, dx, mat, pos, vel, n, u, v, w);
    float *su = (float *)malloc((size_t)nu * sizeof(float));
    float *sv = (float *)malloc((size_t)nv * sizeof(float));
    float *sw = (float *)malloc((size_t)nw * sizeof(float));
    memcpy(su, u, (size_t)nu * sizeof(float));
    memcpy(sv, v, (size_t)nv * sizeof(float));
    memcpy(sw, w, (size_t)nw * sizeof(float));
    gfo_extrapolate(ni, nj, nk, mat, num_layers, su, sv, sw);

    /* 6. body forces */
    gfo_body_force(ni, nj, nk, mat, g, dt, u, v, w);

    /* 7. pressure */
    double *pres = (double *)malloc((size_t)(F > 0 ? F : 1) * sizeof(double));
    int iters = -1;
    double resid = 0.0;
    gfo_pressure_solve(ni, nj, nk, dx, density, dt, mat, u, v, w, 1e-6, 200, pres, &iters, &resid);
    float *pgrid = pressure_grid ? pressure_grid : (float *)malloc((size_t)ncell * sizeof(float));
    gfo_pressure_to_grid(ni, nj, nk, mat, pres, pgrid);

    /* 8. apply pressure */
    gfo_apply_pressure(ni, nj, nk, dx, density, dt, mat, pgrid, u, v, w);

    /* 9. extrapolate MAC */
    gfo_extrapolate(ni, nj, nk, mat, num_layers, u, v, w);

    /* 11. PIC/FLIP */
    gfo_flip_update(ni, nj, nk, dx, ratio_pic, u, v, w, su, sv, sw, pos, n, vel);

    /* 12. advance + collisions + per-cell cap */
    float *p1 = (float *)malloc((size_t)(n > 0 ? n : 1) * 3 * sizeof(float));
    gfo_advect_rk4(ni, nj, nk, dx, u, v, w, dt, pos, n, p1);
    gfo_resolve_collisions(ni, nj, nk, dx, mat, pos, n, p1);
    memcpy(pos, p1, (size_t)n * 3 * sizeof(float));
    n = gfo_cap_particles_per_cell(ni, nj, nk, dx, max_per_cell, pos, vel, ids, n);

    if (stats) {
        stats->num_fluid_cells = F;
        stats->num_particles = n;
        stats->cg_iterations = iters;
        stats->cg_max_resid = resid;
    }
    free(p1); free(pres); free(su); free(sv); free(sw);
    if (!pressure_grid) free(pgrid);
    return n;
}

/* max|b - A p| in double for a compact pressure vector p (lexicographic fluid
   order): the reference's b (pressuresolver.cpp:162-208) and stencil (:388-426). */
double gfo_pressure_residual(int ni, int nj, int nk, double dx, double density, double dt,
                             const uint8_t *mat, const float *u, const float *v, const float *w,
                             const double *p) {
    gfo_ps s;
    memset(&s, 0, sizeof(s));
    s.ni = ni; s.nj = nj; s.nk = nk;
    int64_t ncell = (int64_t)ni * nj * nk, F = 0;
    for (int64_t c = 0; c < ncell; c++) F += (mat[c] == GFO_FLUID);
    if (F == 0) return 0.0;
    s.F = F;
    s.cells = (int32_t *)malloc((size_t)F * sizeof(int32_t));
    s.keymap = (int32_t *)malloc((size_t)ncell * sizeof(int32_t));
    for (int64_t c = 0, r = 0; c < ncell; c++) {
        s.keymap[c] = -1;
        if (mat[c] == GFO_FLUID) { s.cells[r] = (int32_t)c; s.keymap[c] = (int32_t)r; r++; }
    }
    double *b = (double *)malloc((size_t)F * sizeof(double));
    double *Ap = (double *)malloc((size_t)F * sizeof(double));
    s.diag = (uint8_t *)calloc((size_t)F, 1);
    int UW = ni + 1, VH = nj + 1;
    #define U_(i, j, k) (in_range(i, j, k, ni + 1, nj, nk) ? u[idx3(i, j, k, UW, nj)] : 0.0f)
    #define V_(i, j, k) (in_range(i, j, k, ni, nj + 1, nk) ? v[idx3(i, j, k, ni, VH)] : 0.0f)
    #define W_(i, j, k) (in_range(i, j, k, ni, nj, nk + 1) ? w[idx3(i, j, k, ni, nj)] : 0.0f)
    #define SOLID_(i, j, k) (mat_at(mat, i, j, k, ni, nj, nk) == GFO_SOLID)
    double scale_div = 1.0f / (float)dx;
    float fscale = (float)scale_div;
    for (int64_t idx = 0; idx < F; idx++) {
        int32_t c = s.cells[idx];
        int i = c % ni, j = (c / ni) % nj, k = c / (ni * nj);
        float div = U_(i + 1, j, k) - U_(i, j, k) + V_(i, j + 1, k) - V_(i, j, k) +
                    W_(i, j, k + 1) - W_(i, j, k);
        double bv = -scale_div * (double)div;
        if (SOLID_(i - 1, j, k)) bv -= fscale * U_(i, j, k);
        if (SOLID_(i + 1, j, k)) bv += fscale * U_(i + 1, j, k);
        if (SOLID_(i, j - 1, k)) bv -= fscale * V_(i, j, k);
        if (SOLID_(i, j + 1, k)) bv += fscale * V_(i, j + 1, k);
        if (SOLID_(i, j, k - 1)) bv -= fscale * W_(i, j, k);
        if (SOLID_(i, j, k + 1)) bv += fscale * W_(i, j, k + 1);
        b[idx] = bv;
        int nn = 0;
        if (!SOLID_(i - 1, j, k)) nn++;
        if (!SOLID_(i + 1, j, k)) nn++;
        if (!SOLID_(i, j - 1, k)) nn++;
        if (!SOLID_(i, j + 1, k)) nn++;
        if (!SOLID_(i, j, k - 1)) nn++;
        if (!SOLID_(i, j, k + 1)) nn++;
        s.diag[idx] = (uint8_t)nn;
    }
    #undef U_
    #undef V_
    #undef W_
    #undef SOLID_
    s.scale = dt / (density * dx * dx);
    s.negscale = -s.scale;
    ps_apply_matrix(&s, p, Ap);
    double m = 0.0;
    for (int64_t i = 0; i < F; i++) { double r = fabs(b[i] - Ap[i]); if (r > m) m = r; }
    free(b); free(Ap); free(s.diag); free(s.cells); free(s.keymap);
    return m;
}
