// extrapolate.cu -- MACVelocityField::extrapolateVelocityField
// (macvelocityfield.cpp:560-797) on the device.
//
// Layers: the reference grows layer L from layer L-1 with a lexicographic sweep
// (_updateExtrapolationLayer, :560-585) whose writes never feed the same sweep
// (it looks for L-1 and writes L), so the gather form here -- a cell becomes L
// when it is non-solid, still unlabelled and has a 6-neighbour at L-1 -- gives
// the same labels.  Layer 0 is the fluid cells.
//
// Faces: layer pass L writes the faces that border layer L, not layer L-1 and
// not a solid cell, with the mean of their face-neighbours that border L-1
// (_extrapolateVelocitiesForLayerIndexU/V/W :665-718,
// _getExtrapolatedVelocityForFaceU/V/W :602-663).  Those neighbours are never
// written in the same pass, so one kernel per layer needs no ordering.
// The layer grid depends only on the material grid, so one substep builds it
// once and uses it for both extrapolations (saved field and MAC field).
#include "gfs_internal.h"

namespace gfs {

__global__ void k_layer_init(int8_t *__restrict__ layer, const uint8_t *__restrict__ mat, GridDim c) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y, k = blockIdx.z;
    if (i >= c.nx) return;
    long long at = c.at(i, j, k);
    layer[at] = mat[at] == GFS_FLUID ? 0 : -1;
}

__global__ void k_layer_grow(int8_t *__restrict__ layer, const uint8_t *__restrict__ mat, GridDim c, int L) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y, k = blockIdx.z;
    if (i >= c.nx) return;
    long long at = c.at(i, j, k);
    if (layer[at] != -1 || mat[at] == GFS_SOLID) return;
    // the halo holds -1, so out-of-range neighbours never match L-1
    long long sx = 1, sy = c.sx, sz = (long long)c.sx * c.sy;
    int8_t want = (int8_t)(L - 1);
    if (layer[at - sx] == want || layer[at + sx] == want || layer[at - sy] == want ||
        layer[at + sy] == want || layer[at - sz] == want || layer[at + sz] == want)
        layer[at] = (int8_t)L;
}

int build_layers(Sim *s, int num_layers) {
    Ctx *ctx = s->ctx;
    ProfScope prof(ctx, KC_LAYERS);
    const GridDim &c = s->g.c;
    dim3 grid(grid_blocks(c.nx, 128), c.ny, c.nz);
    k_layer_init<<<grid, 128, 0, ctx->stream>>>(s->layer.as<int8_t>(), s->mat.as<uint8_t>(), c);
    ctx->launches++;
    for (int L = 1; L <= num_layers; L++) {
        k_layer_grow<<<grid, 128, 0, ctx->stream>>>(s->layer.as<int8_t>(), s->mat.as<uint8_t>(), c, L);
        ctx->launches++;
    }
    GFS_LAUNCH_CHECK();
    return GFS_OK;
}

// MACVelocityField::_isFaceBorderingGridValueU/V/W (macvelocityfield.h:159-173)
__device__ __forceinline__ bool face_borders_layer(const int8_t *__restrict__ layer, const GridDim &c,
                                                   int d, int i, int j, int k, int value) {
    int n = d == 0 ? c.nx : (d == 1 ? c.ny : c.nz);
    int t = d == 0 ? i : (d == 1 ? j : k);
    int pi = i - (d == 0), pj = j - (d == 1), pk = k - (d == 2);
    if (t == n) return layer[c.at(pi, pj, pk)] == value;
    if (t > 0) return layer[c.at(i, j, k)] == value || layer[c.at(pi, pj, pk)] == value;
    return layer[c.at(i, j, k)] == value;
}

struct ExtrapArgs {
    GridDim c, f[3];
    int L;
};

__global__ void __launch_bounds__(128) k_extrap_reset(GridDim c, GridDim fu, GridDim fv, GridDim fw,
                                                      const uint8_t *__restrict__ mat, float *__restrict__ u,
                                                      float *__restrict__ v, float *__restrict__ w) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i > c.nx || j > c.ny || k > c.nz) return;
    // _resetExtrapolatedFluidVelocities (macvelocityfield.cpp:720-752)
    if (fu.in(i, j, k) && !face_borders(mat, c, 0, i, j, k, GFS_FLUID)) u[fu.at(i, j, k)] = 0.0f;
    if (fv.in(i, j, k) && !face_borders(mat, c, 1, i, j, k, GFS_FLUID)) v[fv.at(i, j, k)] = 0.0f;
    if (fw.in(i, j, k) && !face_borders(mat, c, 2, i, j, k, GFS_FLUID)) w[fw.at(i, j, k)] = 0.0f;
}

__global__ void __launch_bounds__(128) k_extrap_layer(ExtrapArgs A, const uint8_t *__restrict__ mat,
                                                      const int8_t *__restrict__ layer, float *__restrict__ u,
                                                      float *__restrict__ v, float *__restrict__ w) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    int k = blockIdx.z * blockDim.z + threadIdx.z;
    const GridDim &c = A.c;
    if (i > c.nx || j > c.ny || k > c.nz) return;
    float *g[3] = {u, v, w};
    const int L = A.L;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const GridDim &f = A.f[d];
        if (!f.in(i, j, k)) continue;
        bool ext = face_borders_layer(layer, c, d, i, j, k, L) &&
                   !face_borders_layer(layer, c, d, i, j, k, L - 1) &&
                   !face_borders(mat, c, d, i, j, k, GFS_SOLID);
        if (!ext) continue;
        const int nb[6][3] = {{i - 1, j, k}, {i + 1, j, k}, {i, j - 1, k},
                              {i, j + 1, k}, {i, j, k - 1}, {i, j, k + 1}};
        double sum = 0.0, wsum = 0.0;
#pragma unroll
        for (int q = 0; q < 6; q++) {
            int a = nb[q][0], b = nb[q][1], e = nb[q][2];
            if (f.in(a, b, e) && face_borders_layer(layer, c, d, a, b, e, L - 1)) {
                sum += (double)g[d][f.at(a, b, e)];
                wsum += 1.0;
            }
        }
        g[d][f.at(i, j, k)] = (sum == 0.0) ? 0.0f : (float)(sum / wsum);
    }
}

int extrapolate_field(Sim *s, float *const fld[3], int num_layers, bool reset) {
    Ctx *ctx = s->ctx;
    ProfScope prof(ctx, KC_EXTRAP);
    const GridDim &c = s->g.c;
    dim3 block(32, 2, 2);
    dim3 grid(grid_blocks(c.nx + 1, 32), grid_blocks(c.ny + 1, 2), grid_blocks(c.nz + 1, 2));
    if (reset) {
        k_extrap_reset<<<grid, block, 0, ctx->stream>>>(c, s->g.f[0], s->g.f[1], s->g.f[2],
                                                        s->mat.as<uint8_t>(), fld[0], fld[1], fld[2]);
        ctx->launches++;
    }
    ExtrapArgs A;
    A.c = c;
    for (int d = 0; d < 3; d++) A.f[d] = s->g.f[d];
    for (int L = 1; L <= num_layers; L++) {
        A.L = L;
        k_extrap_layer<<<grid, block, 0, ctx->stream>>>(A, s->mat.as<uint8_t>(), s->layer.as<int8_t>(),
                                                        fld[0], fld[1], fld[2]);
        ctx->launches++;
    }
    GFS_LAUNCH_CHECK();
    return GFS_OK;
}

}  // namespace gfs
