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

// Also lists the cells of layer L (their storage indices) for the face passes:
// layer L's list starts after those of layers 1..L-1 (lcnt[l]: count of layer l),
// one atomic per warp; the order within a list does not matter (a face pass reads
// only faces of the layer before).
__global__ void k_layer_grow(int8_t *__restrict__ layer, const uint8_t *__restrict__ mat, GridDim c, int L,
                             uint32_t *__restrict__ lcells, uint32_t *__restrict__ lcnt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y, k = blockIdx.z;
    bool grow = false;
    long long at = 0;
    if (i < c.nx) {
        at = c.at(i, j, k);
        if (layer[at] == -1 && mat[at] != GFS_SOLID) {
            // the halo holds -1, so out-of-range neighbours never match L-1
            long long sx = 1, sy = c.sx, sz = (long long)c.sx * c.sy;
            int8_t want = (int8_t)(L - 1);
            grow = layer[at - sx] == want || layer[at + sx] == want || layer[at - sy] == want ||
                   layer[at + sy] == want || layer[at - sz] == want || layer[at + sz] == want;
        }
    }
    const unsigned m = __ballot_sync(0xffffffffu, grow);
    if (!m) return;
    const int lane = threadIdx.x & 31;
    uint32_t first = 0;
    if (lane == __ffs(m) - 1) {
        uint32_t base = 0;
        for (int l = 1; l < L; l++) base += lcnt[l];
        first = base + atomicAdd(&lcnt[L], (uint32_t)__popc(m));
    }
    first = __shfl_sync(0xffffffffu, first, __ffs(m) - 1);
    if (grow) {
        layer[at] = (int8_t)L;
        lcells[first + __popc(m & ((1u << lane) - 1u))] = (uint32_t)at;
    }
}

int build_layers(Sim *s, int num_layers) {
    Ctx *ctx = s->ctx;
    ProfScope prof(ctx, KC_LAYERS);
    const GridDim &c = s->g.c;
    if (num_layers > GFS_MAX_LAYERS) {
        set_error(GFS_ERR_INVALID, "%d extrapolation layers exceed the supported %d", num_layers, GFS_MAX_LAYERS);
        return GFS_ERR_INVALID;
    }
    dim3 grid(grid_blocks(c.nx, 128), c.ny, c.nz);
    GFS_CUDA_CHECK(cudaMemsetAsync(s->lcnt.p, 0, s->lcnt.bytes, ctx->stream));
    k_layer_init<<<grid, 128, 0, ctx->stream>>>(s->layer.as<int8_t>(), s->mat.as<uint8_t>(), c);
    ctx->launches++;
    for (int L = 1; L <= num_layers; L++) {
        k_layer_grow<<<grid, 128, 0, ctx->stream>>>(s->layer.as<int8_t>(), s->mat.as<uint8_t>(), c, L,
                                                    s->lcells.as<uint32_t>(), s->lcnt.as<uint32_t>());
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

// Face (d; i, j, k) of layer pass L, if it borders layer L, not layer L-1 and not a
// solid cell: the mean of its face-neighbours that border layer L-1.
__device__ __forceinline__ void extrap_face(const ExtrapArgs &A, const uint8_t *__restrict__ mat,
                                            const int8_t *__restrict__ layer, float *__restrict__ g, int d, int i,
                                            int j, int k) {
    const GridDim &c = A.c, &f = A.f[d];
    const int L = A.L;
    if (!f.in(i, j, k)) return;
    if (!(face_borders_layer(layer, c, d, i, j, k, L) && !face_borders_layer(layer, c, d, i, j, k, L - 1) &&
          !face_borders(mat, c, d, i, j, k, GFS_SOLID)))
        return;
    const int nb[6][3] = {{i - 1, j, k}, {i + 1, j, k}, {i, j - 1, k}, {i, j + 1, k}, {i, j, k - 1}, {i, j, k + 1}};
    double sum = 0.0, wsum = 0.0;
#pragma unroll
    for (int q = 0; q < 6; q++) {
        int a = nb[q][0], b = nb[q][1], e = nb[q][2];
        if (f.in(a, b, e) && face_borders_layer(layer, c, d, a, b, e, L - 1)) {
            sum += (double)g[f.at(a, b, e)];
            wsum += 1.0;
        }
    }
    g[f.at(i, j, k)] = (sum == 0.0) ? 0.0f : (float)(sum / wsum);
}

// Layer pass L over the cells of layer L: a face bordering layer L borders one or two
// of them; the upper cell of the two does it (each cell its three lower faces, and an
// upper face only when the cell above it is not in layer L), so every face is written
// once.  The faces it reads border layer L-1 and were written by earlier passes.
__global__ void __launch_bounds__(128) k_extrap_list(ExtrapArgs A, const uint8_t *__restrict__ mat,
                                                     const int8_t *__restrict__ layer,
                                                     const uint32_t *__restrict__ lcells,
                                                     const uint32_t *__restrict__ lcnt, float *__restrict__ u,
                                                     float *__restrict__ v, float *__restrict__ w) {
    const GridDim &c = A.c;
    const int L = A.L;
    uint32_t base = 0;
    for (int l = 1; l < L; l++) base += lcnt[l];
    const uint32_t n = lcnt[L];
    float *g[3] = {u, v, w};
    const long long sx = 1, sy = c.sx, sz = (long long)c.sx * c.sy;
    const long long st[3] = {sx, sy, sz};
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const long long at = lcells[base + e];
        const int i = (int)(at % c.sx) - GFS_PAD;
        const int j = (int)((at / c.sx) % c.sy) - GFS_PAD;
        const int k = (int)(at / ((long long)c.sx * c.sy)) - GFS_PAD;
#pragma unroll
        for (int d = 0; d < 3; d++) {
            extrap_face(A, mat, layer, g[d], d, i, j, k);
            // the face above: this cell's unless the cell above is in layer L too (the halo holds -1)
            if (layer[at + st[d]] != (int8_t)L) extrap_face(A, mat, layer, g[d], d, i + (d == 0), j + (d == 1), k + (d == 2));
        }
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
    const unsigned nb = (unsigned)ctx->num_sms * 8;
    for (int L = 1; L <= num_layers; L++) {
        A.L = L;
        k_extrap_list<<<nb, 128, 0, ctx->stream>>>(A, s->mat.as<uint8_t>(), s->layer.as<int8_t>(),
                                                   s->lcells.as<uint32_t>(), s->lcnt.as<uint32_t>(), fld[0], fld[1],
                                                   fld[2]);
        ctx->launches++;
    }
    GFS_LAUNCH_CHECK();
    return GFS_OK;
}

}  // namespace gfs
