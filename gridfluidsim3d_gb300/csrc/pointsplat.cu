// pointsplat.cu -- general weighted point splat onto a node grid:
// CLScalarField::addPoints / addPointValues (clscalarfield.cpp:68-300) with the
// arithmetic of ScalarField::addPoint / addPointValue (scalarfield.cpp:121-201).
//
// For every point p with value v (1 for addPoints) and every node (i,j,k) at
// (i,j,k)*dx that lies inside the reference's index bounds of p - offset
// (Grid3d::getGridIndexBounds, grid3d.h:350-371) and strictly within `radius`,
//     field(i,j,k) += w * v,   weight(i,j,k) += w,
//     w = 1 - 4/9 s^3 + 17/9 s^2 - 22/9 s,  s = |node - (p - offset)|^2 / radius^2.
//
// Design (deterministic, no atomics on the field):
//   1. k_pt_prepare computes each point's exact reference bounds [lo, hi] (the
//      same double/float steps as the reference) and keys the point by its
//      lower corner lo; points whose bounds are empty reach no node and drop out.
//   2. A counting sort by key (count, exclusive scan, scatter) followed by an
//      insertion sort by point index inside each key puts the points in a fixed
//      order; k_pt_permute copies them into that order (contiguous runs).
//   3. k_pt_gather: one thread per node scans the keys lo in
//      [node - span, node] (span = the largest hi - lo of any point) and, for
//      every point there with node <= hi, forms the exact float distance and
//      the weight.  The (point, node) pairs are therefore exactly the pairs the
//      reference's triple loop visits; each node sums in (key, index) order.
//
// Max-value threshold (CLScalarField::setMaxScalarFieldValueThreshold,
// clscalarfield.cpp:303-318): the reference's OpenCL path skips whole work
// chunks whose minimum field value is already at or above the threshold,
// re-evaluated between batches of chunks (:992-1013), so which contributions
// it drops depends on its chunking.  Here a node whose value before the call
// exceeds the threshold receives nothing (ScalarField's per-node test,
// scalarfield.cpp:141-143, applied to the incoming field), which is
// independent of any work partition.
#include "gfs_internal.h"

namespace gfs {

struct PtArgs {
    float off[3];
    double dx, inv, r;
    int W, H, D;
};

// ScalarField::addPointValue's bounds for one point (p already minus offset).
// Returns false if the point reaches no node of the grid.
__device__ __forceinline__ bool pt_bounds(const PtArgs &A, const float p[3], int lo[3], int hi[3]) {
    const int n[3] = {A.W, A.H, A.D};
#pragma unroll
    for (int d = 0; d < 3; d++) {
        // Grid3d::positionToGridIndex (grid3d.h:58-63): floor(p * (1/dx)) in double
        double x = (double)p[d] * A.inv;
        if (!(x > -1e9 && x < 1e9)) return false;   // non-finite or far outside: reaches no node
        int c = (int)floor(x);
        // cpos = GridIndexToPosition (float), trans = p - cpos (float)
        float cpos = (float)((double)(float)c * A.dx);
        float trans = __fsub_rn(p[d], cpos);
        int gmin = c - (int)fmax(0.0, ceil((A.r - (double)trans) * A.inv));
        int gmax = c + (int)fmax(0.0, ceil((A.r - A.dx + (double)trans) * A.inv));
        lo[d] = max(gmin, 0);
        hi[d] = min(gmax, n[d] - 1);
        if (lo[d] > hi[d]) return false;
    }
    return true;
}

__global__ void k_pt_prepare(PtArgs A, const float *__restrict__ pts, const float *__restrict__ vals, long long n,
                             float4 *__restrict__ pq, int4 *__restrict__ phi, uint32_t *__restrict__ key,
                             uint32_t *__restrict__ count, int *__restrict__ span) {
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    // p -= _gridOffset (vmath::vec3, float)
    float p[3] = {__fsub_rn(pts[3 * q], A.off[0]), __fsub_rn(pts[3 * q + 1], A.off[1]),
                  __fsub_rn(pts[3 * q + 2], A.off[2])};
    int lo[3], hi[3];
    if (!pt_bounds(A, p, lo, hi)) {
        key[q] = 0xFFFFFFFFu;
        return;
    }
    uint32_t k = (uint32_t)lo[0] + (uint32_t)A.W * ((uint32_t)lo[1] + (uint32_t)A.H * (uint32_t)lo[2]);
    key[q] = k;
    pq[q] = make_float4(p[0], p[1], p[2], vals ? vals[q] : 1.0f);
    phi[q] = make_int4(hi[0], hi[1], hi[2], 0);
    atomicAdd(count + k, 1u);
    atomicMax(span + 0, hi[0] - lo[0]);
    atomicMax(span + 1, hi[1] - lo[1]);
    atomicMax(span + 2, hi[2] - lo[2]);
}

__global__ void k_pt_scatter(const uint32_t *__restrict__ key, long long n, const uint32_t *__restrict__ offset,
                             uint32_t *__restrict__ cursor, uint32_t *__restrict__ perm) {
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    uint32_t k = key[q];
    if (k == 0xFFFFFFFFu) return;
    uint32_t slot = offset[k] + atomicAdd(cursor + k, 1u);
    perm[slot] = (uint32_t)q;
}

// Points of one key in increasing index order (the scatter's atomics leave them unordered).
__global__ void k_pt_sort_keys(const uint32_t *__restrict__ offset, long long nkeys, uint32_t *__restrict__ perm) {
    long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nkeys) return;
    uint32_t s = offset[b], e = offset[b + 1];
    for (uint32_t x = s + 1; x < e; x++) {
        uint32_t v = perm[x];
        uint32_t y = x;
        while (y > s && perm[y - 1] > v) {
            perm[y] = perm[y - 1];
            y--;
        }
        perm[y] = v;
    }
}

__global__ void k_pt_permute(const uint32_t *__restrict__ perm, uint32_t m, const float4 *__restrict__ pq,
                             const int4 *__restrict__ phi, float4 *__restrict__ spq, int4 *__restrict__ sphi) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= m) return;
    uint32_t q = perm[t];
    spq[t] = pq[q];
    sphi[t] = phi[q];
}

struct GatherArgs {
    double dx;
    float r2_thresh;   // (double)d2 < r*r  <=>  d2 < r2_thresh
    float inv_r2;
    int W, H, D;
    int span[3];
    int thr_set;
    float thr;
};

__global__ void __launch_bounds__(128) k_pt_gather(GatherArgs A, const uint32_t *__restrict__ offset,
                                                   const float4 *__restrict__ spq, const int4 *__restrict__ sphi,
                                                   float *__restrict__ field, float *__restrict__ weight) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= A.W || j >= A.H || k >= A.D) return;
    long long node = (long long)i + (long long)A.W * ((long long)j + (long long)A.H * k);
    const float before = field[node];
    if (A.thr_set && before > A.thr) return;
    // Grid3d::GridIndexToPosition (grid3d.h:79-81), float
    const float gx = (float)((double)(float)i * A.dx);
    const float gy = (float)((double)(float)j * A.dx);
    const float gz = (float)((double)(float)k * A.dx);
    float sf = 0.f, sw = 0.f;
    int hits = 0;
    const int i0 = max(i - A.span[0], 0), j0 = max(j - A.span[1], 0), k0 = max(k - A.span[2], 0);
    for (int kb = k0; kb <= k; kb++) {
        for (int jb = j0; jb <= j; jb++) {
            long long row = (long long)A.W * ((long long)jb + (long long)A.H * kb);
            uint32_t b = __ldg(offset + row + i0), e = __ldg(offset + row + i + 1);
            for (uint32_t q = b; q < e; q++) {
                int4 h = __ldg(sphi + q);
                if (i > h.x || j > h.y || k > h.z) continue;
                float4 p = __ldg(spq + q);
                // vmath::dot of gpos - p (float, left to right, no FMA)
                float ax = __fsub_rn(gx, p.x), ay = __fsub_rn(gy, p.y), az = __fsub_rn(gz, p.z);
                float d2 = __fadd_rn(__fadd_rn(__fmul_rn(ax, ax), __fmul_rn(ay, ay)), __fmul_rn(az, az));
                if (!(d2 < A.r2_thresh)) continue;
                // _evaluateTricubicFieldFunctionForRadiusSquared, factored: (1-s)^2 (1 - 4s/9)
                float s = d2 * A.inv_r2;
                float a = 1.0f - s;
                float w = a * a * (1.0f - (4.0f / 9.0f) * s);
                sf += w * p.w;
                sw += w;
                hits++;
            }
        }
    }
    if (hits == 0) return;
    field[node] = before + sf;
    if (weight) weight[node] += sw;
}

static float ceil_to_float(double x) {
    float f = (float)x;
    if ((double)f < x) f = nextafterf(f, INFINITY);
    return f;
}

int splat_points(Ctx *ctx, const float *d_pts, const float *d_vals, long long n, double radius,
                 const float offset[3], double dx, int W, int H, int D, float *d_field, float *d_weight,
                 bool thr_set, float thr) {
    if (n == 0) return GFS_OK;
    cudaStream_t st = ctx->stream;
    const long long nkeys = (long long)W * H * D;
    DevMem pq, phi, key, count, offs, perm, spq, sphi, tmp, span;
    if (pq.alloc((size_t)n * sizeof(float4)) || phi.alloc((size_t)n * sizeof(int4)) ||
        key.alloc((size_t)n * sizeof(uint32_t)) || count.alloc((size_t)(nkeys + 1) * sizeof(uint32_t)) ||
        offs.alloc((size_t)(nkeys + 1) * sizeof(uint32_t)) || perm.alloc((size_t)n * sizeof(uint32_t)) ||
        tmp.alloc(scan_temp_elems(nkeys + 1) * sizeof(uint32_t)) || span.alloc(4 * sizeof(int)))
        return GFS_ERR_NOMEM;
    PtArgs P;
    for (int d = 0; d < 3; d++) P.off[d] = offset[d];
    P.dx = dx;
    P.inv = 1.0 / dx;
    P.r = radius;
    P.W = W; P.H = H; P.D = D;
    GFS_CUDA_CHECK(cudaMemsetAsync(count.p, 0, count.bytes, st));
    GFS_CUDA_CHECK(cudaMemsetAsync(span.p, 0, span.bytes, st));
    const int T = 256;
    {
        ProfScope prof(ctx, KC_SORT);
        k_pt_prepare<<<grid_blocks(n, T), T, 0, st>>>(P, d_pts, d_vals, n, pq.as<float4>(), phi.as<int4>(),
                                                      key.as<uint32_t>(), count.as<uint32_t>(), span.as<int>());
        ctx->launches++;
        int rc = exclusive_scan_u32(ctx, count.as<uint32_t>(), offs.as<uint32_t>(), nkeys + 1, tmp.as<uint32_t>(), st);
        if (rc) return rc;
        GFS_CUDA_CHECK(cudaMemsetAsync(count.p, 0, count.bytes, st));
        k_pt_scatter<<<grid_blocks(n, T), T, 0, st>>>(key.as<uint32_t>(), n, offs.as<uint32_t>(),
                                                      count.as<uint32_t>(), perm.as<uint32_t>());
        k_pt_sort_keys<<<grid_blocks(nkeys, T), T, 0, st>>>(offs.as<uint32_t>(), nkeys, perm.as<uint32_t>());
        ctx->launches += 2;
        GFS_LAUNCH_CHECK();
    }
    // number of points that reach the grid, and the largest bound spans
    uint32_t m = 0;
    int hspan[4] = {0, 0, 0, 0};
    GFS_CUDA_CHECK(cudaMemcpyAsync(&m, offs.as<uint32_t>() + nkeys, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    GFS_CUDA_CHECK(cudaMemcpyAsync(hspan, span.p, sizeof(hspan), cudaMemcpyDeviceToHost, st));
    GFS_CUDA_CHECK(cudaStreamSynchronize(st));
    if (m == 0) return GFS_OK;
    if (spq.alloc((size_t)m * sizeof(float4)) || sphi.alloc((size_t)m * sizeof(int4))) return GFS_ERR_NOMEM;
    ProfScope prof(ctx, KC_SPLAT);
    k_pt_permute<<<grid_blocks(m, T), T, 0, st>>>(perm.as<uint32_t>(), m, pq.as<float4>(), phi.as<int4>(),
                                                  spq.as<float4>(), sphi.as<int4>());
    GatherArgs G;
    G.dx = dx;
    G.r2_thresh = ceil_to_float(radius * radius);
    G.inv_r2 = (float)(1.0 / (radius * radius));
    G.W = W; G.H = H; G.D = D;
    for (int d = 0; d < 3; d++) G.span[d] = hspan[d];
    G.thr_set = thr_set ? 1 : 0;
    G.thr = thr;
    dim3 block(32, 2, 2);
    dim3 grid(grid_blocks(W, 32), grid_blocks(H, 2), grid_blocks(D, 2));
    k_pt_gather<<<grid, block, 0, st>>>(G, offs.as<uint32_t>(), spq.as<float4>(), sphi.as<int4>(), d_field, d_weight);
    ctx->launches += 2;
    GFS_LAUNCH_CHECK();
    GFS_CUDA_CHECK(cudaStreamSynchronize(st));   // the scratch buffers are freed on return
    return GFS_OK;
}

}  // namespace gfs
