// particles.cu -- particle ordering and cell classification.
//
// Particles are kept in (cell, id) order.  After every substep (and after an
// upload) a counting sort rebuilds that order:
//   k_keys      cell key per particle (invalid for out-of-grid / solid cells:
//               FluidSimulation::_removeMarkerParticlesInSolidCells,
//               fluidsimulation.cpp:1933-1958) and an atomic slot in its cell;
//   scan        exclusive scan of the per-cell counts -> cell offsets;
//   k_scatter   particles to offset[cell] + slot;
//   k_rank_sort each particle of a cell's run to its rank by particle id in the
//               run, which makes the order independent of the atomic slot
//               order (the splat sums in this order, so every run is bitwise
//               reproducible);
//   cap         cells holding more than max_particles_per_cell keep their
//               smallest ids (FluidSimulation::_removeMarkerParticles,
//               fluidsimulation.cpp:3221-3243, keeps a random subset after a
//               rand() shuffle; the selection here is deterministic).
// k_classify is FluidSimulation::_updateFluidCells (fluidsimulation.cpp:1990-2041)
// on the dense grid: interior fluid cells become air, cells holding particles
// become fluid.  The lexicographic fluid-cell list of the reference is implicit
// in the dense layout.
#include <utility>

#include "gfs_internal.h"

namespace gfs {

#define KEY_INVALID 0xFFFFFFFFu

__device__ __forceinline__ uint32_t pid(const float4 &p) { return __float_as_uint(p.w); }

__global__ void k_keys(const float4 *__restrict__ pos, const uint32_t *__restrict__ num,
                       long long nbound, GridDim c, double invdx_d, float invdx_f, int pow2,
                       const uint8_t *__restrict__ mat, uint32_t *__restrict__ key,
                       uint32_t *__restrict__ slot, uint32_t *__restrict__ count) {
    long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (p >= nbound || p >= (long long)num[0]) return;
    float4 x = pos[p];
    uint32_t kk = KEY_INVALID;
    if (isfinite(x.x) && isfinite(x.y) && isfinite(x.z)) {
        int i, j, k;
        // Grid3d::positionToGridIndex (grid3d.h:58-63): floor(p * (1/dx)).  With
        // a power-of-two dx the float product is exact and equals the double one.
        if (pow2) {
            i = (int)floorf(x.x * invdx_f);
            j = (int)floorf(x.y * invdx_f);
            k = (int)floorf(x.z * invdx_f);
        } else {
            i = (int)floor((double)x.x * invdx_d);
            j = (int)floor((double)x.y * invdx_d);
            k = (int)floor((double)x.z * invdx_d);
        }
        // solid cells, and cells flagged by an outflow source or the removed-cell
        // queue (bit 0x80), keep no particle
        if (c.in(i, j, k)) {
            const uint8_t m = mat[c.at(i, j, k)];
            if (m != GFS_SOLID && !(m & 0x80))
                kk = (uint32_t)i + (uint32_t)c.nx * ((uint32_t)j + (uint32_t)c.ny * (uint32_t)k);
        }
    }
    key[p] = kk;
    if (kk != KEY_INVALID) slot[p] = atomicAdd(&count[kk], 1u);
}

__global__ void k_scatter(const float4 *__restrict__ pos, const float4 *__restrict__ vel,
                          const uint32_t *__restrict__ key, const uint32_t *__restrict__ slot,
                          const uint32_t *__restrict__ offset, const uint32_t *__restrict__ num,
                          long long nbound, float4 *__restrict__ pos_out,
                          float4 *__restrict__ vel_out) {
    long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (p >= nbound || p >= (long long)num[0]) return;
    uint32_t kk = key[p];
    if (kk == KEY_INVALID) return;
    uint32_t d = offset[kk] + slot[p];
    pos_out[d] = pos[p];
    vel_out[d] = vel[p];
}

// One thread per particle of the scattered set: its place in its cell's run is its rank by
// id there (ties, which distinct ids never give, by scattered position).  The (cell, id)
// order is that of an insertion sort of each run by id, reached without a serial pass
// per cell.  The cell is recomputed with k_keys' formula.  A cell keeps its `cap` smallest
// ids, written from dst_off (the scan of min(count, cap); the run offsets themselves when no
// cap applies), and num[0] gets the count after removal and capping.
__global__ void k_rank_sort(const float4 *__restrict__ pos_in, const float4 *__restrict__ vel_in,
                            const uint32_t *__restrict__ offset, const uint32_t *__restrict__ dst_off,
                            long long ncells, long long nbound, GridDim c, double invdx_d, float invdx_f, int pow2,
                            int cap, float4 *__restrict__ pos_out, float4 *__restrict__ vel_out,
                            uint32_t *__restrict__ num) {
    const long long n = (long long)offset[ncells];
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q == 0) num[0] = dst_off[ncells];
    if (q >= n || q >= nbound) return;
    const float4 x = pos_in[q];
    int i, j, k;
    if (pow2) {
        i = (int)floorf(x.x * invdx_f);
        j = (int)floorf(x.y * invdx_f);
        k = (int)floorf(x.z * invdx_f);
    } else {
        i = (int)floor((double)x.x * invdx_d);
        j = (int)floor((double)x.y * invdx_d);
        k = (int)floor((double)x.z * invdx_d);
    }
    if (!c.in(i, j, k)) return;   // never for a scattered set
    const uint32_t kk = (uint32_t)i + (uint32_t)c.nx * ((uint32_t)j + (uint32_t)c.ny * (uint32_t)k);
    const uint32_t b = offset[kk], e = offset[kk + 1];
    if ((uint32_t)q < b || (uint32_t)q >= e) return;   // never for a scattered set
    const uint32_t id = pid(x);
    uint32_t r = 0;
    for (uint32_t a = b; a < e; a++) {
        const uint32_t o = pid(pos_in[a]);
        r += (o < id || (o == id && a < (uint32_t)q)) ? 1u : 0u;
    }
    if (r >= (uint32_t)cap) return;   // the cell's smallest ids stay (dst_off: the capped run starts)
    const uint32_t d = dst_off[kk] + r;
    pos_out[d] = x;
    vel_out[d] = vel_in[q];
}

__global__ void k_cap_counts(const uint32_t *__restrict__ offset, long long ncells, int cap,
                             uint32_t *__restrict__ cnt) {
    long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (c > ncells) return;
    if (c == ncells) { cnt[c] = 0; return; }
    uint32_t m = offset[c + 1] - offset[c];
    cnt[c] = m < (uint32_t)cap ? m : (uint32_t)cap;
}

// One thread per particle of the sorted set: the particle's cell (the sort's own
// formula, k_keys) and its rank in the cell; the first `cap` of each cell (the
// smallest ids) move to the capped offsets, in order -- coalesced reads and writes.
__global__ void k_cap_copy(const float4 *__restrict__ pos, const float4 *__restrict__ vel,
                           const uint32_t *__restrict__ off_in, const uint32_t *__restrict__ off_out,
                           long long ncells, long long n, GridDim c, double invdx_d, float invdx_f, int pow2,
                           int cap, float4 *__restrict__ pos_out, float4 *__restrict__ vel_out,
                           uint32_t *__restrict__ num) {
    long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (p == 0) num[0] = off_out[ncells];
    if (p >= n) return;
    const float4 x = pos[p];
    int i, j, k;
    if (pow2) {
        i = (int)floorf(x.x * invdx_f);
        j = (int)floorf(x.y * invdx_f);
        k = (int)floorf(x.z * invdx_f);
    } else {
        i = (int)floor((double)x.x * invdx_d);
        j = (int)floor((double)x.y * invdx_d);
        k = (int)floor((double)x.z * invdx_d);
    }
    if (!c.in(i, j, k)) return;   // never for a sorted set
    const uint32_t kk = (uint32_t)i + (uint32_t)c.nx * ((uint32_t)j + (uint32_t)c.ny * (uint32_t)k);
    const uint32_t b = off_in[kk];
    if ((uint32_t)p < b || (uint32_t)p >= off_in[kk + 1]) return;   // never for a sorted set
    const uint32_t rank = (uint32_t)p - b;
    if (rank >= (uint32_t)cap) return;
    const uint32_t o = off_out[kk] + rank;
    pos_out[o] = x;
    vel_out[o] = vel[p];
}

// ------------------------------------------------------------------ scan

#define SCAN_THREADS 512
#define SCAN_ITEMS 16
#define SCAN_TILE (SCAN_THREADS * SCAN_ITEMS)

size_t scan_temp_elems(long long n) { return (size_t)((n + SCAN_TILE - 1) / SCAN_TILE) + 1; }

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *total) {
    __shared__ uint32_t warp_sums[SCAN_THREADS / 32];
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < SCAN_THREADS / 32 ? warp_sums[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < SCAN_THREADS / 32) warp_sums[lane] = w;
    }
    __syncthreads();
    uint32_t before = warp > 0 ? warp_sums[warp - 1] : 0;
    *total = warp_sums[SCAN_THREADS / 32 - 1];
    __syncthreads();
    return before + x - v;
}

// in and out may alias (the cap path scans in place).
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_local(const uint32_t *in, uint32_t *out, long long n,
                                                             uint32_t *__restrict__ block_sums) {
    long long base = (long long)blockIdx.x * SCAN_TILE + (long long)threadIdx.x * SCAN_ITEMS;
    uint32_t v[SCAN_ITEMS];
    uint32_t sum = 0;
#pragma unroll
    for (int q = 0; q < SCAN_ITEMS; q++) {
        long long e = base + q;
        v[q] = e < n ? in[e] : 0u;
        sum += v[q];
    }
    uint32_t total;
    uint32_t run = block_exclusive_scan(sum, &total);
#pragma unroll
    for (int q = 0; q < SCAN_ITEMS; q++) {
        long long e = base + q;
        if (e < n) out[e] = run;
        run += v[q];
    }
    if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_top(uint32_t *__restrict__ sums, long long nb) {
    // nb <= SCAN_TILE
    long long base = (long long)threadIdx.x * SCAN_ITEMS;
    uint32_t v[SCAN_ITEMS];
    uint32_t sum = 0;
#pragma unroll
    for (int q = 0; q < SCAN_ITEMS; q++) {
        long long e = base + q;
        v[q] = e < nb ? sums[e] : 0u;
        sum += v[q];
    }
    uint32_t total;
    uint32_t run = block_exclusive_scan(sum, &total);
#pragma unroll
    for (int q = 0; q < SCAN_ITEMS; q++) {
        long long e = base + q;
        if (e < nb) sums[e] = run;
        run += v[q];
    }
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_add(uint32_t *__restrict__ out, long long n,
                                                           const uint32_t *__restrict__ sums) {
    uint32_t add = sums[blockIdx.x];
    long long base = (long long)blockIdx.x * SCAN_TILE;
    for (int q = threadIdx.x; q < SCAN_TILE; q += SCAN_THREADS) {
        long long e = base + q;
        if (e < n) out[e] += add;
    }
}

int exclusive_scan_u32(Ctx *ctx, uint32_t *in, uint32_t *out, long long n, uint32_t *block_sums,
                       cudaStream_t st) {
    long long nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (nb > SCAN_TILE) {
        set_error(GFS_ERR_INVALID, "scan of %lld elements exceeds the supported %lld", n,
                  (long long)SCAN_TILE * SCAN_TILE);
        return GFS_ERR_INVALID;
    }
    k_scan_local<<<(unsigned)nb, SCAN_THREADS, 0, st>>>(in, out, n, block_sums);
    k_scan_top<<<1, SCAN_THREADS, 0, st>>>(block_sums, nb);
    k_scan_add<<<(unsigned)nb, SCAN_THREADS, 0, st>>>(out, n, block_sums);
    ctx->launches += 3;
    GFS_LAUNCH_CHECK();
    return GFS_OK;
}

// --------------------------------------------------------------- driver

// The cap check of k_rank_sort for a set that was already in order: num[0] = the
// particle count after removal, num[1] set if a cell holds more than `cap`.
__global__ void k_cap_flag(const uint32_t *__restrict__ offset, long long ncells, int cap,
                           uint32_t *__restrict__ num) {
    long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (c >= ncells) return;
    if (c == ncells - 1) num[0] = offset[ncells];
    if ((int)(offset[c + 1] - offset[c]) > cap) atomicOr(&num[1], 1u);
}

// After the particles are in (cell, id) order: read the count and the cap flag;
// cells holding more than max_particles_per_cell keep their smallest ids.
static int finish_sort(Sim *s, long long ncells, bool /*was_in_order*/) {
    Ctx *ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    const int T = 256;
    uint32_t *count = s->count.as<uint32_t>();
    uint32_t *offset = s->offset.as<uint32_t>();
    uint32_t *num = s->num.as<uint32_t>();
    int cap = s->params.max_particles_per_cell > 0 ? s->params.max_particles_per_cell : 0x7fffffff;
    uint32_t host_num[2];
    GFS_CUDA_CHECK(cudaMemcpyAsync(host_num, num, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    GFS_CUDA_CHECK(cudaStreamSynchronize(st));
    if (host_num[1]) {
        // Some cell holds more than `cap` particles: keep the smallest ids.
        k_cap_counts<<<grid_blocks(ncells + 1, T), T, 0, st>>>(offset, ncells, cap, count);
        ctx->launches++;
        GFS_LAUNCH_CHECK();
        int rc = exclusive_scan_u32(ctx, count, count, ncells + 1, s->scan_tmp.as<uint32_t>(), st);
        if (rc) return rc;
        const long long n = host_num[0];
        k_cap_copy<<<grid_blocks(n > 0 ? n : 1, T), T, 0, st>>>(
            s->pos.as<float4>(), s->vel.as<float4>(), offset, count, ncells, n, s->g.c, 1.0 / s->g.dx, s->inv_dx_f,
            s->dx_pow2 ? 1 : 0, cap, s->pos_alt.as<float4>(), s->vel_alt.as<float4>(), num);
        ctx->launches++;
        GFS_LAUNCH_CHECK();
        std::swap(s->pos.p, s->pos_alt.p);
        std::swap(s->vel.p, s->vel_alt.p);
        std::swap(s->count.p, s->offset.p);   // capped offsets become the live offsets
        GFS_CUDA_CHECK(cudaMemcpyAsync(host_num, num, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        GFS_CUDA_CHECK(cudaStreamSynchronize(st));
    }
    s->n_bound = host_num[0];
    s->need_sort = false;
    return GFS_OK;
}

// num[3] = 1 unless particles [0, n) are already in (cell, id) order with every
// particle in a cell that keeps particles (keys from k_keys; ids in pos.w)
__global__ void k_check_sorted(const float4 *__restrict__ pos, const uint32_t *__restrict__ key,
                               const uint32_t *__restrict__ num, long long nbound, uint32_t *__restrict__ flag) {
    long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long n = nbound < (long long)num[0] ? nbound : (long long)num[0];
    if (p >= n) return;
    const uint32_t k1 = key[p];
    bool bad = k1 == KEY_INVALID;
    if (!bad && p > 0) {
        const uint32_t k0 = key[p - 1];
        bad = k0 > k1 || (k0 == k1 && pid(pos[p - 1]) >= pid(pos[p]));
    }
    if (bad) *flag = 1u;
}

int sort_particles(Sim *s, bool /*remove_solid*/) {
    Ctx *ctx = s->ctx;
    ProfScope prof(ctx, KC_SORT);
    cudaStream_t st = ctx->stream;
    const GridDim &c = s->g.c;
    long long ncells = (long long)c.nx * c.ny * c.nz;
    long long nb = s->n_bound;
    uint32_t *count = s->count.as<uint32_t>();
    uint32_t *offset = s->offset.as<uint32_t>();
    uint32_t *num = s->num.as<uint32_t>();
    GFS_CUDA_CHECK(cudaMemsetAsync(count, 0, (size_t)(ncells + 1) * sizeof(uint32_t), st));
    GFS_CUDA_CHECK(cudaMemsetAsync(num + 1, 0, sizeof(uint32_t), st));
    GFS_CUDA_CHECK(cudaMemsetAsync(num + 3, 0, sizeof(uint32_t), st));
    const int T = 256;
    if (nb > 0) {
        k_keys<<<grid_blocks(nb, T), T, 0, st>>>(s->pos.as<float4>(), num, nb, c, 1.0 / s->g.dx,
                                                 s->inv_dx_f, s->dx_pow2 ? 1 : 0, s->mat.as<uint8_t>(),
                                                 s->key.as<uint32_t>(), s->slot.as<uint32_t>(), count);
        ctx->launches++;
        GFS_LAUNCH_CHECK();
    }
    int rc = exclusive_scan_u32(ctx, count, offset, ncells + 1, s->scan_tmp.as<uint32_t>(), st);
    if (rc) return rc;
    // A set that is already in (cell, id) order with no particle to remove -- an
    // upload of the particles a step handed back, or a load of a saved state --
    // keeps its place: the offsets are all the sort has to produce.  The cap is
    // then checked the way k_rank_sort checks it.
    bool in_order = false;
    if (s->sorted_hint && nb > 0) {
        k_check_sorted<<<grid_blocks(nb, T), T, 0, st>>>(s->pos.as<float4>(), s->key.as<uint32_t>(), num, nb,
                                                         num + 3);
        ctx->launches++;
        GFS_LAUNCH_CHECK();
        uint32_t host_flag = 1;
        GFS_CUDA_CHECK(cudaMemcpyAsync(&host_flag, num + 3, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        GFS_CUDA_CHECK(cudaStreamSynchronize(st));
        in_order = host_flag == 0;
    }
    s->sorted_hint = false;
    if (in_order) {
        int cap = s->params.max_particles_per_cell > 0 ? s->params.max_particles_per_cell : 0x7fffffff;
        k_cap_flag<<<grid_blocks(ncells, T), T, 0, st>>>(offset, ncells, cap, num);
        ctx->launches++;
        GFS_LAUNCH_CHECK();
        return finish_sort(s, ncells, true);
    }
    if (nb > 0) {
        k_scatter<<<grid_blocks(nb, T), T, 0, st>>>(s->pos.as<float4>(), s->vel.as<float4>(),
                                                    s->key.as<uint32_t>(), s->slot.as<uint32_t>(),
                                                    offset, num, nb, s->pos_alt.as<float4>(),
                                                    s->vel_alt.as<float4>());
        ctx->launches++;
        GFS_LAUNCH_CHECK();
    }
    int cap = s->params.max_particles_per_cell > 0 ? s->params.max_particles_per_cell : 0x7fffffff;
    if (nb > 0) {
        // with a cap, the capped run starts: the scan of min(count, cap), into `count`
        // (FluidSimulation::_removeMarkerParticles, fluidsimulation.cpp:3221-3243)
        const bool capping = s->params.max_particles_per_cell > 0;
        if (capping) {
            k_cap_counts<<<grid_blocks(ncells + 1, T), T, 0, st>>>(offset, ncells, cap, count);
            ctx->launches++;
            GFS_LAUNCH_CHECK();
            rc = exclusive_scan_u32(ctx, count, count, ncells + 1, s->scan_tmp.as<uint32_t>(), st);
            if (rc) return rc;
        }
        // the scattered set (pos_alt) into (cell, id) order, back into pos
        k_rank_sort<<<grid_blocks(nb, T), T, 0, st>>>(s->pos_alt.as<float4>(), s->vel_alt.as<float4>(), offset,
                                                      capping ? count : offset, ncells, nb, c, 1.0 / s->g.dx,
                                                      s->inv_dx_f, s->dx_pow2 ? 1 : 0, cap, s->pos.as<float4>(),
                                                      s->vel.as<float4>(), num);
        ctx->launches++;
        GFS_LAUNCH_CHECK();
        if (capping) std::swap(s->count.p, s->offset.p);   // the capped starts become the live offsets
    } else {
        k_cap_flag<<<grid_blocks(ncells, T), T, 0, st>>>(offset, ncells, cap, num);
        ctx->launches++;
        GFS_LAUNCH_CHECK();
    }
    return finish_sort(s, ncells, false);
}

__global__ void k_classify(uint8_t *__restrict__ mat, GridDim c, const uint32_t *__restrict__ offset,
                           uint32_t *__restrict__ fluid_count) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y, k = blockIdx.z;
    bool fl = false;
    if (i < c.nx) {
        long long at = c.at(i, j, k);
        uint8_t m = mat[at];
        bool interior = i > 0 && j > 0 && k > 0 && i < c.nx - 1 && j < c.ny - 1 && k < c.nz - 1;
        if (interior && m == GFS_FLUID) m = GFS_AIR;
        long long lin = i + (long long)c.nx * (j + (long long)c.ny * k);
        if (offset[lin + 1] > offset[lin]) m = GFS_FLUID;
        mat[at] = m;
        fl = m == GFS_FLUID;
    }
    unsigned b = __ballot_sync(0xffffffffu, fl);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(fluid_count, (uint32_t)__popc(b));
}

int classify_cells(Sim *s) {
    Ctx *ctx = s->ctx;
    ProfScope prof(ctx, KC_CLASSIFY);
    const GridDim &c = s->g.c;
    uint32_t *num = s->num.as<uint32_t>();
    GFS_CUDA_CHECK(cudaMemsetAsync(num + 2, 0, sizeof(uint32_t), ctx->stream));
    dim3 grid(grid_blocks(c.nx, 128), c.ny, c.nz);
    k_classify<<<grid, 128, 0, ctx->stream>>>(s->mat.as<uint8_t>(), c, s->offset.as<uint32_t>(), num + 2);
    ctx->launches++;
    GFS_LAUNCH_CHECK();
    return GFS_OK;
}

}  // namespace gfs
