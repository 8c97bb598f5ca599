// capi.cu -- the extern "C" boundary of libgfs (declared in include/gfs.h).
//
// Status codes plus a thread-local error string replace the reference's
// c_bindings convention (int *err + CBINDINGS_ERROR_MESSAGE, cbindings.h:20-135);
// no exception crosses the ABI.  Host buffers are borrowed for the duration of a
// call.  Standalone entry points (splat, interpolate, advect, pressure) stage the
// caller's arrays into padded device grids, run the same kernels the
// device-resident substep runs, and copy the result back.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "gfs_internal.h"

namespace gfs {

static thread_local char g_err[1024] = "";

void set_error(int code, const char *fmt, ...) {
    (void)code;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

const char *const kKernelClassNames[KC_COUNT] = {
    "sort", "classify", "splat", "face_fill", "layers", "extrapolate", "pressure_setup", "mic0_build",
    "mic0_forward", "mic0_backward", "matvec", "axpy", "update_search", "mixed_refine", "apply_pressure",
    "g2p_advect"};

cudaEvent_t Profiler::take() {
    if (!pool.empty()) {
        cudaEvent_t e = pool.back();
        pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

void Profiler::begin(cudaStream_t st, int cls) {
    open_cls = cls;
    open_ev = take();
    cudaEventRecord(open_ev, st);
}

void Profiler::end(cudaStream_t st, int cls) {
    if (open_cls != cls || !open_ev) return;
    cudaEvent_t b = take();
    cudaEventRecord(b, st);
    pending.push_back({cls, open_ev, b});
    open_ev = nullptr;
    open_cls = -1;
}

void Profiler::flush() {
    for (auto &r : pending) {
        cudaEventSynchronize(r.b);
        float t = 0.f;
        if (cudaEventElapsedTime(&t, r.a, r.b) == cudaSuccess) {
            ms[r.cls] += t;
            count[r.cls] += 1;
        }
        pool.push_back(r.a);
        pool.push_back(r.b);
    }
    pending.clear();
}

void Profiler::reset() {
    flush();
    for (int i = 0; i < KC_COUNT; i++) { ms[i] = 0; count[i] = 0; }
}

Profiler::~Profiler() {
    for (auto &r : pending) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
    for (auto e : pool) cudaEventDestroy(e);
}

int DevMem::alloc(size_t n) {
    release();
    if (n == 0) n = 16;
    cudaError_t e = cudaMalloc(&p, n);
    if (e != cudaSuccess) {
        p = nullptr;
        set_error(GFS_ERR_NOMEM, "cudaMalloc(%zu bytes) failed: %s", n, cudaGetErrorString(e));
        return GFS_ERR_NOMEM;
    }
    bytes = n;
    return GFS_OK;
}

int DevMem::ensure(size_t n) {
    if (p && bytes >= n) return GFS_OK;
    return alloc(n);
}

void DevMem::release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
}

// ------------------------------------------------- padded <-> flat grids

template <class T>
__global__ void k_pad(const T *__restrict__ src, GridDim g, T *__restrict__ dst) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y, k = blockIdx.z;
    if (i >= g.nx) return;
    dst[g.at(i, j, k)] = src[i + (long long)g.nx * (j + (long long)g.ny * k)];
}

template <class T>
__global__ void k_unpad(const T *__restrict__ src, GridDim g, T *__restrict__ dst) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y, k = blockIdx.z;
    if (i >= g.nx) return;
    dst[i + (long long)g.nx * (j + (long long)g.ny * k)] = src[g.at(i, j, k)];
}

// host flat -> device padded (through a device staging buffer)
template <class T>
static int upload_padded(Ctx *ctx, const T *h, const GridDim &g, T *d_padded, DevMem &stage) {
    size_t n = (size_t)g.nx * g.ny * g.nz;
    if (stage.ensure(n * sizeof(T))) return GFS_ERR_NOMEM;
    GFS_CUDA_CHECK(cudaMemcpyAsync(stage.p, h, n * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
    dim3 grid(grid_blocks(g.nx, 128), g.ny, g.nz);
    k_pad<T><<<grid, 128, 0, ctx->stream>>>(stage.as<T>(), g, d_padded);
    ctx->launches++;
    GFS_LAUNCH_CHECK();
    return GFS_OK;
}

template <class T>
static int download_padded(Ctx *ctx, const T *d_padded, const GridDim &g, T *h, DevMem &stage) {
    size_t n = (size_t)g.nx * g.ny * g.nz;
    if (stage.ensure(n * sizeof(T))) return GFS_ERR_NOMEM;
    dim3 grid(grid_blocks(g.nx, 128), g.ny, g.nz);
    k_unpad<T><<<grid, 128, 0, ctx->stream>>>(d_padded, g, stage.as<T>());
    ctx->launches++;
    GFS_LAUNCH_CHECK();
    GFS_CUDA_CHECK(cudaMemcpyAsync(h, stage.p, n * sizeof(T), cudaMemcpyDeviceToHost, ctx->stream));
    GFS_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    return GFS_OK;
}

// ------------------------------------------------------ particle packing

// xyz triples <-> the device's float4 particles (id in pos.w).  A block of 256
// threads moves 1024 particles; with 16-byte aligned triples (vec) and a full
// block, the block's triples travel through shared memory so that every warp
// load or store instruction covers 512 contiguous bytes -- whole lines, which is
// what the host link needs when the triples are host memory read or written in
// place (scattered 16-byte pieces ran at a third of the link rate) -- else one
// particle per thread, one float at a time.
static constexpr int PK_THREADS = 256, PK_PER = 4 * PK_THREADS;   // particles per block

__device__ __forceinline__ void copy_block16(float4 *__restrict__ dst, const float4 *__restrict__ src, int n16) {
    for (int i = threadIdx.x; i < n16; i += PK_THREADS) dst[i] = src[i];
}

__global__ void __launch_bounds__(PK_THREADS) k_pack_particles(const float *__restrict__ p3,
                                                               const float *__restrict__ v3,
                                                               const uint32_t *__restrict__ ids, long long n,
                                                               float4 *__restrict__ pos, float4 *__restrict__ vel,
                                                               int vec) {
    __shared__ __align__(16) float sp[3 * PK_PER], sv[3 * PK_PER];
    const long long b0 = (long long)blockIdx.x * PK_PER;
    const int t = threadIdx.x;
    if (vec && b0 + PK_PER <= n) {
        copy_block16(reinterpret_cast<float4 *>(sp), reinterpret_cast<const float4 *>(p3 + 3 * b0), 3 * PK_PER / 4);
        if (v3) copy_block16(reinterpret_cast<float4 *>(sv), reinterpret_cast<const float4 *>(v3 + 3 * b0), 3 * PK_PER / 4);
        __syncthreads();
        for (int k = t; k < PK_PER; k += PK_THREADS) {   // consecutive threads, consecutive particles
            const long long q = b0 + k;
            const uint32_t id = ids ? ids[q] : (uint32_t)q;
            pos[q] = make_float4(sp[3 * k], sp[3 * k + 1], sp[3 * k + 2], __uint_as_float(id));
            vel[q] = v3 ? make_float4(sv[3 * k], sv[3 * k + 1], sv[3 * k + 2], 0.f) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        return;
    }
    for (long long q = b0 + t; q < b0 + PK_PER && q < n; q += PK_THREADS) {
        const uint32_t id = ids ? ids[q] : (uint32_t)q;
        pos[q] = make_float4(p3[3 * q], p3[3 * q + 1], p3[3 * q + 2], __uint_as_float(id));
        vel[q] = v3 ? make_float4(v3[3 * q], v3[3 * q + 1], v3[3 * q + 2], 0.f) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

__global__ void __launch_bounds__(PK_THREADS) k_unpack_particles(const float4 *__restrict__ pos,
                                                                 const float4 *__restrict__ vel, long long n,
                                                                 float *__restrict__ p3, float *__restrict__ v3,
                                                                 uint32_t *__restrict__ ids, int vec) {
    __shared__ __align__(16) float sp[3 * PK_PER], sv[3 * PK_PER];
    const long long b0 = (long long)blockIdx.x * PK_PER;
    const int t = threadIdx.x;
    if (vec && b0 + PK_PER <= n) {
        for (int k = t; k < PK_PER; k += PK_THREADS) {
            const long long q = b0 + k;
            const float4 p = pos[q], v = vel[q];
            sp[3 * k] = p.x; sp[3 * k + 1] = p.y; sp[3 * k + 2] = p.z;
            sv[3 * k] = v.x; sv[3 * k + 1] = v.y; sv[3 * k + 2] = v.z;
            ids[q] = __float_as_uint(p.w);
        }
        __syncthreads();
        copy_block16(reinterpret_cast<float4 *>(p3 + 3 * b0), reinterpret_cast<const float4 *>(sp), 3 * PK_PER / 4);
        copy_block16(reinterpret_cast<float4 *>(v3 + 3 * b0), reinterpret_cast<const float4 *>(sv), 3 * PK_PER / 4);
        return;
    }
    for (long long q = b0 + t; q < b0 + PK_PER && q < n; q += PK_THREADS) {
        const float4 p = pos[q], v = vel[q];
        p3[3 * q] = p.x; p3[3 * q + 1] = p.y; p3[3 * q + 2] = p.z;
        v3[3 * q] = v.x; v3[3 * q + 1] = v.y; v3[3 * q + 2] = v.z;
        ids[q] = __float_as_uint(p.w);
    }
}

static bool all_a16(const void *a, const void *b, const void *c) {
    auto ok = [](const void *q) { return q == nullptr || ((uintptr_t)q & 15u) == 0; };
    return ok(a) && ok(b) && ok(c);
}

static bool valid_dims(int ni, int nj, int nk) {
    return ni > 0 && nj > 0 && nk > 0 && (long long)ni * nj * nk < (1LL << 31);
}

// -------------------------------------------------------------- sim core

static int sim_init(Sim *s, Ctx *ctx, int ni, int nj, int nk, double dx, int64_t cap) {
    s->ctx = ctx;
    s->g = make_grids(ni, nj, nk, dx);
    gfs_sim_default_params(&s->params);
    s->capacity = cap;
    int e;
    double m = frexp(dx, &e);
    s->dx_pow2 = (m == 0.5);
    s->inv_dx_f = (float)(1.0 / dx);
    cudaStream_t st = ctx->stream;
    const GridDim &c = s->g.c;
    long long ncells = (long long)ni * nj * nk;
    int rc = 0;
    rc |= s->mat.alloc((size_t)c.size);
    rc |= s->layer.alloc((size_t)c.size);
    rc |= s->lcells.alloc((size_t)c.size * sizeof(uint32_t));
    rc |= s->lcnt.alloc((size_t)(GFS_MAX_LAYERS + 1) * sizeof(uint32_t));
    for (int d = 0; d < 3; d++) {
        const GridDim &f = s->g.f[d];
        rc |= s->mac[d].alloc((size_t)f.size * sizeof(float));
        rc |= s->saved[d].alloc((size_t)f.size * sizeof(float));
        rc |= s->quad[d].alloc((size_t)f.size * sizeof(float4));
        rc |= s->sval[d].alloc((size_t)f.size * sizeof(float));
        rc |= s->smask[d].alloc((size_t)f.size);
    }
    size_t pc = (size_t)std::max<int64_t>(cap, 1);
    rc |= s->pos.alloc(pc * sizeof(float4));
    rc |= s->vel.alloc(pc * sizeof(float4));
    rc |= s->pos_alt.alloc(pc * sizeof(float4));
    rc |= s->vel_alt.alloc(pc * sizeof(float4));
    rc |= s->key.alloc(pc * sizeof(uint32_t));
    rc |= s->slot.alloc(pc * sizeof(uint32_t));
    rc |= s->count.alloc((size_t)(ncells + 1) * sizeof(uint32_t));
    rc |= s->offset.alloc((size_t)(ncells + 1) * sizeof(uint32_t));
    rc |= s->scan_tmp.alloc(scan_temp_elems(ncells + 1) * sizeof(uint32_t));
    rc |= s->num.alloc(4 * sizeof(uint32_t));
    if (rc) return GFS_ERR_NOMEM;
    GFS_CUDA_CHECK(cudaMemsetAsync(s->mat.p, GFS_SOLID, s->mat.bytes, st));
    GFS_CUDA_CHECK(cudaMemsetAsync(s->layer.p, 0xFF, s->layer.bytes, st));
    for (int d = 0; d < 3; d++) {
        GFS_CUDA_CHECK(cudaMemsetAsync(s->mac[d].p, 0, s->mac[d].bytes, st));
        GFS_CUDA_CHECK(cudaMemsetAsync(s->saved[d].p, 0, s->saved[d].bytes, st));
        GFS_CUDA_CHECK(cudaMemsetAsync(s->sval[d].p, 0, s->sval[d].bytes, st));
        GFS_CUDA_CHECK(cudaMemsetAsync(s->smask[d].p, 0, s->smask[d].bytes, st));
    }
    GFS_CUDA_CHECK(cudaMemsetAsync(s->num.p, 0, s->num.bytes, st));
    GFS_CUDA_CHECK(cudaMemsetAsync(s->offset.p, 0, s->offset.bytes, st));
    // interior of the material grid: air
    DevMem stage;
    std::vector<uint8_t> air((size_t)ncells, GFS_AIR);
    rc = upload_padded<uint8_t>(ctx, air.data(), c, s->mat.as<uint8_t>(), stage);
    if (rc) return rc;
    GFS_CUDA_CHECK(cudaStreamSynchronize(st));
    GFS_CUDA_CHECK(cudaEventCreate(&s->ev0));
    GFS_CUDA_CHECK(cudaEventCreate(&s->ev1));
    GFS_CUDA_CHECK(cudaEventCreate(&s->evp0));
    GFS_CUDA_CHECK(cudaEventCreate(&s->evp1));
    return GFS_OK;
}

// The device address of a host buffer that the device can read and write in
// place -- page-locked and mapped (cudaHostAlloc / cudaHostRegister) for the
// current device, the whole range in one registration -- else nullptr (pageable
// or managed memory goes through a staged copy).  On GB300 the device then
// reaches it over the NVLink-C2C host link from inside the pack / unpack kernels.
static void *mapped_host(const void *h, size_t bytes) {
    if (!h || bytes == 0) return nullptr;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    cudaPointerAttributes a0, a1;
    if (cudaPointerGetAttributes(&a0, h) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a0.type != cudaMemoryTypeHost || a0.devicePointer == nullptr || a0.device != dev) return nullptr;
    const char *last = (const char *)h + bytes - 1;
    if (cudaPointerGetAttributes(&a1, last) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a1.type != cudaMemoryTypeHost || a1.devicePointer == nullptr ||
        (const char *)a1.devicePointer - (const char *)a0.devicePointer != (ptrdiff_t)(bytes - 1))
        return nullptr;
    return a0.devicePointer;
}

static int sim_set_particles(Sim *s, const float *hp, const float *hv, const uint32_t *hid, int64_t n) {
    Ctx *ctx = s->ctx;
    if (n < 0 || n > s->capacity) {
        set_error(GFS_ERR_INVALID, "particle count %lld outside [0, capacity %lld]", (long long)n,
                  (long long)s->capacity);
        return GFS_ERR_INVALID;
    }
    if (n > 0 && !hp) {
        set_error(GFS_ERR_INVALID, "positions pointer is NULL");
        return GFS_ERR_INVALID;
    }
    cudaStream_t st = ctx->stream;
    // xyz triples: read in place from mapped host buffers, else staged in the
    // alternate buffers (16 B per particle >= 12 B)
    const float *p3 = s->pos_alt.as<float>(), *v3 = s->vel_alt.as<float>();
    const uint32_t *ids = s->key.as<uint32_t>();
    if (n > 0) {
        const size_t b3 = (size_t)n * 3 * sizeof(float), b1 = (size_t)n * sizeof(uint32_t);
        if (const void *d = mapped_host(hp, b3)) p3 = (const float *)d;
        else GFS_CUDA_CHECK(cudaMemcpyAsync(s->pos_alt.p, hp, b3, cudaMemcpyHostToDevice, st));
        if (!hv) v3 = nullptr;
        else if (const void *d = mapped_host(hv, b3)) v3 = (const float *)d;
        else GFS_CUDA_CHECK(cudaMemcpyAsync(s->vel_alt.p, hv, b3, cudaMemcpyHostToDevice, st));
        if (!hid) ids = nullptr;
        else if (const void *d = mapped_host(hid, b1)) ids = (const uint32_t *)d;
        else GFS_CUDA_CHECK(cudaMemcpyAsync(s->key.p, hid, b1, cudaMemcpyHostToDevice, st));
        k_pack_particles<<<grid_blocks(n, PK_PER), PK_THREADS, 0, st>>>(p3, v3, ids, n, s->pos.as<float4>(),
                                                                        s->vel.as<float4>(), all_a16(p3, v3, ids));
        ctx->launches++;
        GFS_LAUNCH_CHECK();
    }
    uint32_t hn = (uint32_t)n;
    GFS_CUDA_CHECK(cudaMemcpyAsync(s->num.p, &hn, sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    s->n_bound = n;
    s->need_sort = true;
    s->sorted_hint = true;   // e.g. the set a step handed back: the sort keeps it in place
    // particles that fluid sources add take ids after every id given so far; with
    // caller ids the maximum is found on the device when a source first needs it
    s->next_id = (uint32_t)n;
    s->next_id_valid = hid == nullptr;
    return GFS_OK;
}

// Device-side staging of the particle set as xyz triples (positions in pos_alt,
// velocities in vel_alt, ids in key), for readers and writers of host formats.
// Unpack: the current particles into the staging buffers, *n_out their count.
int sim_stage_xyz(Sim *s, int64_t *n_out) {
    Ctx *ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    uint32_t hn = 0;
    GFS_CUDA_CHECK(cudaMemcpyAsync(&hn, s->num.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    GFS_CUDA_CHECK(cudaStreamSynchronize(st));
    *n_out = hn;
    if (hn > 0) {
        k_unpack_particles<<<grid_blocks(hn, PK_PER), PK_THREADS, 0, st>>>(
            s->pos.as<float4>(), s->vel.as<float4>(), hn, s->pos_alt.as<float>(), s->vel_alt.as<float>(),
            s->key.as<uint32_t>(), 1);
        ctx->launches++;
        GFS_LAUNCH_CHECK();
    }
    return GFS_OK;
}

// Pack: n staged xyz triples (ids 0..n-1) become the particle set, sorted by
// (cell, id) with the particles in solid cells removed, as set_particles does.
int sim_unstage_xyz(Sim *s, int64_t n) {
    Ctx *ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    if (n < 0 || n > s->capacity) {
        set_error(GFS_ERR_INVALID, "particle count %lld outside [0, capacity %lld]", (long long)n,
                  (long long)s->capacity);
        return GFS_ERR_INVALID;
    }
    if (n > 0) {
        k_pack_particles<<<grid_blocks(n, PK_PER), PK_THREADS, 0, st>>>(s->pos_alt.as<float>(),
                                                                        s->vel_alt.as<float>(), nullptr, n,
                                                                        s->pos.as<float4>(), s->vel.as<float4>(), 1);
        ctx->launches++;
        GFS_LAUNCH_CHECK();
    }
    uint32_t hn = (uint32_t)n;
    GFS_CUDA_CHECK(cudaMemcpyAsync(s->num.p, &hn, sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    s->n_bound = n;
    s->need_sort = true;
    s->next_id = (uint32_t)n;
    s->next_id_valid = true;
    int rc = sort_particles(s, true);
    if (rc) return rc;
    // cells holding particles are fluid, as after the reference's initialisation
    // (_initializeFluidMaterialParticlesFromSaveState, fluidsimulation.cpp:1466)
    return classify_cells(s);
}

static int sim_get_particles(Sim *s, float *hp, float *hv, uint32_t *hid, int64_t *n_out) {
    Ctx *ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    uint32_t hn = 0;
    GFS_CUDA_CHECK(cudaMemcpyAsync(&hn, s->num.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    GFS_CUDA_CHECK(cudaStreamSynchronize(st));
    long long n = hn;
    if (n_out) *n_out = n;
    if (n > 0 && (hp || hv || hid)) {
        // written in place into mapped host buffers, else staged and copied
        const size_t b3 = (size_t)n * 3 * sizeof(float), b1 = (size_t)n * sizeof(uint32_t);
        float *p3 = s->pos_alt.as<float>(), *v3 = s->vel_alt.as<float>();
        uint32_t *ids = s->key.as<uint32_t>();
        float *mp = (float *)mapped_host(hp, b3), *mv = (float *)mapped_host(hv, b3);
        uint32_t *mi = (uint32_t *)mapped_host(hid, b1);
        float *op = mp ? mp : p3, *ov = mv ? mv : v3;
        uint32_t *oi = mi ? mi : ids;
        k_unpack_particles<<<grid_blocks(n, PK_PER), PK_THREADS, 0, st>>>(
            s->pos.as<float4>(), s->vel.as<float4>(), n, op, ov, oi, all_a16(op, ov, oi));
        ctx->launches++;
        GFS_LAUNCH_CHECK();
        if (hp && !mp) GFS_CUDA_CHECK(cudaMemcpyAsync(hp, p3, b3, cudaMemcpyDeviceToHost, st));
        if (hv && !mv) GFS_CUDA_CHECK(cudaMemcpyAsync(hv, v3, b3, cudaMemcpyDeviceToHost, st));
        if (hid && !mi) GFS_CUDA_CHECK(cudaMemcpyAsync(hid, ids, b1, cudaMemcpyDeviceToHost, st));
        GFS_CUDA_CHECK(cudaStreamSynchronize(st));
    }
    return GFS_OK;
}

int sim_step(Sim *s, double dt, gfs_step_stats *stats, int last_stage) {
    Ctx *ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    if (!(dt >= 0.0) || !std::isfinite(dt)) {
        set_error(GFS_ERR_INVALID, "delta time must be >= 0 (got %g)", dt);
        return GFS_ERR_INVALID;
    }
    switch (last_stage) {
    case GFS_STAGE_UPDATE_FLUID_CELLS: case GFS_STAGE_BODY_FORCES: case GFS_STAGE_PRESSURE:
    case GFS_STAGE_APPLY_PRESSURE: case GFS_STAGE_EXTRAPOLATE: case GFS_STAGE_ALL:
        break;
    default:
        set_error(GFS_ERR_INVALID, "stage %d is not a stop of the substep (1, 6, 7, 8, 9 or 12)", last_stage);
        return GFS_ERR_INVALID;
    }
    GFS_CUDA_CHECK(cudaEventRecord(s->ev0, st));
    gfs_step_stats local{};
    int rc = GFS_OK;
    GFS_CUDA_CHECK(cudaEventRecord(s->evp0, st));
    GFS_CUDA_CHECK(cudaEventRecord(s->evp1, st));
    do {
        // stage 1: _updateFluidCells (particle removal happened in the last sort), with
        // the queued fluid cells and the fluid sources first when there are any
        // (fluidsimulation.cpp:1990-1994)
        if (s->need_sort && (rc = sort_particles(s, true))) return rc;
        if (!s->added_cells.empty() || !s->removed_cells.empty()) {
            if ((rc = update_fluid_cell_queues(s, nullptr, nullptr))) return rc;
        }
        if (!s->sources.empty()) {
            if ((rc = update_fluid_sources(s, nullptr, nullptr))) return rc;
        }
        if (s->need_sort && (rc = sort_particles(s, true))) return rc;
        if ((rc = classify_cells(s))) return rc;
        if (last_stage == GFS_STAGE_UPDATE_FLUID_CELLS) break;
        // stage 5: velocity splat, fill, saved field, body forces (stage 6 fused)
        if ((rc = splat_velocity(s))) return rc;
        if ((rc = face_fill(s, dt))) return rc;
        int layers = (int)std::ceil(s->params.cfl + 2.0);
        if (layers > 120) layers = 120;
        if ((rc = build_layers(s, layers))) return rc;
        float *saved[3] = {s->saved[0].as<float>(), s->saved[1].as<float>(), s->saved[2].as<float>()};
        if ((rc = extrapolate_field(s, saved, layers, false))) return rc;
        if (last_stage == GFS_STAGE_BODY_FORCES) break;
        // stage 7: pressure
        GFS_CUDA_CHECK(cudaEventRecord(s->evp0, st));
        float *mac[3] = {s->mac[0].as<float>(), s->mac[1].as<float>(), s->mac[2].as<float>()};
        rc = pressure_solve(ctx, s->ps, s->g, s->mat.as<uint8_t>(), mac, s->params.density, dt,
                            s->params.precision, s->params.tol, s->params.max_cg_iterations, &local);
        if (rc) return rc;
        GFS_CUDA_CHECK(cudaEventRecord(s->evp1, st));
        if (last_stage == GFS_STAGE_PRESSURE) break;
        // stage 8, 9
        if ((rc = pressure_apply(s, dt))) return rc;
        if (last_stage == GFS_STAGE_APPLY_PRESSURE) break;
        if ((rc = extrapolate_field(s, mac, layers, false))) return rc;
        if (last_stage == GFS_STAGE_EXTRAPOLATE) break;
        // stages 11, 12
        if ((rc = g2p_advect(s, dt))) return rc;
        if ((rc = sort_particles(s, true))) return rc;
    } while (false);
    GFS_CUDA_CHECK(cudaEventRecord(s->ev1, st));
    GFS_CUDA_CHECK(cudaEventSynchronize(s->ev1));
    if (ctx->prof.on) ctx->prof.flush();
    uint32_t hnum[4];
    GFS_CUDA_CHECK(cudaMemcpy(hnum, s->num.p, sizeof(hnum), cudaMemcpyDeviceToHost));
    float ms = 0.f, pms = 0.f;
    cudaEventElapsedTime(&ms, s->ev0, s->ev1);
    cudaEventElapsedTime(&pms, s->evp0, s->evp1);
    local.num_particles = hnum[0];
    local.num_fluid_cells = hnum[2];
    local.step_ms = ms;
    local.pressure_ms = pms;
    s->last = local;
    if (stats) *stats = local;
    return GFS_OK;
}

}  // namespace gfs

using namespace gfs;

#define GFS_NONNULL(ptr)                                           \
    do {                                                           \
        if (!(ptr)) {                                              \
            set_error(GFS_ERR_INVALID, "%s must not be NULL", #ptr); \
            return GFS_ERR_INVALID;                                \
        }                                                          \
    } while (0)

extern "C" {

const char *gfs_last_error(void) { return g_err; }

const char *gfs_version(void) { return "gfs-gb300 0.1 (sm_103a)"; }

int gfs_ctx_create(int device, gfs_ctx **out) {
    GFS_NONNULL(out);
    *out = nullptr;
    int ndev = 0;
    GFS_CUDA_CHECK(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) {
        set_error(GFS_ERR_INVALID, "device %d out of range (%d devices)", device, ndev);
        return GFS_ERR_INVALID;
    }
    GFS_CUDA_CHECK(cudaSetDevice(device));
    gfs_ctx *c = new (std::nothrow) gfs_ctx();
    if (!c) {
        set_error(GFS_ERR_NOMEM, "host allocation failed");
        return GFS_ERR_NOMEM;
    }
    c->c.device = device;
    cudaDeviceProp prop;
    cudaError_t e = cudaGetDeviceProperties(&prop, device);
    if (e == cudaSuccess) {
        c->c.num_sms = prop.multiProcessorCount;
        snprintf(c->c.device_name, sizeof(c->c.device_name), "%s", prop.name);
    }
    e = cudaStreamCreateWithFlags(&c->c.stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        set_error(GFS_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
        delete c;
        return GFS_ERR_CUDA;
    }
    *out = c;
    return GFS_OK;
}

static void ctx_free(gfs_ctx *ctx) {
    cudaSetDevice(ctx->c.device);
    cudaStreamSynchronize(ctx->c.stream);
    cudaStreamDestroy(ctx->c.stream);
    delete ctx;
}

int gfs_ctx_destroy(gfs_ctx *ctx) {
    if (!ctx) return GFS_OK;
    cudaSetDevice(ctx->c.device);
    cudaStreamSynchronize(ctx->c.stream);
    ctx->closed.store(true);
    if (ctx->sims.load() == 0) ctx_free(ctx);   // else the last simulation destroyed frees it
    return GFS_OK;
}

int gfs_ctx_synchronize(gfs_ctx *ctx) {
    GFS_NONNULL(ctx);
    GFS_CUDA_CHECK(cudaStreamSynchronize(ctx->c.stream));
    return GFS_OK;
}

int gfs_ctx_stream(gfs_ctx *ctx, void **stream) {
    GFS_NONNULL(ctx);
    GFS_NONNULL(stream);
    *stream = (void *)ctx->c.stream;
    return GFS_OK;
}

int gfs_ctx_device_name(gfs_ctx *ctx, char *buf, int buflen) {
    GFS_NONNULL(ctx);
    GFS_NONNULL(buf);
    snprintf(buf, (size_t)std::max(buflen, 1), "%s", ctx->c.device_name);
    return GFS_OK;
}

int gfs_ctx_launch_count(gfs_ctx *ctx, int64_t *count) {
    GFS_NONNULL(ctx);
    GFS_NONNULL(count);
    *count = ctx->c.launches;
    return GFS_OK;
}

int gfs_ctx_set_sweep_kernel(gfs_ctx *ctx, int kind) {
    GFS_NONNULL(ctx);
    if (kind < GFS_SWEEP_AUTO || kind > GFS_SWEEP_WARP) {
        set_error(GFS_ERR_INVALID, "sweep kernel %d is not one of GFS_SWEEP_AUTO .. GFS_SWEEP_WARP", kind);
        return GFS_ERR_INVALID;
    }
    ctx->c.sweep_kernel = kind;
    return GFS_OK;
}

int gfs_ctx_last_sweep_kernel(gfs_ctx *ctx, int *kind) {
    GFS_NONNULL(ctx);
    GFS_NONNULL(kind);
    *kind = ctx->c.last_sweep_kernel;
    return GFS_OK;
}

int gfs_ctx_set_wait_limit(gfs_ctx *ctx, int64_t polls) {
    GFS_NONNULL(ctx);
    ctx->c.wait_limit = polls > 0 ? (long long)std::min<int64_t>(polls, (int64_t)1 << 30) : GFS_SPIN_LIMIT;
    return GFS_OK;
}

int gfs_ctx_inject_wait_timeout(gfs_ctx *ctx, int sweeps) {
    GFS_NONNULL(ctx);
    if (sweeps < 0) {
        set_error(GFS_ERR_INVALID, "sweeps must be >= 0 (got %d)", sweeps);
        return GFS_ERR_INVALID;
    }
    ctx->c.wait_fault_sweeps = sweeps;
    return GFS_OK;
}

int gfs_ctx_profile_enable(gfs_ctx *ctx, int on) {
    GFS_NONNULL(ctx);
    ctx->c.prof.flush();
    ctx->c.prof.on = on != 0;
    return GFS_OK;
}

int gfs_ctx_profile_reset(gfs_ctx *ctx) {
    GFS_NONNULL(ctx);
    GFS_CUDA_CHECK(cudaStreamSynchronize(ctx->c.stream));
    ctx->c.prof.reset();
    return GFS_OK;
}

int gfs_ctx_profile_read(gfs_ctx *ctx, int index, const char **name, double *total_ms, int64_t *count) {
    GFS_NONNULL(ctx);
    if (index < 0 || index >= KC_COUNT) {
        set_error(GFS_ERR_INVALID, "profile index %d outside [0, %d)", index, (int)KC_COUNT);
        return GFS_ERR_INVALID;
    }
    GFS_CUDA_CHECK(cudaStreamSynchronize(ctx->c.stream));
    ctx->c.prof.flush();
    if (name) *name = kKernelClassNames[index];
    if (total_ms) *total_ms = ctx->c.prof.ms[index];
    if (count) *count = ctx->c.prof.count[index];
    return GFS_OK;
}

int gfs_sim_default_params(gfs_sim_params *p) {
    GFS_NONNULL(p);
    p->density = 20.0;
    p->ratio_pic = (double)0.05f;
    p->cfl = 5.0;
    p->gravity[0] = 0.0f;
    p->gravity[1] = -25.0f;
    p->gravity[2] = 0.0f;
    p->max_particles_per_cell = 100;
    p->precision = GFS_PRECISION_PLAIN;
    p->tol = 1e-6;
    p->max_cg_iterations = 200;
    return GFS_OK;
}

int gfs_sim_create(gfs_ctx *ctx, int ni, int nj, int nk, double dx, int64_t max_particles, gfs_sim **out) {
    GFS_NONNULL(ctx);
    GFS_NONNULL(out);
    *out = nullptr;
    if (!valid_dims(ni, nj, nk) || !(dx > 0.0) || max_particles < 0 || max_particles > 0xFFFFFFF0LL) {
        set_error(GFS_ERR_INVALID, "invalid simulation size %d x %d x %d, dx %g, %lld particles", ni, nj, nk, dx,
                  (long long)max_particles);
        return GFS_ERR_INVALID;
    }
    GFS_CUDA_CHECK(cudaSetDevice(ctx->c.device));
    gfs_sim *s = new (std::nothrow) gfs_sim();
    if (!s) {
        set_error(GFS_ERR_NOMEM, "host allocation failed");
        return GFS_ERR_NOMEM;
    }
    s->owner = ctx;
    ctx->sims.fetch_add(1);
    int rc = sim_init(&s->s, &ctx->c, ni, nj, nk, dx, max_particles);
    if (rc) {
        gfs_sim_destroy(s);
        return rc;
    }
    *out = s;
    return GFS_OK;
}

int gfs_sim_destroy(gfs_sim *sim) {
    if (!sim) return GFS_OK;
    Sim *s = &sim->s;
    if (s->ctx) cudaStreamSynchronize(s->ctx->stream);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    if (s->evp0) cudaEventDestroy(s->evp0);
    if (s->evp1) cudaEventDestroy(s->evp1);
    gfs_ctx *owner = sim->owner;
    delete sim;
    if (owner && owner->sims.fetch_sub(1) == 1 && owner->closed.load()) ctx_free(owner);
    return GFS_OK;
}

int gfs_sim_set_params(gfs_sim *sim, const gfs_sim_params *p) {
    GFS_NONNULL(sim);
    GFS_NONNULL(p);
    if (!(p->density > 0) || !(p->cfl >= 0) || p->max_cg_iterations < 0 ||
        (p->precision != GFS_PRECISION_PLAIN && p->precision != GFS_PRECISION_MIXED)) {
        set_error(GFS_ERR_INVALID, "invalid simulation parameters");
        return GFS_ERR_INVALID;
    }
    sim->s.params = *p;
    if (sim->s.params.tol <= 0) sim->s.params.tol = 1e-6;
    return GFS_OK;
}

int gfs_sim_get_params(gfs_sim *sim, gfs_sim_params *p) {
    GFS_NONNULL(sim);
    GFS_NONNULL(p);
    *p = sim->s.params;
    return GFS_OK;
}

int gfs_sim_set_material(gfs_sim *sim, const uint8_t *h_material) {
    GFS_NONNULL(sim);
    GFS_NONNULL(h_material);
    Sim *s = &sim->s;
    DevMem stage;
    int rc = upload_padded<uint8_t>(s->ctx, h_material, s->g.c, s->mat.as<uint8_t>(), stage);
    if (rc) return rc;
    GFS_CUDA_CHECK(cudaStreamSynchronize(s->ctx->stream));
    s->need_sort = true;   // particles in new solid cells go at the next step
    return GFS_OK;
}

int gfs_sim_get_material(gfs_sim *sim, uint8_t *h_material) {
    GFS_NONNULL(sim);
    GFS_NONNULL(h_material);
    DevMem stage;
    return download_padded<uint8_t>(sim->s.ctx, sim->s.mat.as<uint8_t>(), sim->s.g.c, h_material, stage);
}

static int set_solid_cells(gfs_sim *sim, const int32_t *ijk, int n, bool solid) {
    GFS_NONNULL(sim);
    Sim *s = &sim->s;
    if (n < 0 || (n > 0 && !ijk)) {
        set_error(GFS_ERR_INVALID, "solid cell list: invalid arguments");
        return GFS_ERR_INVALID;
    }
    const int ni = s->g.ni, nj = s->g.nj, nk = s->g.nk;
    for (int q = 0; q < n; q++) {
        const int32_t *c = ijk + 3 * q;
        if (c[0] < 0 || c[1] < 0 || c[2] < 0 || c[0] >= ni || c[1] >= nj || c[2] >= nk) {
            set_error(GFS_ERR_INVALID, "solid cell index out of range: i: %d j: %d k: %d", c[0], c[1], c[2]);
            return GFS_ERR_INVALID;
        }
    }
    if (n == 0) return GFS_OK;
    std::vector<uint8_t> mat((size_t)ni * nj * nk);
    DevMem stage;
    int rc = download_padded<uint8_t>(s->ctx, s->mat.as<uint8_t>(), s->g.c, mat.data(), stage);
    if (rc) return rc;
    for (int q = 0; q < n; q++) {
        const int32_t *c = ijk + 3 * q;
        uint8_t &m = mat[(size_t)c[0] + (size_t)ni * ((size_t)c[1] + (size_t)nj * c[2])];
        if (solid) m = GFS_SOLID;
        else if (m == GFS_SOLID) m = GFS_AIR;
    }
    rc = upload_padded<uint8_t>(s->ctx, mat.data(), s->g.c, s->mat.as<uint8_t>(), stage);
    if (rc) return rc;
    GFS_CUDA_CHECK(cudaStreamSynchronize(s->ctx->stream));
    s->need_sort = true;   // particles in new solid cells go at the next step
    return GFS_OK;
}

int gfs_sim_add_solid_cells(gfs_sim *sim, const int32_t *ijk, int n) { return set_solid_cells(sim, ijk, n, true); }

int gfs_sim_remove_solid_cells(gfs_sim *sim, const int32_t *ijk, int n) { return set_solid_cells(sim, ijk, n, false); }

int gfs_sim_initialize(gfs_sim *sim, const double *points, int npoints, const double *cuboids, int ncuboids,
                       int64_t *num_particles) {
    GFS_NONNULL(sim);
    Sim *s = &sim->s;
    if (npoints < 0 || ncuboids < 0 || (npoints > 0 && !points) || (ncuboids > 0 && !cuboids)) {
        set_error(GFS_ERR_INVALID, "gfs_sim_initialize: invalid arguments");
        return GFS_ERR_INVALID;
    }
    const int ni = s->g.ni, nj = s->g.nj, nk = s->g.nk;
    if (ni < 3 || nj < 3 || nk < 3) {
        set_error(GFS_ERR_INVALID, "gfs_sim_initialize: the grid needs at least 3 cells per axis");
        return GFS_ERR_INVALID;
    }
    std::vector<uint8_t> mat((size_t)ni * nj * nk);
    DevMem stage;
    int rc = download_padded<uint8_t>(s->ctx, s->mat.as<uint8_t>(), s->g.c, mat.data(), stage);
    if (rc) return rc;
    std::vector<float> pos;
    std::vector<uint8_t> mat_out;
    rc = seed_fluid_particles(ni, nj, nk, s->g.dx, mat.data(), points, npoints, cuboids, ncuboids, s->jitter_factor,
                              s->jitter_seed, pos, &mat_out);
    if (rc) return rc;
    const int64_t n = (int64_t)(pos.size() / 3);
    if (n > s->capacity) {
        set_error(GFS_ERR_INVALID, "gfs_sim_initialize: the fluid needs %lld particles, the simulation holds %lld",
                  (long long)n, (long long)s->capacity);
        return GFS_ERR_INVALID;
    }
    rc = upload_padded<uint8_t>(s->ctx, mat_out.data(), s->g.c, s->mat.as<uint8_t>(), stage);
    if (rc) return rc;
    std::vector<float> vel(pos.size(), 0.0f);
    rc = sim_set_particles(s, pos.data(), vel.data(), nullptr, n);
    if (rc) return rc;
    if ((rc = sort_particles(s, true))) return rc;
    if ((rc = classify_cells(s))) return rc;
    GFS_CUDA_CHECK(cudaStreamSynchronize(s->ctx->stream));
    if (num_particles) *num_particles = n;
    return GFS_OK;
}

int gfs_sim_set_particles(gfs_sim *sim, const float *h_positions, const float *h_velocities,
                          const uint32_t *h_ids, int64_t n) {
    GFS_NONNULL(sim);
    int rc = sim_set_particles(&sim->s, h_positions, h_velocities, h_ids, n);
    if (rc) return rc;
    if ((rc = sort_particles(&sim->s, true))) return rc;
    // cells holding particles are fluid, as after the reference's initialisation
    // (FluidSimulation::_initializeFluidMaterial, fluidsimulation.cpp:1383), so that
    // fluid sources see them as fluid
    return classify_cells(&sim->s);
}

int gfs_sim_num_particles(gfs_sim *sim, int64_t *n) {
    GFS_NONNULL(sim);
    GFS_NONNULL(n);
    return sim_get_particles(&sim->s, nullptr, nullptr, nullptr, n);
}

int gfs_sim_get_particles(gfs_sim *sim, float *h_positions, float *h_velocities, uint32_t *h_ids, int64_t *n) {
    GFS_NONNULL(sim);
    return sim_get_particles(&sim->s, h_positions, h_velocities, h_ids, n);
}

int gfs_sim_get_velocity_field(gfs_sim *sim, float *h_u, float *h_v, float *h_w) {
    GFS_NONNULL(sim);
    Sim *s = &sim->s;
    float *h[3] = {h_u, h_v, h_w};
    DevMem stage;
    for (int d = 0; d < 3; d++) {
        if (!h[d]) continue;
        int rc = download_padded<float>(s->ctx, s->mac[d].as<float>(), s->g.f[d], h[d], stage);
        if (rc) return rc;
    }
    return GFS_OK;
}

int gfs_sim_get_pressure_grid(gfs_sim *sim, float *h_pressure) {
    GFS_NONNULL(sim);
    GFS_NONNULL(h_pressure);
    Sim *s = &sim->s;
    if (s->ps.allocated_for < 0) {
        memset(h_pressure, 0, sizeof(float) * (size_t)s->g.ni * s->g.nj * s->g.nk);
        return GFS_OK;
    }
    size_t n = (size_t)s->g.ni * s->g.nj * s->g.nk;
    if (s->pgrid.ensure(n * sizeof(float))) return GFS_ERR_NOMEM;
    int rc = pressure_to_grid(s->ctx, s->ps, s->g, s->pgrid.as<float>());
    if (rc) return rc;
    GFS_CUDA_CHECK(cudaMemcpyAsync(h_pressure, s->pgrid.p, n * sizeof(float), cudaMemcpyDeviceToHost, s->ctx->stream));
    GFS_CUDA_CHECK(cudaStreamSynchronize(s->ctx->stream));
    return GFS_OK;
}

int gfs_sim_get_saved_velocity_field(gfs_sim *sim, float *h_u, float *h_v, float *h_w) {
    GFS_NONNULL(sim);
    Sim *s = &sim->s;
    float *h[3] = {h_u, h_v, h_w};
    DevMem stage;
    for (int d = 0; d < 3; d++) {
        if (!h[d]) continue;
        int rc = download_padded<float>(s->ctx, s->saved[d].as<float>(), s->g.f[d], h[d], stage);
        if (rc) return rc;
    }
    return GFS_OK;
}

int gfs_sim_step(gfs_sim *sim, double dt, gfs_step_stats *stats) {
    GFS_NONNULL(sim);
    return sim_step(&sim->s, dt, stats);
}

int gfs_sim_step_stages(gfs_sim *sim, double dt, int last_stage, gfs_step_stats *stats) {
    GFS_NONNULL(sim);
    return sim_step(&sim->s, dt, stats, last_stage);
}

int gfs_sim_step_host(gfs_sim *sim, double dt, float *h_positions, float *h_velocities, uint32_t *h_ids,
                      int64_t *n, gfs_step_stats *stats) {
    GFS_NONNULL(sim);
    GFS_NONNULL(n);
    GFS_NONNULL(h_positions);
    GFS_NONNULL(h_velocities);
    Sim *s = &sim->s;
    int rc = sim_set_particles(s, h_positions, h_velocities, h_ids, *n);
    if (rc) return rc;
    rc = sim_step(s, dt, stats);
    if (rc) return rc;
    std::vector<uint32_t> tmp;
    uint32_t *ids = h_ids;
    if (!ids) {
        tmp.resize((size_t)std::max<int64_t>(*n, 1));
        ids = tmp.data();
    }
    return sim_get_particles(s, h_positions, h_velocities, ids, n);
}

// ---------------------------------------------------------- standalone

int gfs_velocity_scalar_field(gfs_ctx *ctx, int dir, int ni, int nj, int nk, double dx,
                              const float *h_positions, const float *h_velocities, int64_t n, float *h_field,
                              uint8_t *h_is_set) {
    GFS_NONNULL(ctx);
    GFS_NONNULL(h_field);
    GFS_NONNULL(h_is_set);
    if (dir < 0 || dir > 2 || !valid_dims(ni, nj, nk) || !(dx > 0) || n < 0 || (n > 0 && (!h_positions || !h_velocities))) {
        set_error(GFS_ERR_INVALID, "invalid velocity splat arguments");
        return GFS_ERR_INVALID;
    }
    gfs_sim *sim = nullptr;
    int rc = gfs_sim_create(ctx, ni, nj, nk, dx, n, &sim);
    if (rc) return rc;
    Sim *s = &sim->s;
    rc = sim_set_particles(s, h_positions, h_velocities, nullptr, n);
    if (!rc) rc = sort_particles(s, false);
    if (!rc) rc = splat_velocity(s);
    DevMem stage;
    if (!rc) rc = download_padded<float>(&ctx->c, s->sval[dir].as<float>(), s->g.f[dir], h_field, stage);
    if (!rc) rc = download_padded<uint8_t>(&ctx->c, s->smask[dir].as<uint8_t>(), s->g.f[dir], h_is_set, stage);
    gfs_sim_destroy(sim);
    return rc;
}

static int stage_mac(Ctx *ctx, const Grids &g, const float *hu, const float *hv, const float *hw, DevMem dm[3],
                     DevMem &stage) {
    const float *h[3] = {hu, hv, hw};
    for (int d = 0; d < 3; d++) {
        if (dm[d].alloc((size_t)g.f[d].size * sizeof(float))) return GFS_ERR_NOMEM;
        GFS_CUDA_CHECK(cudaMemsetAsync(dm[d].p, 0, dm[d].bytes, ctx->stream));
        int rc = upload_padded<float>(ctx, h[d], g.f[d], dm[d].as<float>(), stage);
        if (rc) return rc;
    }
    return GFS_OK;
}

static int points_common(gfs_ctx *ctx, int order, int ni, int nj, int nk, double dx, const float *hu,
                         const float *hv, const float *hw, double dt, const float *hp, int64_t n, float *hout,
                         bool validate) {
    GFS_NONNULL(ctx);
    if (!valid_dims(ni, nj, nk) || !(dx > 0) || n < 0 || !hu || !hv || !hw || (n > 0 && (!hp || !hout))) {
        set_error(GFS_ERR_INVALID, "invalid interpolation arguments");
        return GFS_ERR_INVALID;
    }
    Ctx *c = &ctx->c;
    Grids g = make_grids(ni, nj, nk, dx);
    DevMem dm[3], stage, dp, dout;
    int rc = stage_mac(c, g, hu, hv, hw, dm, stage);
    if (rc) return rc;
    if (n == 0) return GFS_OK;
    if (dp.alloc((size_t)n * 3 * sizeof(float)) || dout.alloc((size_t)n * 3 * sizeof(float))) return GFS_ERR_NOMEM;
    GFS_CUDA_CHECK(cudaMemcpyAsync(dp.p, hp, (size_t)n * 3 * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    float *mac[3] = {dm[0].as<float>(), dm[1].as<float>(), dm[2].as<float>()};
    rc = interpolate_points(c, g, mac, dp.as<float>(), n, dout.as<float>(), order, dt, validate);
    if (rc) return rc;
    GFS_CUDA_CHECK(cudaMemcpyAsync(hout, dout.p, (size_t)n * 3 * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    GFS_CUDA_CHECK(cudaStreamSynchronize(c->stream));
    return GFS_OK;
}

int gfs_tricubic_interpolate(gfs_ctx *ctx, int ni, int nj, int nk, double dx, const float *h_u, const float *h_v,
                             const float *h_w, const float *h_points, int64_t n, float *h_out) {
    return points_common(ctx, 0, ni, nj, nk, dx, h_u, h_v, h_w, 0.0, h_points, n, h_out, true);
}

int gfs_advect_particles(gfs_ctx *ctx, int order, int ni, int nj, int nk, double dx, const float *h_u,
                         const float *h_v, const float *h_w, double dt, const float *h_points, int64_t n,
                         float *h_out) {
    if (order < 1 || order > 4) {
        set_error(GFS_ERR_INVALID, "Runge-Kutta order must be 1..4 (got %d)", order);
        return GFS_ERR_INVALID;
    }
    return points_common(ctx, order, ni, nj, nk, dx, h_u, h_v, h_w, dt, h_points, n, h_out, false);
}

int gfs_pressure_solve(gfs_ctx *ctx, int ni, int nj, int nk, double dx, double density, double dt,
                       const uint8_t *h_material, const float *h_u, const float *h_v, const float *h_w, int precision,
                       double tol, int max_iters, double *h_pressure, int64_t *num_fluid_cells, int *iterations,
                       double *max_residual) {
    GFS_NONNULL(ctx);
    GFS_NONNULL(h_material);
    GFS_NONNULL(num_fluid_cells);
    if (!valid_dims(ni, nj, nk) || !(dx > 0) || !(density > 0) || !(dt >= 0) ||
        (precision != GFS_PRECISION_PLAIN && precision != GFS_PRECISION_MIXED)) {
        set_error(GFS_ERR_INVALID, "invalid pressure-solve arguments");
        return GFS_ERR_INVALID;
    }
    size_t ncell = (size_t)ni * nj * nk;
    int64_t F = 0;
    for (size_t q = 0; q < ncell; q++) F += h_material[q] == GFS_FLUID;
    if (!h_pressure) {
        *num_fluid_cells = F;
        return GFS_OK;
    }
    if (*num_fluid_cells < F) {
        set_error(GFS_ERR_INVALID, "pressure array holds %lld entries, %lld fluid cells", (long long)*num_fluid_cells,
                  (long long)F);
        return GFS_ERR_INVALID;
    }
    if (!h_u || !h_v || !h_w) {
        set_error(GFS_ERR_INVALID, "velocity field pointers must not be NULL");
        return GFS_ERR_INVALID;
    }
    *num_fluid_cells = F;
    if (tol <= 0) tol = 1e-6;
    if (max_iters <= 0) max_iters = 200;
    Ctx *c = &ctx->c;
    Grids g = make_grids(ni, nj, nk, dx);
    DevMem dm[3], stage, mat, dout;
    int rc = stage_mac(c, g, h_u, h_v, h_w, dm, stage);
    if (rc) return rc;
    if (mat.alloc((size_t)g.c.size)) return GFS_ERR_NOMEM;
    GFS_CUDA_CHECK(cudaMemsetAsync(mat.p, GFS_SOLID, mat.bytes, c->stream));
    rc = upload_padded<uint8_t>(c, h_material, g.c, mat.as<uint8_t>(), stage);
    if (rc) return rc;
    PressureWs ws;
    float *mac[3] = {dm[0].as<float>(), dm[1].as<float>(), dm[2].as<float>()};
    gfs_step_stats st{};
    rc = pressure_solve(c, ws, g, mat.as<uint8_t>(), mac, density, dt, precision, tol, max_iters, &st);
    if (rc) return rc;
    if (iterations) *iterations = st.cg_iterations;
    if (max_residual) *max_residual = st.cg_max_residual;
    if (F > 0) {
        if (dout.alloc((size_t)F * sizeof(double))) return GFS_ERR_NOMEM;
        rc = pressure_gather_compact(c, ws, g, mat.as<uint8_t>(), dout.as<double>(), F);
        if (rc) return rc;
        GFS_CUDA_CHECK(cudaMemcpyAsync(h_pressure, dout.p, (size_t)F * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        GFS_CUDA_CHECK(cudaStreamSynchronize(c->stream));
    }
    return GFS_OK;
}

int gfs_sim_pressure_check(gfs_sim *sim, double dt, double rel_tol, double *fp64_residual, double *rel_error,
                           int *ref_iterations) {
    GFS_NONNULL(sim);
    Sim *s = &sim->s;
    if (!(dt > 0.0) || !(rel_tol > 0.0)) {
        set_error(GFS_ERR_INVALID, "dt and rel_tol must be > 0");
        return GFS_ERR_INVALID;
    }
    return pressure_check(s->ctx, s->ps, s->g, s->params.density, dt, rel_tol, fp64_residual, rel_error,
                          ref_iterations);
}

// ------------------------------------------------ differentiable rollout

struct gfs_diff {
    gfs::DiffRun *d = nullptr;
};

int gfs_diff_create(gfs_sim *sim, int nsteps, int64_t n, double dt, gfs_diff **out) {
    GFS_NONNULL(sim);
    GFS_NONNULL(out);
    *out = nullptr;
    DiffRun *d = nullptr;
    int rc = diff_create(&sim->s, nsteps, (long long)n, dt, &d);
    if (rc) return rc;
    gfs_diff *h = new gfs_diff();
    h->d = d;
    *out = h;
    return GFS_OK;
}

int gfs_diff_destroy(gfs_diff *d) {
    if (!d) return GFS_OK;
    diff_destroy(d->d);
    delete d;
    return GFS_OK;
}

int gfs_diff_forward(gfs_diff *d, const float *d_positions, const float *d_velocities, const float *d_u0,
                     const float *d_v0, const float *d_w0, float *d_density, float *d_centroids) {
    GFS_NONNULL(d);
    GFS_NONNULL(d_positions);
    if (!d_velocities && (!d_u0 || !d_v0 || !d_w0)) {
        set_error(GFS_ERR_INVALID, "give initial velocities or the parameter field (u0, v0, w0)");
        return GFS_ERR_INVALID;
    }
    const float *u0[3] = {d_u0, d_v0, d_w0};
    return diff_forward(d->d, d_positions, d_velocities, u0, d_density, d_centroids);
}

int gfs_diff_backward(gfs_diff *d, const float *d_grad_density, const float *d_grad_centroids, float *d_grad_u0,
                      float *d_grad_v0, float *d_grad_w0, float *d_grad_velocities, float *d_grad_positions) {
    GFS_NONNULL(d);
    if ((d_grad_u0 || d_grad_v0 || d_grad_w0) && !(d_grad_u0 && d_grad_v0 && d_grad_w0)) {
        set_error(GFS_ERR_INVALID, "the parameter-field gradient needs all three of u0, v0, w0");
        return GFS_ERR_INVALID;
    }
    float *g[3] = {d_grad_u0, d_grad_v0, d_grad_w0};
    return diff_backward(d->d, d_grad_density, d_grad_centroids, g, d_grad_velocities, d_grad_positions);
}

int gfs_diff_info(gfs_diff *d, double *forward_ms, double *backward_ms, int64_t *device_bytes) {
    GFS_NONNULL(d);
    long long b = 0;
    diff_info(d->d, forward_ms, backward_ms, &b);
    if (device_bytes) *device_bytes = b;
    return GFS_OK;
}

int gfs_sim_add_marker_particle_points(gfs_sim *sim, double radius, const float offset[3], double dx, int W,
                                       int H, int D, float *h_field, int threshold_set, double threshold) {
    GFS_NONNULL(sim);
    GFS_NONNULL(offset);
    GFS_NONNULL(h_field);
    const long long nodes = (long long)W * H * D;
    if (W <= 0 || H <= 0 || D <= 0 || nodes >= 0xFFFFFFFFll || !(dx > 0) || !(radius > 0) || !std::isfinite(radius)) {
        set_error(GFS_ERR_INVALID, "invalid point splat arguments (W=%d H=%d D=%d dx=%g radius=%g)", W, H, D, dx,
                  radius);
        return GFS_ERR_INVALID;
    }
    Sim *s = &sim->s;
    Ctx *c = s->ctx;
    int64_t n = 0;
    int rc = sim_stage_xyz(s, &n);   // the resident particles as xyz triples, in the simulation's scratch
    if (rc) return rc;
    if (n == 0) return GFS_OK;
    DevMem df;
    const size_t fbytes = (size_t)nodes * sizeof(float);
    if (df.alloc(fbytes)) return GFS_ERR_NOMEM;
    GFS_CUDA_CHECK(cudaMemcpyAsync(df.p, h_field, fbytes, cudaMemcpyHostToDevice, c->stream));
    rc = splat_points(c, s->pos_alt.as<float>(), nullptr, n, radius, offset, dx, W, H, D, df.as<float>(), nullptr,
                      threshold_set != 0, (float)threshold);
    if (rc) return rc;
    GFS_CUDA_CHECK(cudaMemcpyAsync(h_field, df.p, fbytes, cudaMemcpyDeviceToHost, c->stream));
    GFS_CUDA_CHECK(cudaStreamSynchronize(c->stream));
    return GFS_OK;
}

int gfs_scalar_field_add_point_values(gfs_ctx *ctx, const float *h_points, const float *h_values, int64_t n,
                                      double radius, const float offset[3], double dx, int W, int H, int D,
                                      float *h_scalarfield, float *h_weightfield, int threshold_set,
                                      double threshold) {
    GFS_NONNULL(ctx);
    GFS_NONNULL(offset);
    GFS_NONNULL(h_scalarfield);
    const long long nodes = (long long)W * H * D;
    if (W <= 0 || H <= 0 || D <= 0 || nodes >= 0xFFFFFFFFll || !(dx > 0) || !(radius > 0) ||
        !std::isfinite(radius) || n < 0 || n > 0x7FFFFFFFll || (n > 0 && !h_points)) {
        set_error(GFS_ERR_INVALID, "invalid point splat arguments (W=%d H=%d D=%d dx=%g radius=%g n=%lld)", W, H, D,
                  dx, radius, (long long)n);
        return GFS_ERR_INVALID;
    }
    if (n == 0) return GFS_OK;
    Ctx *c = &ctx->c;
    DevMem dp, dv, df, dw;
    const size_t fbytes = (size_t)nodes * sizeof(float);
    if (dp.alloc((size_t)n * 3 * sizeof(float)) || (h_values && dv.alloc((size_t)n * sizeof(float))) ||
        df.alloc(fbytes) || (h_weightfield && dw.alloc(fbytes)))
        return GFS_ERR_NOMEM;
    GFS_CUDA_CHECK(cudaMemcpyAsync(dp.p, h_points, (size_t)n * 3 * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    if (h_values)
        GFS_CUDA_CHECK(cudaMemcpyAsync(dv.p, h_values, (size_t)n * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    GFS_CUDA_CHECK(cudaMemcpyAsync(df.p, h_scalarfield, fbytes, cudaMemcpyHostToDevice, c->stream));
    if (h_weightfield) GFS_CUDA_CHECK(cudaMemcpyAsync(dw.p, h_weightfield, fbytes, cudaMemcpyHostToDevice, c->stream));
    int rc = splat_points(c, dp.as<float>(), h_values ? dv.as<float>() : nullptr, n, radius, offset, dx, W, H, D,
                          df.as<float>(), h_weightfield ? dw.as<float>() : nullptr, threshold_set != 0,
                          (float)threshold);
    if (rc) return rc;
    GFS_CUDA_CHECK(cudaMemcpyAsync(h_scalarfield, df.p, fbytes, cudaMemcpyDeviceToHost, c->stream));
    if (h_weightfield) GFS_CUDA_CHECK(cudaMemcpyAsync(h_weightfield, dw.p, fbytes, cudaMemcpyDeviceToHost, c->stream));
    GFS_CUDA_CHECK(cudaStreamSynchronize(c->stream));
    return GFS_OK;
}

}  // extern "C"
