// gfs_internal.h -- host-side structures shared by the libgfs translation units.
#pragma once

#include <atomic>

#include <cstdarg>
#include <cstdint>
#include <vector>
#include <cuda_runtime.h>

#include "gfs.h"
#include "gfs_common.cuh"

namespace gfs {

void set_error(int code, const char *fmt, ...);

// A device allocation that frees itself.
struct DevMem {
    void *p = nullptr;
    size_t bytes = 0;
    int alloc(size_t n);          // GFS_OK or GFS_ERR_NOMEM (sets the message)
    int ensure(size_t n);         // grow-only
    void release();
    ~DevMem() { release(); }
    template <class T> T *as() const { return static_cast<T *>(p); }
};

// Kernel classes timed by the optional profiler (CUDA events on the stream).
enum KernelClass {
    KC_SORT = 0, KC_CLASSIFY, KC_SPLAT, KC_FILL, KC_LAYERS, KC_EXTRAP, KC_PS_SETUP, KC_PRECON,
    KC_SWEEP_FWD, KC_SWEEP_BWD, KC_MATVEC, KC_AXPY, KC_UPDATE_S, KC_MIXED_AUX, KC_APPLY, KC_G2P,
    KC_COUNT
};
extern const char *const kKernelClassNames[KC_COUNT];

struct Profiler {
    bool on = false;
    struct Rec { int cls; cudaEvent_t a, b; };
    std::vector<Rec> pending;
    std::vector<cudaEvent_t> pool;
    double ms[KC_COUNT] = {0};
    long long count[KC_COUNT] = {0};
    int open_cls = -1;
    cudaEvent_t open_ev = nullptr;
    cudaEvent_t take();
    void begin(cudaStream_t st, int cls);
    void end(cudaStream_t st, int cls);
    void flush();     // waits for the recorded events and accumulates their times
    void reset();
    ~Profiler();
};

struct Ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    int64_t launches = 0;
    char device_name[256] = {0};
    Profiler prof;
    // wavefront kernels of the MIC(0) triangular solves (GFS_SWEEP_*): the one
    // asked for, and the one the last solve ran
    int sweep_kernel = GFS_SWEEP_AUTO;
    int last_sweep_kernel = GFS_SWEEP_AUTO;
    // bound of every wavefront wait, in polls, and the number of coming sweeps
    // whose waits look for an exchange tag that no producer writes
    long long wait_limit = GFS_SPIN_LIMIT;
    int wait_fault_sweeps = 0;
};

// Scoped timing of one kernel class (no-op unless the profiler is on).
struct ProfScope {
    Ctx *c;
    int cls;
    ProfScope(Ctx *ctx, int k) : c(ctx), cls(k) { if (c->prof.on) c->prof.begin(c->stream, cls); }
    ~ProfScope() { if (c->prof.on) c->prof.end(c->stream, cls); }
};

// Controls of the pressure solve, kept in device memory so that the CG loop
// needs no host round trip per iteration.
struct PsCtrl {
    double sigma, alpha, beta;   // CG scalars
    double maxb;                 // max|b|
    double maxr;                 // max|r| of the iteration (FP64 for PLAIN, FP32 r promoted for MIXED inner)
    double maxr64;               // MIXED: FP64 max|b - A p| of the last refinement
    double inner_tol;            // MIXED: inner stopping threshold
    double tol;
    int iter;                    // CG iteration number (reference numbering)
    int max_iters;
    int done;                    // loop finished (converged or capped)
    int converged;
    int total_inner;             // MIXED: inner iterations so far
    int refinements;
    unsigned err;                // GFS_DEV_ERR_* bits
    unsigned tickets[4];         // last-block-done tickets of fused reductions
    unsigned sweep_ticket[3];    // dispatch tickets of the wavefront kernels, by kind (precon, fwd, bwd)
    unsigned epoch;              // tag of the current wavefront's exchange words
};

// Pressure workspace.  flags / b / p are dense over the padded cell grid; the
// solver's vectors use the skewed block layout of pressure.cu (skew_size slots).
struct PressureWs {
    GridDim c{};
    int nbj = 0, nbk = 0;        // wavefront block grid
    long long skew_size = 0;
    DevMem flags, b, p;          // padded cell layout: uint8, FP64, FP64 (the solution)
    DevMem fsk;                  // skewed flags
    DevMem bsk, psk, r, z, s, As, q, precon;        // FP64, skewed
    DevMem mpc;                  // FP64 negscale * precon (the FP64 block solves read it)
    DevMem r32, z32, s32, As32, q32, e32, precon32; // FP32 (mixed), skewed
    DevMem partials;             // double per block
    DevMem ctrl;                 // PsCtrl
    DevMem xch;                  // block-boundary exchange words of the wavefronts
    DevMem nbstd, nbsk;          // MIC(0) neighbour bits, padded cell and skewed layouts
    DevMem blkf;                 // per skew block: 1 if it holds a fluid cell
    DevMem slist, soff, stmp;    // strips holding fluid (uint32 indices, in order); per-strip scan, scan temp
    DevMem snum;                 // uint32: the length of slist
    size_t nblocks_red = 0;      // blocks of the reduction kernels
    long long allocated_for = -1;
    bool mixed_alloc = false;
};

struct Sim {
    Ctx *ctx = nullptr;
    Grids g{};
    gfs_sim_params params{};
    int64_t capacity = 0;
    int64_t n_bound = 0;         // host-side upper bound of the particle count
    bool need_sort = false;      // particles not yet in (cell, id) order
    bool sorted_hint = false;    // uploaded set may already be in order: the next sort checks first
    bool dx_pow2 = false;
    float inv_dx_f = 0.f;
    float bound_f[3] = {0, 0, 0}; // smallest floats >= dx*n (exact in-grid test)

    DevMem mat;                  // uint8 padded cell grid
    DevMem mac[3], saved[3];     // float padded face grids
    DevMem quad[3];              // float4 row quads of mac, rebuilt for each G2P pass
    DevMem sval[3], smask[3];    // splat value / is-set mask
    DevMem layer;                // int8 padded cell grid
    DevMem lcells, lcnt;         // cells of each extrapolation layer (storage indices, layer by layer); counts
    DevMem pos, vel, pos_alt, vel_alt;   // float4 x capacity
    DevMem key, slot;            // uint32 x capacity
    DevMem count, offset, scan_tmp;      // uint32 x (ncells + 1), scan block sums
    DevMem num;                  // uint32[4]: [0] particle count, [1] overflow flag
    DevMem pgrid;                // float pressure grid (unpadded) for get_pressure
    PressureWs ps;
    std::vector<gfs_fluid_source> sources;   // FluidSimulation::_fluidSources
    double jitter_factor = 0.1;              // _markerParticleJitterFactor (fluidsimulation.h:1111)
    unsigned long long jitter_seed = 0;
    uint32_t next_id = 0;                    // first id not yet given to a particle
    bool next_id_valid = true;               // false: recompute from the particles' ids
    DevMem src_mark, src_a, src_b, src_tmp;  // fluid-source work buffers
    // FluidSimulation::_addedFluidCellQueue / _removedFluidCellQueue
    // (fluidsimulation.h:1108-1109): cell triples (i, j, k), applied at the next step
    struct CellGroup {
        std::vector<int32_t> ijk;
        float vel[3];
    };
    std::vector<CellGroup> added_cells;
    std::vector<int32_t> removed_cells;
    gfs_step_stats last{};
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, evp0 = nullptr, evp1 = nullptr;
};

// ---- particles.cu
int sort_particles(Sim *s, bool remove_solid);
int classify_cells(Sim *s);
int exclusive_scan_u32(Ctx *ctx, uint32_t *data_in, uint32_t *data_out, long long n,
                       uint32_t *block_sums, cudaStream_t st);
size_t scan_temp_elems(long long n);

// ---- splat.cu
int splat_velocity(Sim *s, float *const wsum[3] = nullptr);   // P2G for U, V, W into sval/smask (+ weight sums)
int face_fill(Sim *s, double dt);     // a3 + saved copy + body forces

// ---- capi.cu
// one device-resident substep, or its stages up to last_stage (GFS_STAGE_*)
int sim_step(Sim *s, double dt, gfs_step_stats *stats, int last_stage = GFS_STAGE_ALL);
int sim_stage_xyz(Sim *s, int64_t *n_out);   // particles -> xyz triples in pos_alt / vel_alt (ids in key)
int sim_unstage_xyz(Sim *s, int64_t n);      // n staged triples (ids 0..n-1) -> particles, sorted

// ---- seeding.cu: FluidSimulation::_initializeFluidMaterial on the host (points: x y z r,
// cuboids: x y z w h d); the material gets the solid border; out: xyz triples
int seed_fluid_particles(int ni, int nj, int nk, double dx, const uint8_t *mat_in, const double *points,
                         int npoints, const double *cuboids, int ncuboids, double jitter_factor,
                         unsigned long long seed, std::vector<float> &out, std::vector<uint8_t> *mat_out);

// ---- sources.cu
int update_fluid_sources(Sim *s, int64_t *added, int64_t *removed);   // _updateFluidSources
// _updateAddedFluidCellQueue + _updateRemovedFluidCellQueue
int update_fluid_cell_queues(Sim *s, int64_t *added, int64_t *removed);

// ---- adjoint.cu: the differentiable rollout
struct DiffRun;
int diff_create(Sim *s, int nsteps, long long n, double dt, DiffRun **out);
void diff_destroy(DiffRun *d);
int diff_forward(DiffRun *d, const float *d_pos, const float *d_vel0, const float *const d_u0[3], float *d_density,
                 float *d_centroids);
int diff_backward(DiffRun *d, const float *d_rho_bar, const float *d_grad_centroids, float *const d_grad[3],
                  float *d_grad_vel0, float *d_grad_pos0);
void diff_info(DiffRun *d, double *fwd_ms, double *bwd_ms, long long *bytes);

// ---- pointsplat.cu
// General weighted point splat on a W x H x D node grid (device buffers; d_vals
// NULL = value 1, d_weight may be NULL).  Adds into d_field / d_weight.
int splat_points(Ctx *ctx, const float *d_pts, const float *d_vals, long long n, double radius,
                 const float offset[3], double dx, int W, int H, int D, float *d_field, float *d_weight,
                 bool thr_set, float thr);

// ---- extrapolate.cu
#define GFS_MAX_LAYERS 126       // layers fit in the int8 layer grid
int build_layers(Sim *s, int num_layers);
int extrapolate_field(Sim *s, float *const f[3], int num_layers, bool reset);

// ---- pressure.cu
int pressure_solve(Ctx *ctx, PressureWs &ws, const Grids &g, const uint8_t *mat,
                   float *const mac[3], double density, double dt, int precision, double tol,
                   int max_iters, gfs_step_stats *stats);
// Accuracy of the last solve on this workspace: FP64 residual max|b - A p| of its
// solution, and max|p - p_ref| / max|p_ref| against an FP64 PCG solve of the same
// system to rel_tol (the workspace's pressure is left as it was).
int pressure_check(Ctx *ctx, PressureWs &ws, const Grids &g, double density, double dt, double rel_tol,
                   double *fp64_residual, double *rel_error, int *ref_iterations);
// The system's flags, b and neighbour bits only (no solve).
int pressure_setup(Ctx *ctx, PressureWs &ws, const Grids &g, const uint8_t *mat, float *const mac[3]);
// Solve A x = rhs (padded cell layout, FP64) on the matrix of the last
// pressure_solve on this workspace, to max|r| < rel_tol * max|rhs|; the
// solution is left in ws.p.
int pressure_solve_rhs(Ctx *ctx, PressureWs &ws, const Grids &g, const double *rhs, double density, double dt,
                       double rel_tol, int max_iters, gfs_step_stats *stats, bool mixed = false);
int pressure_apply(Sim *s, double dt);
int pressure_to_grid(Ctx *ctx, PressureWs &ws, const Grids &g, float *pgrid_unpadded);
int pressure_gather_compact(Ctx *ctx, PressureWs &ws, const Grids &g, const uint8_t *mat,
                            double *d_out, int64_t F);

// ---- advect.cu
int g2p_advect(Sim *s, double dt);
int interpolate_points(Ctx *ctx, const Grids &g, float *const mac[3], const float *d_points,
                       int64_t n, float *d_out, int rk_order, double dt, bool validate);

}  // namespace gfs

// A context stays allocated while simulations built on it are alive: destroying
// it only marks it closed, and the last simulation destroyed frees it.
struct gfs_ctx {
    gfs::Ctx c;
    std::atomic<int> sims{0};
    std::atomic<bool> closed{false};
};

struct gfs_sim {
    gfs::Sim s;
    gfs_ctx *owner = nullptr;
};
