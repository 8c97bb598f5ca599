// pressure.cu -- MICCG(0) pressure projection (PressureSolver, pressuresolver.cpp)
// and the pressure update of the MAC field.
//
// Layout: every vector is dense over the padded cell grid (GridDim), zero on
// non-fluid cells and on the halo.  A one-byte flag per cell holds "fluid" and
// the MatrixCell diagonal (number of non-solid neighbours).  With zeros off the
// fluid set, the reference's keymap lookups (found -> value, not found -> 0)
// become plain 7-point stencils, and every per-cell formula keeps the
// reference's operation order; the FP64 (PLAIN) kernels use explicitly rounded
// intrinsics (no FMA contraction), so the preconditioner, the stencil and the
// triangular solves reproduce the reference's doubles bit for bit.  Only the
// dot products differ (parallel summation order).
//
// MIC(0) triangular solves.  The forward solve L q = r and the build of the
// preconditioner are recurrences over i-1, j-1, k-1; the backward solve over
// i+1, j+1, k+1 (pressuresolver.cpp:246-386).  A cell depends only on cells of
// a lower i+j+k plane, so a wavefront reproduces the sequential result.  Each
// CTA owns a BJ x BK block of (j, k) pencils, one thread per pencil, and walks
// i: at step s thread (jl, kl) updates cell i = s - jl - kl.  The j-1 / k-1
// neighbours were produced by the adjacent threads at step s-1 (shared-memory
// exchange, one barrier per step), i-1 by the thread itself.  Neighbouring
// CTAs exchange their boundary rows through global memory: a CTA publishes how
// many steps it has completed (st.release) and a consumer waits (ld.acquire,
// bounded spin) only when it has caught up with its producer, so the CTAs form
// a pipeline over the (j, k) block grid.  CTAs take dispatch tickets in
// dependency order, so every CTA they wait for is already resident.
//
// The CG loop runs on the device: each kernel first checks a device "done"
// flag, reductions finish in the last CTA to arrive (fixed order, so results
// are deterministic), and the host only polls the flag every few iterations.
#include <cstring>

#include "gfs_internal.h"

namespace gfs {

// ------------------------------------------------------------ arithmetic

template <class T> struct Ar;
template <> struct Ar<double> {
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
};
template <> struct Ar<float> {
    static __device__ __forceinline__ float mul(float a, float b) { return a * b; }
    static __device__ __forceinline__ float add(float a, float b) { return a + b; }
    static __device__ __forceinline__ float sub(float a, float b) { return a - b; }
};

template <class T> __device__ __forceinline__ T ldcg(const T *p) { return __ldcg(p); }

#define RED_THREADS 256

template <int OP>  // 0 = sum, 1 = max
__device__ __forceinline__ double block_reduce(double v) {
    __shared__ double sh[32];
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int nw = (blockDim.x * blockDim.y * blockDim.z + 31) >> 5;
    int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    lane = tid & 31;
    warp = tid >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        double y = __shfl_down_sync(0xffffffffu, v, o);
        v = OP == 0 ? v + y : fmax(v, y);
    }
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    if (warp == 0) {
        v = lane < nw ? sh[lane] : (OP == 0 ? 0.0 : 0.0);
        for (int o = 16; o > 0; o >>= 1) {
            double y = __shfl_down_sync(0xffffffffu, v, o);
            v = OP == 0 ? v + y : fmax(v, y);
        }
    }
    __syncthreads();
    return v;  // valid in thread 0
}

// Last-CTA-done reduction: every CTA writes its partial, the last CTA to take a
// ticket combines all partials in index order.  Returns true in the last CTA
// (thread 0 holds *out).
template <int OP>
__device__ __forceinline__ bool finish_reduce(double part, double *partials, unsigned *ticket,
                                              unsigned nblocks, double *out) {
    __shared__ bool last;
    int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    int nthr = blockDim.x * blockDim.y * blockDim.z;
    unsigned bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    if (tid == 0) {
        partials[bid] = part;
        __threadfence();
        unsigned t = atomicAdd(ticket, 1u);
        last = (t == nblocks - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double acc = 0.0;
    // fixed assignment of partials to threads, fixed tree: deterministic
    for (unsigned q = tid; q < nblocks; q += nthr) {
        double v = __ldcg(partials + q);
        acc = OP == 0 ? acc + v : fmax(acc, v);
    }
    acc = block_reduce<OP>(acc);
    if (tid == 0) {
        *out = acc;
        *ticket = 0;
    }
    return true;
}

// ------------------------------------------------------------------ setup

struct SetupArgs {
    GridDim c, fu, fv, fw;
    float fscale;        // (float)(1.0f / (float)dx)
    double scale_div;    // 1.0f / (float)dx as double (pressuresolver.cpp:164)
    double tol;
};

// _calculateNegativeDivergenceVector (pressuresolver.cpp:162-208) and
// _calculateMatrixCoefficients (:222-244) for one cell; also resets p, r, s.
__global__ void __launch_bounds__(RED_THREADS) k_ps_setup(SetupArgs A, const uint8_t *__restrict__ mat,
                                                          const float *__restrict__ u, const float *__restrict__ v,
                                                          const float *__restrict__ w, uint8_t *__restrict__ flags,
                                                          double *__restrict__ b, double *__restrict__ r,
                                                          double *__restrict__ p, double *__restrict__ s,
                                                          double *__restrict__ partials, PsCtrl *ctrl) {
    const GridDim &c = A.c;
    double mx = 0.0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < c.size;
         e += (long long)gridDim.x * blockDim.x) {
        long long kq = e / ((long long)c.sx * c.sy);
        long long rem = e - kq * (long long)c.sx * c.sy;
        int k = (int)kq - GFS_PAD, j = (int)(rem / c.sx) - GFS_PAD, i = (int)(rem % c.sx) - GFS_PAD;
        uint8_t fl = 0;
        double bv = 0.0;
        if (c.in(i, j, k) && mat[e] == GFS_FLUID) {
            long long sx = 1, sy = c.sx, sz = (long long)c.sx * c.sy;
            float u0 = u[A.fu.at(i, j, k)], u1 = u[A.fu.at(i + 1, j, k)];
            float v0 = v[A.fv.at(i, j, k)], v1 = v[A.fv.at(i, j + 1, k)];
            float w0 = w[A.fw.at(i, j, k)], w1 = w[A.fw.at(i, j, k + 1)];
            float div = __fsub_rn(__fadd_rn(__fsub_rn(__fadd_rn(__fsub_rn(u1, u0), v1), v0), w1), w0);
            bv = __dmul_rn(-A.scale_div, (double)div);
            bool sim = mat[e - sx] == GFS_SOLID, sip = mat[e + sx] == GFS_SOLID;
            bool sjm = mat[e - sy] == GFS_SOLID, sjp = mat[e + sy] == GFS_SOLID;
            bool skm = mat[e - sz] == GFS_SOLID, skp = mat[e + sz] == GFS_SOLID;
            if (sim) bv = __dsub_rn(bv, (double)__fmul_rn(A.fscale, __fsub_rn(u0, 0.0f)));
            if (sip) bv = __dadd_rn(bv, (double)__fmul_rn(A.fscale, __fsub_rn(u1, 0.0f)));
            if (sjm) bv = __dsub_rn(bv, (double)__fmul_rn(A.fscale, __fsub_rn(v0, 0.0f)));
            if (sjp) bv = __dadd_rn(bv, (double)__fmul_rn(A.fscale, __fsub_rn(v1, 0.0f)));
            if (skm) bv = __dsub_rn(bv, (double)__fmul_rn(A.fscale, __fsub_rn(w0, 0.0f)));
            if (skp) bv = __dadd_rn(bv, (double)__fmul_rn(A.fscale, __fsub_rn(w1, 0.0f)));
            int diag = (!sim) + (!sip) + (!sjm) + (!sjp) + (!skm) + (!skp);
            fl = (uint8_t)(GFS_PF_FLUID | (diag << 1));
            mx = fmax(mx, fabs(bv));
        }
        flags[e] = fl;
        b[e] = bv;
        r[e] = bv;
        p[e] = 0.0;
        s[e] = 0.0;
    }
    double part = block_reduce<1>(mx);
    double res;
    if (finish_reduce<1>(part, partials, &ctrl->tickets[0], gridDim.x, &res) && threadIdx.x == 0) {
        ctrl->maxb = res;
        ctrl->maxr = res;
        ctrl->maxr64 = res;
        ctrl->iter = 0;
        ctrl->converged = 0;
        ctrl->total_inner = 0;
        ctrl->refinements = 0;
        ctrl->sigma = 0.0;
        ctrl->alpha = 0.0;
        ctrl->beta = 0.0;
        // PressureSolver::solve returns before CG when max|b| < tol (:128-130)
        ctrl->done = res < A.tol ? 1 : 0;
        if (ctrl->done) ctrl->iter = -1;
    }
}

// ------------------------------------------------------------ wavefronts

enum { SW_PRECON = 0, SW_FWD = 1, SW_BWD = 2 };

template <class T>
struct SweepArgs {
    GridDim c;
    int nbj, nbk, S;
    const uint8_t *flags;
    const T *in;          // FWD: r, BWD: q
    T *out;               // FWD: q, BWD: z, PRECON: precon (double)
    const T *precon;      // FWD/BWD
    const T *rdot;        // BWD: r, for dot(z, r)
    float *out32;         // PRECON: float copy of precon (MIXED)
    T negscale;
    double scale, dnegscale;
    unsigned *progress;   // nbj * nbk
    unsigned *ticket;     // dispatch ticket
    unsigned *done_ticket;
    double *partials;
    PsCtrl *ctrl;
    int init;             // BWD: first solve of a CG run (sets sigma, no beta)
};

__device__ __forceinline__ void wait_progress(const unsigned *p, unsigned need, unsigned &cached,
                                              bool &timed_out, PsCtrl *ctrl) {
    if (cached >= need || timed_out) return;
    int spins = 0;
    while ((cached = ld_acquire_u32(p)) < need) {
        if (++spins > GFS_SPIN_LIMIT) {
            atomicOr(&ctrl->err, GFS_DEV_ERR_TIMEOUT);
            timed_out = true;
            return;
        }
    }
}

// MIC(0) diagonal for one fluid cell (pressuresolver.cpp:255-301).  pim1/pjm1/pkm1
// are the preconditioner values of the i-1, j-1, k-1 neighbours (0 if not fluid).
__device__ __forceinline__ double mic0_precon(const uint8_t *__restrict__ flags, const GridDim &c,
                                              long long e, uint8_t fl, double pim1, double pjm1,
                                              double pkm1, double scale, double negscale) {
    const double tau = 0.97, sigma = 0.25;
    long long sx = 1, sy = c.sx, sz = (long long)c.sx * c.sy;
    bool fim1 = flags[e - sx] & GFS_PF_FLUID, fjm1 = flags[e - sy] & GFS_PF_FLUID,
         fkm1 = flags[e - sz] & GFS_PF_FLUID;
    // MatrixCell plus flags of the lower neighbours: A[n].plusX = fluid(n + e_X)
    double plusi_im1 = fim1 ? __dmul_rn(1.0, negscale) : 0.0;
    double plusj_im1 = fim1 ? __dmul_rn((double)((flags[e - sx + sy] & GFS_PF_FLUID) ? 1 : 0), negscale) : 0.0;
    double plusk_im1 = fim1 ? __dmul_rn((double)((flags[e - sx + sz] & GFS_PF_FLUID) ? 1 : 0), negscale) : 0.0;
    double plusi_jm1 = fjm1 ? __dmul_rn((double)((flags[e - sy + sx] & GFS_PF_FLUID) ? 1 : 0), negscale) : 0.0;
    double plusj_jm1 = fjm1 ? __dmul_rn(1.0, negscale) : 0.0;
    double plusk_jm1 = fjm1 ? __dmul_rn((double)((flags[e - sy + sz] & GFS_PF_FLUID) ? 1 : 0), negscale) : 0.0;
    double plusi_km1 = fkm1 ? __dmul_rn((double)((flags[e - sz + sx] & GFS_PF_FLUID) ? 1 : 0), negscale) : 0.0;
    double plusj_km1 = fkm1 ? __dmul_rn((double)((flags[e - sz + sy] & GFS_PF_FLUID) ? 1 : 0), negscale) : 0.0;
    double plusk_km1 = fkm1 ? __dmul_rn(1.0, negscale) : 0.0;
    double precon_im1 = fim1 ? pim1 : 0.0, precon_jm1 = fjm1 ? pjm1 : 0.0, precon_km1 = fkm1 ? pkm1 : 0.0;
    double diag = __dmul_rn((double)(fl >> 1), scale);
    double v1 = __dmul_rn(plusi_im1, precon_im1);
    double v2 = __dmul_rn(plusj_jm1, precon_jm1);
    double v3 = __dmul_rn(plusk_km1, precon_km1);
    double v4 = __dmul_rn(precon_im1, precon_im1);
    double v5 = __dmul_rn(precon_jm1, precon_jm1);
    double v6 = __dmul_rn(precon_km1, precon_km1);
    double ta = __dmul_rn(__dmul_rn(plusi_im1, __dadd_rn(plusj_im1, plusk_im1)), v4);
    double tb = __dmul_rn(__dmul_rn(plusj_jm1, __dadd_rn(plusi_jm1, plusk_jm1)), v5);
    double tc = __dmul_rn(__dmul_rn(plusk_km1, __dadd_rn(plusi_km1, plusj_km1)), v6);
    double ee = __dsub_rn(__dsub_rn(__dsub_rn(__dsub_rn(diag, __dmul_rn(v1, v1)), __dmul_rn(v2, v2)),
                                    __dmul_rn(v3, v3)),
                          __dmul_rn(tau, __dadd_rn(__dadd_rn(ta, tb), tc)));
    if (ee < __dmul_rn(sigma, diag)) ee = diag;
    return fabs(ee) > 10e-9 ? __ddiv_rn(1.0, __dsqrt_rn(ee)) : 0.0;
}

template <class T, int BJ, int BK, int MODE>
__global__ void __launch_bounds__(BJ *BK) k_sweep(SweepArgs<T> A) {
    using Op = Ar<T>;
    if (A.ctrl->done) return;
    __shared__ T xb[2][BK][BJ];
    __shared__ unsigned sh_ticket;
    const int tid = threadIdx.x;
    const int jl = tid % BJ, kl = tid / BJ;
    if (tid == 0) sh_ticket = atomicAdd(A.ticket, 1u);
    __syncthreads();
    const unsigned t = sh_ticket;
    int bj, bk;
    if (MODE == SW_BWD) {
        bj = A.nbj - 1 - (int)(t % A.nbj);
        bk = A.nbk - 1 - (int)(t / A.nbj);
    } else {
        bj = (int)(t % A.nbj);
        bk = (int)(t / A.nbj);
    }
    const GridDim &c = A.c;
    const int j = bj * BJ + jl, k = bk * BK + kl;
    const bool valid = j < c.ny && k < c.nz;
    const long long sy = c.sx, sz = (long long)c.sx * c.sy;
    const int S = A.S;

    // producers of this block's boundary rows
    const unsigned *prod_j = nullptr, *prod_k = nullptr;
    if (MODE == SW_BWD) {
        if (bj + 1 < A.nbj) prod_j = A.progress + (bk * A.nbj + bj + 1);
        if (bk + 1 < A.nbk) prod_k = A.progress + ((bk + 1) * A.nbj + bj);
    } else {
        if (bj > 0) prod_j = A.progress + (bk * A.nbj + bj - 1);
        if (bk > 0) prod_k = A.progress + ((bk - 1) * A.nbj + bj);
    }
    unsigned *mine = A.progress + (bk * A.nbj + bj);
    unsigned cj = 0, ck = 0;
    bool timed_out = false;

    if (tid == 0) {
        if (prod_j) wait_progress(prod_j, min(BJ, S), cj, timed_out, A.ctrl);
        if (prod_k) wait_progress(prod_k, min(BK, S), ck, timed_out, A.ctrl);
    }
    __syncthreads();

    // exchanged value: FWD w = (negscale*precon)*q; BWD z; PRECON precon
    T prev = T(0);
    double dot = 0.0;
    for (int s = 0; s < S; s++) {
        int i;
        if (MODE == SW_BWD) i = (c.nx - 1) - (s - (BJ - 1 - jl) - (BK - 1 - kl));
        else i = s - jl - kl;
        const bool act = valid && i >= 0 && i < c.nx;
        T xch = T(0);
        if (act) {
            const long long e = c.at(i, j, k);
            const uint8_t fl = A.flags[e];
            // neighbour values of the previous step
            T nj_, nk_;
            if (MODE == SW_BWD) {
                if (jl < BJ - 1) nj_ = xb[(s - 1) & 1][kl][jl + 1];
                else nj_ = ldcg(A.out + e + sy);
                if (kl < BK - 1) nk_ = xb[(s - 1) & 1][kl + 1][jl];
                else nk_ = ldcg(A.out + e + sz);
            } else if (MODE == SW_FWD) {
                if (jl > 0) nj_ = xb[(s - 1) & 1][kl][jl - 1];
                else nj_ = Op::mul(Op::mul(A.negscale, A.precon[e - sy]), ldcg(A.out + e - sy));
                if (kl > 0) nk_ = xb[(s - 1) & 1][kl - 1][jl];
                else nk_ = Op::mul(Op::mul(A.negscale, A.precon[e - sz]), ldcg(A.out + e - sz));
            } else {
                if (jl > 0) nj_ = xb[(s - 1) & 1][kl][jl - 1];
                else nj_ = ldcg(A.out + e - sy);
                if (kl > 0) nk_ = xb[(s - 1) & 1][kl - 1][jl];
                else nk_ = ldcg(A.out + e - sz);
            }
            T val = T(0);
            if (fl & GFS_PF_FLUID) {
                if (MODE == SW_FWD) {
                    // _applyPreconditioner forward solve (pressuresolver.cpp:311-351)
                    T pc = A.precon[e];
                    T tt = Op::sub(Op::sub(Op::sub(A.in[e], prev), nj_), nk_);
                    val = Op::mul(tt, pc);
                    xch = Op::mul(Op::mul(A.negscale, pc), val);
                } else if (MODE == SW_BWD) {
                    // backward solve (pressuresolver.cpp:354-385)
                    T pc = A.precon[e];
                    T m = Op::mul(A.negscale, pc);
                    T tt = Op::sub(Op::sub(Op::sub(A.in[e], Op::mul(m, prev)), Op::mul(m, nj_)),
                                   Op::mul(m, nk_));
                    val = Op::mul(tt, pc);
                    xch = val;
                    dot += (double)val * (double)A.rdot[e];
                } else {
                    val = (T)mic0_precon(A.flags, c, e, fl, (double)prev, (double)nj_, (double)nk_,
                                         A.scale, A.dnegscale);
                    xch = val;
                    if (A.out32) A.out32[e] = (float)val;
                }
            } else if (MODE == SW_PRECON && A.out32) {
                A.out32[e] = 0.0f;
            }
            A.out[e] = val;
        }
        xb[s & 1][kl][jl] = xch;
        prev = xch;
        if (tid == 0 && !timed_out) {
            st_release_u32(mine, (unsigned)s);   // steps 0..s-1 are complete
            unsigned nxt = (unsigned)min(s + 1 + BJ, S), nxk = (unsigned)min(s + 1 + BK, S);
            if (prod_j) wait_progress(prod_j, nxt, cj, timed_out, A.ctrl);
            if (prod_k) wait_progress(prod_k, nxk, ck, timed_out, A.ctrl);
        }
        __syncthreads();
    }
    if (tid == 0) st_release_u32(mine, (unsigned)S);

    // block partial of dot(z, r) and the last-CTA epilogue
    double part = 0.0;
    if (MODE == SW_BWD) part = block_reduce<0>(dot);
    __shared__ bool last;
    unsigned nblocks = (unsigned)(A.nbj * A.nbk);
    if (tid == 0) {
        if (MODE == SW_BWD) A.partials[bj + A.nbj * bk] = part;
        __threadfence();
        unsigned tk = atomicAdd(A.done_ticket, 1u);
        last = tk == nblocks - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    for (unsigned q = tid; q < nblocks; q += BJ * BK) A.progress[q] = 0;
    if (MODE == SW_BWD) {
        double acc = 0.0;
        for (unsigned q = tid; q < nblocks; q += BJ * BK) acc += __ldcg(A.partials + q);
        acc = block_reduce<0>(acc);
        if (tid == 0) {
            PsCtrl *C = A.ctrl;
            if (A.init) {
                C->sigma = acc;
                C->beta = 0.0;
            } else {
                // _solvePressureSystem (pressuresolver.cpp:481-486)
                C->beta = acc / C->sigma;
                C->sigma = acc;
                C->iter += 1;
                if (C->iter >= C->max_iters) C->done = 1;
            }
        }
    }
    if (tid == 0) {
        *A.ticket = 0;
        *A.done_ticket = 0;
    }
}

// -------------------------------------------------------- vector kernels

template <class T>
struct VecArgs {
    GridDim c;
    const uint8_t *flags;
    T negscale, scale;
    double *partials;
    PsCtrl *ctrl;
    int mixed;
};

// As = A s and dot(As, s) -> alpha (pressuresolver.cpp:388-426, :472-473)
template <class T>
__global__ void __launch_bounds__(RED_THREADS) k_matvec(VecArgs<T> A, const T *__restrict__ s,
                                                        T *__restrict__ As) {
    using Op = Ar<T>;
    if (A.ctrl->done) return;
    const GridDim &c = A.c;
    const long long sy = c.sx, sz = (long long)c.sx * c.sy;
    double dot = 0.0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < c.size;
         e += (long long)gridDim.x * blockDim.x) {
        uint8_t fl = A.flags[e];
        if (!(fl & GFS_PF_FLUID)) continue;
        T x = s[e];
        T val = Op::add(Op::add(Op::add(Op::add(Op::add(s[e - 1], s[e + 1]), s[e - sy]), s[e + sy]), s[e - sz]),
                        s[e + sz]);
        val = Op::mul(val, A.negscale);
        val = Op::add(val, Op::mul(Op::mul((T)(fl >> 1), A.scale), x));
        As[e] = val;
        dot += (double)val * (double)x;
    }
    double part = block_reduce<0>(dot);
    double res;
    if (finish_reduce<0>(part, A.partials, &A.ctrl->tickets[1], gridDim.x, &res) && threadIdx.x == 0)
        A.ctrl->alpha = A.ctrl->sigma / res;
}

// p += alpha s; r -= alpha As; max|r| and the stopping test (pressuresolver.cpp:474-479)
template <class T>
__global__ void __launch_bounds__(RED_THREADS) k_axpy(VecArgs<T> A, T *__restrict__ p, T *__restrict__ r,
                                                      const T *__restrict__ s, const T *__restrict__ As) {
    using Op = Ar<T>;
    PsCtrl *C = A.ctrl;
    if (C->done) return;
    const GridDim &c = A.c;
    const T alpha = (T)C->alpha, nalpha = (T)(-C->alpha);
    double mx = 0.0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < c.size;
         e += (long long)gridDim.x * blockDim.x) {
        if (!(A.flags[e] & GFS_PF_FLUID)) continue;
        p[e] = Op::add(p[e], Op::mul(s[e], alpha));
        T rv = Op::add(r[e], Op::mul(As[e], nalpha));
        r[e] = rv;
        mx = fmax(mx, fabs((double)rv));
    }
    double part = block_reduce<1>(mx);
    double res;
    if (finish_reduce<1>(part, A.partials, &C->tickets[2], gridDim.x, &res) && threadIdx.x == 0) {
        C->maxr = res;
        double thr = A.mixed ? C->inner_tol : C->tol;
        if (res < thr) {
            C->done = 1;
            C->converged = 1;
        }
    }
}

// s = z + beta s (pressuresolver.cpp:483)
template <class T>
__global__ void __launch_bounds__(RED_THREADS) k_update_s(VecArgs<T> A, const T *__restrict__ z,
                                                          T *__restrict__ s) {
    using Op = Ar<T>;
    if (A.ctrl->done) return;
    const GridDim &c = A.c;
    const T beta = (T)A.ctrl->beta;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < c.size;
         e += (long long)gridDim.x * blockDim.x) {
        if (!(A.flags[e] & GFS_PF_FLUID)) continue;
        s[e] = Op::add(Op::mul(z[e], (T)1.0), Op::mul(s[e], beta));
    }
}

// MIXED: r32 = (float) r64, e32 = 0, s32 = 0; inner threshold from max|r64|.
__global__ void __launch_bounds__(RED_THREADS) k_mixed_prepare(GridDim c, const uint8_t *__restrict__ flags,
                                                               const double *__restrict__ r64,
                                                               float *__restrict__ r32, float *__restrict__ e32,
                                                               float *__restrict__ s32, PsCtrl *ctrl,
                                                               double eta) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < c.size;
         e += (long long)gridDim.x * blockDim.x) {
        bool f = flags[e] & GFS_PF_FLUID;
        r32[e] = f ? (float)r64[e] : 0.0f;
        e32[e] = 0.0f;
        s32[e] = 0.0f;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        double m = ctrl->maxr64;
        ctrl->inner_tol = fmax(eta * m, 0.25 * ctrl->tol);
        ctrl->done = 0;
        ctrl->converged = 0;
        ctrl->iter = 0;
        ctrl->sigma = 0.0;
        ctrl->beta = 0.0;
    }
}

// MIXED: p64 += e32, then r64 = b - A p64 in FP64 and max|r64| (outer refinement).
__global__ void __launch_bounds__(RED_THREADS) k_mixed_correct(GridDim c, const uint8_t *__restrict__ flags,
                                                               double *__restrict__ p64,
                                                               const float *__restrict__ e32) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < c.size;
         e += (long long)gridDim.x * blockDim.x)
        if (flags[e] & GFS_PF_FLUID) p64[e] += (double)e32[e];
}

__global__ void __launch_bounds__(RED_THREADS) k_residual64(VecArgs<double> A, const double *__restrict__ b,
                                                            const double *__restrict__ p,
                                                            double *__restrict__ r) {
    using Op = Ar<double>;
    const GridDim &c = A.c;
    const long long sy = c.sx, sz = (long long)c.sx * c.sy;
    double mx = 0.0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < c.size;
         e += (long long)gridDim.x * blockDim.x) {
        uint8_t fl = A.flags[e];
        if (!(fl & GFS_PF_FLUID)) continue;
        double val = p[e - 1] + p[e + 1] + p[e - sy] + p[e + sy] + p[e - sz] + p[e + sz];
        val = Op::add(Op::mul(val, A.negscale), Op::mul(Op::mul((double)(fl >> 1), A.scale), p[e]));
        double rv = b[e] - val;
        r[e] = rv;
        mx = fmax(mx, fabs(rv));
    }
    double part = block_reduce<1>(mx);
    double res;
    PsCtrl *C = A.ctrl;
    if (finish_reduce<1>(part, A.partials, &C->tickets[3], gridDim.x, &res) && threadIdx.x == 0) {
        C->maxr64 = res;
        C->refinements += 1;
    }
}

// --------------------------------------------------------------- driver

static constexpr int BJ64 = 8, BK64 = 8;     // FP64 sweeps: FP64 issue rate favours small CTAs
static constexpr int BJ32 = 16, BK32 = 16;   // FP32 sweeps

static int ensure_ws(Ctx *ctx, PressureWs &ws, const Grids &g, bool mixed) {
    long long n = g.c.size;
    if (ws.allocated_for != n) {
        ws.c = g.c;
        int rc = 0;
        rc |= ws.flags.alloc((size_t)n);
        DevMem *v64[] = {&ws.b, &ws.p, &ws.r, &ws.z, &ws.s, &ws.As, &ws.q, &ws.precon};
        for (DevMem *m : v64) rc |= m->alloc((size_t)n * sizeof(double));
        if (rc) return GFS_ERR_NOMEM;
        for (DevMem *m : v64) GFS_CUDA_CHECK(cudaMemsetAsync(m->p, 0, m->bytes, ctx->stream));
        GFS_CUDA_CHECK(cudaMemsetAsync(ws.flags.p, 0, ws.flags.bytes, ctx->stream));
        ws.nblocks_red = (size_t)ctx->num_sms * 8;
        int nbmax = (int)(((g.c.ny + 7) / 8) * ((g.c.nz + 7) / 8));
        size_t np = ws.nblocks_red > (size_t)nbmax ? ws.nblocks_red : (size_t)nbmax;
        if (ws.partials.alloc(np * sizeof(double))) return GFS_ERR_NOMEM;
        if (ws.ctrl.alloc(sizeof(PsCtrl))) return GFS_ERR_NOMEM;
        GFS_CUDA_CHECK(cudaMemsetAsync(ws.ctrl.p, 0, sizeof(PsCtrl), ctx->stream));
        if (ws.progress.alloc((size_t)nbmax * sizeof(unsigned))) return GFS_ERR_NOMEM;
        GFS_CUDA_CHECK(cudaMemsetAsync(ws.progress.p, 0, ws.progress.bytes, ctx->stream));
        ws.allocated_for = n;
        ws.mixed_alloc = false;
    }
    if (mixed && !ws.mixed_alloc) {
        DevMem *v32[] = {&ws.r32, &ws.z32, &ws.s32, &ws.As32, &ws.q32, &ws.e32, &ws.precon32};
        for (DevMem *m : v32) {
            if (m->alloc((size_t)n * sizeof(float))) return GFS_ERR_NOMEM;
            GFS_CUDA_CHECK(cudaMemsetAsync(m->p, 0, m->bytes, ctx->stream));
        }
        ws.mixed_alloc = true;
    }
    return GFS_OK;
}

template <class T, int BJ, int BK, int MODE>
static int launch_sweep(Ctx *ctx, PressureWs &ws, const T *in, T *out, const T *precon, const T *rdot,
                        float *out32, double scale, int init) {
    SweepArgs<T> A;
    A.c = ws.c;
    A.nbj = (ws.c.ny + BJ - 1) / BJ;
    A.nbk = (ws.c.nz + BK - 1) / BK;
    A.S = ws.c.nx + BJ + BK - 2;
    A.flags = ws.flags.as<uint8_t>();
    A.in = in;
    A.out = out;
    A.precon = precon;
    A.rdot = rdot;
    A.out32 = out32;
    A.negscale = (T)(-scale);
    A.scale = scale;
    A.dnegscale = -scale;
    A.progress = ws.progress.as<unsigned>();
    PsCtrl *C = ws.ctrl.as<PsCtrl>();
    A.ticket = &C->sweep_ticket[MODE];
    A.done_ticket = &C->tickets[0];
    A.partials = ws.partials.as<double>();
    A.ctrl = C;
    A.init = init;
    k_sweep<T, BJ, BK, MODE><<<A.nbj * A.nbk, BJ * BK, 0, ctx->stream>>>(A);
    ctx->launches++;
    GFS_LAUNCH_CHECK();
    return GFS_OK;
}

template <class T>
static VecArgs<T> vec_args(PressureWs &ws, double scale, int mixed) {
    VecArgs<T> A;
    A.c = ws.c;
    A.flags = ws.flags.as<uint8_t>();
    A.negscale = (T)(-scale);
    A.scale = (T)scale;
    A.partials = ws.partials.as<double>();
    A.ctrl = ws.ctrl.as<PsCtrl>();
    A.mixed = mixed;
    return A;
}

// One CG iteration (matvec, update, forward + backward MIC(0) solve, new search direction).
template <class T, int BJ, int BK>
static int cg_iteration(Ctx *ctx, PressureWs &ws, double scale, int mixed, T *p, T *r, T *z, T *s, T *As,
                        T *q, const T *precon) {
    unsigned nb = (unsigned)ws.nblocks_red;
    VecArgs<T> V = vec_args<T>(ws, scale, mixed);
    k_matvec<T><<<nb, RED_THREADS, 0, ctx->stream>>>(V, s, As);
    k_axpy<T><<<nb, RED_THREADS, 0, ctx->stream>>>(V, p, r, s, As);
    ctx->launches += 2;
    int rc = launch_sweep<T, BJ, BK, SW_FWD>(ctx, ws, r, q, precon, nullptr, nullptr, scale, 0);
    if (rc) return rc;
    rc = launch_sweep<T, BJ, BK, SW_BWD>(ctx, ws, q, z, precon, r, nullptr, scale, 0);
    if (rc) return rc;
    k_update_s<T><<<nb, RED_THREADS, 0, ctx->stream>>>(V, z, s);
    ctx->launches++;
    GFS_LAUNCH_CHECK();
    return GFS_OK;
}

static int read_ctrl(Ctx *ctx, PressureWs &ws, PsCtrl *h) {
    GFS_CUDA_CHECK(cudaMemcpyAsync(h, ws.ctrl.p, sizeof(PsCtrl), cudaMemcpyDeviceToHost, ctx->stream));
    GFS_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    if (h->err & GFS_DEV_ERR_TIMEOUT) {
        set_error(GFS_ERR_TIMEOUT, "pressure solve: a wavefront wait exceeded its bound");
        return GFS_ERR_TIMEOUT;
    }
    return GFS_OK;
}

#define CG_CHUNK 8

int pressure_solve(Ctx *ctx, PressureWs &ws, const Grids &g, const uint8_t *mat, float *const mac[3],
                   double density, double dt, int precision, double tol, int max_iters,
                   gfs_step_stats *stats) {
    bool mixed = precision == GFS_PRECISION_MIXED;
    int rc = ensure_ws(ctx, ws, g, mixed);
    if (rc) return rc;
    cudaStream_t st = ctx->stream;
    const double dx = g.dx;
    const double scale = dt / (density * dx * dx);   // pressuresolver.cpp:250
    PsCtrl *C = ws.ctrl.as<PsCtrl>();
    // tolerance / cap into the control block
    {
        PsCtrl h;
        memset(&h, 0, sizeof(h));
        GFS_CUDA_CHECK(cudaMemcpyAsync(&h, C, sizeof(PsCtrl), cudaMemcpyDeviceToHost, st));
        GFS_CUDA_CHECK(cudaStreamSynchronize(st));
        h.tol = tol;
        h.max_iters = max_iters;
        h.err = 0;
        GFS_CUDA_CHECK(cudaMemcpyAsync(C, &h, sizeof(PsCtrl), cudaMemcpyHostToDevice, st));
    }
    SetupArgs SA;
    SA.c = g.c;
    SA.fu = g.f[0];
    SA.fv = g.f[1];
    SA.fw = g.f[2];
    SA.fscale = 1.0f / (float)dx;
    SA.scale_div = (double)(1.0f / (float)dx);
    SA.tol = tol;
    unsigned nb = (unsigned)ws.nblocks_red;
    k_ps_setup<<<nb, RED_THREADS, 0, st>>>(SA, mat, mac[0], mac[1], mac[2], ws.flags.as<uint8_t>(),
                                            ws.b.as<double>(), ws.r.as<double>(), ws.p.as<double>(),
                                            ws.s.as<double>(), ws.partials.as<double>(), C);
    ctx->launches++;
    GFS_LAUNCH_CHECK();
    PsCtrl h;
    rc = read_ctrl(ctx, ws, &h);
    if (rc) return rc;
    int iterations = h.iter;
    double final_res = h.maxb;
    int refinements = 0;
    if (!h.done) {
        // MIC(0) preconditioner (pressuresolver.cpp:246-302), FP64 in both modes
        rc = launch_sweep<double, BJ64, BK64, SW_PRECON>(ctx, ws, nullptr, ws.precon.as<double>(), nullptr,
                                                         nullptr, mixed ? ws.precon32.as<float>() : nullptr,
                                                         scale, 0);
        if (rc) return rc;
        if (!mixed) {
            double *p = ws.p.as<double>(), *r = ws.r.as<double>(), *z = ws.z.as<double>(),
                   *s = ws.s.as<double>(), *As = ws.As.as<double>(), *q = ws.q.as<double>(),
                   *pc = ws.precon.as<double>();
            rc = launch_sweep<double, BJ64, BK64, SW_FWD>(ctx, ws, r, q, pc, nullptr, nullptr, scale, 0);
            if (rc) return rc;
            rc = launch_sweep<double, BJ64, BK64, SW_BWD>(ctx, ws, q, z, pc, r, nullptr, scale, 1);
            if (rc) return rc;
            VecArgs<double> V = vec_args<double>(ws, scale, 0);
            k_update_s<double><<<nb, RED_THREADS, 0, st>>>(V, z, s);
            ctx->launches++;
            for (;;) {
                for (int it = 0; it < CG_CHUNK; it++) {
                    rc = cg_iteration<double, BJ64, BK64>(ctx, ws, scale, 0, p, r, z, s, As, q, pc);
                    if (rc) return rc;
                }
                rc = read_ctrl(ctx, ws, &h);
                if (rc) return rc;
                if (h.done) break;
            }
            iterations = h.iter;
            final_res = h.maxr;
        } else {
            const double eta = 1e-3;
            float *r32 = ws.r32.as<float>(), *z32 = ws.z32.as<float>(), *s32 = ws.s32.as<float>(),
                  *As32 = ws.As32.as<float>(), *q32 = ws.q32.as<float>(), *e32 = ws.e32.as<float>(),
                  *pc32 = ws.precon32.as<float>();
            int total = 0;
            bool converged = false;
            double res64 = h.maxb;
            VecArgs<double> V64 = vec_args<double>(ws, scale, 1);
            VecArgs<float> V32 = vec_args<float>(ws, scale, 1);
            while (total < max_iters) {
                k_mixed_prepare<<<nb, RED_THREADS, 0, st>>>(g.c, ws.flags.as<uint8_t>(), ws.r.as<double>(), r32,
                                                           e32, s32, C, eta);
                ctx->launches++;
                // the inner cap is what is left of the total budget
                {
                    int left = max_iters - total;
                    GFS_CUDA_CHECK(cudaMemcpyAsync(&C->max_iters, &left, sizeof(int), cudaMemcpyHostToDevice, st));
                }
                rc = launch_sweep<float, BJ32, BK32, SW_FWD>(ctx, ws, r32, q32, pc32, nullptr, nullptr, scale, 0);
                if (rc) return rc;
                rc = launch_sweep<float, BJ32, BK32, SW_BWD>(ctx, ws, q32, z32, pc32, r32, nullptr, scale, 1);
                if (rc) return rc;
                k_update_s<float><<<nb, RED_THREADS, 0, st>>>(V32, z32, s32);
                ctx->launches++;
                for (;;) {
                    for (int it = 0; it < CG_CHUNK; it++) {
                        rc = cg_iteration<float, BJ32, BK32>(ctx, ws, scale, 1, e32, r32, z32, s32, As32, q32,
                                                             pc32);
                        if (rc) return rc;
                    }
                    rc = read_ctrl(ctx, ws, &h);
                    if (rc) return rc;
                    if (h.done) break;
                }
                // h.iter counts the inner iterations that completed without converging;
                // the converging iteration is one more.
                total += h.converged ? h.iter + 1 : h.iter;
                k_mixed_correct<<<nb, RED_THREADS, 0, st>>>(g.c, ws.flags.as<uint8_t>(), ws.p.as<double>(), e32);
                k_residual64<<<nb, RED_THREADS, 0, st>>>(V64, ws.b.as<double>(), ws.p.as<double>(),
                                                          ws.r.as<double>());
                ctx->launches += 2;
                rc = read_ctrl(ctx, ws, &h);
                if (rc) return rc;
                res64 = h.maxr64;
                refinements = h.refinements;
                if (res64 < tol) {
                    converged = true;
                    break;
                }
            }
            // reference numbering: the converging iteration is not counted
            iterations = converged ? total - 1 : total;
            if (iterations < 0) iterations = 0;
            final_res = res64;
            // restore the cap for later solves
            GFS_CUDA_CHECK(cudaMemcpyAsync(&C->max_iters, &max_iters, sizeof(int), cudaMemcpyHostToDevice, st));
            int one = 1;
            GFS_CUDA_CHECK(cudaMemcpyAsync(&C->done, &one, sizeof(int), cudaMemcpyHostToDevice, st));
        }
    }
    if (stats) {
        stats->cg_iterations = iterations;
        stats->cg_max_residual = final_res;
        stats->refinements = refinements;
    }
    return GFS_OK;
}

// ------------------------------------------------------ apply pressure

struct ApplyArgs {
    GridDim c, f[3];
    double scale, invscale;  // dt/(density*dx) (fluidsimulation.cpp:2900-2901)
};

// _applyPressureToVelocityField (fluidsimulation.cpp:2895-3061): each face's new
// value depends only on its own old value and the pressure grid, so the update
// is done in place (the reference goes through a temporary field).
__global__ void __launch_bounds__(128) k_apply_pressure(ApplyArgs A, const uint8_t *__restrict__ mat,
                                                        const double *__restrict__ p, float *__restrict__ u,
                                                        float *__restrict__ v, float *__restrict__ w) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    int k = blockIdx.z * blockDim.z + threadIdx.z;
    const GridDim &c = A.c;
    if (i > c.nx || j > c.ny || k > c.nz) return;
    float *g[3] = {u, v, w};
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const GridDim &f = A.f[d];
        if (!f.in(i, j, k)) continue;
        if (!face_borders(mat, c, d, i, j, k, GFS_FLUID)) continue;
        long long at = f.at(i, j, k);
        if (face_borders(mat, c, d, i, j, k, GFS_SOLID)) {
            g[d][at] = 0.0f;
            continue;
        }
        int ci = i - (d == 0), cj = j - (d == 1), ck = k - (d == 2);
        long long c0 = c.at(ci, cj, ck), c1 = c.at(ci + (d == 0), cj + (d == 1), ck + (d == 2));
        // pressureGrid holds (float) pressure (fluidsimulation.cpp:2884-2888)
        double p0 = (double)(float)p[c0], p1 = (double)(float)p[c1];
        double face = (double)g[d][at];
        bool s0 = mat[c0] == GFS_SOLID, s1 = mat[c1] == GFS_SOLID;
        if (s0) p0 = __dsub_rn(p1, __dmul_rn(A.invscale, face));
        else if (s1) p1 = __dadd_rn(p0, __dmul_rn(A.invscale, face));
        g[d][at] = (float)__dsub_rn(face, __dmul_rn(A.scale, __dsub_rn(p1, p0)));
    }
}

int pressure_apply(Sim *s, double dt) {
    Ctx *ctx = s->ctx;
    ApplyArgs A;
    A.c = s->g.c;
    for (int d = 0; d < 3; d++) A.f[d] = s->g.f[d];
    A.scale = dt / (s->params.density * s->g.dx);
    A.invscale = 1.0 / A.scale;
    dim3 block(32, 2, 2);
    dim3 grid(grid_blocks(A.c.nx + 1, 32), grid_blocks(A.c.ny + 1, 2), grid_blocks(A.c.nz + 1, 2));
    k_apply_pressure<<<grid, block, 0, ctx->stream>>>(A, s->mat.as<uint8_t>(), s->ps.p.as<double>(),
                                                      s->mac[0].as<float>(), s->mac[1].as<float>(),
                                                      s->mac[2].as<float>());
    ctx->launches++;
    GFS_LAUNCH_CHECK();
    return GFS_OK;
}

__global__ void k_pressure_grid(GridDim c, const uint8_t *__restrict__ flags, const double *__restrict__ p,
                                float *__restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y, k = blockIdx.z;
    if (i >= c.nx) return;
    long long e = c.at(i, j, k);
    out[i + (long long)c.nx * (j + (long long)c.ny * k)] = (flags[e] & GFS_PF_FLUID) ? (float)p[e] : 0.0f;
}

int pressure_to_grid(Ctx *ctx, PressureWs &ws, const Grids &g, float *out) {
    dim3 grid(grid_blocks(g.c.nx, 128), g.c.ny, g.c.nz);
    k_pressure_grid<<<grid, 128, 0, ctx->stream>>>(g.c, ws.flags.as<uint8_t>(), ws.p.as<double>(), out);
    ctx->launches++;
    GFS_LAUNCH_CHECK();
    return GFS_OK;
}

__global__ void k_fluid_indicator(GridDim c, const uint8_t *__restrict__ mat, uint32_t *__restrict__ ind) {
    long long lin = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    long long n = (long long)c.nx * c.ny * c.nz;
    if (lin > n) return;
    if (lin == n) { ind[lin] = 0; return; }
    int i = (int)(lin % c.nx), j = (int)((lin / c.nx) % c.ny), k = (int)(lin / ((long long)c.nx * c.ny));
    ind[lin] = mat[c.at(i, j, k)] == GFS_FLUID ? 1u : 0u;
}

__global__ void k_gather_compact(GridDim c, const uint8_t *__restrict__ mat, const uint32_t *__restrict__ idx,
                                 const double *__restrict__ p, double *__restrict__ out) {
    long long lin = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    long long n = (long long)c.nx * c.ny * c.nz;
    if (lin >= n) return;
    int i = (int)(lin % c.nx), j = (int)((lin / c.nx) % c.ny), k = (int)(lin / ((long long)c.nx * c.ny));
    long long e = c.at(i, j, k);
    if (mat[e] == GFS_FLUID) out[idx[lin]] = p[e];
}

int pressure_gather_compact(Ctx *ctx, PressureWs &ws, const Grids &g, const uint8_t *mat, double *d_out,
                            int64_t F) {
    (void)F;
    long long n = (long long)g.c.nx * g.c.ny * g.c.nz;
    DevMem ind, tmp;
    if (ind.alloc((size_t)(n + 1) * sizeof(uint32_t))) return GFS_ERR_NOMEM;
    if (tmp.alloc(scan_temp_elems(n + 1) * sizeof(uint32_t))) return GFS_ERR_NOMEM;
    k_fluid_indicator<<<grid_blocks(n + 1, 256), 256, 0, ctx->stream>>>(g.c, mat, ind.as<uint32_t>());
    ctx->launches++;
    int rc = exclusive_scan_u32(ctx, ind.as<uint32_t>(), ind.as<uint32_t>(), n + 1, tmp.as<uint32_t>(),
                                ctx->stream);
    if (rc) return rc;
    k_gather_compact<<<grid_blocks(n, 256), 256, 0, ctx->stream>>>(g.c, mat, ind.as<uint32_t>(),
                                                                    ws.p.as<double>(), d_out);
    ctx->launches++;
    GFS_LAUNCH_CHECK();
    GFS_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    return GFS_OK;
}

}  // namespace gfs
