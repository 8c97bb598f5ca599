// pressure.cu -- MICCG(0) pressure projection (PressureSolver, pressuresolver.cpp)
// and the pressure update of the MAC field.
//
// Vector layout.  The solver's vectors live in a "skewed" layout built for the
// MIC(0) triangular solves.  The forward solve L q = r and the preconditioner
// build are recurrences over i-1, j-1, k-1, the backward solve over i+1, j+1,
// k+1 (pressuresolver.cpp:246-386).  A cell depends only on cells of a lower
// i+j+k plane, so a wavefront reproduces the sequential result.  Each CTA owns
// one block: SBJ*SBK threads, one per pencil, walk the block's planes (step t
// handles plane t forwards, plane S-1-t backwards).  The j / k neighbours were
// produced by the adjacent threads one step earlier (shared-memory exchange,
// one barrier per step), the i neighbour by the thread itself.  Per-cell
// inputs are prefetched P steps ahead (cp.async into shared memory for the
// triangular solves, k_tri; registers for the build, k_sweep).  Blocks without
// fluid are skipped: they hand over zeros only.  Blocks hand their edge
// values to the downstream blocks through tagged 64-bit exchange words (value
// bits | sweep epoch): a consumer prefetches the word it will need P steps
// later and only re-reads it (bounded) if the tag is not yet this sweep's, so
// no fence or progress counter sits on the per-step path.  CTAs take dispatch
// tickets in dependency order, so every CTA they wait for is already resident.
// The FP32 triangular solves normally run k_tri_cl, the same wavefront in
// thread-block clusters whose blocks hand over through distributed shared memory.
//
// The CG loop runs on the device: each kernel first checks a device "done"
// flag, reductions finish in the last CTA to arrive (fixed order, so results
// are deterministic), and the host only polls the flag every few iterations.
#include <cstdlib>
#include <cstring>
#include <mutex>

#include <cooperative_groups.h>

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

__device__ __forceinline__ unsigned ld_acquire_cta_shared(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.cta.shared.u32 %0, [%1];" : "=r"(v) : "r"((unsigned)__cvta_generic_to_shared(p)) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_cta_shared(unsigned *p, unsigned v) {
    asm volatile("st.release.cta.shared.u32 [%0], %1;" ::"r"((unsigned)__cvta_generic_to_shared(p)), "r"(v) : "memory");
}

__device__ __forceinline__ void named_barrier(int id, int nthreads) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

#define RED_THREADS 256

template <int OP>  // 0 = sum, 1 = max
__device__ __forceinline__ double block_reduce(double v) {
    __shared__ double sh[32];
    int nw = (blockDim.x * blockDim.y * blockDim.z + 31) >> 5;
    int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    int lane = tid & 31, warp = tid >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        double y = __shfl_down_sync(0xffffffffu, v, o);
        v = OP == 0 ? v + y : fmax(v, y);
    }
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    if (warp == 0) {
        v = lane < nw ? sh[lane] : 0.0;
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

// ---------------------------------------------------------- skewed layout

static constexpr int SBJ = 16, SBK = 16, SPLANE = SBJ * SBK;

struct Skew {
    int nx, ny, nz, nbj, nbk, S;
    long long size;
    __host__ __device__ __forceinline__ long long base(int bj, int bk) const {
        return ((long long)bk * nbj + bj) * (long long)S * SPLANE;
    }
    __host__ __device__ __forceinline__ long long slot(int bj, int bk, int s, int jl, int kl) const {
        return base(bj, bk) + (long long)s * SPLANE + kl * SBJ + jl;
    }
    // slot -> block, plane and pencil position
    __device__ __forceinline__ void decode(long long q, int &bj, int &bk, int &s, int &jl, int &kl) const {
        long long per = (long long)S * SPLANE;
        long long blk = q / per;
        int rem = (int)(q - blk * per);
        s = rem / SPLANE;
        int w = rem - s * SPLANE;
        kl = w / SBJ;
        jl = w - kl * SBJ;
        bk = (int)(blk / nbj);
        bj = (int)(blk - (long long)bk * nbj);
    }
};

static Skew make_skew(const GridDim &c) {
    Skew K;
    K.nx = c.nx; K.ny = c.ny; K.nz = c.nz;
    K.nbj = (c.ny + SBJ - 1) / SBJ;
    K.nbk = (c.nz + SBK - 1) / SBK;
    K.S = c.nx + SBJ + SBK - 2;
    K.size = (long long)K.nbj * K.nbk * K.S * SPLANE;
    return K;
}

// ------------------------------------------------------------------ setup

struct SetupArgs {
    GridDim c, fu, fv, fw;
    float fscale;        // (float)(1.0f / (float)dx)
    double scale_div;    // 1.0f / (float)dx as double (pressuresolver.cpp:164)
    double tol;
};

// _calculateNegativeDivergenceVector (pressuresolver.cpp:162-208) and
// _calculateMatrixCoefficients (:222-244) for one cell, in the padded cell layout.
__global__ void __launch_bounds__(RED_THREADS) k_ps_setup(SetupArgs A, const uint8_t *__restrict__ mat,
                                                          const float *__restrict__ u, const float *__restrict__ v,
                                                          const float *__restrict__ w, uint8_t *__restrict__ flags,
                                                          double *__restrict__ b, double *__restrict__ partials,
                                                          PsCtrl *ctrl) {
    const GridDim &c = A.c;
    const unsigned plane = (unsigned)c.sx * (unsigned)c.sy;
    double mx = 0.0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < c.size;
         e += (long long)gridDim.x * blockDim.x) {
        unsigned ue = (unsigned)e;
        int k = (int)(ue / plane) - GFS_PAD;
        unsigned rem = ue % plane;
        int j = (int)(rem / (unsigned)c.sx) - GFS_PAD, i = (int)(rem % (unsigned)c.sx) - GFS_PAD;
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

// padded cell layout -> skewed layout: flags, b; r = b, p = 0, s = 0
__global__ void __launch_bounds__(RED_THREADS) k_to_skew(Skew K, GridDim c, const uint8_t *__restrict__ flags,
                                                         const double *__restrict__ b,
                                                         const uint16_t *__restrict__ nbits,
                                                         uint8_t *__restrict__ fsk, uint16_t *__restrict__ nbsk,
                                                         double *__restrict__ bsk, double *__restrict__ rsk,
                                                         double *__restrict__ psk, double *__restrict__ ssk,
                                                         uint8_t *__restrict__ blkf) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < K.size;
         q += (long long)gridDim.x * blockDim.x) {
        int bj, bk, s, jl, kl;
        K.decode(q, bj, bk, s, jl, kl);
        int i = s - jl - kl, j = bj * SBJ + jl, k = bk * SBK + kl;
        uint8_t fl = 0;
        uint16_t nb = 0;
        double bv = 0.0;
        if (c.in(i, j, k)) {
            long long e = c.at(i, j, k);
            fl = flags[e];
            bv = b[e];
            nb = nbits[e];
        }
        fsk[q] = fl;
        nbsk[q] = nb;
        if (fl & GFS_PF_FLUID) blkf[bk * K.nbj + bj] = 1;   // same value from every writer
        bsk[q] = bv;
        rsk[q] = bv;
        psk[q] = 0.0;
        ssk[q] = 0.0;
    }
}

// skewed pressure -> padded cell layout (0 off the fluid set)
__global__ void k_from_skew(Skew K, GridDim c, const uint8_t *__restrict__ flags, const double *__restrict__ psk,
                            double *__restrict__ p) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y, k = blockIdx.z;
    if (i >= c.nx) return;
    long long e = c.at(i, j, k);
    double v = 0.0;
    if (flags[e] & GFS_PF_FLUID) {
        int bj = j / SBJ, bk = k / SBK, jl = j - bj * SBJ, kl = k - bk * SBK;
        v = psk[K.slot(bj, bk, i + jl + kl, jl, kl)];
    }
    p[e] = v;
}

// ------------------------------------------------------------ wavefronts

enum { SW_PRECON = 0, SW_FWD = 1, SW_BWD = 2 };

template <class T>
struct SweepArgs {
    Skew K;
    GridDim c;               // padded cell layout (neighbour flags of the MIC(0) build)
    const uint8_t *fsk;      // skewed flags
    const uint8_t *fstd;     // padded-layout flags
    const T *in;             // FWD: r, BWD: q
    T *out;                  // FWD: q, BWD: z, PRECON: precon (double)
    const T *precon;         // FWD/BWD
    const T *rdot;           // BWD: r, for dot(z, r)
    const T *mpc;            // FWD/BWD in FP64: negscale * precon, precomputed (k_tri)
    float *out32;            // PRECON: float copy of precon (MIXED)
    T negscale;
    double scale, dnegscale;
    unsigned long long *xch; // block-boundary exchange words
    const uint16_t *nbits;   // PRECON: skewed MIC(0) neighbour bits
    const uint8_t *blkf;     // per skew block: 1 if it holds a fluid cell
    unsigned *ticket;        // dispatch ticket
    unsigned *done_ticket;
    double *partials;
    PsCtrl *ctrl;
    int init;                // BWD: first solve of a CG run (sets sigma, no beta)
    int spin_limit;          // bound of every exchange wait, in polls
    unsigned wait_skew;      // 0; nonzero (fault injection) makes every wait look for a tag nobody writes
};

// Fluid bits of the neighbours the MIC(0) diagonal needs, packed:
//   0 i-1, 1 j-1, 2 k-1, 3 (i-1,j+1), 4 (i-1,k+1), 5 (i+1,j-1), 6 (j-1,k+1),
//   7 (i+1,k-1), 8 (j+1,k-1).
__device__ __forceinline__ unsigned mic0_neighbour_bits(const uint8_t *__restrict__ flags, const GridDim &c,
                                                        long long e) {
    const long long sx = 1, sy = c.sx, sz = (long long)c.sx * c.sy;
    const long long off[9] = {-sx, -sy, -sz, -sx + sy, -sx + sz, sx - sy, -sy + sz, sx - sz, sy - sz};
    unsigned bits = 0;
#pragma unroll
    for (int q = 0; q < 9; q++) bits |= (flags[e + off[q]] & GFS_PF_FLUID) ? (1u << q) : 0u;
    return bits;
}

// neighbour bits of every fluid cell, padded cell layout (input of the MIC(0) build)
__global__ void k_nbits(GridDim c, const uint8_t *__restrict__ flags, uint16_t *__restrict__ nbits) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y, k = blockIdx.z;
    if (i >= c.nx) return;
    long long e = c.at(i, j, k);
    nbits[e] = (flags[e] & GFS_PF_FLUID) ? (uint16_t)mic0_neighbour_bits(flags, c, e) : (uint16_t)0;
}

// MIC(0) diagonal for one fluid cell (pressuresolver.cpp:255-301).  pim1/pjm1/pkm1
// are the preconditioner values of the i-1, j-1, k-1 neighbours (0 if not fluid).
// In double it reproduces the reference's arithmetic exactly; the MIXED solver
// builds its FP32 preconditioner with the same formula in float.
template <class T>
__device__ __forceinline__ T mic0_precon(unsigned nb, uint8_t fl, T pim1, T pjm1, T pkm1, T scale, T negscale) {
    using Op = Ar<T>;
    const T tau = (T)0.97, sigma = (T)0.25, zero = T(0), one = T(1);
    bool fim1 = nb & 1u, fjm1 = nb & 2u, fkm1 = nb & 4u;
    // MatrixCell plus flags of the lower neighbours: A[n].plusX = fluid(n + e_X)
    T plusi_im1 = fim1 ? Op::mul(one, negscale) : zero;
    T plusj_im1 = fim1 ? Op::mul((nb & 8u) ? one : zero, negscale) : zero;
    T plusk_im1 = fim1 ? Op::mul((nb & 16u) ? one : zero, negscale) : zero;
    T plusi_jm1 = fjm1 ? Op::mul((nb & 32u) ? one : zero, negscale) : zero;
    T plusj_jm1 = fjm1 ? Op::mul(one, negscale) : zero;
    T plusk_jm1 = fjm1 ? Op::mul((nb & 64u) ? one : zero, negscale) : zero;
    T plusi_km1 = fkm1 ? Op::mul((nb & 128u) ? one : zero, negscale) : zero;
    T plusj_km1 = fkm1 ? Op::mul((nb & 256u) ? one : zero, negscale) : zero;
    T plusk_km1 = fkm1 ? Op::mul(one, negscale) : zero;
    T precon_im1 = fim1 ? pim1 : zero, precon_jm1 = fjm1 ? pjm1 : zero, precon_km1 = fkm1 ? pkm1 : zero;
    T diag = Op::mul((T)(fl >> 1), scale);
    T v1 = Op::mul(plusi_im1, precon_im1);
    T v2 = Op::mul(plusj_jm1, precon_jm1);
    T v3 = Op::mul(plusk_km1, precon_km1);
    T v4 = Op::mul(precon_im1, precon_im1);
    T v5 = Op::mul(precon_jm1, precon_jm1);
    T v6 = Op::mul(precon_km1, precon_km1);
    T ta = Op::mul(Op::mul(plusi_im1, Op::add(plusj_im1, plusk_im1)), v4);
    T tb = Op::mul(Op::mul(plusj_jm1, Op::add(plusi_jm1, plusk_jm1)), v5);
    T tc = Op::mul(Op::mul(plusk_km1, Op::add(plusi_km1, plusj_km1)), v6);
    T ee = Op::sub(Op::sub(Op::sub(Op::sub(diag, Op::mul(v1, v1)), Op::mul(v2, v2)), Op::mul(v3, v3)),
                   Op::mul(tau, Op::add(Op::add(ta, tb), tc)));
    if (ee < Op::mul(sigma, diag)) ee = diag;
    if (!(fabs((double)ee) > 10e-9)) return zero;
    if (sizeof(T) == 8) return (T)__ddiv_rn(1.0, __dsqrt_rn((double)ee));
    return (T)(1.0f / sqrtf((float)ee));
}

#define SWEEP_THREADS SPLANE
#define XCH_PER_PLANE (SBJ + SBK)   // exchange entries per block plane: j edge (by kl), k edge (by jl)

// Block-boundary exchange.  The threads on a block's downstream j / k edge write
// the value each of their cells hands to the neighbouring block into an
// exchange buffer as 64-bit words (32 value bits | 32-bit sweep epoch).  A
// 64-bit aligned store is single-copy atomic, so a consumer that reads a word
// whose tag equals the current epoch holds the producer's value for this sweep:
// no progress counters and no memory fences are needed.  FP64 values travel as
// two tagged words.
// Exchange words are read and written with relaxed gpu-scope (strong) accesses.
// A poll loop of weak loads may legally be collapsed into a single load by the
// compiler (nothing in the loop orders it), after which it never sees the
// producer's store; a strong load is performed on every iteration and must
// eventually observe the strong store.  Both go to L2, like .cg accesses.
__device__ __forceinline__ unsigned long long ld_cg_u64(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed_u64(unsigned long long *p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
template <class T> struct Xch;
template <> struct Xch<float> {
    static constexpr int W = 1;
    static __device__ __forceinline__ void put(unsigned long long *p, float v, unsigned tag) {
        unsigned long long w = ((unsigned long long)tag << 32) | (unsigned long long)__float_as_uint(v);
        st_relaxed_u64(p, w);
    }
    static __device__ __forceinline__ void fetch(const unsigned long long *p, unsigned long long w[1]) {
        w[0] = ld_cg_u64(p);
    }
    static __device__ __forceinline__ bool ready(const unsigned long long w[1], unsigned tag) {
        return (unsigned)(w[0] >> 32) == tag;
    }
    static __device__ __forceinline__ float value(const unsigned long long w[1]) {
        return __uint_as_float((unsigned)(w[0] & 0xFFFFFFFFull));
    }
};
template <> struct Xch<double> {
    static constexpr int W = 2;
    static __device__ __forceinline__ void put(unsigned long long *p, double v, unsigned tag) {
        unsigned long long bits = (unsigned long long)__double_as_longlong(v);
        st_relaxed_u64(p, ((unsigned long long)tag << 32) | (bits & 0xFFFFFFFFull));
        st_relaxed_u64(p + 1, ((unsigned long long)tag << 32) | (bits >> 32));
    }
    static __device__ __forceinline__ void fetch(const unsigned long long *p, unsigned long long w[2]) {
        w[0] = ld_cg_u64(p);
        w[1] = ld_cg_u64(p + 1);
    }
    static __device__ __forceinline__ bool ready(const unsigned long long w[2], unsigned tag) {
        return (unsigned)(w[0] >> 32) == tag && (unsigned)(w[1] >> 32) == tag;
    }
    static __device__ __forceinline__ double value(const unsigned long long w[2]) {
        return __longlong_as_double((long long)((w[0] & 0xFFFFFFFFull) | (w[1] << 32)));
    }
};

// Take a prefetched exchange word, re-reading it (bounded) until it carries this sweep's tag.
template <class T>
__device__ __forceinline__ T xch_take(unsigned long long w[], const unsigned long long *src, unsigned tag,
                                      int limit, PsCtrl *ctrl, bool &timed_out) {
    if (!Xch<T>::ready(w, tag) && !timed_out) {
        int spins = 0;
        do {
            Xch<T>::fetch(src, w);
            if (++spins > limit) {
                atomicOr(&ctrl->err, GFS_DEV_ERR_TIMEOUT);
                timed_out = true;
                break;
            }
        } while (!Xch<T>::ready(w, tag));
    }
    return Xch<T>::value(w);
}

// Compensated (double-float) accumulation: s + c tracks a running sum with
// about twice float precision (Knuth's TwoSum), so the FP32 kernels form their
// dot-product partials without FP64 arithmetic.
struct Acc2f {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        float t = s + x;
        float bp = t - s;
        float err = (s - (t - bp)) + (x - bp);
        s = t;
        c += err;
    }
    __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }


// In-place loads for the wavefront's prefetch ring: asm volatile keeps each load
// where it is written (P steps before its use), so its latency overlaps the
// intervening steps instead of sitting on the step's critical path.
__device__ __forceinline__ float ld_nc(const float *p) {
    float v;
    asm volatile("ld.global.nc.f32 %0, [%1];" : "=f"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ double ld_nc(const double *p) {
    double v;
    asm volatile("ld.global.nc.f64 %0, [%1];" : "=d"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ unsigned ld_nc_u8(const uint8_t *p) {
    unsigned v;
    asm volatile("ld.global.nc.u8 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ unsigned ld_nc_u16(const uint16_t *p) {
    unsigned short v;
    asm volatile("ld.global.nc.u16 %0, [%1];" : "=h"(v) : "l"(p));
    return v;
}

// Per-thread asynchronous copies (cp.async) into the shared-memory ring: one
// commit group per step, waited for P-1 groups later, so the copy of step st+P
// overlaps P steps of the recurrence without holding any register scoreboard.
template <int N>
__device__ __forceinline__ void cp_async(void *dst, const void *src, bool pred) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;" ::"r"(smem_addr(dst)), "l"(src), "n"(N),
                 "r"(pred ? N : 0)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

template <class T, int MODE, int P, int PE>
__global__ void __launch_bounds__(SWEEP_THREADS, 1) k_sweep(SweepArgs<T> A) {
    using Op = Ar<T>;
    using X = Xch<T>;
    constexpr bool bwd = MODE == SW_BWD;
    constexpr long long PS = bwd ? -(long long)SPLANE : (long long)SPLANE;   // slot advance per step
    constexpr long long XP = (long long)XCH_PER_PLANE * X::W;               // exchange words per plane
    constexpr long long XS = bwd ? -XP : XP;                                // exchange advance per step
    __shared__ T xb[2][SBK][SBJ];
    // ring of P steps per input (FWD: r, precon; BWD: q, precon, r); each thread owns column tid
    __shared__ __align__(16) T ring[(MODE == SW_PRECON) ? 1 : (MODE == SW_BWD ? 3 : 2)][P][SPLANE];
    __shared__ unsigned sh_ticket, sh_epoch;
    if (A.ctrl->done) return;
    const int tid = threadIdx.x;
    const Skew &K = A.K;
    const int S = K.S;
    if (tid == 0) {
        sh_ticket = atomicAdd(A.ticket, 1u);
        sh_epoch = A.ctrl->epoch;
    }
    __syncthreads();
    const unsigned t = sh_ticket, tag = sh_epoch;
    const unsigned wtag = tag + A.wait_skew;   // the tag the waits look for (tag itself unless a test skews it)
    int bj = (int)(t % K.nbj), bk = (int)(t / K.nbj);
    if (bwd) {
        bj = K.nbj - 1 - bj;
        bk = K.nbk - 1 - bk;
    }
    const int pbj = bwd ? bj + 1 : bj - 1, pbk = bwd ? bk + 1 : bk - 1;
    // a block without fluid hands over zeros only (precon is 0 off the fluid set), so it
    // does no work and its consumers take 0 instead of waiting for it
    const bool live = A.blkf[bk * K.nbj + bj] != 0;
    const bool has_pj = pbj >= 0 && pbj < K.nbj && A.blkf[bk * K.nbj + pbj],
               has_pk = pbk >= 0 && pbk < K.nbk && A.blkf[pbk * K.nbj + bj];
    bool timed_out = false;

    const int jl = tid % SBJ, kl = tid / SBJ;
    const int j = bj * SBJ + jl, k = bk * SBK + kl;
    const bool valid = live && j < K.ny && k < K.nz;
    const int xj = bwd ? jl + 1 : jl - 1, xk = bwd ? kl + 1 : kl - 1;
    const bool at_j = bwd ? jl == SBJ - 1 : jl == 0;                // on the upstream j edge
    const bool at_k = bwd ? kl == SBK - 1 : kl == 0;
    const bool in_j = at_j && has_pj, in_k = at_k && has_pk;        // read a producer block
    const bool out_j = bwd ? jl == 0 : jl == SBJ - 1;               // write for the j consumer
    const bool out_k = bwd ? kl == 0 : kl == SBK - 1;
    // step st handles plane S-1-st (backward) or st (forward); the cell exists for st in [st_lo, st_hi)
    const int st_lo = valid ? (bwd ? S - K.nx - jl - kl : jl + kl) : S;
    const int st_hi = valid ? st_lo + K.nx : S;
    const long long q0 = K.base(bj, bk) + kl * SBJ + jl + (bwd ? (long long)(S - 1) * SPLANE : 0);
    const long long xblock = (long long)S * XP;
    const long long xo0 = (long long)(bk * K.nbj + bj) * xblock + (bwd ? (long long)(S - 1) * XP : 0);
    const long long xj0 = has_pj ? (long long)(bk * K.nbj + pbj) * xblock +
                                       (bwd ? (long long)(S - 1 - (SBJ - 1)) : (long long)(SBJ - 1)) * XP +
                                       (long long)kl * X::W
                                 : 0;
    const long long xk0 = has_pk ? (long long)(pbk * K.nbj + bj) * xblock +
                                       (bwd ? (long long)(S - 1 - (SBK - 1)) : (long long)(SBK - 1)) * XP +
                                       (long long)(SBJ + jl) * X::W
                                 : 0;
    // per-thread pointers at step 0 (every step moves them by PS slots)
    const T *pa = MODE == SW_PRECON ? nullptr : A.in + q0;        // FWD r, BWD q
    const T *pb = MODE == SW_PRECON ? nullptr : A.precon + q0;
    const T *pc_ = MODE == SW_BWD ? A.rdot + q0 : nullptr;        // BWD r
    const uint8_t *pf = MODE == SW_PRECON ? A.fsk + q0 : nullptr;
    const uint16_t *pn = MODE == SW_PRECON ? A.nbits + q0 : nullptr;
    T *pout = A.out + q0;
    float *pout32 = A.out32 ? A.out32 + q0 : nullptr;
    unsigned long long *xbuf = A.xch;
    const unsigned long long *pxj = xbuf + xj0, *pxk = xbuf + xk0;
    unsigned long long *pxo = xbuf + xo0;

    // ring slot u holds the inputs of step s0 + u (FWD/BWD: cp.async into shared
    // memory; PRECON, once per solve: registers)
    unsigned r_f[P], r_n[P];
    unsigned long long r_wj[PE][X::W], r_wk[PE][X::W];
    auto prefetch = [&](int st, int u) {
        const bool ok = st >= st_lo && st < st_hi;
        const long long o = (long long)st * PS;
        if (MODE == SW_PRECON) {
            r_f[u] = ok ? ld_nc_u8(pf + o) : 0u;
            r_n[u] = ok ? ld_nc_u16(pn + o) : 0u;
        } else {
            // a zero-size source fills the slot with zeros
            cp_async<sizeof(T)>(&ring[0][u][tid], ok ? pa + o : pa, ok);
            cp_async<sizeof(T)>(&ring[1][u][tid], ok ? pb + o : pb, ok);
            if (MODE == SW_BWD) cp_async<sizeof(T)>(&ring[MODE == SW_BWD ? 2 : 0][u][tid], ok ? pc_ + o : pc_, ok);
            cp_async_commit();
        }
    };
    auto prefetch_x = [&](int st, int v) {
        const bool ok = st >= st_lo && st < st_hi;
        if (in_j && ok) {
            const unsigned long long *q = pxj + (long long)st * XS;
            r_wj[v][0] = ld_cg_u64(q);
            if (X::W == 2) r_wj[v][X::W - 1] = ld_cg_u64(q + 1);
        }
        if (in_k && ok) {
            const unsigned long long *q = pxk + (long long)st * XS;
            r_wk[v][0] = ld_cg_u64(q);
            if (X::W == 2) r_wk[v][X::W - 1] = ld_cg_u64(q + 1);
        }
    };
#pragma unroll
    for (int u = 0; u < P; u++) prefetch(u, u);
#pragma unroll
    for (int v = 0; v < PE; v++) prefetch_x(v, v);

    T prev = T(0);       // exchanged value of this pencil's previous cell
    Acc2f dot32;         // BWD, FP32: compensated dot(z, r)
    double dot64 = 0.0;  // BWD, FP64
    static_assert(P % PE == 0, "exchange ring must divide the input ring");
    const int SP = live ? ((S + P - 1) / P) * P : 0;
    for (int s0 = 0; s0 < SP; s0 += P) {
#pragma unroll
        for (int u = 0; u < P; u++) {
            const int st = s0 + u;
            const int v = u % PE;
            if (MODE != SW_PRECON) cp_async_wait<P - 1>();   // this step's copies have landed
            T xch = T(0);
            if (st >= st_lo && st < st_hi) {
                const long long o = (long long)st * PS;
                T nj_, nk_;
                if (!at_j) nj_ = xb[(st - 1) & 1][kl][xj];
                else nj_ = in_j ? xch_take<T>(r_wj[v], pxj + (long long)st * XS, wtag, A.spin_limit, A.ctrl, timed_out) : T(0);
                if (!at_k) nk_ = xb[(st - 1) & 1][xk][jl];
                else nk_ = in_k ? xch_take<T>(r_wk[v], pxk + (long long)st * XS, wtag, A.spin_limit, A.ctrl, timed_out) : T(0);
                T val = T(0);
                if (MODE == SW_FWD) {
                    // _applyPreconditioner forward solve (pressuresolver.cpp:311-351); neighbours hand
                    // over (negscale*precon)*q.  precon is 0 off the fluid set, so those cells give 0.
                    T pc = ring[1][u][tid];
                    T tt = Op::sub(Op::sub(Op::sub(ring[0][u][tid], prev), nj_), nk_);
                    val = Op::mul(tt, pc);
                    xch = Op::mul(Op::mul(A.negscale, pc), val);
                } else if (MODE == SW_BWD) {
                    // backward solve (pressuresolver.cpp:354-385)
                    T pc = ring[1][u][tid];
                    T m = Op::mul(A.negscale, pc);
                    T tt = Op::sub(Op::sub(Op::sub(ring[0][u][tid], Op::mul(m, prev)), Op::mul(m, nj_)),
                                   Op::mul(m, nk_));
                    val = Op::mul(tt, pc);
                    xch = val;
                    const T rv = ring[MODE == SW_BWD ? 2 : 0][u][tid];
                    if (sizeof(T) == 4) dot32.add((float)val * (float)rv);
                    else dot64 += (double)val * (double)rv;
                } else {
                    const uint8_t fl = (uint8_t)r_f[u];
                    if (fl & GFS_PF_FLUID) val = mic0_precon<T>(r_n[u], fl, prev, nj_, nk_, (T)A.scale, A.negscale);
                    xch = val;
                }
                pout[o] = val;
                if (MODE == SW_PRECON && pout32) pout32[o] = (float)val;
                if (out_j) X::put(pxo + (long long)st * XS + (long long)kl * X::W, xch, tag);
                if (out_k) X::put(pxo + (long long)st * XS + (long long)(SBJ + jl) * X::W, xch, tag);
            }
            xb[st & 1][kl][jl] = xch;
            prev = xch;
            prefetch(st + P, u);
            prefetch_x(st + PE, v);
            __syncthreads();
        }
    }
    if (MODE != SW_PRECON) cp_async_wait<0>();

    // block partial of dot(z, r) and the last-CTA epilogue
    double part = 0.0;
    if (MODE == SW_BWD) part = block_reduce<0>(sizeof(T) == 4 ? dot32.value() : dot64);
    __shared__ bool last;
    const unsigned nblocks = (unsigned)(K.nbj * K.nbk);
    if (tid == 0) {
        if (MODE == SW_BWD) A.partials[bj + K.nbj * bk] = part;
        __threadfence();
        unsigned tk = atomicAdd(A.done_ticket, 1u);
        last = tk == nblocks - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    if (MODE == SW_BWD) {
        double acc = 0.0;
        for (unsigned q = tid; q < nblocks; q += SWEEP_THREADS) acc += __ldcg(A.partials + q);
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
        A.ctrl->epoch = tag + 1 == 0 ? 1u : tag + 1;   // the next sweep's tag (0 marks never written)
    }
}

// ---------------------------------------------------- receiver warps
//
// The L2 hand-over between blocks.  A block's 32 upstream edge pencils (16 on
// the j edge, 16 on the k edge) each need one exchange word per step from a
// producer block.  Polled by the pencils themselves, a word that is not there
// yet costs the whole block an L2 round trip per step; near a block's start,
// where it runs just behind its producer, that is every step, and the polling
// branches and fences lengthen every step of the edge warps.  Instead, RX_NR
// extra warps per block (the receivers) poll the words: lane l of receiver warp
// r takes the steps s = r (mod RX_NR) of edge pencil l, with one read in flight
// (several reads in flight from one thread do not overlap: each extra one added
// about a round trip to every hand-over), and publishes each word in a shared
// ring: value, then the class's progress (every step of the class below it is in
// the ring).  Before the barrier that ends step st, warp 0 (the gate) waits until
// every edge pencil's input of step st+1 is there -- in the ring, or for a
// hand-over inside a thread-block cluster in the block's receive buffer -- so the
// compute threads read their neighbours with plain loads, and the gate hands
// ring slots back for all pencils together every RX_CB steps.
static constexpr int RX_R = 32;    // ring steps per pencil
static constexpr int RX_NR = 4;    // receiver warps (step classes)
static constexpr int RX_CB = 8;    // steps between slot hand-backs
static constexpr int RX_THREADS = 32 * RX_NR;
static constexpr int RX_DONE = 0x7fffffff;   // progress of a pencil with nothing (more) to receive

template <class T>
struct RxRing {
    T val[RX_R][32];
    int prog[RX_NR][32];   // class r, lane l: the steps of class r below prog[r][l] are in val
    int cons;              // steps below cons have been read by the compute threads
};

__device__ __forceinline__ int ld_volatile_s32(const int *p) { return *(const volatile int *)p; }
__device__ __forceinline__ void st_volatile_s32(int *p, int v) { *(volatile int *)p = v; }

// Receiver lane: the steps s = cls (mod RX_NR) in [s_lo, s_hi) of one edge pencil,
// whose word of step s is at src + s * xs.  A read that has not seen the tag after
// `limit` rounds marks the timeout; either way the lane ends by publishing
// RX_DONE, so that the gate never waits on it again.
template <class T>
__device__ void rx_receive(RxRing<T> &R, int cls, int lane, const unsigned long long *src, long long xs, int s_lo,
                           int s_hi, unsigned tag, int limit, PsCtrl *ctrl) {
    using X = Xch<T>;
    unsigned long long w[X::W];
    int s = s_lo + ((cls - s_lo) % RX_NR + RX_NR) % RX_NR;   // the first step of the class at or after s_lo
    st_volatile_s32(&R.prog[cls][lane], s);
    bool inflight = false;
    int rounds = 0;
    while (s < s_hi) {
        if (++rounds > limit) {
            atomicOr(&ctrl->err, GFS_DEV_ERR_TIMEOUT);
            break;
        }
        if (!inflight) {
            // ring slot s & (RX_R-1) is free once the compute threads have read step s - RX_R
            if (s < max(ld_volatile_s32(&R.cons), s_lo) + RX_R - RX_CB) {
                X::fetch(src + (long long)s * xs, w);
                inflight = true;
            } else {
                __nanosleep(32);   // ahead of the compute threads: leave them the issue slots
            }
        } else if (X::ready(w, tag)) {
            R.val[s & (RX_R - 1)][lane] = X::value(w);
            s += RX_NR;
            __threadfence_block();   // the value before the progress
            st_volatile_s32(&R.prog[cls][lane], s);
            inflight = false;
            if (s < s_hi && s < max(ld_volatile_s32(&R.cons), s_lo) + RX_R - RX_CB) {
                X::fetch(src + (long long)s * xs, w);
                inflight = true;
            }
        } else {
            X::fetch(src + (long long)s * xs, w);
        }
    }
    __threadfence_block();
    st_volatile_s32(&R.prog[cls][lane], RX_DONE);
}

// Gate (warp 0, lane l for edge pencil l): wait until the input of step `need` of
// every edge pencil is readable -- L2 pencils: every class's progress is past it
// (their minimum cached in `seen`); cluster pencils: the tagged word is in the
// receive buffer (rxw: the word of step 0, stride rxs words per step); pencils that
// need nothing at `need` pass.  Bounded; a timeout marks the error and lets every
// later gate pass.
template <class T>
__device__ __forceinline__ void rx_gate(RxRing<T> &R, int lane, int need, bool l2, bool cl, int lo, int hi,
                                        const unsigned long long *rxw, long long rxs, unsigned tag, int &seen,
                                        int limit, PsCtrl *ctrl, bool &timed_out) {
    using X = Xch<T>;
    const bool wants = need >= lo && need < hi;
    int spins = 0;
    for (;;) {
        bool ok = true;
        if (wants && !timed_out) {
            if (l2 && need >= seen) {
                int m = ld_volatile_s32(&R.prog[0][lane]);
#pragma unroll
                for (int r = 1; r < RX_NR; r++) m = min(m, ld_volatile_s32(&R.prog[r][lane]));
                seen = m;
                ok = need < seen;
            } else if (cl) {
                unsigned long long w[X::W];
#pragma unroll
                for (int q = 0; q < X::W; q++) w[q] = *(const volatile unsigned long long *)(rxw + need * rxs + q);
                ok = X::ready(w, tag);
            }
        }
        if (__all_sync(0xffffffffu, ok)) break;
        if (++spins > limit) {
            if (!timed_out && lane == 0) atomicOr(&ctrl->err, GFS_DEV_ERR_TIMEOUT);
            timed_out = true;
        }
    }
    __threadfence_block();   // what the gate saw before the barrier that follows
}

__device__ __forceinline__ void compute_barrier() { asm volatile("bar.sync 1, %0;" ::"n"(SPLANE) : "memory"); }

// Lean triangular solve (FWD / BWD).  One pencil per thread; everything that
// does not depend on the step is hoisted, per-step addresses are pointer
// increments, every slot of the block's plane is copied and stored (slots of
// cells outside the grid store 0, which they already hold), and only the value
// select, the dot product and the exchange words are predicated on the cell
// being inside the grid.  This keeps the per-step instruction count -- the issue-rate limit of
// the SMs hosting two such CTAs -- low.
template <class T, int MODE, int P, int PE>
__global__ void __launch_bounds__(SPLANE + RX_THREADS, 1) k_tri(SweepArgs<T> A) {
    using Op = Ar<T>;
    using X = Xch<T>;
    static_assert(MODE == SW_FWD || MODE == SW_BWD, "triangular solves only");
    constexpr bool bwd = MODE == SW_BWD;
    constexpr long long PS = bwd ? -(long long)SPLANE : (long long)SPLANE;
    constexpr long long XP = (long long)XCH_PER_PLANE * X::W;
    constexpr long long XS = bwd ? -XP : XP;
    // FP64 solves read negscale * precon (one FP64 multiply per cell fewer: GB300's FP64
    // rate bounds them) from ring array IM; FP32 solves form it
    constexpr bool PM = sizeof(T) == 8;
    constexpr int IM = bwd ? 3 : 2;
    constexpr int NARR = (bwd ? 3 : 2) + (PM ? 1 : 0);
    __shared__ T xb[2][SBK][SBJ];
    __shared__ __align__(16) T ring[NARR][P][SPLANE];
    __shared__ unsigned sh_ticket, sh_epoch;
    __shared__ RxRing<T> rxr;
    if (A.ctrl->done) return;
    const int tid = threadIdx.x;
    const Skew &K = A.K;
    const int S = K.S;
    if (tid == 0) {
        sh_ticket = atomicAdd(A.ticket, 1u);
        sh_epoch = A.ctrl->epoch;
    }
    for (int q = tid; q < RX_NR * 32; q += blockDim.x) (&rxr.prog[0][0])[q] = 0;
    if (tid == 0) rxr.cons = 0;
    __syncthreads();
    const unsigned t = sh_ticket, tag = sh_epoch;
    const unsigned wtag = tag + A.wait_skew;   // the tag the waits look for (tag itself unless a test skews it)
    int bj = (int)(t % K.nbj), bk = (int)(t / K.nbj);
    if (bwd) {
        bj = K.nbj - 1 - bj;
        bk = K.nbk - 1 - bk;
    }
    const int pbj = bwd ? bj + 1 : bj - 1, pbk = bwd ? bk + 1 : bk - 1;
    const int cbj = bwd ? bj - 1 : bj + 1, cbk = bwd ? bk - 1 : bk + 1;
    // blocks without fluid are skipped; their consumers take 0 (see k_sweep)
    const bool live = A.blkf[bk * K.nbj + bj] != 0;
    const bool has_pj = pbj >= 0 && pbj < K.nbj && A.blkf[bk * K.nbj + pbj],
               has_pk = pbk >= 0 && pbk < K.nbk && A.blkf[pbk * K.nbj + bj];
    const bool has_cj = cbj >= 0 && cbj < K.nbj && A.blkf[bk * K.nbj + cbj],
               has_ck = cbk >= 0 && cbk < K.nbk && A.blkf[cbk * K.nbj + bj];
    bool timed_out = false;
    const long long xblock = (long long)S * XP;
    Acc2f dot32;
    double dot64 = 0.0;
    if (tid >= SPLANE) {
        // receiver warps (class cls): lane l < 16 feeds the j-edge pencil kl = l, lane 16 + l the k-edge pencil jl = l
        const int cls = (tid - SPLANE) >> 5, lane = (tid - SPLANE) & 31, e = lane >> 4, idx = lane & 15;
        const int jl_c = e == 0 ? (bwd ? SBJ - 1 : 0) : idx, kl_c = e == 0 ? idx : (bwd ? SBK - 1 : 0);
        const bool valid_c = live && bj * SBJ + jl_c < K.ny && bk * SBK + kl_c < K.nz;
        if (valid_c && (e == 0 ? has_pj : has_pk)) {
            const int lo = bwd ? S - K.nx - jl_c - kl_c : jl_c + kl_c;
            const unsigned long long *src =
                e == 0 ? A.xch + (long long)(bk * K.nbj + pbj) * xblock +
                             (bwd ? (long long)(S - 1 - (SBJ - 1)) : (long long)(SBJ - 1)) * XP + (long long)idx * X::W
                       : A.xch + (long long)(pbk * K.nbj + bj) * xblock +
                             (bwd ? (long long)(S - 1 - (SBK - 1)) : (long long)(SBK - 1)) * XP +
                             (long long)(SBJ + idx) * X::W;
            rx_receive<T>(rxr, cls, lane, src, XS, lo, lo + K.nx, wtag, A.spin_limit, A.ctrl);
        }
    } else {
    const int jl = tid % SBJ, kl = tid / SBJ;
    const bool valid = live && bj * SBJ + jl < K.ny && bk * SBK + kl < K.nz;
    const int xj = bwd ? jl + 1 : jl - 1, xk = bwd ? kl + 1 : kl - 1;
    const bool at_j = bwd ? jl == SBJ - 1 : jl == 0;
    const bool at_k = bwd ? kl == SBK - 1 : kl == 0;
    const bool in_j = at_j && has_pj, in_k = at_k && has_pk;
    const bool out_j = (bwd ? jl == 0 : jl == SBJ - 1) && has_cj;
    const bool out_k = (bwd ? kl == 0 : kl == SBK - 1) && has_ck;
    const int st_lo = valid ? (bwd ? S - K.nx - jl - kl : jl + kl) : S;
    const int st_hi = valid ? st_lo + K.nx : S;
    const long long q0 = K.base(bj, bk) + kl * SBJ + jl + (bwd ? (long long)(S - 1) * SPLANE : 0);
    // inputs: each plane of a block is SPLANE contiguous slots, copied in 16-byte
    // pieces by NCP threads starting at thread NCP (the first and last warps
    // carry the k-edge exchange); 16-byte aligned: allocation bases, and plane
    // offsets that are multiples of SPLANE elements
    constexpr int E = 16 / (int)sizeof(T), NCP = SPLANE / E;
    const int cpi = tid - NCP;
    const bool copier = cpi >= 0 && cpi < NCP;
    const long long qp = K.base(bj, bk) + (bwd ? (long long)(S - 1) * SPLANE : 0) + (long long)(copier ? cpi : 0) * E;
    const T *ca = A.in + qp, *cb = A.precon + qp, *cc = (bwd ? A.rdot : A.in) + qp, *cm = (PM ? A.mpc : A.in) + qp;
    const T *fa = ca + P * PS, *fb = cb + P * PS, *fc = cc + P * PS, *fm = cm + P * PS;   // the first refill: step P
    T *po = A.out + q0;
    unsigned long long *xbuf = A.xch;
    unsigned long long *pxj_out = xbuf + (long long)(bk * K.nbj + bj) * xblock + (bwd ? (long long)(S - 1) * XP : 0) +
                                  (long long)kl * X::W;
    unsigned long long *pxk_out = xbuf + (long long)(bk * K.nbj + bj) * xblock + (bwd ? (long long)(S - 1) * XP : 0) +
                                  (long long)(SBJ + jl) * X::W;
    // warp 0 is the gate: lane l watches edge pencil l (lanes 0-15 the j edge, kl = l;
    // lanes 16-31 the k edge, jl = l - 16), all of them fed through L2 here
    const int g_e = tid >> 4, g_idx = tid & 15;
    const int g_jl = g_e == 0 ? (bwd ? SBJ - 1 : 0) : g_idx, g_kl = g_e == 0 ? g_idx : (bwd ? SBK - 1 : 0);
    const bool g_valid = tid < 32 && live && bj * SBJ + g_jl < K.ny && bk * SBK + g_kl < K.nz;
    const bool g_l2 = g_valid && (g_e == 0 ? has_pj : has_pk);
    const int g_lo = bwd ? S - K.nx - g_jl - g_kl : g_jl + g_kl, g_hi = g_lo + K.nx;
    int g_seen = 0;

    // fill the ring with steps 0..P-1
#pragma unroll
    for (int u = 0; u < P; u++) {
        if (copier && u < S && live) {
            cp_async<16>(&ring[0][u][cpi * E], ca + u * PS, true);
            cp_async<16>(&ring[1][u][cpi * E], cb + u * PS, true);
            if (bwd) cp_async<16>(&ring[2][u][cpi * E], cc + u * PS, true);
            if (PM) cp_async<16>(&ring[IM][u][cpi * E], cm + u * PS, true);
        }
        cp_async_commit();
    }
    cp_async_wait<P - 1>();   // step 0 has landed ...
    if (tid < 32 && live)
        rx_gate<T>(rxr, tid, 0, g_l2, false, g_lo, g_hi, nullptr, 0, wtag, g_seen, A.spin_limit, A.ctrl, timed_out);
    compute_barrier();        // ... and, with the edge inputs of step 0, is visible to every compute thread

    T prev = T(0);
    const int SP = live ? ((S + P - 1) / P) * P : 0;
    for (int s0 = 0; s0 < SP; s0 += P) {
#pragma unroll
        for (int u = 0; u < P; u++) {
            const int st = s0 + u;
            // the slot step st-1 read is free (the barrier of step st-1 has passed):
            // refill it with step st-1+P
            if (copier && st >= 1) {   // warp-uniform: the other warps skip it
                if (st - 1 + P < S) {
                    cp_async<16>(&ring[0][(u + P - 1) % P][cpi * E], fa, true);
                    cp_async<16>(&ring[1][(u + P - 1) % P][cpi * E], fb, true);
                    if (bwd) cp_async<16>(&ring[2][(u + P - 1) % P][cpi * E], fc, true);
                    if (PM) cp_async<16>(&ring[IM][(u + P - 1) % P][cpi * E], fm, true);
                }
                fa += PS;
                fb += PS;
                fc += PS;
                fm += PS;
            }
            cp_async_commit();
            const bool act = st >= st_lo && st < st_hi;
            T nj_ = at_j ? T(0) : xb[(st - 1) & 1][kl][xj];
            T nk_ = at_k ? T(0) : xb[(st - 1) & 1][xk][jl];
            if (in_j && act) nj_ = rxr.val[st & (RX_R - 1)][kl];         // the gate saw it arrive
            if (in_k && act) nk_ = rxr.val[st & (RX_R - 1)][SBJ + jl];
            const T ra = ring[0][u][tid], pc = ring[1][u][tid];
            T val, xch;
            if (MODE == SW_FWD) {
                // _applyPreconditioner forward solve (pressuresolver.cpp:311-351); neighbours hand
                // over (negscale*precon)*q; precon is 0 off the fluid set, so those cells give 0
                val = Op::mul(Op::sub(Op::sub(Op::sub(ra, prev), nj_), nk_), pc);
                xch = Op::mul(PM ? ring[IM][u][tid] : Op::mul(A.negscale, pc), val);
            } else {
                // backward solve (pressuresolver.cpp:354-385)
                const T m = PM ? ring[IM][u][tid] : Op::mul(A.negscale, pc);
                val = Op::mul(Op::sub(Op::sub(Op::sub(ra, Op::mul(m, prev)), Op::mul(m, nj_)), Op::mul(m, nk_)), pc);
                xch = val;
            }
            // slots outside the grid (and steps past the last plane) store and hand over 0
            val = act ? val : T(0);
            xch = act ? xch : T(0);
            if (MODE == SW_BWD && act) {
                const T rv = ring[2][u][tid];
                if (sizeof(T) == 4) dot32.add((float)val * (float)rv);
                else dot64 += (double)val * (double)rv;
            }
            if (st < S) {
                *po = val;
                if (out_j && act) X::put(pxj_out + (long long)st * XS, xch, tag);
                if (out_k && act) X::put(pxk_out + (long long)st * XS, xch, tag);
            }
            po += PS;
            xb[st & 1][kl][jl] = xch;
            prev = xch;
            cp_async_wait<P - 2>();   // step st+1 has landed (its group is older than the last P-2)
            if (tid < 32) {
                if (st + 1 < S)
                    rx_gate<T>(rxr, tid, st + 1, g_l2, false, g_lo, g_hi, nullptr, 0, wtag, g_seen, A.spin_limit,
                               A.ctrl, timed_out);
                if (tid == 0 && ((st + 1) & (RX_CB - 1)) == 0) st_volatile_s32(&rxr.cons, st);   // steps < st are read
            }
            compute_barrier();
        }
    }
    cp_async_wait<0>();
    }

    double part = 0.0;
    if (MODE == SW_BWD) part = block_reduce<0>(sizeof(T) == 4 ? dot32.value() : dot64);
    __shared__ bool last;
    const unsigned nblocks = (unsigned)(K.nbj * K.nbk);
    if (tid == 0) {
        if (MODE == SW_BWD) A.partials[bj + K.nbj * bk] = part;
        __threadfence();
        unsigned tk = atomicAdd(A.done_ticket, 1u);
        last = tk == nblocks - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    if (MODE == SW_BWD) {
        double acc = 0.0;
        for (unsigned q = tid; q < nblocks; q += blockDim.x) acc += __ldcg(A.partials + q);
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
        A.ctrl->epoch = tag + 1 == 0 ? 1u : tag + 1;
    }
}

// Clustered triangular solve (FWD / BWD): k_tri with the hand-overs inside a
// thread-block cluster moved from L2 to distributed shared memory.  A cluster
// of CL_J x CL_K blocks takes one dispatch ticket (clusters in dependency
// order, 4 x 2 or 2 x 2 blocks); within it, a producer block stores each edge value, tagged as in the
// L2 exchange, straight into the consumer block's shared receive buffer, where
// the consumer block's gate warp checks the tag in its own shared memory.  Hand-overs between clusters go
// through L2 and the receiver warp.  On a monotone path through the 16 x 16 blocks of a
// 256^3 grid that leaves 3 + 7 (4 x 2) or 7 + 7 (2 x 2) of the 30 hand-overs in L2.  The receive
// buffers hold every step (no slot is reused within a launch), so producers
// need no flow control; a cluster barrier after zeroing them orders the first
// remote store after the zeroing, and one before exit keeps every block
// resident while its peers may still store into it.  Arithmetic, summation
// order and outputs are k_tri's.

// A receive-buffer word whose tag has been seen (by the gate).
template <class T>
__device__ __forceinline__ T rx_read(const unsigned long long *p) {
    using X = Xch<T>;
    unsigned long long w[X::W];
#pragma unroll
    for (int q = 0; q < X::W; q++) w[q] = *(const volatile unsigned long long *)(p + q);
    return X::value(w);
}

template <class T>
__device__ __forceinline__ void rx_put(unsigned long long *p, T v, unsigned tag) {
    if constexpr (sizeof(T) == 4) {
        *(volatile unsigned long long *)p = ((unsigned long long)tag << 32) | (unsigned long long)__float_as_uint(v);
    } else {
        unsigned long long bits = (unsigned long long)__double_as_longlong(v);
        *(volatile unsigned long long *)p = ((unsigned long long)tag << 32) | (bits & 0xFFFFFFFFull);
        *(volatile unsigned long long *)(p + 1) = ((unsigned long long)tag << 32) | (bits >> 32);
    }
}

// receive-buffer steps: the first edge value a producer hands over is its step SBJ-1 (= SBK-1)
__host__ __device__ __forceinline__ int rx_steps(int S) { return S - (SBJ - 1); }

template <class T, int MODE, int P, int PE, int CL_J, int CL_K>
__global__ void __cluster_dims__(CL_J * CL_K, 1, 1) __launch_bounds__(SPLANE + RX_THREADS, 1) k_tri_cl(SweepArgs<T> A) {
    namespace cg = cooperative_groups;
    using Op = Ar<T>;
    using X = Xch<T>;
    static_assert(MODE == SW_FWD || MODE == SW_BWD, "triangular solves only");
    static_assert(SBJ == SBK, "one receive-buffer step count for both edges");
    constexpr bool bwd = MODE == SW_BWD;
    constexpr long long PS = bwd ? -(long long)SPLANE : (long long)SPLANE;
    constexpr long long XP = (long long)XCH_PER_PLANE * X::W;
    constexpr long long XS = bwd ? -XP : XP;
    constexpr int NARR = bwd ? 3 : 2;
    constexpr int W = X::W;
    __shared__ T xb[2][SBK][SBJ];
    __shared__ __align__(16) T ring[NARR][P][SPLANE];
    __shared__ unsigned sh_ticket, sh_epoch;
    __shared__ RxRing<T> rxr;   // the L2 hand-overs (receiver warp)
    // receive buffers: j edge [step][kl][W], then k edge [step][jl][W]
    extern __shared__ __align__(16) unsigned long long rx[];
    if (A.ctrl->done) return;   // the same value in every block of the launch
    cg::cluster_group cl = cg::this_cluster();
    const unsigned rank = cl.block_rank();
    const int tid = threadIdx.x;
    const Skew &K = A.K;
    const int S = K.S;
    const int NR = rx_steps(S);
    unsigned long long *rxj = rx, *rxk = rx + (long long)NR * SBK * W;
    for (int q = tid; q < 2 * NR * SBK * W; q += blockDim.x) rx[q] = 0ull;
    for (int q = tid; q < RX_NR * 32; q += blockDim.x) (&rxr.prog[0][0])[q] = 0;
    if (tid == 0) rxr.cons = 0;
    if (tid == 0) {
        if (rank == 0) sh_ticket = atomicAdd(A.ticket, 1u);
        sh_epoch = A.ctrl->epoch;
    }
    cl.sync();
    const unsigned t = *cl.map_shared_rank(&sh_ticket, 0u), tag = sh_epoch;
    const unsigned wtag = tag + A.wait_skew;
    const int ncj = (K.nbj + CL_J - 1) / CL_J, nck = (K.nbk + CL_K - 1) / CL_K;
    int cj = (int)(t % (unsigned)ncj), ck = (int)(t / (unsigned)ncj);
    if (bwd) {
        cj = ncj - 1 - cj;
        ck = nck - 1 - ck;
    }
    const int j0 = cj * CL_J, k0 = ck * CL_K;
    const int bj = j0 + (int)(rank % CL_J), bk = k0 + (int)(rank / CL_J);
    const bool exists = bj < K.nbj && bk < K.nbk;
    const bool live = exists && A.blkf[bk * K.nbj + bj] != 0;
    const int pbj = bwd ? bj + 1 : bj - 1, pbk = bwd ? bk + 1 : bk - 1;
    const int cbj = bwd ? bj - 1 : bj + 1, cbk = bwd ? bk - 1 : bk + 1;
    const bool has_pj = exists && pbj >= 0 && pbj < K.nbj && A.blkf[bk * K.nbj + pbj],
               has_pk = exists && pbk >= 0 && pbk < K.nbk && A.blkf[pbk * K.nbj + bj];
    const bool has_cj = exists && cbj >= 0 && cbj < K.nbj && A.blkf[bk * K.nbj + cbj],
               has_ck = exists && cbk >= 0 && cbk < K.nbk && A.blkf[cbk * K.nbj + bj];
    // neighbours inside this cluster hand over through shared memory
    const bool pj_cl = pbj >= j0 && pbj < j0 + CL_J, pk_cl = pbk >= k0 && pbk < k0 + CL_K;
    const bool cj_cl = cbj >= j0 && cbj < j0 + CL_J, ck_cl = cbk >= k0 && cbk < k0 + CL_K;
    bool timed_out = false;
    const long long xblock = (long long)S * XP;
    Acc2f dot32;
    double dot64 = 0.0;
    if (tid >= SPLANE) {
        // receiver warps (class cls) for the edges fed through L2: lane l < 16 feeds
        // the j-edge pencil kl = l, lane 16 + l the k-edge pencil jl = l
        const int cls = (tid - SPLANE) >> 5, lane = (tid - SPLANE) & 31, e = lane >> 4, idx = lane & 15;
        const int jl_c = e == 0 ? (bwd ? SBJ - 1 : 0) : idx, kl_c = e == 0 ? idx : (bwd ? SBK - 1 : 0);
        const bool valid_c = live && bj * SBJ + jl_c < K.ny && bk * SBK + kl_c < K.nz;
        if (valid_c && (e == 0 ? has_pj && !pj_cl : has_pk && !pk_cl)) {
            const int lo = bwd ? S - K.nx - jl_c - kl_c : jl_c + kl_c;
            const unsigned long long *src =
                e == 0 ? A.xch + (long long)(bk * K.nbj + pbj) * xblock +
                             (bwd ? (long long)(S - 1 - (SBJ - 1)) : (long long)(SBJ - 1)) * XP + (long long)idx * W
                       : A.xch + (long long)(pbk * K.nbj + bj) * xblock +
                             (bwd ? (long long)(S - 1 - (SBK - 1)) : (long long)(SBK - 1)) * XP +
                             (long long)(SBJ + idx) * W;
            rx_receive<T>(rxr, cls, lane, src, XS, lo, lo + K.nx, wtag, A.spin_limit, A.ctrl);
        }
    } else {
    const int jl = tid % SBJ, kl = tid / SBJ;
    const bool valid = live && bj * SBJ + jl < K.ny && bk * SBK + kl < K.nz;
    const int xj = bwd ? jl + 1 : jl - 1, xk = bwd ? kl + 1 : kl - 1;
    const bool at_j = bwd ? jl == SBJ - 1 : jl == 0;
    const bool at_k = bwd ? kl == SBK - 1 : kl == 0;
    const bool in_j = at_j && has_pj, in_k = at_k && has_pk;
    const bool out_j = (bwd ? jl == 0 : jl == SBJ - 1) && has_cj;
    const bool out_k = (bwd ? kl == 0 : kl == SBK - 1) && has_ck;
    const int st_lo = valid ? (bwd ? S - K.nx - jl - kl : jl + kl) : S;
    const int st_hi = valid ? st_lo + K.nx : S;
    const long long q0 = K.base(bj, bk) + kl * SBJ + jl + (bwd ? (long long)(S - 1) * SPLANE : 0);
    // inputs: each plane of a block is SPLANE contiguous slots, copied in 16-byte
    // pieces by NCP threads starting at thread NCP, so that the first and last
    // warps, which carry the k-edge exchange, copy nothing in FP32 (16-byte
    // aligned: allocation bases, and plane offsets that are multiples of SPLANE)
    constexpr int E = 16 / (int)sizeof(T), NCP = SPLANE / E;
    const int cpi = tid - NCP;
    const bool copier = cpi >= 0 && cpi < NCP;
    const long long qp = K.base(bj, bk) + (bwd ? (long long)(S - 1) * SPLANE : 0) + (long long)(copier ? cpi : 0) * E;
    const T *ca = A.in + qp, *cb = A.precon + qp, *cc = (bwd ? A.rdot : A.in) + qp;
    const T *fa = ca + P * PS, *fb = cb + P * PS, *fc = cc + P * PS;
    T *po = A.out + q0;
    unsigned long long *xbuf = A.xch;
    const long long bself = exists ? (long long)(bk * K.nbj + bj) * xblock : 0;
    unsigned long long *pxj_out = xbuf + bself + (bwd ? (long long)(S - 1) * XP : 0) + (long long)kl * W;
    unsigned long long *pxk_out = xbuf + bself + (bwd ? (long long)(S - 1) * XP : 0) + (long long)(SBJ + jl) * W;
    // warp 0 is the gate: lane l watches edge pencil l (lanes 0-15 the j edge, kl = l;
    // lanes 16-31 the k edge, jl = l - 16), fed through L2 or, inside the cluster,
    // through this block's receive buffer
    const int g_e = tid >> 4, g_idx = tid & 15;
    const int g_jl = g_e == 0 ? (bwd ? SBJ - 1 : 0) : g_idx, g_kl = g_e == 0 ? g_idx : (bwd ? SBK - 1 : 0);
    const bool g_valid = tid < 32 && live && bj * SBJ + g_jl < K.ny && bk * SBK + g_kl < K.nz;
    const bool g_has = g_valid && (g_e == 0 ? has_pj : has_pk), g_incl = g_e == 0 ? pj_cl : pk_cl;
    const bool g_l2 = g_has && !g_incl, g_cl = g_has && g_incl;
    const int g_lo = bwd ? S - K.nx - g_jl - g_kl : g_jl + g_kl, g_hi = g_lo + K.nx;
    const unsigned long long *g_rxw = (g_e == 0 ? rxj : rxk) + (long long)g_idx * W;
    int g_seen = 0;
    // this thread's receive words (step 0) and, on a downstream edge inside the
    // cluster, the consumer's (its step 0 is this block's step SBJ-1)
    const unsigned long long *rj_in = rxj + (long long)kl * W;
    const unsigned long long *rk_in = rxk + (long long)jl * W;
    unsigned long long *rj_out = nullptr, *rk_out = nullptr;
    if (out_j && cj_cl) rj_out = cl.map_shared_rank(rxj, rank + (unsigned)(cbj - bj)) + (long long)kl * W;
    if (out_k && ck_cl) rk_out = cl.map_shared_rank(rxk, rank + (unsigned)((cbk - bk) * CL_J)) + (long long)jl * W;

#pragma unroll
    for (int u = 0; u < P; u++) {
        if (copier && u < S && live) {
            cp_async<16>(&ring[0][u][cpi * E], ca + u * PS, true);
            cp_async<16>(&ring[1][u][cpi * E], cb + u * PS, true);
            if (bwd) cp_async<16>(&ring[NARR - 1][u][cpi * E], cc + u * PS, true);
        }
        cp_async_commit();
    }
    cp_async_wait<P - 1>();   // step 0 has landed ...
    if (tid < 32 && live)
        rx_gate<T>(rxr, tid, 0, g_l2, g_cl, g_lo, g_hi, g_rxw, (long long)SBK * W, wtag, g_seen, A.spin_limit, A.ctrl,
                   timed_out);
    compute_barrier();        // ... and, with the edge inputs of step 0, is visible to every compute thread

    T prev = T(0);
    const int SP = live ? ((S + P - 1) / P) * P : 0;
    for (int s0 = 0; s0 < SP; s0 += P) {
#pragma unroll
        for (int u = 0; u < P; u++) {
            const int st = s0 + u;
            // the slot step st-1 read is free (the barrier of step st-1 has passed):
            // refill it with step st-1+P
            if (copier && st >= 1) {   // warp-uniform: the other warps skip it
                if (st - 1 + P < S) {
                    cp_async<16>(&ring[0][(u + P - 1) % P][cpi * E], fa, true);
                    cp_async<16>(&ring[1][(u + P - 1) % P][cpi * E], fb, true);
                    if (bwd) cp_async<16>(&ring[NARR - 1][(u + P - 1) % P][cpi * E], fc, true);
                }
                fa += PS;
                fb += PS;
                fc += PS;
            }
            cp_async_commit();
            const bool act = st >= st_lo && st < st_hi;
            T nj_ = at_j ? T(0) : xb[(st - 1) & 1][kl][xj];
            T nk_ = at_k ? T(0) : xb[(st - 1) & 1][xk][jl];
            // the gate saw these inputs arrive
            if (in_j && act)
                nj_ = pj_cl ? rx_read<T>(rj_in + (long long)st * SBK * W) : rxr.val[st & (RX_R - 1)][kl];
            if (in_k && act)
                nk_ = pk_cl ? rx_read<T>(rk_in + (long long)st * SBJ * W) : rxr.val[st & (RX_R - 1)][SBJ + jl];
            const T ra = ring[0][u][tid], pc = ring[1][u][tid];
            T val, xch;
            if (MODE == SW_FWD) {
                // _applyPreconditioner forward solve (pressuresolver.cpp:311-351)
                val = Op::mul(Op::sub(Op::sub(Op::sub(ra, prev), nj_), nk_), pc);
                xch = Op::mul(Op::mul(A.negscale, pc), val);
            } else {
                // backward solve (pressuresolver.cpp:354-385)
                const T m = Op::mul(A.negscale, pc);
                val = Op::mul(Op::sub(Op::sub(Op::sub(ra, Op::mul(m, prev)), Op::mul(m, nj_)), Op::mul(m, nk_)), pc);
                xch = val;
            }
            val = act ? val : T(0);
            xch = act ? xch : T(0);
            if (MODE == SW_BWD && act) {
                const T rv = ring[NARR - 1][u][tid];
                if (sizeof(T) == 4) dot32.add((float)val * (float)rv);
                else dot64 += (double)val * (double)rv;
            }
            if (st < S) {
                *po = val;
                if (out_j && act) {
                    if (rj_out) rx_put<T>(rj_out + (long long)(st - (SBJ - 1)) * SBK * W, xch, tag);
                    else X::put(pxj_out + (long long)st * XS, xch, tag);
                }
                if (out_k && act) {
                    if (rk_out) rx_put<T>(rk_out + (long long)(st - (SBK - 1)) * SBJ * W, xch, tag);
                    else X::put(pxk_out + (long long)st * XS, xch, tag);
                }
            }
            po += PS;
            xb[st & 1][kl][jl] = xch;
            prev = xch;
            cp_async_wait<P - 2>();   // step st+1 has landed (its group is older than the last P-2)
            if (tid < 32) {
                if (st + 1 < S)
                    rx_gate<T>(rxr, tid, st + 1, g_l2, g_cl, g_lo, g_hi, g_rxw, (long long)SBK * W, wtag, g_seen,
                               A.spin_limit, A.ctrl, timed_out);
                if (tid == 0 && ((st + 1) & (RX_CB - 1)) == 0) st_volatile_s32(&rxr.cons, st);   // steps < st are read
            }
            compute_barrier();
        }
    }
    cp_async_wait<0>();
    }
    // no block of the cluster leaves while a peer may still store into it
    cl.sync();

    double part = 0.0;
    if (MODE == SW_BWD) part = block_reduce<0>(sizeof(T) == 4 ? dot32.value() : dot64);
    __shared__ bool last;
    if (tid == 0) {
        if (MODE == SW_BWD && exists) A.partials[bj + K.nbj * bk] = part;
        __threadfence();
        unsigned tk = atomicAdd(A.done_ticket, 1u);
        last = tk == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    if (MODE == SW_BWD) {
        const unsigned nblocks = (unsigned)(K.nbj * K.nbk);
        double acc = 0.0;
        for (unsigned q = tid; q < nblocks; q += blockDim.x) acc += __ldcg(A.partials + q);
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
        A.ctrl->epoch = tag + 1 == 0 ? 1u : tag + 1;
    }
}

// dynamic shared memory of k_tri_cl: the two receive buffers
template <class T>
static size_t tri_cl_smem(int S) {
    return (size_t)2 * rx_steps(S) * SBJ * Xch<T>::W * sizeof(unsigned long long);
}
// ------------------------------------------------- one-warp triangular solve
//
// k_tri_warp (FP32 FWD / BWD): the triangular solves with ONE compute warp per
// 16 x 16 pencil block and no per-plane barrier.  Lane L (a = L & 3, b = L >> 2)
// owns the pencils jl' = 4a..4a+3 of the rows kl' = b and kl' = b + 8, where the
// primed coordinates are the block's own for the forward solve and mirrored
// (jl' = 15 - jl, kl' = 15 - kl) for the backward one, so that both walk the
// same upstream direction: a lane's two rows are the 16-byte plane chunks L and
// L + 32 (forward) or 63 - L and 31 - L with the four pencils reversed
// (backward), one conflict-free 16-byte shared-memory read per row and array.
// Per step, the i neighbour is the lane's own previous value, the j neighbour
// the previous pencil of the row (a shuffle across the lane's left boundary),
// the k neighbour the row below (a shuffle), and the block edges the receiver
// ring.  The plane inputs arrive by bulk copies (cp.async.bulk, WT_G planes per
// copy and array, WT_NG copies in flight, full / empty mbarriers) issued by one
// loader lane; the edge words by the RX_NR receiver warps (one read in flight per
// lane, classes of steps mod RX_NR), each publishing the step below which every
// edge word of its class is in the ring.  Slots of cells outside the grid hold 0
// in the input and preconditioner vectors, so such a cell computes +-0 without a
// select and hands over +-0.  Arithmetic per cell is k_tri's; the backward
// solve's dot(z, r) sums each lane's eight rounded products of a step pairwise
// before its compensated running sum (deterministic; its rounding differs from
// k_tri's per-pencil sums; measured at 256^3 it takes as many inner iterations).
static constexpr int WT_G = 8;                             // planes per bulk copy
static constexpr int WT_NG = 4;                            // copies in flight
// The compute warp checks the receivers' progress once per WT_POLL steps, for all of
// them: the check (volatile reads and a fence) holds the compiler back from scheduling
// loads across it, so fewer checks buy a faster step (a block with no upstream: 101 ns
// per plane checking every step, 83 every 4, 74 never) for up to WT_POLL - 1 steps of
// extra lag behind each producer; at 256^3 every 4 steps was fastest (2: 11.3, 4: 11.8,
// 8: 11.7 substeps/s).
static constexpr int WT_POLL = 4;
static_assert(WT_G % WT_POLL == 0, "a poll chunk never straddles two copy groups");
static constexpr int WT_THREADS = 32 + RX_THREADS + 32;    // compute warp, receiver warps, loader warp
static_assert(RX_CB == WT_G, "receive-ring slots are handed back once per copy group");

struct WtRx {
    float val[RX_R][32];   // step s, lane l: the edge word (l < 16: j edge of kl = l; 16 + l: k edge of jl = l)
    int prog[RX_NR];       // class r: every edge word of the class's steps below prog[r] is in val
    int cons;              // steps below cons have been read by the compute warp
};

template <int MODE>
static constexpr size_t tri_warp_smem() {
    return (size_t)WT_NG * (MODE == SW_BWD ? 3 : 2) * WT_G * SPLANE * sizeof(float) +
           2 * WT_NG * sizeof(unsigned long long);
}

__device__ __forceinline__ void mbar_init(unsigned long long *mb, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(mb)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long *mb, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(mb)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long *mb) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(mb)) : "memory");
}
// potentially blocking test of the phase with the given parity (the thread may be
// suspended for a bounded time); true once that phase has completed
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *mb, unsigned parity) {
    unsigned ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(ok)
                 : "r"(smem_addr(mb)), "r"(parity)
                 : "memory");
    return ok != 0;
}
// bulk copy global -> shared (16-byte aligned addresses, size a multiple of 16),
// completing bytes on the mbarrier
__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *mb) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(mb))
                 : "memory");
}
// tagged exchange words without a branch: stored only where pred is nonzero
__device__ __forceinline__ void put_word(unsigned long long *p, float v, unsigned tag, unsigned pred) {
    const unsigned long long w = ((unsigned long long)tag << 32) | (unsigned long long)__float_as_uint(v);
    asm volatile("{\n .reg .pred q;\n setp.ne.u32 q, %2, 0;\n @q st.relaxed.gpu.global.u64 [%0], %1;\n}\n"
                 ::"l"(p), "l"(w), "r"(pred)
                 : "memory");
}
__device__ __forceinline__ void put_words2(unsigned long long *p, float v0, float v1, unsigned tag, unsigned pred) {
    const unsigned long long w0 = ((unsigned long long)tag << 32) | (unsigned long long)__float_as_uint(v0);
    const unsigned long long w1 = ((unsigned long long)tag << 32) | (unsigned long long)__float_as_uint(v1);
    asm volatile("{\n .reg .pred q;\n setp.ne.u32 q, %3, 0;\n @q st.relaxed.gpu.global.v2.u64 [%0], {%1, %2};\n}\n"
                 ::"l"(p), "l"(w0), "l"(w1), "r"(pred)
                 : "memory");
}
// the four floats of a 16-byte chunk in pencil order (reversed for the mirrored backward solve)
template <bool REV>
__device__ __forceinline__ void unpack4(const float4 v, float o[4]) {
    if (REV) { o[0] = v.w; o[1] = v.z; o[2] = v.y; o[3] = v.x; }
    else { o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w; }
}
template <bool REV>
__device__ __forceinline__ float4 pack4(const float o[4]) {
    return REV ? make_float4(o[3], o[2], o[1], o[0]) : make_float4(o[0], o[1], o[2], o[3]);
}

template <int MODE>
__global__ void __launch_bounds__(WT_THREADS, 1) k_tri_warp(SweepArgs<float> A) {
    using Op = Ar<float>;
    static_assert(MODE == SW_FWD || MODE == SW_BWD, "triangular solves only");
    constexpr bool bwd = MODE == SW_BWD;
    constexpr int NARR = bwd ? 3 : 2;
    constexpr unsigned FULL = 0xffffffffu;
    constexpr long long XP = XCH_PER_PLANE;   // words per block plane (one per FP32 entry)
    constexpr long long XS = bwd ? -XP : XP;
    constexpr long long PS = bwd ? -(long long)SPLANE : (long long)SPLANE;
    extern __shared__ __align__(128) unsigned char wt_smem[];
    float (*ring)[NARR][WT_G][SPLANE] = reinterpret_cast<float (*)[NARR][WT_G][SPLANE]>(wt_smem);
    unsigned long long *mfull =
        reinterpret_cast<unsigned long long *>(wt_smem + (size_t)WT_NG * NARR * WT_G * SPLANE * sizeof(float));
    unsigned long long *mempty = mfull + WT_NG;
    __shared__ __align__(16) WtRx rx;
    __shared__ unsigned sh_ticket, sh_epoch;
    if (A.ctrl->done) return;   // the same value in every block of the launch
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const Skew &K = A.K;
    const int S = K.S;
    if (tid == 0) {
        sh_ticket = atomicAdd(A.ticket, 1u);
        sh_epoch = A.ctrl->epoch;
        rx.cons = 0;
    }
    if (tid < RX_NR) rx.prog[tid] = 0;
    for (int q = tid; q < RX_R * 32; q += WT_THREADS) (&rx.val[0][0])[q] = 0.f;
    if (tid == WT_THREADS - 32) {
        for (int u = 0; u < WT_NG; u++) {
            mbar_init(&mfull[u], 1);
            mbar_init(&mempty[u], 1);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    const unsigned t = sh_ticket, tag = sh_epoch;
    const unsigned wtag = tag + A.wait_skew;   // the tag the waits look for (tag itself unless a test skews it)
    int bj = (int)(t % K.nbj), bk = (int)(t / K.nbj);
    if (bwd) {
        bj = K.nbj - 1 - bj;
        bk = K.nbk - 1 - bk;
    }
    const int pbj = bwd ? bj + 1 : bj - 1, pbk = bwd ? bk + 1 : bk - 1;
    const int cbj = bwd ? bj - 1 : bj + 1, cbk = bwd ? bk - 1 : bk + 1;
    // blocks without fluid are skipped; their consumers take 0 (as k_tri)
    const bool live = A.blkf[bk * K.nbj + bj] != 0;
    const bool has_pj = pbj >= 0 && pbj < K.nbj && A.blkf[bk * K.nbj + pbj],
               has_pk = pbk >= 0 && pbk < K.nbk && A.blkf[pbk * K.nbj + bj];
    const bool has_cj = cbj >= 0 && cbj < K.nbj && A.blkf[bk * K.nbj + cbj],
               has_ck = cbk >= 0 && cbk < K.nbk && A.blkf[cbk * K.nbj + bj];
    const long long xblock = (long long)S * XP;
    const long long base = K.base(bj, bk);
    const int ngroups = live ? (S + WT_G - 1) / WT_G : 0;
    Acc2f dot32;
    if (warp == WT_THREADS / 32 - 1) {
        // loader: copy group g (steps g*G .. g*G+np-1) into slot g % WT_NG once the compute warp released it
        if (lane == 0 && ngroups > 0) {
            int g = 0;
            bool to = false;
            for (; g < ngroups; g++) {
                const int slot = g % WT_NG;
                if (g >= WT_NG) {
                    int k = 0;
                    while (!mbar_try_wait(&mempty[slot], (unsigned)((g / WT_NG - 1) & 1))) {
                        if (++k > A.spin_limit) {
                            atomicOr(&A.ctrl->err, GFS_DEV_ERR_TIMEOUT);
                            to = true;
                            break;
                        }
                    }
                    if (to) break;
                }
                const int np = min(WT_G, S - g * WT_G);
                // forward: planes g*G ..; backward: planes S-g*G-np .. S-1-g*G, step u at np-1-u
                const long long p0 = base + (long long)(bwd ? S - g * WT_G - np : g * WT_G) * SPLANE;
                const unsigned bytes = (unsigned)(np * SPLANE * sizeof(float));
                mbar_arrive_expect_tx(&mfull[slot], (unsigned)NARR * bytes);
                bulk_copy_g2s(&ring[slot][0][0][0], A.in + p0, bytes, &mfull[slot]);
                bulk_copy_g2s(&ring[slot][1][0][0], A.precon + p0, bytes, &mfull[slot]);
                if (bwd) bulk_copy_g2s(&ring[slot][NARR - 1][0][0], A.rdot + p0, bytes, &mfull[slot]);
            }
            // copies still in flight land before the block may exit
            for (int q = max(0, g - WT_NG); q < g; q++) {
                int k = 0;
                while (!mbar_try_wait(&mfull[q % WT_NG], (unsigned)((q / WT_NG) & 1)) && ++k < A.spin_limit) {
                }
            }
        }
    } else if (warp >= 1) {
        // receiver warp of class r: lane l < 16 the j-edge pencil kl = l, lane 16 + l the
        // k-edge pencil jl = l; its steps s = r (mod RX_NR), one read in flight
        const int r = warp - 1, e = lane >> 4, idx = lane & 15;
        const int jl_c = e == 0 ? (bwd ? SBJ - 1 : 0) : idx, kl_c = e == 0 ? idx : (bwd ? SBK - 1 : 0);
        const bool valid_c = live && bj * SBJ + jl_c < K.ny && bk * SBK + kl_c < K.nz;
        const bool act = valid_c && (e == 0 ? has_pj : has_pk);
        const int lo = bwd ? S - K.nx - jl_c - kl_c : jl_c + kl_c;
        const int end = act ? lo + K.nx : 0;
        const unsigned long long *src =
            !act ? A.xch
            : e == 0 ? A.xch + (long long)(bk * K.nbj + pbj) * xblock +
                           (bwd ? (long long)(S - 1 - (SBJ - 1)) : (long long)(SBJ - 1)) * XP + idx
                     : A.xch + (long long)(pbk * K.nbj + bj) * xblock +
                           (bwd ? (long long)(S - 1 - (SBK - 1)) : (long long)(SBK - 1)) * XP + SBJ + idx;
        int s = lo + ((r - lo) % RX_NR + RX_NR) % RX_NR;   // the first step of the class at or after lo
        bool inflight = false;
        unsigned long long w = 0ull;
        int pub = 0, rounds = 0;
        while (__any_sync(FULL, s < end)) {
            if (++rounds > A.spin_limit) {
                if (lane == 0) atomicOr(&A.ctrl->err, GFS_DEV_ERR_TIMEOUT);
                break;
            }
            // a round: take the word that arrived, publish, and only then issue the next
            // reads -- a fence behind a read still in flight would wait for its round trip
            if (s < end && inflight) {
                if ((unsigned)(w >> 32) == wtag) {
                    rx.val[s & (RX_R - 1)][lane] = __uint_as_float((unsigned)(w & 0xFFFFFFFFull));
                    s += RX_NR;
                }
                inflight = false;   // arrived (taken or stale): read again below
            }
            const int m = __reduce_min_sync(FULL, s < end ? s : S);
            if (m > pub) {
                __syncwarp();
                if (lane == 0) {
                    __threadfence_block();   // the values before the progress
                    st_volatile_s32(&rx.prog[r], m);
                }
                pub = m;
            }
            if (s < end) {
                // ring slot s & (RX_R-1) is free once the compute warp has read step s - RX_R
                if (s < max(ld_volatile_s32(&rx.cons), lo) + RX_R - RX_CB) {
                    w = ld_cg_u64(src + (long long)s * XS);
                    inflight = true;
                } else {
                    __nanosleep(32);
                }
            }
        }
        __syncwarp();
        if (lane == 0) {
            __threadfence_block();
            st_volatile_s32(&rx.prog[r], S);   // nothing more (or given up): no step waits on this class
        }
    } else if (ngroups > 0) {
        // the compute warp
        const int a = lane & 3, b = lane >> 2;
        const int c0 = bwd ? 63 - lane : lane, c1 = bwd ? 31 - lane : lane + 32;   // 16-byte chunks of rows 0, 1
        float px[2][4];
#pragma unroll
        for (int r = 0; r < 2; r++)
#pragma unroll
            for (int p = 0; p < 4; p++) px[r][p] = 0.f;
        float *po = A.out + base + (bwd ? (long long)(S - 1) * SPLANE : 0);
        unsigned long long *pxo = A.xch + (long long)(bk * K.nbj + bj) * xblock + (bwd ? (long long)(S - 1) * XP : 0);
        // hand-overs: j edge (jl' = 15: a == 3, pencil 3) of rows kl' = b, b + 8 at words kl;
        // k edge (kl' = 15: b == 7, row 1) of pencils jl' = 4a + p at words 16 + jl
        const int wj0 = bwd ? 15 - b : b, wj1 = bwd ? 7 - b : b + 8;
        const int wk = bwd ? 28 - 4 * a : 16 + 4 * a;
        const unsigned out_j = a == 3 && has_cj, out_k = b == 7 && has_ck;
        // edge inputs: j edge (jl' = 0: a == 0) of rows r at ring words wj0 / wj1; k edge
        // (kl' = 0: b == 0, row 0) of pencils jl' = 4a + p in the 16-byte chunk at ring word ek0
        const int ek0 = wk;
        const float ns = A.negscale;
        int seen = 0;
        bool to = false;
        for (int g = 0; g < ngroups && !to; g++) {
            const int slot = g % WT_NG;
            {
                int k = 0;
                while (!mbar_try_wait(&mfull[slot], (unsigned)((g / WT_NG) & 1))) {
                    if (++k > A.spin_limit) {
                        if (lane == 0) atomicOr(&A.ctrl->err, GFS_DEV_ERR_TIMEOUT);
                        to = true;
                        break;
                    }
                }
                if (to) break;
            }
            const int np = min(WT_G, S - g * WT_G);
            auto step = [&](const int u) {
                const int st = g * WT_G + u;
                const int ui = bwd ? np - 1 - u : u;
                // the edge words of steps st .. st + WT_POLL - 1, checked once per chunk of steps
                const int need = min(st + WT_POLL - 1, S - 1);
                if ((u % WT_POLL) == 0 && need >= seen) {
                    int k = 0;
                    for (;;) {
                        int m = ld_volatile_s32(&rx.prog[0]);
#pragma unroll
                        for (int r = 1; r < RX_NR; r++) m = min(m, ld_volatile_s32(&rx.prog[r]));
                        seen = m;
                        if (seen > need) break;
                        if (++k > A.spin_limit) {
                            if (lane == 0) atomicOr(&A.ctrl->err, GFS_DEV_ERR_TIMEOUT);
                            seen = S;
                            break;
                        }
                    }
                    __threadfence_block();   // the ring values after the progress that covers them
                }
                float ra[2][4], pc[2][4], rv[2][4], ek[4];
                unpack4<bwd>(*reinterpret_cast<const float4 *>(&ring[slot][0][ui][4 * c0]), ra[0]);
                unpack4<bwd>(*reinterpret_cast<const float4 *>(&ring[slot][0][ui][4 * c1]), ra[1]);
                unpack4<bwd>(*reinterpret_cast<const float4 *>(&ring[slot][1][ui][4 * c0]), pc[0]);
                unpack4<bwd>(*reinterpret_cast<const float4 *>(&ring[slot][1][ui][4 * c1]), pc[1]);
                if (bwd) {
                    unpack4<bwd>(*reinterpret_cast<const float4 *>(&ring[slot][NARR - 1][ui][4 * c0]), rv[0]);
                    unpack4<bwd>(*reinterpret_cast<const float4 *>(&ring[slot][NARR - 1][ui][4 * c1]), rv[1]);
                }
                const float *xr = &rx.val[st & (RX_R - 1)][0];
                const float ej[2] = {xr[wj0], xr[wj1]};
                unpack4<bwd>(*reinterpret_cast<const float4 *>(xr + ek0), ek);
                float nj[2][4], nk[2][4];
#pragma unroll
                for (int r = 0; r < 2; r++) {
                    const float sj = __shfl_up_sync(FULL, px[r][3], 1, 4);
                    nj[r][0] = a ? sj : ej[r];
#pragma unroll
                    for (int p = 1; p < 4; p++) nj[r][p] = px[r][p - 1];
                }
#pragma unroll
                for (int p = 0; p < 4; p++) {
                    const float up0 = __shfl_up_sync(FULL, px[0][p], 4);
                    nk[0][p] = b ? up0 : ek[p];
                    const float send = b == 7 ? px[0][p] : px[1][p];   // row 1's lower row: lane - 4's row 1, or row 0 of b = 7
                    nk[1][p] = __shfl_sync(FULL, send, (lane - 4) & 31);
                }
                float val[2][4];
#pragma unroll
                for (int r = 0; r < 2; r++)
#pragma unroll
                    for (int p = 0; p < 4; p++) {
                        if (!bwd) {
                            // _applyPreconditioner forward solve (pressuresolver.cpp:311-351), as k_tri
                            val[r][p] = Op::mul(Op::sub(Op::sub(Op::sub(ra[r][p], px[r][p]), nj[r][p]), nk[r][p]), pc[r][p]);
                            px[r][p] = Op::mul(Op::mul(ns, pc[r][p]), val[r][p]);
                        } else {
                            // backward solve (pressuresolver.cpp:354-385), as k_tri
                            const float m = Op::mul(ns, pc[r][p]);
                            val[r][p] = Op::mul(Op::sub(Op::sub(Op::sub(ra[r][p], Op::mul(m, px[r][p])), Op::mul(m, nj[r][p])),
                                                        Op::mul(m, nk[r][p])),
                                                pc[r][p]);
                            px[r][p] = val[r][p];
                        }
                    }
                if (bwd) {
                    // dot(z, r): the eight rounded products summed pairwise, then the compensated running sum
                    float pr[8];
#pragma unroll
                    for (int r = 0; r < 2; r++)
#pragma unroll
                        for (int p = 0; p < 4; p++) pr[4 * r + p] = val[r][p] * rv[r][p];
                    dot32.add(((pr[0] + pr[1]) + (pr[2] + pr[3])) + ((pr[4] + pr[5]) + (pr[6] + pr[7])));
                }
                *reinterpret_cast<float4 *>(po + 4 * c0) = pack4<bwd>(val[0]);
                *reinterpret_cast<float4 *>(po + 4 * c1) = pack4<bwd>(val[1]);
                po += PS;
                put_word(pxo + wj0, px[0][3], tag, out_j);
                put_word(pxo + wj1, px[1][3], tag, out_j);
                if (!bwd) {
                    put_words2(pxo + wk, px[1][0], px[1][1], tag, out_k);
                    put_words2(pxo + wk + 2, px[1][2], px[1][3], tag, out_k);
                } else {
                    put_words2(pxo + wk, px[1][3], px[1][2], tag, out_k);
                    put_words2(pxo + wk + 2, px[1][1], px[1][0], tag, out_k);
                }
                pxo += XS;
            };
            if (np == WT_G) {
#pragma unroll
                for (int u = 0; u < WT_G; u++) step(u);
            } else {
                for (int u = 0; u < np; u++) step(u);
            }
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(&mempty[slot]);
                st_volatile_s32(&rx.cons, g * WT_G + np - 1);   // the steps up to it have been read
            }
        }
        if (to && lane == 0) st_volatile_s32(&rx.cons, S);
    }

    // block partial of dot(z, r) (the compute warp's lanes in order) and the last-CTA epilogue
    double part = 0.0;
    if (MODE == SW_BWD && warp == 0) {
        part = dot32.value();
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) part += __shfl_down_sync(FULL, part, o);
    }
    __shared__ bool last;
    const unsigned nblocks = (unsigned)(K.nbj * K.nbk);
    if (tid == 0) {
        if (MODE == SW_BWD) A.partials[bj + K.nbj * bk] = part;
        __threadfence();
        unsigned tk = atomicAdd(A.done_ticket, 1u);
        last = tk == nblocks - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    if (MODE == SW_BWD) {
        double acc = 0.0;
        for (unsigned q = tid; q < nblocks; q += blockDim.x) acc += __ldcg(A.partials + q);
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
        A.ctrl->epoch = tag + 1 == 0 ? 1u : tag + 1;
    }
}

// -------------------------------------------------------- vector kernels

template <class T>
struct VecArgs {
    Skew K;
    const uint8_t *fsk;
    T negscale, scale;
    double *partials;
    PsCtrl *ctrl;
    int mixed;
    const unsigned *slist;   // the strips (of Strip<T>::W slots) that hold fluid, in order
    const unsigned *snum;    // their number
    T dcoef[8];              // (T)n * scale for n non-solid neighbours, formed once on the host
};

// x at the six neighbours of slot q in the skewed layout, in the reference's
// summation order i-1, i+1, j-1, j+1, k-1, k+1 (0 outside the grid).
template <class T>
__device__ __forceinline__ T neighbour_sum(const Skew &K, const T *__restrict__ x, long long q) {
    using Op = Ar<T>;
    int bj, bk, s, jl, kl;
    K.decode(q, bj, bk, s, jl, kl);
    const int i = s - jl - kl;
    T xim = i > 0 ? x[q - SPLANE] : T(0);
    T xip = i < K.nx - 1 ? x[q + SPLANE] : T(0);
    T xjm = jl > 0 ? x[q - SPLANE - 1] : (bj > 0 ? x[K.slot(bj - 1, bk, s + SBJ - 1, SBJ - 1, kl)] : T(0));
    T xjp = jl < SBJ - 1 ? x[q + SPLANE + 1] : (bj + 1 < K.nbj ? x[K.slot(bj + 1, bk, s - SBJ + 1, 0, kl)] : T(0));
    T xkm = kl > 0 ? x[q - SPLANE - SBJ] : (bk > 0 ? x[K.slot(bj, bk - 1, s + SBK - 1, jl, SBK - 1)] : T(0));
    T xkp = kl < SBK - 1 ? x[q + SPLANE + SBJ] : (bk + 1 < K.nbk ? x[K.slot(bj, bk + 1, s - SBK + 1, jl, 0)] : T(0));
    return Op::add(Op::add(Op::add(Op::add(Op::add(xim, xip), xjm), xjp), xkm), xkp);
}

// ------------------------------------------------- strip-wise vector kernels
//
// The per-iteration vector kernels take one strip per thread: 32 bytes of
// consecutive slots of one row (fixed plane s and kl) of a pencil block -- 8
// FP32 or 4 FP64 slots.  A strip costs one flag load and two 16-byte loads per
// operand, all issued together, so the kernels stream at HBM rate instead of
// waiting on a byte load before each slot's operands.  The kernels walk the list
// of strips that hold fluid (built once per solve, in strip order; at 256^3 about
// a third of all strips), so strips without fluid cost neither a flag load nor a
// thread.  Stores stay per slot and on fluid slots only, so the per-slot results
// are those of the slot-wise loops in the reference (pressuresolver.cpp:388-486)
// bit for bit; the reductions sum in the walk's fixed order.

template <class T>
struct Strip {
    static constexpr int W = 32 / (int)sizeof(T);   // slots per strip
    static constexpr int PER_ROW = SBJ / W, PER_PLANE = SPLANE / W;
    static constexpr int NF = W / 4;                 // 32-bit flag words
};

struct StripPos {
    int bj, bk, s, kl, jl0;
    long long q0;   // first slot
};

template <class T>
__device__ __forceinline__ StripPos strip_pos(const Skew &K, unsigned u) {
    using St = Strip<T>;
    const unsigned per = (unsigned)K.S * St::PER_PLANE;   // strips per pencil block
    StripPos P;
    const unsigned pb = u / per, rem = u - pb * per;
    P.s = (int)(rem / St::PER_PLANE);
    const unsigned w = rem - (unsigned)P.s * St::PER_PLANE;
    P.kl = (int)(w / St::PER_ROW);
    P.jl0 = (int)(w - (unsigned)P.kl * St::PER_ROW) * St::W;
    P.bk = (int)(pb / (unsigned)K.nbj);
    P.bj = (int)(pb - (unsigned)P.bk * K.nbj);
    P.q0 = (long long)u * St::W;
    return P;
}

template <class T>
struct StripFlags {
    unsigned w[Strip<T>::NF];
    __device__ __forceinline__ void load(const uint8_t *fsk, long long q0) {
        if constexpr (Strip<T>::NF == 2) {
            const uint2 v = *reinterpret_cast<const uint2 *>(fsk + q0);
            w[0] = v.x;
            w[1] = v.y;
        } else {
            w[0] = *reinterpret_cast<const unsigned *>(fsk + q0);
        }
    }
    __device__ __forceinline__ unsigned at(int e) const { return (w[e >> 2] >> (8 * (e & 3))) & 0xffu; }
    __device__ __forceinline__ bool fluid(int e) const { return (at(e) & GFS_PF_FLUID) != 0u; }
    __device__ __forceinline__ bool any() const {
        unsigned o = 0u;
#pragma unroll
        for (int h = 0; h < Strip<T>::NF; h++) o |= w[h];
        return (o & 0x01010101u) != 0u;
    }
    __device__ __forceinline__ bool all() const {
        unsigned a = 0x01010101u;
#pragma unroll
        for (int h = 0; h < Strip<T>::NF; h++) a &= w[h];
        return a == 0x01010101u;
    }
};

// d[0..W-1] = p[0..W-1] (two 16-byte loads; p is 32-byte aligned), or 0 when !ok
template <class T>
__device__ __forceinline__ void load_strip(T (&d)[Strip<T>::W], const T *p, bool ok = true) {
    if constexpr (sizeof(T) == 4) {
        float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
        if (ok) {
            a = *reinterpret_cast<const float4 *>(p);
            b = *reinterpret_cast<const float4 *>(p + 4);
        }
        d[0] = a.x; d[1] = a.y; d[2] = a.z; d[3] = a.w;
        d[4] = b.x; d[5] = b.y; d[6] = b.z; d[7] = b.w;
    } else {
        double2 a = make_double2(0.0, 0.0), b = a;
        if (ok) {
            a = *reinterpret_cast<const double2 *>(p);
            b = *reinterpret_cast<const double2 *>(p + 2);
        }
        d[0] = a.x; d[1] = a.y; d[2] = b.x; d[3] = b.y;
    }
}

// p = d on the fluid slots of the strip (two 16-byte stores when all are fluid)
template <class T>
__device__ __forceinline__ void store_strip_fluid(T *p, const T (&d)[Strip<T>::W], const StripFlags<T> &f) {
    if (f.all()) {
        if constexpr (sizeof(T) == 4) {
            *reinterpret_cast<float4 *>(p) = make_float4(d[0], d[1], d[2], d[3]);
            *reinterpret_cast<float4 *>(p + 4) = make_float4(d[4], d[5], d[6], d[7]);
        } else {
            *reinterpret_cast<double2 *>(p) = make_double2(d[0], d[1]);
            *reinterpret_cast<double2 *>(p + 2) = make_double2(d[2], d[3]);
        }
        return;
    }
#pragma unroll
    for (int e = 0; e < Strip<T>::W; e++)
        if (f.fluid(e)) p[e] = d[e];
}

// x at the six neighbours of each slot of a strip, summed in the reference's
// order i-1, i+1, j-1, j+1, k-1, k+1 (0 outside the grid).  Neighbours in
// plane s-1 / s+1 of the same pencil block are strip loads of the rows
// (s-1, kl), (s+1, kl), (s-1, kl-1), (s+1, kl+1); j-1 / j+1 of slot jl are
// rows (s-1, kl) / (s+1, kl) shifted by one, whose two outermost values are
// scalar loads (from the adjacent pencil block at jl = 0 / 15).  Slots outside
// the grid hold 0 in x, so a neighbour slot outside the grid reads 0; the
// guards only keep the addresses inside the array.
template <class T>
__device__ __forceinline__ void neighbour_sum_strip(const Skew &K, const T *__restrict__ x, const StripPos &P,
                                                    T (&sum)[Strip<T>::W]) {
    using Op = Ar<T>;
    constexpr int W = Strip<T>::W;
    const long long q0 = P.q0;
    const bool has_m = P.s > 0, has_p = P.s + 1 < K.S;
    T im[W], ip[W], km[W], kp[W];
    load_strip<T>(im, x + (has_m ? q0 - SPLANE : q0), has_m);
    load_strip<T>(ip, x + (has_p ? q0 + SPLANE : q0), has_p);
    T jm0 = T(0), jpl = T(0);
    if (P.jl0 > 0) {
        if (has_m) jm0 = x[q0 - SPLANE - 1];
    } else if (P.bj > 0 && P.s + SBJ - 1 < K.S) {
        jm0 = x[K.slot(P.bj - 1, P.bk, P.s + SBJ - 1, SBJ - 1, P.kl)];
    }
    if (P.jl0 + W < SBJ) {
        if (has_p) jpl = x[q0 + SPLANE + W];
    } else if (P.bj + 1 < K.nbj && P.s >= SBJ - 1) {
        jpl = x[K.slot(P.bj + 1, P.bk, P.s - SBJ + 1, 0, P.kl)];
    }
    if (P.kl > 0) {
        load_strip<T>(km, x + (has_m ? q0 - SPLANE - SBJ : q0), has_m);
    } else {
        const bool ok = P.bk > 0 && P.s + SBK - 1 < K.S;
        load_strip<T>(km, x + (ok ? K.slot(P.bj, P.bk - 1, P.s + SBK - 1, P.jl0, SBK - 1) : 0), ok);
    }
    if (P.kl < SBK - 1) {
        load_strip<T>(kp, x + (has_p ? q0 + SPLANE + SBJ : q0), has_p);
    } else {
        const bool ok = P.bk + 1 < K.nbk && P.s >= SBK - 1;
        load_strip<T>(kp, x + (ok ? K.slot(P.bj, P.bk + 1, P.s - SBK + 1, P.jl0, 0) : 0), ok);
    }
#pragma unroll
    for (int e = 0; e < W; e++) {
        const T jm = e == 0 ? jm0 : im[e - 1];
        const T jp = e == W - 1 ? jpl : ip[e + 1];
        sum[e] = Op::add(Op::add(Op::add(Op::add(Op::add(im[e], ip[e]), jm), jp), km[e]), kp[e]);
    }
}

// The strips that hold a fluid slot, in strip order, for the per-iteration vector
// kernels (built once per solve: the fluid set is fixed during it).  off[u] = 1 if
// strip u holds fluid; an exclusive scan of off turns it into list positions.
template <class T>
__global__ void __launch_bounds__(RED_THREADS) k_strip_mark(Skew K, const uint8_t *__restrict__ fsk,
                                                            unsigned *__restrict__ off) {
    constexpr int W = Strip<T>::W;
    const unsigned nstrip = (unsigned)(K.size / W);
    for (unsigned u = blockIdx.x * blockDim.x + threadIdx.x; u <= nstrip; u += gridDim.x * blockDim.x) {
        if (u == nstrip) {
            off[u] = 0u;
            continue;
        }
        StripFlags<T> f;
        f.load(fsk, (long long)u * W);
        off[u] = f.any() ? 1u : 0u;
    }
}
__global__ void __launch_bounds__(RED_THREADS) k_strip_list(unsigned nstrip, const unsigned *__restrict__ off,
                                                            unsigned *__restrict__ list, unsigned *__restrict__ num) {
    for (unsigned u = blockIdx.x * blockDim.x + threadIdx.x; u < nstrip; u += gridDim.x * blockDim.x)
        if (off[u + 1] != off[u]) list[off[u]] = u;
    if (blockIdx.x == 0 && threadIdx.x == 0) *num = off[nstrip];
}

// The next strip of a thread's walk over the list: loaded one step ahead, so the
// list read does not sit in front of the strip's own loads.
struct StripWalk {
    const unsigned *list;
    unsigned n, i, stride, next;
    __device__ __forceinline__ StripWalk(const unsigned *l, const unsigned *num) : list(l) {
        n = *num;
        i = blockIdx.x * blockDim.x + threadIdx.x;
        stride = gridDim.x * blockDim.x;
        next = i < n ? list[i] : 0u;
    }
    __device__ __forceinline__ bool more() const { return i < n; }
    __device__ __forceinline__ unsigned take() {
        const unsigned u = next;
        i += stride;
        if (i < n) next = list[i];
        return u;
    }
};

// As = A s and dot(As, s) -> alpha (pressuresolver.cpp:388-426, :472-473)
template <class T>
__global__ void __launch_bounds__(RED_THREADS) k_matvec(VecArgs<T> A, const T *__restrict__ s,
                                                        T *__restrict__ As) {
    using Op = Ar<T>;
    constexpr int W = Strip<T>::W;
    if (A.ctrl->done) return;
    const Skew &K = A.K;
    double dot = 0.0;   // FP64 operands
    Acc2f dot32;        // FP32 operands: compensated
    for (StripWalk sw(A.slist, A.snum); sw.more();) {
        const StripPos P = strip_pos<T>(K, sw.take());
        StripFlags<T> f;
        f.load(A.fsk, P.q0);
        T xc[W], val[W];
        load_strip<T>(xc, s + P.q0);
        neighbour_sum_strip<T>(K, s, P, val);
#pragma unroll
        for (int e = 0; e < W; e++) {
            const unsigned fl = f.at(e);
            T v = Op::mul(val[e], A.negscale);
            v = Op::add(v, Op::mul(A.dcoef[(fl >> 1) & 7u], xc[e]));
            val[e] = v;
            if (fl & GFS_PF_FLUID) {
                if (sizeof(T) == 4) dot32.add((float)v * (float)xc[e]);
                else dot += (double)v * (double)xc[e];
            }
        }
        store_strip_fluid<T>(As + P.q0, val, f);
    }
    double part = block_reduce<0>(sizeof(T) == 4 ? dot32.value() : dot);
    double res;
    if (finish_reduce<0>(part, A.partials, &A.ctrl->tickets[1], gridDim.x, &res) && threadIdx.x == 0)
        A.ctrl->alpha = A.ctrl->sigma / res;
}

// p += alpha s; r -= alpha As; max|r| and the stopping test (pressuresolver.cpp:474-479)
template <class T>
__global__ void __launch_bounds__(RED_THREADS) k_axpy(VecArgs<T> A, T *__restrict__ p, T *__restrict__ r,
                                                      const T *__restrict__ s, const T *__restrict__ As) {
    using Op = Ar<T>;
    constexpr int W = Strip<T>::W;
    PsCtrl *C = A.ctrl;
    if (C->done) return;
    const T alpha = (T)C->alpha, nalpha = (T)(-C->alpha);
    T mx = T(0);
    for (StripWalk sw(A.slist, A.snum); sw.more();) {
        const long long q0 = (long long)sw.take() * W;
        StripFlags<T> f;
        f.load(A.fsk, q0);
        T pv[W], sv[W], rv[W], av[W];
        load_strip<T>(pv, p + q0);
        load_strip<T>(sv, s + q0);
        load_strip<T>(rv, r + q0);
        load_strip<T>(av, As + q0);
#pragma unroll
        for (int e = 0; e < W; e++) {
            pv[e] = Op::add(pv[e], Op::mul(sv[e], alpha));
            rv[e] = Op::add(rv[e], Op::mul(av[e], nalpha));
            if (f.fluid(e)) mx = fmax(mx, fabs(rv[e]));
        }
        store_strip_fluid<T>(p + q0, pv, f);
        store_strip_fluid<T>(r + q0, rv, f);
    }
    double part = block_reduce<1>((double)mx);
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
    constexpr int W = Strip<T>::W;
    if (A.ctrl->done) return;
    const T beta = (T)A.ctrl->beta;
    for (StripWalk sw(A.slist, A.snum); sw.more();) {
        const long long q0 = (long long)sw.take() * W;
        StripFlags<T> f;
        f.load(A.fsk, q0);
        T zv[W], sv[W];
        load_strip<T>(zv, z + q0);
        load_strip<T>(sv, s + q0);
#pragma unroll
        for (int e = 0; e < W; e++) {
            // FP64: z * 1 is z exactly, so the multiply is left out (GB300's FP64 rate);
            // FP32 keeps the expression as compiled so far
            if constexpr (sizeof(T) == 8) sv[e] = Op::add(zv[e], Op::mul(sv[e], beta));
            else sv[e] = Op::add(Op::mul(zv[e], (T)1.0), Op::mul(sv[e], beta));
        }
        store_strip_fluid<T>(s + q0, sv, f);
    }
}

// MIXED: r32 = (float) r64, e32 = 0, s32 = 0; inner threshold from max|r64|.
__global__ void __launch_bounds__(RED_THREADS) k_mixed_prepare(Skew K, const uint8_t *__restrict__ fsk,
                                                               const double *__restrict__ r64,
                                                               float *__restrict__ r32, float *__restrict__ e32,
                                                               float *__restrict__ s32, PsCtrl *ctrl, double eta) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < K.size;
         q += (long long)gridDim.x * blockDim.x) {
        bool f = fsk[q] & GFS_PF_FLUID;
        r32[q] = f ? (float)r64[q] : 0.0f;
        e32[q] = 0.0f;
        s32[q] = 0.0f;
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

// The per-update kernels of the MIXED form below walk the solve's FP32 strip
// list (8 slots per strip, the list the inner PCG builds); each FP32 strip is two
// 4-slot FP64 strips of the FP64 vectors.  Slots outside the listed strips hold no
// fluid, and the vectors' non-fluid slots keep the 0 that k_mixed_prepare wrote
// at the start of the solve (the inner PCG stores fluid slots only).

// MIXED, reliable update: the inner FP32 CG goes on with the true residual.
// r32 = r64 (the FP64 residual of the corrected p64), e32 = 0, and the search
// direction s32 and sigma are kept, so the Krylov information of the earlier
// inner iterations is not thrown away.  The pending preconditioner apply of the
// iteration that met the inner threshold completes that iteration, so the
// iteration counter restarts at -1 (that apply brings it to 0).
__global__ void __launch_bounds__(RED_THREADS) k_mixed_reliable(VecArgs<float> A, const double *__restrict__ r64,
                                                                float *__restrict__ r32, float *__restrict__ e32,
                                                                double eta) {
    for (StripWalk sw(A.slist, A.snum); sw.more();) {
        const long long q0 = (long long)sw.take() * Strip<float>::W;
        StripFlags<float> f;
        f.load(A.fsk, q0);
        double lo[4], hi[4];
        load_strip<double>(lo, r64 + q0);
        load_strip<double>(hi, r64 + q0 + 4);
        float rv[8];
#pragma unroll
        for (int e = 0; e < 4; e++) {
            rv[e] = f.fluid(e) ? (float)lo[e] : 0.0f;
            rv[e + 4] = f.fluid(e + 4) ? (float)hi[e] : 0.0f;
        }
        *reinterpret_cast<float4 *>(r32 + q0) = make_float4(rv[0], rv[1], rv[2], rv[3]);
        *reinterpret_cast<float4 *>(r32 + q0 + 4) = make_float4(rv[4], rv[5], rv[6], rv[7]);
        *reinterpret_cast<float4 *>(e32 + q0) = make_float4(0.f, 0.f, 0.f, 0.f);
        *reinterpret_cast<float4 *>(e32 + q0 + 4) = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        PsCtrl *ctrl = A.ctrl;
        double m = ctrl->maxr64;
        ctrl->inner_tol = fmax(eta * m, 0.25 * ctrl->tol);
        ctrl->done = 0;
        ctrl->converged = 0;
        ctrl->iter = -1;
    }
}

// MIXED: p64 += e32 (outer refinement)
__global__ void __launch_bounds__(RED_THREADS) k_mixed_correct(VecArgs<float> A, double *__restrict__ p64,
                                                               const float *__restrict__ e32) {
    for (StripWalk sw(A.slist, A.snum); sw.more();) {
        const long long q0 = (long long)sw.take() * Strip<float>::W;
        StripFlags<float> f;
        f.load(A.fsk, q0);
        float ev[8];
        load_strip<float>(ev, e32 + q0);
#pragma unroll
        for (int h = 0; h < 2; h++) {
            StripFlags<double> fh;
            fh.w[0] = f.w[h];
            double pv[4];
            load_strip<double>(pv, p64 + q0 + 4 * h);
#pragma unroll
            for (int e = 0; e < 4; e++) pv[e] += (double)ev[4 * h + e];
            store_strip_fluid<double>(p64 + q0 + 4 * h, pv, fh);
        }
    }
}

// MIXED: r64 = b - A p64 in FP64 and max|r64|.  A carries the FP32 strip list.
__global__ void __launch_bounds__(RED_THREADS) k_residual64(VecArgs<double> A, const double *__restrict__ b,
                                                            const double *__restrict__ p,
                                                            double *__restrict__ r) {
    using Op = Ar<double>;
    constexpr int W = Strip<double>::W;
    const Skew &K = A.K;
    double mx = 0.0;
    for (StripWalk sw(A.slist, A.snum); sw.more();) {
        const unsigned u = sw.take() * 2u;   // the FP32 strip's two FP64 strips
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const StripPos P = strip_pos<double>(K, u + (unsigned)h);
            StripFlags<double> f;
            f.load(A.fsk, P.q0);
            double xc[W], bv[W], val[W];
            load_strip<double>(xc, p + P.q0);
            load_strip<double>(bv, b + P.q0);
            neighbour_sum_strip<double>(K, p, P, val);
#pragma unroll
            for (int e = 0; e < W; e++) {
                const unsigned fl = f.at(e);
                double v = Op::mul(val[e], A.negscale);
                v = Op::add(v, Op::mul(A.dcoef[(fl >> 1) & 7u], xc[e]));
                val[e] = bv[e] - v;
                if (fl & GFS_PF_FLUID) mx = fmax(mx, fabs(val[e]));
            }
            store_strip_fluid<double>(r + P.q0, val, f);
        }
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

static int ensure_ws(Ctx *ctx, PressureWs &ws, const Grids &g, bool mixed) {
    long long n = g.c.size;
    Skew K = make_skew(g.c);
    if (ws.allocated_for != n) {
        ws.c = g.c;
        ws.nbj = K.nbj;
        ws.nbk = K.nbk;
        ws.skew_size = K.size;
        int rc = 0;
        rc |= ws.flags.alloc((size_t)n);
        rc |= ws.b.alloc((size_t)n * sizeof(double));
        rc |= ws.p.alloc((size_t)n * sizeof(double));
        rc |= ws.fsk.alloc((size_t)K.size);
        DevMem *v64[] = {&ws.bsk, &ws.psk, &ws.r, &ws.z, &ws.s, &ws.As, &ws.q, &ws.precon};
        for (DevMem *m : v64) rc |= m->alloc((size_t)K.size * sizeof(double));
        if (rc) return GFS_ERR_NOMEM;
        for (DevMem *m : v64) GFS_CUDA_CHECK(cudaMemsetAsync(m->p, 0, m->bytes, ctx->stream));
        GFS_CUDA_CHECK(cudaMemsetAsync(ws.flags.p, 0, ws.flags.bytes, ctx->stream));
        GFS_CUDA_CHECK(cudaMemsetAsync(ws.fsk.p, 0, ws.fsk.bytes, ctx->stream));
        GFS_CUDA_CHECK(cudaMemsetAsync(ws.b.p, 0, ws.b.bytes, ctx->stream));
        GFS_CUDA_CHECK(cudaMemsetAsync(ws.p.p, 0, ws.p.bytes, ctx->stream));
        ws.nblocks_red = (size_t)ctx->num_sms * 8;
        size_t nbl = (size_t)K.nbj * K.nbk;
        size_t np = ws.nblocks_red > nbl ? ws.nblocks_red : nbl;
        if (ws.partials.alloc(np * sizeof(double))) return GFS_ERR_NOMEM;
        if (ws.ctrl.alloc(sizeof(PsCtrl)) || ws.blkf.alloc(nbl)) return GFS_ERR_NOMEM;
        GFS_CUDA_CHECK(cudaMemsetAsync(ws.ctrl.p, 0, sizeof(PsCtrl), ctx->stream));
        // exchange words: per block and plane XCH_PER_PLANE entries of up to 2 words
        size_t nx_words = nbl * (size_t)K.S * XCH_PER_PLANE * 2;
        if (ws.xch.alloc(nx_words * sizeof(unsigned long long))) return GFS_ERR_NOMEM;
        GFS_CUDA_CHECK(cudaMemsetAsync(ws.xch.p, 0, ws.xch.bytes, ctx->stream));
        if (ws.nbstd.alloc((size_t)n * sizeof(uint16_t)) || ws.nbsk.alloc((size_t)K.size * sizeof(uint16_t)))
            return GFS_ERR_NOMEM;
        // strip list: at most K.size / 4 strips (FP64 strips of 4 slots)
        const size_t maxstrip = (size_t)(K.size / 4);
        if (ws.slist.alloc(maxstrip * sizeof(unsigned)) || ws.soff.alloc((maxstrip + 1) * sizeof(unsigned)) ||
            ws.stmp.alloc(scan_temp_elems((long long)maxstrip + 1) * sizeof(unsigned)) || ws.snum.alloc(sizeof(unsigned)))
            return GFS_ERR_NOMEM;
        GFS_CUDA_CHECK(cudaMemsetAsync(ws.snum.p, 0, sizeof(unsigned), ctx->stream));
        GFS_CUDA_CHECK(cudaMemsetAsync(ws.nbsk.p, 0, ws.nbsk.bytes, ctx->stream));
        ws.allocated_for = n;
        ws.mixed_alloc = false;
    }
    if (mixed && !ws.mixed_alloc) {
        DevMem *v32[] = {&ws.r32, &ws.z32, &ws.s32, &ws.As32, &ws.q32, &ws.e32, &ws.precon32};
        for (DevMem *m : v32) {
            if (m->alloc((size_t)K.size * sizeof(float))) return GFS_ERR_NOMEM;
            GFS_CUDA_CHECK(cudaMemsetAsync(m->p, 0, m->bytes, ctx->stream));
        }
        ws.mixed_alloc = true;
    }
    return GFS_OK;
}

// k_tri_cl<.., CJ, CK> fits when its receive buffers fit in shared memory and
// every cluster of the launch can be resident at once (a cluster that waits for
// a free SM would serialise the wavefront); checked, and the shared-memory
// limit raised, once per instantiation, device and size.
template <class T, int MODE, int P, int PE, int CJ, int CK>
static bool tri_cl_usable(int S, int ncl) {
    constexpr int MAXDEV = 64;
    static std::mutex mu;
    static size_t attr_dev[MAXDEV] = {};
    static int active_dev[MAXDEV] = {};   // clusters that fit at once, 0 unknown (stored + 1)
    const size_t dyn = tri_cl_smem<T>(S);
    if (dyn > 160 * 1024) return false;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAXDEV) {
        cudaGetLastError();
        return false;
    }
    std::lock_guard<std::mutex> lock(mu);
    size_t &attr = attr_dev[dev];
    int &active1 = active_dev[dev];
    if (dyn > attr) {
        if (cudaFuncSetAttribute(k_tri_cl<T, MODE, P, PE, CJ, CK>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)dyn) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        attr = dyn;
        active1 = 0;
    }
    if (active1 == 0) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(CJ * CK);
        cfg.blockDim = dim3(SPLANE + RX_THREADS);
        cfg.dynamicSmemBytes = attr;
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, k_tri_cl<T, MODE, P, PE, CJ, CK>, &cfg) != cudaSuccess) n = 0;
        cudaGetLastError();
        active1 = n + 1;
    }
    return active1 - 1 >= ncl;
}

// k_tri_warp's dynamic shared memory limit, raised once per device
template <int MODE>
static void launch_tri_warp(Ctx *ctx, const SweepArgs<float> &A) {
    constexpr int MAXDEV = 64;
    static bool raised[MAXDEV] = {};
    static std::mutex mu;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) dev = -1;
    {
        std::lock_guard<std::mutex> lk(mu);
        const bool known = dev >= 0 && dev < MAXDEV;
        if (!known || !raised[dev]) {
            cudaFuncSetAttribute(k_tri_warp<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)tri_warp_smem<MODE>());
            if (known) raised[dev] = true;
        }
    }
    k_tri_warp<MODE><<<A.K.nbj * A.K.nbk, WT_THREADS, tri_warp_smem<MODE>(), ctx->stream>>>(A);
}

template <class T, int MODE, int P, int PE, int CJ, int CK>
static bool launch_tri_cl(Ctx *ctx, const SweepArgs<T> &A) {
    const int ncl = ((A.K.nbj + CJ - 1) / CJ) * ((A.K.nbk + CK - 1) / CK);
    auto a16 = [](const void *q) { return ((uintptr_t)q & 15u) == 0; };
    if (!a16(A.in) || !a16(A.precon) || (MODE == SW_BWD && !a16(A.rdot))) return false;   // 16-byte copies
    if (!tri_cl_usable<T, MODE, P, PE, CJ, CK>(A.K.S, ncl)) return false;
    k_tri_cl<T, MODE, P, PE, CJ, CK><<<ncl * CJ * CK, SPLANE + RX_THREADS, tri_cl_smem<T>(A.K.S), ctx->stream>>>(A);
    return true;
}

// PE: how many steps ahead a pencil on a block edge loads the upstream block's
// exchange words (the L2 round trip must fit in PE steps)
#ifndef GFS_SWEEP_PE
#define GFS_SWEEP_PE 4
#endif
template <class T, int MODE, int P = (sizeof(T) == 8 ? 4 : 8),
          int PE = (GFS_SWEEP_PE < P ? GFS_SWEEP_PE : P)>
static int launch_sweep(Ctx *ctx, PressureWs &ws, const T *in, T *out, const T *precon, const T *rdot,
                        float *out32, double scale, int init) {
    if (MODE != SW_PRECON) {
        // the triangular solves copy their input planes in 16-byte pieces
        auto a16 = [](const void *q) { return ((uintptr_t)q & 15u) == 0; };
        if (!a16(in) || !a16(precon) || (MODE == SW_BWD && !a16(rdot))) {
            set_error(GFS_ERR_INVALID, "pressure sweep: input vectors must be 16-byte aligned");
            return GFS_ERR_INVALID;
        }
    }
    SweepArgs<T> A;
    A.K = make_skew(ws.c);
    A.c = ws.c;
    A.fsk = ws.fsk.as<uint8_t>();
    A.fstd = ws.flags.as<uint8_t>();
    A.in = in;
    A.out = out;
    A.precon = precon;
    A.rdot = rdot;
    A.mpc = sizeof(T) == 8 ? (const T *)ws.mpc.p : nullptr;
    A.out32 = out32;
    A.negscale = (T)(-scale);
    A.scale = scale;
    A.dnegscale = -scale;
    A.xch = ws.xch.as<unsigned long long>();
    A.nbits = ws.nbsk.as<uint16_t>();
    A.blkf = ws.blkf.as<uint8_t>();
    PsCtrl *C = ws.ctrl.as<PsCtrl>();
    A.ticket = &C->sweep_ticket[MODE];
    A.done_ticket = &C->tickets[0];
    A.partials = ws.partials.as<double>();
    A.ctrl = C;
    A.init = init;
    A.spin_limit = (int)ctx->wait_limit;
    A.wait_skew = 0u;
    if (ctx->wait_fault_sweeps > 0) {
        A.wait_skew = 0x40000000u;
        ctx->wait_fault_sweeps--;
    }
    ProfScope prof(ctx, MODE == SW_FWD ? KC_SWEEP_FWD : (MODE == SW_BWD ? KC_SWEEP_BWD : KC_PRECON));
    // the build runs k_sweep, the triangular solves the context's kernel (only the
    // launched kernels are instantiated)
    if constexpr (MODE == SW_PRECON) {
        k_sweep<T, MODE, P, PE><<<A.K.nbj * A.K.nbk, SWEEP_THREADS, 0, ctx->stream>>>(A);
    } else {
        const int want = ctx->sweep_kernel;
        int ran = 0;
        // AUTO: FP32 solves run the one-warp kernel, FP64 solves the block kernel (the
        // one-warp kernel is FP32 only; an explicit WARP on an FP64 solve runs BLOCK)
        bool warp_ran = false;
        if constexpr (sizeof(T) == 4) {
            if (want == GFS_SWEEP_AUTO || want == GFS_SWEEP_WARP) {
                launch_tri_warp<MODE>(ctx, A);
                ran = GFS_SWEEP_WARP;
                warp_ran = true;
            }
        }
        if (warp_ran) {
        } else if (want == GFS_SWEEP_CLUSTER_4X2 && launch_tri_cl<T, MODE, P, PE, 4, 2>(ctx, A))
            ran = GFS_SWEEP_CLUSTER_4X2;
        else if (want == GFS_SWEEP_CLUSTER_2X2 && launch_tri_cl<T, MODE, P, PE, 2, 2>(ctx, A))
            ran = GFS_SWEEP_CLUSTER_2X2;
        else if (want == GFS_SWEEP_AUTO || want == GFS_SWEEP_BLOCK || want == GFS_SWEEP_WARP) {
            k_tri<T, MODE, P, PE><<<A.K.nbj * A.K.nbk, SPLANE + RX_THREADS, 0, ctx->stream>>>(A);
            ran = GFS_SWEEP_BLOCK;
        } else {
            set_error(GFS_ERR_INVALID, "sweep kernel %d cannot run this %dx%dx%d solve: its clusters do not all "
                      "fit on the device at once", want, A.K.nx, A.K.ny, A.K.nz);
            return GFS_ERR_INVALID;
        }
        ctx->last_sweep_kernel = ran;
    }
    ctx->launches++;
    GFS_LAUNCH_CHECK();
    return GFS_OK;
}

template <class T>
static VecArgs<T> vec_args(PressureWs &ws, double scale, int mixed) {
    VecArgs<T> A;
    A.K = make_skew(ws.c);
    A.fsk = ws.fsk.as<uint8_t>();
    A.negscale = (T)(-scale);
    A.scale = (T)scale;
    A.partials = ws.partials.as<double>();
    A.ctrl = ws.ctrl.as<PsCtrl>();
    A.mixed = mixed;
    A.slist = ws.slist.as<unsigned>();
    A.snum = ws.snum.as<unsigned>();
    // the diagonal coefficient of a cell with n non-solid neighbours, (T)n * scale, as the
    // device forms it (one IEEE multiply in T)
    for (int n = 0; n < 8; n++) A.dcoef[n] = (T)n * A.scale;
    return A;
}

// One CG iteration (matvec, update, forward + backward MIC(0) solve, new search direction).
template <class T>
static int cg_iteration(Ctx *ctx, PressureWs &ws, double scale, int mixed, T *p, T *r, T *z, T *s, T *As,
                        T *q, const T *precon) {
    unsigned nb = (unsigned)ws.nblocks_red;
    VecArgs<T> V = vec_args<T>(ws, scale, mixed);
    {
        ProfScope prof(ctx, KC_MATVEC);
        k_matvec<T><<<nb, RED_THREADS, 0, ctx->stream>>>(V, s, As);
    }
    {
        ProfScope prof(ctx, KC_AXPY);
        k_axpy<T><<<nb, RED_THREADS, 0, ctx->stream>>>(V, p, r, s, As);
    }
    ctx->launches += 2;
    int rc = launch_sweep<T, SW_FWD>(ctx, ws, r, q, precon, nullptr, nullptr, scale, 0);
    if (rc) return rc;
    rc = launch_sweep<T, SW_BWD>(ctx, ws, q, z, precon, r, nullptr, scale, 0);
    if (rc) return rc;
    ProfScope prof(ctx, KC_UPDATE_S);
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
#ifndef GFS_MIXED_ETA
#define GFS_MIXED_ETA 1e-2
#endif

// MICCG(0) on the system set up in ws (b, r = b, p = s = 0 in the skewed layout,
// control block reset by the set-up kernel), to max|r| < tol or max_iters:
// PLAIN is the reference's FP64 PCG (pressuresolver.cpp:448-498); MIXED runs the
// inner PCG in FP32 with FP64 reliable updates of the residual.  Fills the
// reference-numbered iteration count, the final max-norm residual, the number
// of FP64 updates and of forward (= backward) MIC(0) solves.
// mpc = negscale * precon over every slot, with the solves' own FP64 multiply
__global__ void __launch_bounds__(RED_THREADS) k_neg_precon(long long n, double negscale,
                                                            const double *__restrict__ precon,
                                                            double *__restrict__ mpc) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
        mpc[q] = Ar<double>::mul(negscale, precon[q]);
}

// The list of strips (of Strip<T>::W slots) that hold fluid, for this solve's vector kernels.
template <class T>
static int build_strip_list(Ctx *ctx, PressureWs &ws, const Skew &K) {
    const long long nstrip = K.size / Strip<T>::W;
    cudaStream_t st = ctx->stream;
    unsigned nb = (unsigned)ws.nblocks_red;
    unsigned *off = ws.soff.as<unsigned>();
    k_strip_mark<T><<<nb, RED_THREADS, 0, st>>>(K, ws.fsk.as<uint8_t>(), off);
    ctx->launches++;
    GFS_LAUNCH_CHECK();
    int rc = exclusive_scan_u32(ctx, off, off, nstrip + 1, ws.stmp.as<unsigned>(), st);
    if (rc) return rc;
    k_strip_list<<<nb, RED_THREADS, 0, st>>>((unsigned)nstrip, off, ws.slist.as<unsigned>(), ws.snum.as<unsigned>());
    ctx->launches++;
    GFS_LAUNCH_CHECK();
    return GFS_OK;
}

static int run_cg(Ctx *ctx, PressureWs &ws, const Skew &K, double scale, bool mixed, double tol, int max_iters,
                  PsCtrl &h, int &iterations, double &final_res, int &refinements, int &sweeps) {
    cudaStream_t st = ctx->stream;
    PsCtrl *C = ws.ctrl.as<PsCtrl>();
    unsigned nb = (unsigned)ws.nblocks_red;
    int rc = mixed ? build_strip_list<float>(ctx, ws, K) : build_strip_list<double>(ctx, ws, K);
    if (rc) return rc;
    // MIC(0) preconditioner (pressuresolver.cpp:246-302): FP64 for PLAIN, FP32 for the MIXED inner solve
    if (mixed) rc = launch_sweep<float, SW_PRECON>(ctx, ws, nullptr, ws.precon32.as<float>(), nullptr, nullptr,
                                                   nullptr, scale, 0);
    else rc = launch_sweep<double, SW_PRECON>(ctx, ws, nullptr, ws.precon.as<double>(), nullptr, nullptr, nullptr,
                                              scale, 0);
    if (rc) return rc;
    if (!mixed) {
        // negscale * precon for the FP64 triangular solves
        if (ws.mpc.ensure((size_t)K.size * sizeof(double))) return GFS_ERR_NOMEM;
        k_neg_precon<<<nb, RED_THREADS, 0, st>>>(K.size, -scale, ws.precon.as<double>(), ws.mpc.as<double>());
        ctx->launches++;
        GFS_LAUNCH_CHECK();
    }
    if (!mixed) {
        double *p = ws.psk.as<double>(), *r = ws.r.as<double>(), *z = ws.z.as<double>(),
               *s = ws.s.as<double>(), *As = ws.As.as<double>(), *q = ws.q.as<double>(),
               *pc = ws.precon.as<double>();
        rc = launch_sweep<double, SW_FWD>(ctx, ws, r, q, pc, nullptr, nullptr, scale, 0);
        if (rc) return rc;
        rc = launch_sweep<double, SW_BWD>(ctx, ws, q, z, pc, r, nullptr, scale, 1);
        if (rc) return rc;
        VecArgs<double> V = vec_args<double>(ws, scale, 0);
        {
            ProfScope prof(ctx, KC_UPDATE_S);
            k_update_s<double><<<nb, RED_THREADS, 0, st>>>(V, z, s);
        }
        ctx->launches++;
        for (;;) {
            for (int it = 0; it < CG_CHUNK; it++) {
                rc = cg_iteration<double>(ctx, ws, scale, 0, p, r, z, s, As, q, pc);
                if (rc) return rc;
            }
            rc = read_ctrl(ctx, ws, &h);
            if (rc) return rc;
            if (h.done) break;
        }
        iterations = h.iter;
        final_res = h.maxr;
        sweeps = 1 + h.iter;
    } else {
        // inner FP32 rounds end when max|r32| has dropped below eta * max|r64| of the last update
        const double eta = GFS_MIXED_ETA;
        float *r32 = ws.r32.as<float>(), *z32 = ws.z32.as<float>(), *s32 = ws.s32.as<float>(),
              *As32 = ws.As32.as<float>(), *q32 = ws.q32.as<float>(), *e32 = ws.e32.as<float>(),
              *pc32 = ws.precon32.as<float>();
        int total = 0;
        bool converged = false;
        double res64 = h.maxb;
        VecArgs<double> V64 = vec_args<double>(ws, scale, 1);
        VecArgs<float> V32 = vec_args<float>(ws, scale, 1);
        bool first = true;
        while (total < max_iters) {
            {
                ProfScope prof(ctx, KC_MIXED_AUX);
                if (first)
                    k_mixed_prepare<<<nb, RED_THREADS, 0, st>>>(K, ws.fsk.as<uint8_t>(), ws.r.as<double>(), r32,
                                                               e32, s32, C, eta);
                else
                    k_mixed_reliable<<<nb, RED_THREADS, 0, st>>>(V32, ws.r.as<double>(), r32, e32, eta);
            }
            ctx->launches++;
            // the inner cap is what is left of the total budget
            {
                int left = max_iters - total;
                GFS_CUDA_CHECK(cudaMemcpyAsync(&C->max_iters, &left, sizeof(int), cudaMemcpyHostToDevice, st));
            }
            rc = launch_sweep<float, SW_FWD>(ctx, ws, r32, q32, pc32, nullptr, nullptr, scale, 0);
            if (rc) return rc;
            // first round: s = z = M^-1 r (init); later rounds: the pending half of the
            // iteration that met the inner threshold, beta = sigma_new / sigma, s = z + beta s
            rc = launch_sweep<float, SW_BWD>(ctx, ws, q32, z32, pc32, r32, nullptr, scale, first ? 1 : 0);
            if (rc) return rc;
            first = false;
            {
                ProfScope prof(ctx, KC_UPDATE_S);
                k_update_s<float><<<nb, RED_THREADS, 0, st>>>(V32, z32, s32);
            }
            ctx->launches++;
            for (;;) {
                for (int it = 0; it < CG_CHUNK; it++) {
                    rc = cg_iteration<float>(ctx, ws, scale, 1, e32, r32, z32, s32, As32, q32, pc32);
                    if (rc) return rc;
                }
                rc = read_ctrl(ctx, ws, &h);
                if (rc) return rc;
                if (h.done) break;
            }
            // h.iter counts the inner iterations that completed without converging;
            // the converging iteration is one more.
            total += h.converged ? h.iter + 1 : h.iter;
            sweeps += 1 + h.iter;
            {
                ProfScope prof(ctx, KC_MIXED_AUX);
                k_mixed_correct<<<nb, RED_THREADS, 0, st>>>(V32, ws.psk.as<double>(), e32);
                k_residual64<<<nb, RED_THREADS, 0, st>>>(V64, ws.bsk.as<double>(), ws.psk.as<double>(),
                                                          ws.r.as<double>());
            }
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
    return GFS_OK;
}

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
    const Skew K = make_skew(g.c);
    // tolerance / cap into the control block
    {
        PsCtrl h;
        memset(&h, 0, sizeof(h));
        GFS_CUDA_CHECK(cudaMemcpyAsync(&h, C, sizeof(PsCtrl), cudaMemcpyDeviceToHost, st));
        GFS_CUDA_CHECK(cudaStreamSynchronize(st));
        h.tol = tol;
        h.max_iters = max_iters;
        h.err = 0;
        if (h.epoch == 0) h.epoch = 1;   // exchange words start zeroed: tag 0 means "never written"
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
    {
        ProfScope prof(ctx, KC_PS_SETUP);
        k_ps_setup<<<nb, RED_THREADS, 0, st>>>(SA, mat, mac[0], mac[1], mac[2], ws.flags.as<uint8_t>(),
                                                ws.b.as<double>(), ws.partials.as<double>(), C);
        dim3 cgrid(grid_blocks(g.c.nx, 128), g.c.ny, g.c.nz);
        k_nbits<<<cgrid, 128, 0, st>>>(g.c, ws.flags.as<uint8_t>(), ws.nbstd.as<uint16_t>());
        GFS_CUDA_CHECK(cudaMemsetAsync(ws.blkf.p, 0, ws.blkf.bytes, st));
        k_to_skew<<<nb, RED_THREADS, 0, st>>>(K, g.c, ws.flags.as<uint8_t>(), ws.b.as<double>(),
                                               ws.nbstd.as<uint16_t>(), ws.fsk.as<uint8_t>(), ws.nbsk.as<uint16_t>(), ws.bsk.as<double>(), ws.r.as<double>(),
                                               ws.psk.as<double>(), ws.s.as<double>(), ws.blkf.as<uint8_t>());
    }
    ctx->launches += 3;
    GFS_LAUNCH_CHECK();
    PsCtrl h;
    rc = read_ctrl(ctx, ws, &h);
    if (rc) return rc;
    int iterations = h.iter;
    double final_res = h.maxb;
    int refinements = 0;
    int sweeps = 0;   // forward (= backward) MIC(0) solves that did work
    if (!h.done) {
        rc = run_cg(ctx, ws, K, scale, mixed, tol, max_iters, h, iterations, final_res, refinements, sweeps);
        if (rc) return rc;
    }
    // solution back to the padded cell layout
    {
        dim3 grid(grid_blocks(g.c.nx, 128), g.c.ny, g.c.nz);
        k_from_skew<<<grid, 128, 0, st>>>(K, g.c, ws.flags.as<uint8_t>(), ws.psk.as<double>(), ws.p.as<double>());
        ctx->launches++;
        GFS_LAUNCH_CHECK();
    }
    if (stats) {
        stats->cg_iterations = iterations;
        stats->cg_max_residual = final_res;
        stats->refinements = refinements;
        stats->sweeps = sweeps;
    }
    return GFS_OK;
}

// ------------------------------------------------ setup without a solve

// Flags, b and neighbour bits of the system for (mat, mac) -- what
// pressure_solve does before its first sweep -- so that pressure_solve_rhs
// can solve with the same matrix and a caller can supply the pressure itself.
int pressure_setup(Ctx *ctx, PressureWs &ws, const Grids &g, const uint8_t *mat, float *const mac[3]) {
    int rc = ensure_ws(ctx, ws, g, false);
    if (rc) return rc;
    cudaStream_t st = ctx->stream;
    const double dx = g.dx;
    PsCtrl *C = ws.ctrl.as<PsCtrl>();
    SetupArgs SA;
    SA.c = g.c;
    SA.fu = g.f[0];
    SA.fv = g.f[1];
    SA.fw = g.f[2];
    SA.fscale = 1.0f / (float)dx;
    SA.scale_div = (double)(1.0f / (float)dx);
    SA.tol = 1e-6;
    unsigned nb = (unsigned)ws.nblocks_red;
    ProfScope prof(ctx, KC_PS_SETUP);
    k_ps_setup<<<nb, RED_THREADS, 0, st>>>(SA, mat, mac[0], mac[1], mac[2], ws.flags.as<uint8_t>(), ws.b.as<double>(),
                                            ws.partials.as<double>(), C);
    dim3 cgrid(grid_blocks(g.c.nx, 128), g.c.ny, g.c.nz);
    k_nbits<<<cgrid, 128, 0, st>>>(g.c, ws.flags.as<uint8_t>(), ws.nbstd.as<uint16_t>());
    ctx->launches += 2;
    GFS_LAUNCH_CHECK();
    return GFS_OK;
}

// ------------------------------------------- solve with a given right-hand side

// b = rhs on the fluid cells of the current flags; control block reset as
// k_ps_setup does, with the stopping threshold relative to max|rhs|.
__global__ void __launch_bounds__(RED_THREADS) k_set_rhs(GridDim c, const uint8_t *__restrict__ flags,
                                                         const double *__restrict__ rhs, double *__restrict__ b,
                                                         double *__restrict__ partials, PsCtrl *ctrl,
                                                         double rel_tol) {
    double mx = 0.0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < c.size;
         e += (long long)gridDim.x * blockDim.x) {
        double v = (flags[e] & GFS_PF_FLUID) ? rhs[e] : 0.0;
        b[e] = v;
        mx = fmax(mx, fabs(v));
    }
    double part = block_reduce<1>(mx);
    double res;
    if (finish_reduce<1>(part, partials, &ctrl->tickets[0], gridDim.x, &res) && threadIdx.x == 0) {
        ctrl->maxb = res;
        ctrl->maxr = res;
        ctrl->maxr64 = res;
        ctrl->tol = rel_tol * res;
        ctrl->iter = 0;
        ctrl->converged = 0;
        ctrl->total_inner = 0;
        ctrl->refinements = 0;
        ctrl->sigma = 0.0;
        ctrl->alpha = 0.0;
        ctrl->beta = 0.0;
        ctrl->done = res > 0.0 ? 0 : 1;
    }
}

int pressure_solve_rhs(Ctx *ctx, PressureWs &ws, const Grids &g, const double *rhs, double density, double dt,
                       double rel_tol, int max_iters, gfs_step_stats *stats, bool mixed) {
    if (ws.allocated_for != g.c.size) {
        set_error(GFS_ERR_STATE, "pressure_solve_rhs needs a pressure solve on this grid first");
        return GFS_ERR_STATE;
    }
    if (mixed) {
        int rc0 = ensure_ws(ctx, ws, g, true);
        if (rc0) return rc0;
    }
    cudaStream_t st = ctx->stream;
    const double dx = g.dx;
    const double scale = dt / (density * dx * dx);
    PsCtrl *C = ws.ctrl.as<PsCtrl>();
    const Skew K = make_skew(g.c);
    {
        PsCtrl h;
        memset(&h, 0, sizeof(h));
        GFS_CUDA_CHECK(cudaMemcpyAsync(&h, C, sizeof(PsCtrl), cudaMemcpyDeviceToHost, st));
        GFS_CUDA_CHECK(cudaStreamSynchronize(st));
        h.max_iters = max_iters;
        h.err = 0;
        if (h.epoch == 0) h.epoch = 1;
        GFS_CUDA_CHECK(cudaMemcpyAsync(C, &h, sizeof(PsCtrl), cudaMemcpyHostToDevice, st));
    }
    unsigned nb = (unsigned)ws.nblocks_red;
    {
        ProfScope prof(ctx, KC_PS_SETUP);
        k_set_rhs<<<nb, RED_THREADS, 0, st>>>(g.c, ws.flags.as<uint8_t>(), rhs, ws.b.as<double>(),
                                               ws.partials.as<double>(), C, rel_tol);
        GFS_CUDA_CHECK(cudaMemsetAsync(ws.blkf.p, 0, ws.blkf.bytes, st));
        k_to_skew<<<nb, RED_THREADS, 0, st>>>(K, g.c, ws.flags.as<uint8_t>(), ws.b.as<double>(),
                                               ws.nbstd.as<uint16_t>(), ws.fsk.as<uint8_t>(), ws.nbsk.as<uint16_t>(),
                                               ws.bsk.as<double>(), ws.r.as<double>(), ws.psk.as<double>(),
                                               ws.s.as<double>(), ws.blkf.as<uint8_t>());
    }
    ctx->launches += 2;
    GFS_LAUNCH_CHECK();
    PsCtrl h;
    int rc = read_ctrl(ctx, ws, &h);
    if (rc) return rc;
    int sweeps = 0, iterations = h.iter, refinements = 0;
    double final_res = h.maxb;
    if (!h.done) {
        rc = run_cg(ctx, ws, K, scale, mixed, h.tol, max_iters, h, iterations, final_res, refinements, sweeps);
        if (rc) return rc;
    }
    {
        dim3 grid(grid_blocks(g.c.nx, 128), g.c.ny, g.c.nz);
        k_from_skew<<<grid, 128, 0, st>>>(K, g.c, ws.flags.as<uint8_t>(), ws.psk.as<double>(), ws.p.as<double>());
        ctx->launches++;
        GFS_LAUNCH_CHECK();
    }
    if (h.err) {
        set_error(GFS_ERR_TIMEOUT, "a wavefront wait of the pressure solve timed out");
        return GFS_ERR_TIMEOUT;
    }
    if (stats) {
        stats->cg_iterations = iterations;
        stats->cg_max_residual = final_res;
        stats->refinements = refinements;
        stats->sweeps = sweeps;
    }
    return GFS_OK;
}

// ------------------------------------------------- accuracy check

__device__ __forceinline__ void atomic_max_nonneg(double *addr, double v) {
    // non-negative doubles order like their bit patterns
    atomicMax(reinterpret_cast<unsigned long long *>(addr), (unsigned long long)__double_as_longlong(v));
}

// out[0] = max |b - A p| (FP64, the matrix of the flags), out[1] = max |p - q|, out[2] = max |q|
__global__ void __launch_bounds__(RED_THREADS) k_check(GridDim c, const uint8_t *__restrict__ flags,
                                                       const double *__restrict__ b, const double *__restrict__ p,
                                                       const double *__restrict__ q, double scale,
                                                       double *__restrict__ out) {
    double r = 0.0, e = 0.0, m = 0.0;
    const long long sx = 1, sy = c.sx, sz = (long long)c.sx * c.sy;
    for (long long at = blockIdx.x * (long long)blockDim.x + threadIdx.x; at < c.size;
         at += (long long)gridDim.x * blockDim.x) {
        uint8_t fl = flags[at];
        if (!(fl & GFS_PF_FLUID)) continue;
        // _applyMatrix (pressuresolver.cpp:388-426): diag*scale*x - scale * sum of fluid neighbours
        double nb = 0.0;
        const long long off[6] = {-sx, sx, -sy, sy, -sz, sz};
        for (int k = 0; k < 6; k++)
            if (flags[at + off[k]] & GFS_PF_FLUID) nb += p[at + off[k]];
        double ap = (double)(fl >> 1) * scale * p[at] - scale * nb;
        r = fmax(r, fabs(b[at] - ap));
        e = fmax(e, fabs(p[at] - q[at]));
        m = fmax(m, fabs(q[at]));
    }
    r = block_reduce<1>(r);
    e = block_reduce<1>(e);
    m = block_reduce<1>(m);
    if (threadIdx.x == 0) {
        atomic_max_nonneg(out, r);
        atomic_max_nonneg(out + 1, e);
        atomic_max_nonneg(out + 2, m);
    }
}

int pressure_check(Ctx *ctx, PressureWs &ws, const Grids &g, double density, double dt, double rel_tol,
                   double *fp64_residual, double *rel_error, int *ref_iterations) {
    if (ws.allocated_for != g.c.size) {
        set_error(GFS_ERR_STATE, "no pressure solve to check on this grid");
        return GFS_ERR_STATE;
    }
    cudaStream_t st = ctx->stream;
    const size_t bytes = (size_t)g.c.size * sizeof(double);
    DevMem pm, bc, out;
    if (pm.alloc(bytes) || bc.alloc(bytes) || out.alloc(3 * sizeof(double))) return GFS_ERR_NOMEM;
    GFS_CUDA_CHECK(cudaMemcpyAsync(pm.p, ws.p.p, bytes, cudaMemcpyDeviceToDevice, st));
    GFS_CUDA_CHECK(cudaMemcpyAsync(bc.p, ws.b.p, bytes, cudaMemcpyDeviceToDevice, st));
    gfs_step_stats stats{};
    int rc = pressure_solve_rhs(ctx, ws, g, bc.as<double>(), density, dt, rel_tol, 20000, &stats);
    if (rc) return rc;
    GFS_CUDA_CHECK(cudaMemsetAsync(out.p, 0, out.bytes, st));
    const double scale = dt / (density * g.dx * g.dx);
    k_check<<<(unsigned)ws.nblocks_red, RED_THREADS, 0, st>>>(g.c, ws.flags.as<uint8_t>(), bc.as<double>(),
                                                              pm.as<double>(), ws.p.as<double>(), scale,
                                                              out.as<double>());
    ctx->launches++;
    GFS_LAUNCH_CHECK();
    double h[3];
    GFS_CUDA_CHECK(cudaMemcpyAsync(h, out.p, sizeof(h), cudaMemcpyDeviceToHost, st));
    // the checked solution back in place (the workspace's pressure is the substep's)
    GFS_CUDA_CHECK(cudaMemcpyAsync(ws.p.p, pm.p, bytes, cudaMemcpyDeviceToDevice, st));
    GFS_CUDA_CHECK(cudaStreamSynchronize(st));
    if (fp64_residual) *fp64_residual = h[0];
    if (rel_error) *rel_error = h[2] > 0.0 ? h[1] / h[2] : 0.0;
    if (ref_iterations) *ref_iterations = stats.cg_iterations;
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
    ProfScope prof(ctx, KC_APPLY);
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
