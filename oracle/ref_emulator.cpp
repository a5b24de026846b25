/*
 * ref_emulator.cpp -- the reference's own kernel files, compiled for the host.
 *
 * TEST INFRASTRUCTURE ONLY: builds oracle/_ref/libxrdt_ref.so, used to pin the
 * FP64 oracle (xrdt_oracle.c) and to generate the golden fixtures in
 * tests/golden.  It is built only where the reference sources are present.
 *
 * The files Forward_projector_kernels/{Copy2Vector,GetIntersection,attenuator,
 * find_src_nrg_range,wvt_value,integrate_diffraction}.cu are #included
 * unmodified from the reference tree (include path given by the Makefile).
 * Around them this file provides:
 *   - the compile-time configuration of Forward_XRD.cu:16-53 (same names and
 *     values; the float constants are typed double so that every expression
 *     of the kernels evaluates in FP64 on the float-rounded values);
 *   - `float` redefined as `double` for the kernel bodies;
 *   - CUDA intrinsics mapped to their exact FP64 counterparts;
 *   - tex2D as exact bilinear interpolation with a zero border (the texture
 *     setup of Forward_XRD.cu:229-233);
 *   - a SIMT block emulator: each CUDA thread runs as a user-level fiber;
 *     __syncthreads and __shfl_down_sync are rendezvous points.  Fibers are
 *     resumed in thread order after every rendezvous, so every read of the
 *     attenuator's shared partial sums (attenuator.cu:96-101) happens before
 *     the next write to them; the emulated block is free of that data race.
 * Uninitialised locals are zeroed (-ftrivial-auto-var-init=zero), so the
 * stale voxel coordinates read at integrate_diffraction.cu:181 start at (0,0).
 */
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <climits>
#include <limits>
#include <vector>
#include <deque>
#include <ucontext.h>

struct float2 {
    double x, y;
};
struct EmuDim3 {
    int x, y, z;
};

namespace emu {

constexpr int kWarp = 32;
constexpr size_t kStack = 256 * 1024;

struct Block;
thread_local Block *g_block = nullptr;
thread_local EmuDim3 g_block_idx = {0, 0, 0};

enum State { RUN = 0, WAIT_SYNC = 1, WAIT_SHFL = 2, DONE = 3 };

struct Block {
    int nthreads = 0;
    std::vector<ucontext_t> ctx;
    std::vector<char *> stacks;
    std::vector<int> state;
    std::vector<EmuDim3> tidx;
    ucontext_t sched;
    int cur = -1;
    int sync_arrived = 0;
    std::vector<int> shfl_arrived;   // per warp
    std::vector<double> shfl_val;    // per thread
    std::vector<int> shfl_off;       // per thread
    std::vector<double> shfl_res;    // per thread
    std::deque<int> runq;
    void (*entry)(void *) = nullptr;
    void *arg = nullptr;
    bool failed = false;

    ~Block() {
        for (char *s : stacks) free(s);
    }
};

inline const EmuDim3 &thread_idx() { return g_block->tidx[g_block->cur]; }

inline void yield_to_sched() {
    Block *b = g_block;
    swapcontext(&b->ctx[b->cur], &b->sched);
}

inline void syncthreads() {
    Block *b = g_block;
    b->state[b->cur] = WAIT_SYNC;
    if (++b->sync_arrived == b->nthreads) {
        b->sync_arrived = 0;
        for (int t = 0; t < b->nthreads; t++) {
            b->state[t] = RUN;
            b->runq.push_back(t);
        }
    }
    yield_to_sched();
}

inline double shfl_down(double v, int off) {
    Block *b = g_block;
    int t = b->cur, w = t / kWarp;
    b->shfl_val[t] = v;
    b->shfl_off[t] = off;
    b->state[t] = WAIT_SHFL;
    if (++b->shfl_arrived[w] == kWarp) {
        b->shfl_arrived[w] = 0;
        for (int l = 0; l < kWarp; l++) {
            int tt = w * kWarp + l;
            int src = l + b->shfl_off[tt];
            b->shfl_res[tt] = (src < kWarp) ? b->shfl_val[w * kWarp + src] : b->shfl_val[tt];
        }
        for (int l = 0; l < kWarp; l++) {
            b->state[w * kWarp + l] = RUN;
            b->runq.push_back(w * kWarp + l);
        }
    }
    yield_to_sched();
    return b->shfl_res[t];
}

void trampoline(int t) {
    Block *b = g_block;
    (void)t;
    b->entry(b->arg);
    b->state[b->cur] = DONE;
    yield_to_sched();
}

/* Runs entry(arg) as a block of n threads; returns false on deadlock. */
bool run_block(Block &b, int n, void (*entry)(void *), void *arg) {
    b.nthreads = n;
    if ((int)b.ctx.size() < n) {
        b.ctx.resize(n);
        while ((int)b.stacks.size() < n) b.stacks.push_back((char *)malloc(kStack));
    }
    b.state.assign(n, RUN);
    b.tidx.resize(n);
    b.shfl_arrived.assign((n + kWarp - 1) / kWarp, 0);
    b.shfl_val.assign(n, 0.0);
    b.shfl_off.assign(n, 0);
    b.shfl_res.assign(n, 0.0);
    b.sync_arrived = 0;
    b.runq.clear();
    b.entry = entry;
    b.arg = arg;
    g_block = &b;
    for (int t = 0; t < n; t++) {
        b.tidx[t] = {t, 0, 0};
        getcontext(&b.ctx[t]);
        b.ctx[t].uc_stack.ss_sp = b.stacks[t];
        b.ctx[t].uc_stack.ss_size = kStack;
        b.ctx[t].uc_link = nullptr;
        makecontext(&b.ctx[t], (void (*)())trampoline, 1, t);
        b.runq.push_back(t);
    }
    int done = 0;
    while (!b.runq.empty()) {
        int t = b.runq.front();
        b.runq.pop_front();
        b.cur = t;
        swapcontext(&b.sched, &b.ctx[t]);
        if (b.state[t] == DONE) done++;
    }
    g_block = nullptr;
    return done == n;
}

inline int f2i_rd(double x) {
    if (std::isnan(x)) return 0;
    double f = std::floor(x);
    if (f >= 2147483647.0) return INT_MAX;
    if (f <= -2147483648.0) return INT_MIN;
    return (int)f;
}
inline int f2i_ru(double x) {
    if (std::isnan(x)) return 0;
    double f = std::ceil(x);
    if (f >= 2147483647.0) return INT_MAX;
    if (f <= -2147483648.0) return INT_MIN;
    return (int)f;
}

struct Tex {
    const double *a1 = nullptr, *a2 = nullptr;
    int nx = 0, ny = 0;
};

} // namespace emu

/* ---- texture: exact bilinear, border 0, unnormalised coordinates ---- */
static thread_local emu::Tex texRef;
static inline float2 tex2D(const emu::Tex &t, double x, double y) {
    double xb = x - 0.5, yb = y - 0.5;
    double fi = std::floor(xb), fj = std::floor(yb);
    double fx = xb - fi, fy = yb - fj;
    long i0 = (long)fi, j0 = (long)fj;
    float2 r = {0.0, 0.0};
    for (int dj = 0; dj < 2; dj++) {
        long j = j0 + dj;
        if (j < 0 || j >= t.ny) continue;
        double wy = dj ? fy : 1.0 - fy;
        for (int di = 0; di < 2; di++) {
            long i = i0 + di;
            if (i < 0 || i >= t.nx) continue;
            double w = wy * (di ? fx : 1.0 - fx);
            r.x += w * t.a1[i + j * (long)t.nx];
            r.y += w * t.a2[i + j * (long)t.nx];
        }
    }
    return r;
}

/* ---- compile-time configuration of Forward_XRD.cu:16-53 ---- */
#ifndef SRC
#define SRC 32
#endif
#ifndef COL
#define COL 1024
#endif
#ifndef ROW
#define ROW 1
#endif
#define DET COL*ROW
#ifndef NRG
#define NRG 64
#endif
#ifndef DNRG
#define DNRG 5
#endif
#ifndef NWT
#define NWT 256
#endif
#ifndef NQF
#define NQF 768
#endif
#ifndef MAT
#define MAT 3
#endif
#define FULL_MASK 0xffffffff
#define warpSize 32
#define maxNumThreads 1024
#define numWarps NWT/warpSize
#define NQBatch NQF/NWT
#define rsqrt2pi ((double)0.398942280401433f)
#define twopi ((double)6.28318530717959f)
#define hbarc ((double)1.973269804f)
#define qmin ((double)0.5f)
#define qmax ((double)6.0f)
#define dq0 ((double)0.01f)
#define dq_fine (qmax-qmin)/__int2float_rn(NQF)
#define DQ ((double)0.25f)
#ifndef NQ
#define NQ 64
#endif
#ifndef NA
#define NA 64
#endif
#define KN0 ((double)0.751691286166726f)
#define KN1 ((double)1.4599683207703f)
#define KN2 ((double)-0.64597532690936f)

/* ---- CUDA device environment for the kernel bodies ---- */
#define __device__
#define __global__
#define __shared__ thread_local
#define threadIdx (emu::thread_idx())
#define blockIdx (emu::g_block_idx)
#define __syncthreads() emu::syncthreads()
#define __shfl_down_sync(mask, v, off) emu::shfl_down((v), (off))
#define __int2float_rn(x) ((double)(x))
#define __int2float_rd(x) ((double)(x))
#define __float2int_rd(x) emu::f2i_rd((double)(x))
#define __float2int_ru(x) emu::f2i_ru((double)(x))
#define __int_as_float(x) (std::numeric_limits<double>::quiet_NaN())
#define __fsqrt_rn(x) std::sqrt((double)(x))
#define __frsqrt_rn(x) (1.0 / std::sqrt((double)(x)))
#define rsqrtf(x) (1.0 / std::sqrt((double)(x)))
#define sqrtf(x) std::sqrt((double)(x))
#define __log2f(x) std::log2((double)(x))
#define __expf(x) std::exp((double)(x))
#define expf(x) std::exp((double)(x))
#define sinf(x) std::sin((double)(x))
#define cosf(x) std::cos((double)(x))
#define tanf(x) std::tan((double)(x))
#define fabsf(x) std::fabs((double)(x))
#define fminf(a, b) std::fmin((double)(a), (double)(b))
#define fmaxf(a, b) std::fmax((double)(a), (double)(b))

#define float double
#include "Copy2Vector.cu"
#include "GetIntersection.cu"
#include "attenuator.cu"
#include "find_src_nrg_range.cu"
#include "wvt_value.cu"
#include "integrate_diffraction.cu"
#undef float

/* ---- host entry points ---- */
namespace {

struct KernelArgs {
    double *spectrum, *Nphotons, *Amatrix, *Ifine;
    int *seg;
    int NX, NY;
    double *Cphotons, *S2;
    double q_min, q_max, a_min, a_max;
};

void kernel_entry(void *p) {
    KernelArgs *a = (KernelArgs *)p;
    integrate_diffraction(a->spectrum, a->Nphotons, a->Amatrix, a->Ifine, a->seg, a->NX, a->NY,
                          a->Cphotons, a->S2, a->q_min, a->q_max, a->a_min, a->a_max);
}

template <class T>
T *shifted(T *base, int64_t idx) {
    return (T *)((uintptr_t)base - (uintptr_t)(idx * (int64_t)sizeof(T)));
}

} // namespace

extern "C" {

/* Compile-time configuration: SRC, COL, ROW, NRG, DNRG, NWT, NQF, MAT, NQ, NA. */
void xrdt_ref_config(int32_t *out) {
    const int32_t v[10] = {SRC, COL, ROW, NRG, DNRG, NWT, NQF, MAT, NQ, NA};
    memcpy(out, v, sizeof(v));
}

void xrdt_ref_wvt_value(int32_t nwt, double *q, double *dq) { wvt_value(nwt, q, dq); }

void xrdt_ref_find_src_nrg_range(int32_t nrg, int32_t *lo, int32_t *hi) {
    find_src_nrg_range(nrg, lo, hi);
}

void xrdt_ref_get_intersection(double x1, double y1, double x2, double y2, int32_t nx, int32_t ny,
                               double *rx, double *ry) {
    float2 r = GetIntersection(x1, y1, x2, y2, nx, ny);
    *rx = r.x;
    *ry = r.y;
}

/* integrate_diffraction for the listed rays (linear index src + det*SRC +
 * nrg*SRC*DET), one emulated block of NWT threads per ray.  Outputs:
 * N[n_rays], C[n_rays], A[n_rays][MAT][NWT] (may be NULL: then a scratch row
 * receives the model matrix).  Returns the number of blocks that failed. */
int32_t xrdt_ref_integrate_diffraction(const float *spectrum, const float *Ifine, const int32_t *seg,
                                       const float *a1, const float *a2, const float *S2,
                                       int32_t NXv, int32_t NYv, float q_min, float q_max,
                                       float a_min, float a_max, const int64_t *rays, int64_t n_rays,
                                       double *N, double *C, double *A, int32_t n_threads) {
    std::vector<double> spec(spectrum, spectrum + (size_t)NRG * NRG);
    std::vector<double> ifine(Ifine, Ifine + (size_t)NQF * MAT);
    std::vector<double> s2(S2, S2 + (size_t)NQ * NA);
    size_t nvox = (size_t)NXv * NYv;
    std::vector<double> A1(a1, a1 + nvox), A2(a2, a2 + nvox);
    std::vector<int> segv(seg, seg + nvox);
    int failed = 0;
#pragma omp parallel num_threads(n_threads > 0 ? n_threads : 1) reduction(+ : failed)
    {
        emu::Block block;
        std::vector<double> arow((size_t)MAT * NWT);
        texRef.a1 = A1.data();
        texRef.a2 = A2.data();
        texRef.nx = NXv;
        texRef.ny = NYv;
#pragma omp for schedule(dynamic, 1)
        for (int64_t i = 0; i < n_rays; i++) {
            int64_t r = rays[i];
            int src = (int)(r % SRC);
            int det = (int)((r / SRC) % (DET));
            int nrg = (int)(r / ((int64_t)SRC * (DET)));
            emu::g_block_idx = {src, det, nrg};
            double *arow_dst = A ? A + i * (int64_t)MAT * NWT : arow.data();
            int64_t out_idx = (int64_t)src + (int64_t)det * SRC + (int64_t)nrg * SRC * (DET);
            int64_t a_idx = (int64_t)src * NWT * MAT + (int64_t)det * NWT * MAT * SRC +
                            (int64_t)nrg * NWT * MAT * SRC * (DET);
            KernelArgs ka;
            ka.spectrum = spec.data();
            ka.Nphotons = shifted(&N[i], out_idx);
            ka.Cphotons = shifted(&C[i], out_idx);
            ka.Amatrix = shifted(arow_dst, a_idx);
            ka.Ifine = ifine.data();
            ka.seg = segv.data();
            ka.NX = NXv;
            ka.NY = NYv;
            ka.S2 = s2.data();
            ka.q_min = q_min;
            ka.q_max = q_max;
            ka.a_min = a_min;
            ka.a_max = a_max;
            if (!emu::run_block(block, NWT, kernel_entry, &ka)) failed++;
        }
    }
    return failed;
}

} // extern "C"
