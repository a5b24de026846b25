// k_vox.cu -- the model with per-voxel coefficients: forward, adjoint and
// the MLEM update, matrix-free, for a batch of independent problems.
//
// The reference's model matrix has one unknown per (coarse q bin, material):
// Amatrix[k, m, ray] = sum over the voxels of material m of the coarse-q
// term of integrate_diffraction.cu:311-315,
//
//   Av[ray, v, k] = sum_{e in window(nrg)} RF[e,nrg] Pin Pout geom Rayleigh
//                   * G(wvt(v,e) - q_k; sigma(v,e)) * dq_k .
//
// With one unknown per (voxel, coarse bin), x[v, k], the forward model is
// y = Av x and its adjoint g = Av^T w.  Both are computed on the fly; the
// source-side attenuation comes from the per-(source, voxel) table.
//
// Every kernel takes a batch of problems (phantoms and scanners of any
// size, VoxJob); a single operator is a batch of one.  The two heavy kernels
// are persistent: a grid sized to the GPU takes work items from an atomic
// counter -- the (source, pixel) pairs of all problems for the forward, the
// (voxel chunk, pair group) tiles of all problems for the adjoint -- so that
// uneven problems share one launch and the tail stays short.
//
// The detector-side integrals of each (pair, voxel) come from a table: the
// operator's own (VoxOp::walk, walked once by k_walk.cu when the operator is
// created) or the current tile of a walk streamed inside the call.
//
//  * forward (k_vox_fwd): one item = one (source, pixel) pair, as in
//    k_fwd.cu; lane = source energy (or, for windows that are not a multiple
//    of 32 energies, the chunk's (voxel, energy) items 32 at a time) sums the
//    coarse bins within 7.5 sigma of the wavevector transfer, weighted by
//    x[v, k] dq_k, into compensated per-energy sums; the banded spectrum
//    weights give the detector bins.  In
//    MLEM mode the block goes on to form the ratios y / (Av x + c + 1e-20) of
//    main.m:162 for its detector bins and folds them back through the same
//    spectrum band into per-energy weights what[pair, e] = sum_nrg RF[e,nrg]
//    ratio[nrg].
//  * adjoint (k_vox_adj): voxel-major, so that g stays on chip.  A warp owns
//    32 voxels and loops over a group of pairs; per (pair, voxel) lane =
//    energy forms what[pair,e] * (the energy's prefactor) and its coarse-bin
//    window (13.25 sigma), then lane = coarse bin k adds the terms of the
//    energies whose windows can hold k to the voxel's compensated sum.  The
//    groups' partial sums (float pairs) are added in FP64 by k_vox_reduce,
//    which also applies the MLEM update (main.m:163-176).
#include "scatter.cuh"

namespace xrdt {

namespace {

constexpr int kFwdThreads = 256;
constexpr int kFwdWarps = kFwdThreads / 32;

// Per-(voxel, energy) factors shared by the forward and the adjoint: the
// prefactor pref = Pin Pout geom Rayleigh / (sigma sqrt(2 pi)) without RF,
// the wavevector transfer as a pair, the Gaussian exponent scale (log2
// units, as a pair) and the window half-width.
struct EnergyTerm {
    float pref, w_hi, w_lo, c_hi, c_lo, half;
};

// Per-(pair, voxel) parts of sigma^2 = c1 s^2 + c2(e) sg / s^2 as pairs:
// c1 s^2 (c1, the energy-bin width term, is the same for every source bin)
// and sg / s^2.
struct SigmaGeom {
    ff t1, sg_s2;
};

__device__ __forceinline__ SigmaGeom sigma_geom(float sh, float sl, ff sg, ff c1)
{
    SigmaGeom g;
    const ff s2 = ff_sqr(ff{sh, sl});
    g.t1 = ff_mul(c1, s2);
    g.sg_s2 = ff_div(sg, s2);
    return g;
}

__device__ __forceinline__ EnergyTerm energy_term(const float *en, int E, int el, float Adx, float Ady, float Asx,
                                                  float Asy, float sh, float sl, const SigmaGeom &sgm, float Wg,
                                                  float rsqrt2pi)
{
    const float if1 = en[el], if2 = en[E + el];
    const float Xin = fmaf(Adx, if1, Ady * if2);
    const float Xout = fmaf(Asx, if1, Asy * if2);
    const float wh0 = en[2 * E + el], wl0 = en[3 * E + el];
    EnergyTerm t;
    float w_hi = wh0 * sh;
    float w_lo = fmaf(wh0, sh, -w_hi) + fmaf(wh0, sl, wl0 * sh);
    {
        const float s = w_hi + w_lo;
        w_lo = w_lo - (s - w_hi);
        w_hi = s;
    }
    // sigma^2 as a pair: deep in the Gaussian's tail the exponent amplifies
    // its relative error by (q distance / sigma)^2 / 2
    const ff sig2 = ff_add(sgm.t1, ff_mul(ff{en[5 * E + el], en[7 * E + el]}, sgm.sg_s2));
    // 1/sigma to within an ulp: one Newton step on rsqrt, with the low part
    const float r0 = rsqrtf(sig2.hi);
    const float h = fmaf(-0.5f * sig2.hi * r0, r0, 0.5f) - 0.5f * sig2.lo * r0 * r0;
    const float rs = fmaf(r0, h, r0);
    const ff c = gauss_scale(sig2);
    t.c_hi = c.hi;
    t.c_lo = c.lo;
    // exp(-X) as 2^(-X log2 e) with log2 e as a pair
    const float X = Xin + Xout;
    const float PP = ex2_approx(-fmaf(X, kLog2e, X * kLog2e_lo));
    t.pref = PP * Wg * rsqrt2pi * rs;
    t.half = kSig * sig2.hi * rs;
    t.w_hi = w_hi;
    t.w_lo = w_lo;
    return t;
}

// Energy rows in shared memory: 1/f1, 1/f2, wfac_hi, wfac_lo, sig_c1,
// sig_c2, and the low parts of sig_c1, sig_c2.
constexpr int kEnRows = 8;
__device__ __forceinline__ void stage_energy_rows(const VoxJob &J, float *en, int tid, int nthreads)
{
    for (int i = tid; i < J.E; i += nthreads) {
        const EnergyRow r = J.op.energy[J.op.P.e_lo + i];
        en[i] = r.inv_f1;
        en[J.E + i] = r.inv_f2;
        en[2 * J.E + i] = r.wfac_hi;
        en[3 * J.E + i] = r.wfac_lo;
        en[4 * J.E + i] = r.sig_c1;
        en[5 * J.E + i] = r.sig_c2;
        en[6 * J.E + i] = r.sig_c1_lo;
        en[7 * J.E + i] = r.sig_c2_lo;
    }
}

// The problem that work item t belongs to: the last p with off[p] <= t.
__device__ __forceinline__ int find_job(const int64_t *__restrict__ off, int n, int64_t t)
{
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(off + mid) <= t) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Copies a job into shared memory with every thread of the block.
__device__ __forceinline__ void load_job(const VoxJob *__restrict__ jobs, int p, VoxJob *dst)
{
    static_assert(sizeof(VoxJob) % 4 == 0, "job size");
    const int *src = reinterpret_cast<const int *>(jobs + p);
    int *d = reinterpret_cast<int *>(dst);
    for (int i = threadIdx.x; i < (int)(sizeof(VoxJob) / 4); i += blockDim.x) d[i] = __ldg(src + i);
}

struct FwdLayout {
    size_t tn, tns, en, rf, winlo, wn, cq, ratio, total;
};

__host__ __device__ inline size_t al16(size_t x) { return (x + 15) & ~(size_t)15; }

__host__ __device__ inline FwdLayout vox_fwd_layout(const DevProblem &P, int E)
{
    const int W = 2 * P.dnrg + 1;
    FwdLayout L;
    size_t o = 0;
    L.tn = o; o = al16(o + sizeof(double) * E);
    L.tns = o; o = al16(o + sizeof(float2) * kFwdWarps * E);
    L.en = o; o = al16(o + sizeof(float) * kEnRows * E);
    L.rf = o; o = al16(o + sizeof(float) * P.nrg_det * W);
    L.winlo = o; o = al16(o + sizeof(int) * P.nrg_det);
    L.wn = o; o = al16(o + sizeof(int) * 2 * E);
    L.cq = o; o = al16(o + sizeof(float4) * P.nwt);
    L.ratio = o; o = al16(o + sizeof(double) * P.nrg_det);
    L.total = o;
    return L;
}

// One (source, pixel) pair of job J, by the whole block.
template <bool MLEM>
__device__ __forceinline__ void vox_fwd_pair(const VoxJob &J, int64_t pidx, unsigned char *sm, PairRec &pair)
{
    const DevProblem &P = J.op.P;
    const F32Consts &c = J.c;
    const int E = J.E, K = P.nwt, W = 2 * P.dnrg + 1;
    const FwdLayout L = vox_fwd_layout(P, E);
    double *TN = (double *)(sm + L.tn);
    float2 *TNs = (float2 *)(sm + L.tns);
    float *en = (float *)(sm + L.en);
    float *rf = (float *)(sm + L.rf);
    int *winlo = (int *)(sm + L.winlo);
    int *wn = (int *)(sm + L.wn);
    float4 *cq = (float4 *)(sm + L.cq);
    double *ratio = (double *)(sm + L.ratio);   // kept in FP64: see the weights below

    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int64_t npairs = (int64_t)P.n_src * P.n_det;
    const int src = (int)(pidx % P.n_src);

    stage_energy_rows(J, en, tid, kFwdThreads);
    for (int i = tid; i < kFwdWarps * E; i += kFwdThreads) TNs[i] = make_float2(0.f, 0.f);
    for (int i = tid; i < 2 * E; i += kFwdThreads) wn[i] = J.op.win_n[2 * P.e_lo + i];
    for (int i = tid; i < P.nrg_det * W; i += kFwdThreads) rf[i] = J.op.rf_win[i];
    for (int i = tid; i < P.nrg_det; i += kFwdThreads) winlo[i] = J.op.win_lo[i];
    for (int i = tid; i < K; i += kFwdThreads) cq[i] = J.op.coarse_q[i];
    static_assert(sizeof(PairRec) / 4 <= kFwdThreads, "one word per thread");
    if (tid < (int)(sizeof(PairRec) / 4))
        reinterpret_cast<int *>(&pair)[tid] = reinterpret_cast<const int *>(J.op.pairs + pidx)[tid];
    const float rsqrt2pi = c.rsqrt2pi;
    const float qlo_f = c.q_lo;
    const float *__restrict__ xd = J.xd;
    __syncthreads();

    float2 *TNw = TNs + wid * E;
    const int nv = J.op.nv;
    const int nchunks = (nv + 31) >> 5;
    for (int chunk = wid; chunk < nchunks; chunk += kFwdWarps) {
        const int v = min(chunk * 32 + lane, nv - 1);
        const int xy = J.op.vox_xy[v];
        const float vx = ((float)(xy & 0xffff) + 0.5f) * c.vox;
        const float vy = ((float)(xy >> 16) + 0.5f) * c.vox;
        const VoxGeom vg = vox_geom<true>(pair.G, vx, vy);
        const float2 Asv = J.op.atten_src[(int64_t)src * nv + v];
        // the detector-side integral feeds Pin (integrate_diffraction.cu:259-260),
        // read from the table of this job's pairs (kept, or walked for the tile)
        const float2 Adv = J.op.walk[(pidx - J.pair0) * nv + v];

        const int nin = min(32, nv - chunk * 32);
        // the (voxel, energy) term: lane's energy el for voxel i of the chunk
        auto term = [&](int i, int el, float2 Ad, float sh, float sl, float Wg, float Asx, float Asy,
                        const SigmaGeom &sgm) {
            const float *xrow = xd + (int64_t)(chunk * 32 + i) * K;
            const EnergyTerm t = energy_term(en, E, el, Ad.x, Ad.y, Asx, Asy, sh, sl, sgm, Wg, rsqrt2pi);
            if (t.pref == 0.f) return;   // attenuation underflow: no contribution
            int klo, khi;
            coarse_window(t.w_hi, t.half, qlo_f, c.qpar_a, c.qpar_b, K, &klo, &khi);
            float acc = 0.f;
            for (int k = klo; k <= khi; k++) {
                const float4 q = cq[k];
                acc = fmaf(gauss_f32(t.w_hi, t.w_lo, q.x, q.y, t.c_hi, t.c_lo), __ldg(xrow + k), acc);
            }
            float2 s = TNw[el];
            kahan_add(s.x, s.y, t.pref * acc);
            TNw[el] = s;
        };
        if (E > 32 && (E & 31)) {
            // E not a multiple of 32 (40 on the 128x128 workload): the chunk's
            // (voxel, energy) items nin*E, 32 consecutive ones per step, so
            // that no step runs with a few lanes.  Consecutive items of a step
            // have distinct energies (32 < E), hence distinct sums TNw[el].
            // Each lane's voxel constants come from the lane that holds them.
            const SigmaGeom sgv = sigma_geom(vg.s.hi, vg.s.lo, vg.sg, ff{en[4 * E], en[6 * E]});
            int i = 0, el = lane;
            for (int t0 = 0; t0 < nin * E; t0 += 32) {
                const bool act = i < nin;
                const float2 Ad = make_float2(__shfl_sync(0xffffffffu, Adv.x, i), __shfl_sync(0xffffffffu, Adv.y, i));
                const float sh = __shfl_sync(0xffffffffu, vg.s.hi, i);
                const float sl = __shfl_sync(0xffffffffu, vg.s.lo, i);
                const float Wg = __shfl_sync(0xffffffffu, vg.Wg, i);
                const float Asx = __shfl_sync(0xffffffffu, Asv.x, i);
                const float Asy = __shfl_sync(0xffffffffu, Asv.y, i);
                SigmaGeom sgm;
                sgm.t1 = ff{__shfl_sync(0xffffffffu, sgv.t1.hi, i), __shfl_sync(0xffffffffu, sgv.t1.lo, i)};
                sgm.sg_s2 = ff{__shfl_sync(0xffffffffu, sgv.sg_s2.hi, i), __shfl_sync(0xffffffffu, sgv.sg_s2.lo, i)};
                if (act) term(i, el, Ad, sh, sl, Wg, Asx, Asy, sgm);
                el += 32;
                if (el >= E) {
                    el -= E;
                    i++;
                }
            }
        } else {
            for (int i = 0; i < nin; i++) {
                const float2 Ad = make_float2(__shfl_sync(0xffffffffu, Adv.x, i), __shfl_sync(0xffffffffu, Adv.y, i));
                const float sh = __shfl_sync(0xffffffffu, vg.s.hi, i);
                const float sl = __shfl_sync(0xffffffffu, vg.s.lo, i);
                const ff sg = {__shfl_sync(0xffffffffu, vg.sg.hi, i), __shfl_sync(0xffffffffu, vg.sg.lo, i)};
                const float Wg = __shfl_sync(0xffffffffu, vg.Wg, i);
                const float Asx = __shfl_sync(0xffffffffu, Asv.x, i);
                const float Asy = __shfl_sync(0xffffffffu, Asv.y, i);
                const SigmaGeom sgm = sigma_geom(sh, sl, sg, ff{en[4 * E], en[6 * E]});
#pragma unroll 1
                for (int el = lane; el < E; el += 32) term(i, el, Ad, sh, sl, Wg, Asx, Asy, sgm);
            }
        }
    }
    __syncthreads();
    for (int el = tid; el < E; el += kFwdThreads) {
        double s = 0.0;
        for (int w = 0; w < kFwdWarps; w++) s += (double)TNs[w * E + el].x - (double)TNs[w * E + el].y;
        TN[el] = s;
    }
    __syncthreads();
    const int lo_e = P.e_lo;
    for (int n = tid; n < P.nrg_det; n += kFwdThreads) {
        double acc = 0.0;
        for (int j = 0; j < W; j++) acc += (double)rf[n * W + j] * TN[winlo[n] + j - lo_e];
        const int64_t ray = pidx + (int64_t)n * npairs;
        if (MLEM) ratio[n] = (double)J.ymeas[ray] / (acc + (double)J.cbg[ray] + 1e-20);   // main.m:162
        else J.y[ray] = (float)acc;
    }
    if (MLEM) {
        __syncthreads();
        // what[pair, e] = sum over the detector bins whose window holds e
        for (int el = tid; el < E; el += kFwdThreads) {
            const int e = lo_e + el;
            double s = 0.0;
            for (int n = wn[2 * el]; n <= wn[2 * el + 1]; n++) {
                const int j = e - winlo[n];
                if (j >= 0 && j < W) s += (double)rf[n * W + j] * ratio[n];
            }
            J.what[pidx * E + el] = (float)s;
        }
    }
}

// Persistent forward over the pairs of every job (offsets off[0 .. n]).
template <bool MLEM>
__global__ void __launch_bounds__(kFwdThreads, 3)
k_vox_fwd(const VoxBatch B)
{
    extern __shared__ __align__(16) unsigned char sm[];
    __shared__ PairRec pair;
    __shared__ VoxJob job;
    __shared__ long long item_s;
    const int64_t *off = B.off + 0 * (B.n + 1);
    const int64_t total = off[B.n];
    int cur = -1;
    for (;;) {
        __syncthreads();   // the previous item is done with shared memory
        if (threadIdx.x == 0) item_s = (long long)atomicAdd(B.counters + 0, 1ull);
        __syncthreads();
        const int64_t item = item_s;
        if (item >= total) break;
        const int p = find_job(off, B.n, item);
        if (p != cur) {
            load_job(B.jobs, p, &job);
            cur = p;
            __syncthreads();
        }
        vox_fwd_pair<MLEM>(job, job.pair0 + (item - off[p]), sm, pair);
    }
}

// Adjoint tile (voxel-chunk block bx, pair group by) of job J.  Shared
// memory: energy rows and coarse bins, then per warp E rows of (coefficient,
// wvt pair, exponent scale), 32 x K compensated sums and the current pair's
// record.
__global__ void __launch_bounds__(128)
k_vox_adj(const VoxBatch B)
{
    extern __shared__ __align__(16) unsigned char sm[];
    __shared__ VoxJob J;
    __shared__ long long item_s;
    const int nwarps = blockDim.x >> 5;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int64_t *off = B.off + 1 * (B.n + 1);
    const int64_t total = off[B.n];
    int cur = -1;
    for (;;) {
        __syncthreads();
        if (tid == 0) item_s = (long long)atomicAdd(B.counters + 1, 1ull);
        __syncthreads();
        const int64_t item = item_s;
        if (item >= total) break;
        const int p = find_job(off, B.n, item);
        if (p != cur) {
            load_job(B.jobs, p, &J);
            cur = p;
            __syncthreads();
        }
        const DevProblem &P = J.op.P;
        const F32Consts &c = J.c;
        const int E = J.E, K = P.nwt;
        float *en = (float *)sm;                                            // [6][E]
        float4 *cq = (float4 *)(sm + al16(sizeof(float) * kEnRows * E));    // [K]
        float4 *rows = cq + K;                                              // [warps][E]
        float2 *gacc = (float2 *)(rows + (size_t)nwarps * E);               // [warps][32][K]
        PairRec *prs = (PairRec *)(gacc + (size_t)nwarps * 32 * K);         // [warps]
        float *rows_lo = (float *)(prs + nwarps);                           // [warps][E]
        int2 *wins = (int2 *)(sm + al16((size_t)((unsigned char *)(rows_lo + (size_t)nwarps * E) - sm)));
                                                                            // [warps][E]
        unsigned char *eranges = (unsigned char *)(wins + (size_t)nwarps * E);   // [warps][2][K]
        float4 *rw = rows + (size_t)wid * E;
        float *rwl = rows_lo + (size_t)wid * E;
        int2 *ww = wins + (size_t)wid * E;
        unsigned char *e_first = eranges + (size_t)wid * 2 * K, *e_end = e_first + K;
        float2 *gw = gacc + (size_t)wid * 32 * K;
        PairRec &pr = prs[wid];
        stage_energy_rows(J, en, tid, blockDim.x);
        for (int i = tid; i < K; i += blockDim.x) cq[i] = J.op.coarse_q[i];
        for (int i = lane; i < 32 * K; i += 32) gw[i] = make_float2(0.f, 0.f);
        __syncthreads();

        const int64_t r = item - off[p];
        const int bx = (int)(r % J.chunk_blocks), by = (int)(r / J.chunk_blocks);
        const int nv = J.op.nv;
        const int chunk = bx * nwarps + wid;
        if (chunk * 32 >= nv) continue;   // an idle warp; the next item starts with a barrier
        const int64_t p0 = J.pair0 + (int64_t)by * J.ppg;
        const int64_t p1 = min(J.pair1, p0 + J.ppg);
        const float rsqrt2pi = c.rsqrt2pi;
        const float q_lo = c.q_lo, q_hi = c.q_hi;
        const int nin = min(32, nv - chunk * 32);
        const int v = chunk * 32 + min(lane, nin - 1);
        const int xy = J.op.vox_xy[v];
        const float vx = ((float)(xy & 0xffff) + 0.5f) * c.vox;
        const float vy = ((float)(xy >> 16) + 0.5f) * c.vox;

        for (int64_t pp = p0; pp < p1; pp++) {
            __syncwarp();   // the previous pair's constants are no longer read
            for (int i = lane; i < (int)(sizeof(PairRec) / 4); i += 32)
                reinterpret_cast<int *>(&pr)[i] = reinterpret_cast<const int *>(J.op.pairs + pp)[i];
            __syncwarp();
            const int src = (int)(pp % P.n_src);
            const VoxGeom vg = vox_geom<true>(pr.G, vx, vy);
            const float2 Asv = J.op.atten_src[(int64_t)src * nv + v];
            const float2 Adv = J.op.walk[(pp - J.pair0) * nv + v];
            const float *wp = J.what + pp * E;
            for (int i = 0; i < nin; i++) {
                const float2 Ad = make_float2(__shfl_sync(0xffffffffu, Adv.x, i), __shfl_sync(0xffffffffu, Adv.y, i));
                const float sh = __shfl_sync(0xffffffffu, vg.s.hi, i);
                const float sl = __shfl_sync(0xffffffffu, vg.s.lo, i);
                const ff sg = {__shfl_sync(0xffffffffu, vg.sg.hi, i), __shfl_sync(0xffffffffu, vg.sg.lo, i)};
                const float Wg = __shfl_sync(0xffffffffu, vg.Wg, i);
                const float Asx = __shfl_sync(0xffffffffu, Asv.x, i);
                const float Asy = __shfl_sync(0xffffffffu, Asv.y, i);
                const SigmaGeom sgm = sigma_geom(sh, sl, sg, ff{en[4 * E], en[6 * E]});
                // lane = energy: the energy's factors and its coarse-bin
                // window (the bins within 13.25 sigma: every term FP32 can
                // represent), with the running maximum of the windows' upper
                // ends in ww[e].x
                int run_max = -1;
                for (int eb = 0; eb < E; eb += 32) {
                    const int el = eb + lane;
                    int klo = K, khi = -1;
                    if (el < E) {
                        const EnergyTerm t =
                            energy_term(en, E, el, Ad.x, Ad.y, Asx, Asy, sh, sl, sgm, Wg, rsqrt2pi);
                        const float cf = __ldg(wp + el) * t.pref;
                        const float half = t.half * (kSigAdj / kSig);
                        // a window entirely outside the coarse grid contributes nothing
                        if (cf != 0.f && !(t.w_hi + half < q_lo || t.w_hi - half > q_hi))
                            coarse_window(t.w_hi, half, q_lo, c.qpar_a, c.qpar_b, K, &klo, &khi);
                        rw[el] = make_float4(cf, t.w_hi, t.w_lo, t.c_hi);
                        rwl[el] = t.c_lo;
                        ww[el].y = klo;
                    }
                    int m = khi;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const int n = __shfl_up_sync(0xffffffffu, m, o);
                        if (lane >= o) m = max(m, n);
                    }
                    m = max(m, run_max);
                    if (el < E) ww[el].x = m;
                    run_max = __shfl_sync(0xffffffffu, m, 31);
                }
                __syncwarp();
                // running minimum of the windows' lower ends from the top
                // energy down, in ww[e].y
                int run_min = K;
                for (int eb = ((E - 1) >> 5) << 5; eb >= 0; eb -= 32) {
                    const int el = eb + lane;
                    int m = el < E ? ww[el].y : K;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const int n = __shfl_down_sync(0xffffffffu, m, o);
                        if (lane + o < 32) m = min(m, n);
                    }
                    m = min(m, run_min);
                    if (el < E) ww[el].y = m;
                    run_min = __shfl_sync(0xffffffffu, m, 0);
                }
                __syncwarp();
                // The energies whose window holds bin k lie in [e0(k), e1(k)):
                // below e0 every window ends before k (the running maximum of
                // the upper ends is below k), from e1 on every window starts
                // after it (the running minimum of the lower ends is above
                // k).  Both bounds are monotone in k, so energy e is e0 for the
                // bins (M[e-1], M[e]] and e1 for [m[e-1], m[e]); lane = energy
                // writes those entries for the bins in [kmin, kmax].
                const int kmin = run_min, kmax = run_max;
                for (int eb = 0; eb < E && kmin <= kmax; eb += 32) {
                    const int el = eb + lane;
                    if (el < E) {
                        const int2 cur = ww[el];
                        const int2 prv = el > 0 ? ww[el - 1] : make_int2(-1, kmin);
                        for (int k = max(prv.x + 1, kmin); k <= min(cur.x, kmax); k++) e_first[k] = (unsigned char)el;
                        if (el > 0)
                            for (int k = max(prv.y, kmin); k <= min(cur.y - 1, kmax); k++) e_end[k] = (unsigned char)el;
                        if (el == E - 1)
                            for (int k = max(cur.y, kmin); k <= kmax; k++) e_end[k] = (unsigned char)E;
                    }
                }
                __syncwarp();
                // lane = coarse bin k over the bins some window reaches
                float2 *gi = gw + i * K;
                for (int kb = kmin; kb <= kmax; kb += 32) {
                    const int k = kb + lane;
                    if (k > kmax) break;
                    const int e0 = e_first[k], e1 = e_end[k];
                    const float4 q = cq[k];
                    float acc = 0.f;
                    for (int e = e0; e < e1; e++) {
                        const float4 rr = rw[e];
                        acc = fmaf(rr.x, gauss_f32(rr.y, rr.z, q.x, q.y, rr.w, rwl[e]), acc);
                    }
                    float2 sacc = gi[k];
                    kahan_add(sacc.x, sacc.y, acc * q.z);
                    gi[k] = sacc;
                }
                __syncwarp();
            }
        }
        // The partial rows keep the compensated sums as pairs (sum, minus
        // the compensation): rounded to one float, each row would carry the
        // same relative error into every MLEM iteration, where the update
        // multiplies it in again and again.  A job that is one tile of a
        // problem adds to the rows the earlier tiles left (tiles run in a
        // fixed order on one stream), with a two-sum.
        float2 *out = J.part + ((int64_t)by * nv + (int64_t)chunk * 32) * K;
        if (J.accumulate)
            for (int i = lane; i < nin * K; i += 32) {
                const float2 o = out[i];
                const float s = o.x + gw[i].x;
                const float bb = s - o.x;
                const float err = (o.x - (s - bb)) + (gw[i].x - bb);
                out[i] = make_float2(s, o.y + (err - gw[i].y));
            }
        else
            for (int i = lane; i < nin * K; i += 32) out[i] = make_float2(gw[i].x, -gw[i].y);
    }
}

// what[p, e] = sum_nrg RF[e, nrg] w[p + nrg * npairs].  mode 0: the weights
// w; mode 1: every w = 1, the sum rounded to float; mode 2: every w = 1, the
// part of the sum that rounding to float dropped.  The sensitivity is the
// adjoint of mode 1 plus that of mode 2: with one float per energy shared by
// every pair, its rounding would be the same relative error in every term of
// an energy, which no sum over pairs averages out, and MLEM multiplies each
// unknown by (1 + that error) again in every iteration.
__global__ void k_vox_wtab(const VoxBatch B, int mode)
{
    const int64_t *off = B.off + 4 * (B.n + 1);
    const int64_t total = off[B.n];
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int pj = find_job(off, B.n, t);
        const VoxJob &J = B.jobs[pj];
        const DevProblem &P = J.op.P;
        const int W = 2 * P.dnrg + 1, E = J.E;
        const int64_t npairs = (int64_t)P.n_src * P.n_det;
        const int64_t loc = t - off[pj];
        const int64_t p = loc / E;
        const int el = (int)(loc - p * E), e = P.e_lo + el;
        double s = 0.0;
        for (int n = J.op.win_n[2 * e]; n <= J.op.win_n[2 * e + 1]; n++) {
            const int j = e - J.op.win_lo[n];
            if (j < 0 || j >= W) continue;
            const double wv = mode ? 1.0 : (double)J.w[p + (int64_t)n * npairs];
            s += (double)J.op.rf_win[n * W + j] * wv;
        }
        J.what[loc] = mode == 2 ? (float)(s - (double)(float)s) : (float)s;
    }
}

// Sum of the adjoint's partial rows in FP64 and what follows from it:
//   mode 0: sens = sum (the sensitivity, Av^T 1)
//   mode 4: sens += sum (its second part, k_vox_wtab)
//   mode 1: the MLEM update x <- x * sum / (sens + 1e-7), non-finite -> 0,
//           negative -> 0 (main.m:162-176), and xd = x dq
//   mode 2: g[voxel] = sum in the full-grid layout (nx + ny*NX)*nwt + k
//   mode 3: g = sum in the compact voxel order [nv][nwt]
__global__ void k_vox_reduce(const VoxBatch B, int mode)
{
    const int64_t *off = B.off + 2 * (B.n + 1);
    const int64_t total = off[B.n];
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int pj = find_job(off, B.n, t);
        const VoxJob &J = B.jobs[pj];
        const int K = J.op.P.nwt;
        const int64_t loc = t - off[pj];
        const int64_t n = (int64_t)J.op.nv * K;
        double s = 0.0;
        for (int gi = 0; gi < J.groups; gi++) {
            const float2 pv = J.part[(int64_t)gi * n + loc];
            s += (double)pv.x + (double)pv.y;
        }
        if (mode == 0) {
            J.sens[loc] = s;
        } else if (mode == 4) {
            J.sens[loc] += s;
        } else if (mode == 1) {
            float v = (float)((double)J.xc[loc] * s / (J.sens[loc] + 1e-7));
            if (!isfinite(v)) v = 0.f;
            if (v < 0.f) v = 0.f;
            J.xc[loc] = v;
            J.xd[loc] = v * J.op.coarse_q[loc % K].z;
        } else if (mode == 2) {
            const int64_t vi = loc / K;
            const int xy = J.op.vox_xy[vi];
            J.g[((int64_t)(xy & 0xffff) + (int64_t)(xy >> 16) * J.op.P.nx) * K + (loc - vi * K)] = (float)s;
        } else {
            J.g[loc] = (float)s;   // compact voxel order [nv][NWT]
        }
    }
}

// Full grid -> compact voxel order: xd = x dq (and xc = x when with_xc).
__global__ void k_vox_gather(const VoxBatch B, int with_xc)
{
    const int64_t *off = B.off + 2 * (B.n + 1);
    const int64_t total = off[B.n];
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int pj = find_job(off, B.n, t);
        const VoxJob &J = B.jobs[pj];
        const int K = J.op.P.nwt;
        const int64_t loc = t - off[pj];
        const int64_t vi = loc / K;
        const int k = (int)(loc - vi * K);
        const int xy = J.op.vox_xy[vi];
        const float v = J.xfull[((int64_t)(xy & 0xffff) + (int64_t)(xy >> 16) * J.op.P.nx) * K + k];
        if (with_xc) J.xc[loc] = v;
        J.xd[loc] = v * J.op.coarse_q[k].z;
    }
}

// Compact -> full grid (the other voxels are left as they are).
__global__ void k_vox_scatter(const VoxBatch B)
{
    const int64_t *off = B.off + 2 * (B.n + 1);
    const int64_t total = off[B.n];
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int pj = find_job(off, B.n, t);
        const VoxJob &J = B.jobs[pj];
        const int K = J.op.P.nwt;
        const int64_t loc = t - off[pj];
        const int64_t vi = loc / K;
        const int xy = J.op.vox_xy[vi];
        J.xout[((int64_t)(xy & 0xffff) + (int64_t)(xy >> 16) * J.op.P.nx) * K + (loc - vi * K)] = J.xc[loc];
    }
}

// Pair table: the (source, pixel) constants of every pair, once per operator.
__global__ void k_pair_table(DevProblem P, const SrcGeom *__restrict__ sg, PairRec *__restrict__ out)
{
    const int64_t npairs = (int64_t)P.n_src * P.n_det;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < npairs;
         p += (int64_t)gridDim.x * blockDim.x) {
        const int src = (int)(p % P.n_src), det = (int)(p / P.n_src);
        PairRec r;
        pair_geom(P, sg[src], det, &r.G, &r.Rdx, &r.Rdy);
        out[p] = r;
    }
}

// a grid-stride loop over n items: at most 32 blocks per SM
int grid_for(int64_t n, int threads)
{
    int64_t b = (n + threads - 1) / threads;
    const int64_t cap = 32LL * current_sm_count();
    if (b > cap) b = cap;
    return (int)(b < 1 ? 1 : b);
}

template <class F>
cudaError_t allow_dynamic_smem(F *kernel, int max_smem)
{
    // the limit covers static and dynamic shared memory together
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, kernel);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem - (int)fa.sharedSizeBytes);
}

template <class F>
size_t static_smem(F *kernel)
{
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, kernel) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return fa.sharedSizeBytes;
}

} // namespace

size_t pair_rec_bytes() { return sizeof(PairRec); }

cudaError_t launch_pair_table(const DevProblem &P, const SrcGeom *sg, PairRec *out, cudaStream_t s,
                              int64_t *launches)
{
    const int64_t n = (int64_t)P.n_src * P.n_det;
    k_pair_table<<<grid_for(n, 128), 128, 0, s>>>(P, sg, out);
    if (launches) (*launches)++;
    return cudaGetLastError();
}

cudaError_t vox_set_attributes(int max_smem)
{
    // the launches stay free of attribute calls, so they can be captured
    cudaError_t e = allow_dynamic_smem(k_vox_fwd<true>, max_smem);
    if (e == cudaSuccess) e = allow_dynamic_smem(k_vox_fwd<false>, max_smem);
    if (e == cudaSuccess) e = allow_dynamic_smem(k_vox_adj, max_smem);
    return e;
}

size_t vox_fwd_static_smem() { return static_smem(k_vox_fwd<true>); }
size_t vox_adj_static_smem() { return static_smem(k_vox_adj); }

size_t vox_fwd_smem(const DevProblem &P) { return vox_fwd_layout(P, P.e_hi - P.e_lo + 1).total; }

size_t vox_adj_smem(const DevProblem &P, int warps)
{
    const int E = P.e_hi - P.e_lo + 1, K = P.nwt;
    return al16(sizeof(float) * kEnRows * E) + sizeof(float4) * K + sizeof(float4) * (size_t)warps * E +
           sizeof(float2) * (size_t)warps * 32 * K + sizeof(PairRec) * warps + sizeof(float) * (size_t)warps * E +
           16 + sizeof(int2) * (size_t)warps * E + (size_t)warps * 2 * K;
}

int vox_fwd_blocks_per_sm(size_t smem)
{
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_vox_fwd<true>, kFwdThreads, smem) != cudaSuccess) {
        cudaGetLastError();
        n = 1;
    }
    return n < 1 ? 1 : n;
}

int vox_adj_blocks_per_sm(int warps, size_t smem)
{
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_vox_adj, 32 * warps, smem) != cudaSuccess) {
        cudaGetLastError();
        n = 1;
    }
    return n < 1 ? 1 : n;
}

cudaError_t launch_vox_forward(const VoxBatch &B, bool mlem, int grid, size_t smem, cudaStream_t s,
                               int64_t *launches)
{
    cudaError_t e = cudaMemsetAsync(B.counters + 0, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    if (mlem) k_vox_fwd<true><<<grid, kFwdThreads, smem, s>>>(B);
    else k_vox_fwd<false><<<grid, kFwdThreads, smem, s>>>(B);
    if (launches) (*launches)++;
    return cudaGetLastError();
}

cudaError_t launch_vox_adjoint(const VoxBatch &B, int grid, size_t smem, cudaStream_t s, int64_t *launches)
{
    cudaError_t e = cudaMemsetAsync(B.counters + 1, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    k_vox_adj<<<grid, 32 * B.adj_warps, smem, s>>>(B);
    if (launches) (*launches)++;
    return cudaGetLastError();
}

cudaError_t launch_vox_wtab(const VoxBatch &B, int64_t total, int mode, cudaStream_t s, int64_t *launches)
{
    k_vox_wtab<<<grid_for(total, 256), 256, 0, s>>>(B, mode);
    if (launches) (*launches)++;
    return cudaGetLastError();
}

cudaError_t launch_vox_reduce(const VoxBatch &B, int64_t total, int mode, cudaStream_t s, int64_t *launches)
{
    k_vox_reduce<<<grid_for(total, 256), 256, 0, s>>>(B, mode);
    if (launches) (*launches)++;
    return cudaGetLastError();
}

cudaError_t launch_vox_gather(const VoxBatch &B, int64_t total, bool with_xc, cudaStream_t s, int64_t *launches)
{
    k_vox_gather<<<grid_for(total, 256), 256, 0, s>>>(B, with_xc ? 1 : 0);
    if (launches) (*launches)++;
    return cudaGetLastError();
}

cudaError_t launch_vox_scatter(const VoxBatch &B, int64_t total, cudaStream_t s, int64_t *launches)
{
    k_vox_scatter<<<grid_for(total, 256), 256, 0, s>>>(B);
    if (launches) (*launches)++;
    return cudaGetLastError();
}

} // namespace xrdt
