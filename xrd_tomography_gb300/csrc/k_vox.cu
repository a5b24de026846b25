// k_vox.cu -- the model with per-voxel coefficients: forward, adjoint and
// the MLEM update, matrix-free.
//
// The reference's model matrix has one unknown per (coarse q bin, material):
// Amatrix[k, m, ray] = sum over the voxels of material m of the coarse-q
// term of integrate_diffraction.cu:311-315,
//
//   Av[ray, v, k] = sum_{e in window(nrg)} RF[e,nrg] Pin Pout geom Rayleigh
//                   * G(wvt(v,e) - q_k; sigma(v,e)) * dq_k .
//
// With one unknown per (voxel, coarse bin), x[v, k], the forward model is
// y = Av x and its adjoint g = Av^T w.  Both are computed on the fly: the
// detector-side attenuation of every (pair, voxel) is walked again in each
// call, the source-side one comes from the per-(source, voxel) table.
//
//  * forward (k_vox_fwd): one block per (source, pixel) as in k_fwd.cu; lane =
//    source energy sums the coarse bins within 7.5 sigma of the wavevector
//    transfer, weighted by x[v, k] dq_k, into compensated per-energy sums; the
//    banded spectrum weights give the detector bins.  In MLEM mode the block
//    goes on to form the ratios y / (Av x + c + 1e-20) of main.m:162 for its
//    detector bins and folds them back through the same spectrum band into
//    per-energy weights  what[pair, e] = sum_nrg RF[e,nrg] ratio[nrg].
//  * adjoint (k_vox_adj): voxel-major, so that g stays on chip.  A warp owns
//    32 voxels and loops over a range of pairs; per (pair, voxel) lane =
//    energy forms what[pair,e] * (the energy's prefactor), then lane = coarse
//    bin k adds sum_e of those times G(wvt_e - q_k) to the voxel's compensated
//    sum.  Ranges of pairs run in parallel blocks and are added in FP64 by
//    k_vox_reduce, which also applies the MLEM update (main.m:163-176).
#include "scatter.cuh"

namespace xrdt {

namespace {

constexpr int kFwdThreads = 256;
constexpr int kFwdWarps = kFwdThreads / 32;

struct VoxArgs {
    DevProblem P;
    const PairRec *pairs;     // [n_src * n_det], index src + det * n_src
    const EnergyRow *energy;  // [nrg_src]
    const float *rf_win;      // [nrg_det][2*dnrg+1]
    const int *win_lo;        // [nrg_det]
    const int *win_n;         // [nrg_src][2]
    const float4 *coarse_q;   // [nwt] (q_hi, q_lo, dq, 0)
    const int *vox_xy;
    const float4 *cells;
    const float2 *atten_src;  // [n_src][nv]
    int nv, E;
    F32Consts c;
};

// Per-(voxel, energy) factors shared by the forward and the adjoint:
// the prefactor RF-less term pref = Pin Pout geom Rayleigh / (sigma sqrt(2 pi)),
// the wavevector transfer as a pair, the Gaussian exponent scale (log2 units)
// and the window half-width.
struct EnergyTerm {
    float pref, w_hi, w_lo, cexp, half;
};

__device__ __forceinline__ EnergyTerm energy_term(const float *en, int E, int el, float Adx, float Ady, float Asx,
                                                  float Asy, float sh, float sl, float s2f, float sg_s2, float Wg,
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
    const float sig2 = fmaf(en[4 * E + el], s2f, en[5 * E + el] * sg_s2);
    const float rs = rsqrtf(sig2);
    t.cexp = -0.5f * kLog2e * rs * rs;
    const float PP = ex2_approx(-(Xin + Xout) * kLog2e);
    t.pref = PP * Wg * rsqrt2pi * rs;
    t.half = kSig * sig2 * rs;
    t.w_hi = w_hi;
    t.w_lo = w_lo;
    return t;
}

// Energy rows in shared memory: 1/f1, 1/f2, wfac_hi, wfac_lo, sig_c1, sig_c2.
__device__ __forceinline__ void stage_energy_rows(const VoxArgs &a, float *en, int tid, int nthreads)
{
    for (int i = tid; i < a.E; i += nthreads) {
        const EnergyRow r = a.energy[a.P.e_lo + i];
        en[i] = r.inv_f1;
        en[a.E + i] = r.inv_f2;
        en[2 * a.E + i] = r.wfac_hi;
        en[3 * a.E + i] = r.wfac_lo;
        en[4 * a.E + i] = r.sig_c1;
        en[5 * a.E + i] = r.sig_c2;
    }
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
    L.en = o; o = al16(o + sizeof(float) * 6 * E);
    L.rf = o; o = al16(o + sizeof(float) * P.nrg_det * W);
    L.winlo = o; o = al16(o + sizeof(int) * P.nrg_det);
    L.wn = o; o = al16(o + sizeof(int) * 2 * E);
    L.cq = o; o = al16(o + sizeof(float4) * P.nwt);
    L.ratio = o; o = al16(o + sizeof(float) * P.nrg_det);
    L.total = o;
    return L;
}

// y = Av x (MLEM = false), or the per-energy weights of the MLEM ratios
// (MLEM = true).  xd = x * dq_k in the compact voxel order, [nv][nwt].
template <bool MLEM>
__global__ void __launch_bounds__(kFwdThreads, 3)
k_vox_fwd(const VoxArgs a, const float *__restrict__ xd, float *__restrict__ y, const float *__restrict__ ymeas,
          const float *__restrict__ cbg, float *__restrict__ what)
{
    extern __shared__ __align__(16) unsigned char sm[];
    __shared__ PairRec pair;
    const DevProblem &P = a.P;
    const F32Consts &c = a.c;
    const int E = a.E, K = P.nwt, W = 2 * P.dnrg + 1;
    const FwdLayout L = vox_fwd_layout(P, E);
    double *TN = (double *)(sm + L.tn);
    float2 *TNs = (float2 *)(sm + L.tns);
    float *en = (float *)(sm + L.en);
    float *rf = (float *)(sm + L.rf);
    int *winlo = (int *)(sm + L.winlo);
    int *wn = (int *)(sm + L.wn);
    float4 *cq = (float4 *)(sm + L.cq);
    float *ratio = (float *)(sm + L.ratio);

    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int det = blockIdx.x, src = blockIdx.y;
    const int64_t npairs = (int64_t)P.n_src * P.n_det;
    const int64_t pidx = (int64_t)src + (int64_t)det * P.n_src;

    stage_energy_rows(a, en, tid, kFwdThreads);
    for (int i = tid; i < kFwdWarps * E; i += kFwdThreads) TNs[i] = make_float2(0.f, 0.f);
    for (int i = tid; i < 2 * E; i += kFwdThreads) wn[i] = a.win_n[2 * P.e_lo + i];
    for (int i = tid; i < P.nrg_det * W; i += kFwdThreads) rf[i] = a.rf_win[i];
    for (int i = tid; i < P.nrg_det; i += kFwdThreads) winlo[i] = a.win_lo[i];
    for (int i = tid; i < K; i += kFwdThreads) cq[i] = a.coarse_q[i];

    if (tid < (int)(sizeof(PairRec) / 4))
        reinterpret_cast<int *>(&pair)[tid] = reinterpret_cast<const int *>(a.pairs + pidx)[tid];
    const PairRec &pr = pair;
    const float rsqrt2pi = c.rsqrt2pi;
    const float DQf = c.DQ;
    const float qlo_f = c.q_lo;
    __syncthreads();

    float2 *TNw = TNs + wid * E;
    const int nv = a.nv;
    const int nchunks = (nv + 31) >> 5;
    for (int chunk = wid; chunk < nchunks; chunk += kFwdWarps) {
        const int v = min(chunk * 32 + lane, nv - 1);
        const int xy = a.vox_xy[v];
        const float vx = ((float)(xy & 0xffff) + 0.5f) * c.vox;
        const float vy = ((float)(xy >> 16) + 0.5f) * c.vox;
        const VoxGeom vg = vox_geom(pr.G, vx, vy);
        const float2 Asv = a.atten_src[(int64_t)src * nv + v];
        WalkSetup ws;
        if (!walk_setup_f32(P, c, pr.G.Rdx.hi, pr.G.Rdy.hi, vx, vy, &ws))
            walk_setup_f64(P, pr.Rdx, pr.Rdy, (double)vx, (double)vy, &ws);

        const int nin = min(32, nv - chunk * 32);
        for (int i = 0; i < nin; i++) {
            WalkSetup wi;
            wi.rx = __shfl_sync(0xffffffffu, ws.rx, i);
            wi.ry = __shfl_sync(0xffffffffu, ws.ry, i);
            wi.Lx = __shfl_sync(0xffffffffu, ws.Lx, i);
            wi.Ly = __shfl_sync(0xffffffffu, ws.Ly, i);
            wi.n = __shfl_sync(0xffffffffu, ws.n, i);
            // the detector-side integral feeds Pin (integrate_diffraction.cu:259-260)
            const float2 Ad = walk_coop(a.cells, P.nx, P.ny, wi, DQf, lane);
            const float sh = __shfl_sync(0xffffffffu, vg.s.hi, i);
            const float sl = __shfl_sync(0xffffffffu, vg.s.lo, i);
            const float sg = __shfl_sync(0xffffffffu, vg.sg, i);
            const float Wg = __shfl_sync(0xffffffffu, vg.Wg, i);
            const float Asx = __shfl_sync(0xffffffffu, Asv.x, i);
            const float Asy = __shfl_sync(0xffffffffu, Asv.y, i);
            const float s2f = sh * sh;
            const float sg_s2 = __fdividef(sg, s2f);
            const float *xrow = xd + (int64_t)(chunk * 32 + i) * K;
#pragma unroll 1
            for (int el = lane; el < E; el += 32) {
                const EnergyTerm t = energy_term(en, E, el, Ad.x, Ad.y, Asx, Asy, sh, sl, s2f, sg_s2, Wg, rsqrt2pi);
                if (t.pref == 0.f) continue;   // attenuation underflow: no contribution
                int klo, khi;
                coarse_window(t.w_hi, t.half, qlo_f, c.qpar_a, c.qpar_b, K, &klo, &khi);
                float acc = 0.f;
                for (int k = klo; k <= khi; k++) {
                    const float4 c = cq[k];
                    const float d = (t.w_hi - c.x) + (t.w_lo - c.y);
                    acc = fmaf(ex2_approx(t.cexp * d * d), __ldg(xrow + k), acc);
                }
                float2 s = TNw[el];
                kahan_add(s.x, s.y, t.pref * acc);
                TNw[el] = s;
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
        if (MLEM) ratio[n] = (float)((double)ymeas[ray] / (acc + (double)cbg[ray] + 1e-20));   // main.m:162
        else y[ray] = (float)acc;
    }
    if (MLEM) {
        __syncthreads();
        // what[pair, e] = sum over the detector bins whose window holds e
        for (int el = tid; el < E; el += kFwdThreads) {
            const int e = lo_e + el;
            double s = 0.0;
            for (int n = wn[2 * el]; n <= wn[2 * el + 1]; n++) {
                const int j = e - winlo[n];
                if (j >= 0 && j < W) s += (double)rf[n * W + j] * (double)ratio[n];
            }
            what[pidx * E + el] = (float)s;
        }
    }
}

// Adjoint: part[group][v][k] = sum over the group's pairs p of
// sum_e what[p, e] pref(p,v,e) G(wvt - q_k) dq_k.
__global__ void __launch_bounds__(128)
k_vox_adj(const VoxArgs a, const float *__restrict__ what, int pairs_per_group, float *__restrict__ part)
{
    extern __shared__ __align__(16) unsigned char sm[];
    const DevProblem &P = a.P;
    const F32Consts &c = a.c;
    const int E = a.E, K = P.nwt;
    const int nwarps = blockDim.x >> 5;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    float *en = (float *)sm;                                            // [6][E]
    float4 *cq = (float4 *)(sm + al16(sizeof(float) * 6 * E));          // [K]
    float4 *rows = cq + K;                                              // [warps][E]
    float2 *gacc = (float2 *)(rows + (size_t)nwarps * E);               // [warps][32][K]
    PairRec *prs = (PairRec *)(gacc + (size_t)nwarps * 32 * K);         // [warps]
    float4 *rw = rows + (size_t)wid * E;
    float2 *gw = gacc + (size_t)wid * 32 * K;
    PairRec &pr = prs[wid];

    stage_energy_rows(a, en, tid, blockDim.x);
    for (int i = tid; i < K; i += blockDim.x) cq[i] = a.coarse_q[i];
    for (int i = lane; i < 32 * K; i += 32) gw[i] = make_float2(0.f, 0.f);
    __syncthreads();

    const int nv = a.nv;
    const int chunk = blockIdx.x * nwarps + wid;
    if (chunk * 32 >= nv) return;   // no block-wide barrier follows
    const int64_t npairs = (int64_t)P.n_src * P.n_det;
    const int64_t p0 = (int64_t)blockIdx.y * pairs_per_group;
    const int64_t p1 = min(npairs, p0 + pairs_per_group);
    const float rsqrt2pi = c.rsqrt2pi;
    const float DQf = c.DQ;
    const float q_lo = c.q_lo, q_hi = c.q_hi;
    const int nin = min(32, nv - chunk * 32);
    const int v = chunk * 32 + min(lane, nin - 1);
    const int xy = a.vox_xy[v];
    const float vx = ((float)(xy & 0xffff) + 0.5f) * c.vox;
    const float vy = ((float)(xy >> 16) + 0.5f) * c.vox;

    for (int64_t p = p0; p < p1; p++) {
        __syncwarp();   // the previous pair's constants are no longer read
        if (lane < (int)(sizeof(PairRec) / 4))
            reinterpret_cast<int *>(&pr)[lane] = reinterpret_cast<const int *>(a.pairs + p)[lane];
        __syncwarp();
        const int src = (int)(p % P.n_src);
        const VoxGeom vg = vox_geom(pr.G, vx, vy);
        const float2 Asv = a.atten_src[(int64_t)src * nv + v];
        WalkSetup ws;
        if (!walk_setup_f32(P, c, pr.G.Rdx.hi, pr.G.Rdy.hi, vx, vy, &ws))
            walk_setup_f64(P, pr.Rdx, pr.Rdy, (double)vx, (double)vy, &ws);
        const float *wp = what + p * E;
        for (int i = 0; i < nin; i++) {
            WalkSetup wi;
            wi.rx = __shfl_sync(0xffffffffu, ws.rx, i);
            wi.ry = __shfl_sync(0xffffffffu, ws.ry, i);
            wi.Lx = __shfl_sync(0xffffffffu, ws.Lx, i);
            wi.Ly = __shfl_sync(0xffffffffu, ws.Ly, i);
            wi.n = __shfl_sync(0xffffffffu, ws.n, i);
            const float2 Ad = walk_coop(a.cells, P.nx, P.ny, wi, DQf, lane);
            const float sh = __shfl_sync(0xffffffffu, vg.s.hi, i);
            const float sl = __shfl_sync(0xffffffffu, vg.s.lo, i);
            const float sg = __shfl_sync(0xffffffffu, vg.sg, i);
            const float Wg = __shfl_sync(0xffffffffu, vg.Wg, i);
            const float Asx = __shfl_sync(0xffffffffu, Asv.x, i);
            const float Asy = __shfl_sync(0xffffffffu, Asv.y, i);
            const float s2f = sh * sh;
            const float sg_s2 = __fdividef(sg, s2f);
            for (int el = lane; el < E; el += 32) {
                const EnergyTerm t = energy_term(en, E, el, Ad.x, Ad.y, Asx, Asy, sh, sl, s2f, sg_s2, Wg, rsqrt2pi);
                float c = __ldg(wp + el) * t.pref;
                // a window entirely outside the coarse grid contributes nothing
                if (t.w_hi + t.half < q_lo || t.w_hi - t.half > q_hi) c = 0.f;
                rw[el] = make_float4(c, t.w_hi, t.w_lo, t.cexp);
            }
            __syncwarp();
            float2 *gi = gw + i * K;
            for (int k = lane; k < K; k += 32) {
                const float4 q = cq[k];
                float acc = 0.f;
                for (int e = 0; e < E; e++) {
                    const float4 r = rw[e];
                    if (r.x == 0.f) continue;   // uniform across the warp
                    const float d = (r.y - q.x) + (r.z - q.y);
                    acc = fmaf(r.x, ex2_approx(r.w * d * d), acc);
                }
                float2 s = gi[k];
                kahan_add(s.x, s.y, acc * q.z);
                gi[k] = s;
            }
            __syncwarp();
        }
    }
    float *out = part + ((int64_t)blockIdx.y * nv + (int64_t)chunk * 32) * K;
    for (int i = lane; i < nin * K; i += 32) out[i] = gw[i].x - gw[i].y;
}

// what[p, e] = sum_nrg RF[e, nrg] w[p + nrg * npairs] (w == NULL: all ones).
__global__ void k_vox_wtab(DevProblem P, int E, const float *__restrict__ rf_win, const int *__restrict__ win_lo,
                           const int *__restrict__ win_n, const float *__restrict__ w, float *__restrict__ what)
{
    const int W = 2 * P.dnrg + 1;
    const int64_t npairs = (int64_t)P.n_src * P.n_det;
    const int64_t total = npairs * E;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = t / E;
        const int el = (int)(t - p * E), e = P.e_lo + el;
        double s = 0.0;
        for (int n = win_n[2 * e]; n <= win_n[2 * e + 1]; n++) {
            const int j = e - win_lo[n];
            if (j < 0 || j >= W) continue;
            const double wv = w ? (double)w[p + (int64_t)n * npairs] : 1.0;
            s += (double)rf_win[n * W + j] * wv;
        }
        what[t] = (float)s;
    }
}

// Sum of the adjoint's partial rows in FP64 and what follows from it:
//   mode 0: sens = sum (the sensitivity, Av^T 1)
//   mode 1: the MLEM update x <- x * sum / (sens + 1e-7), non-finite -> 0,
//           negative -> 0 (main.m:162-176), and xd = x dq
//   mode 2: g[voxel] = sum in the full-grid layout (nx + ny*NX)*nwt + k
__global__ void k_vox_reduce(const float *__restrict__ part, int groups, int nv, int K, int mode,
                             double *__restrict__ sens, float *__restrict__ xc, float *__restrict__ xd,
                             const float4 *__restrict__ coarse_q, const int *__restrict__ vox_xy, int nx,
                             float *__restrict__ g)
{
    const int64_t total = (int64_t)nv * K;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int gi = 0; gi < groups; gi++) s += (double)part[(int64_t)gi * total + t];
        if (mode == 0) {
            sens[t] = s;
        } else if (mode == 1) {
            float v = (float)((double)xc[t] * s / (sens[t] + 1e-7));
            if (!isfinite(v)) v = 0.f;
            if (v < 0.f) v = 0.f;
            xc[t] = v;
            xd[t] = v * coarse_q[t % K].z;
        } else {
            const int64_t vi = t / K;
            const int xy = vox_xy[vi];
            g[((int64_t)(xy & 0xffff) + (int64_t)(xy >> 16) * nx) * K + (t - vi * K)] = (float)s;
        }
    }
}

// Full grid [ny][nx][K] -> compact voxel order: xc = x, xd = x dq.
__global__ void k_vox_gather(const float *__restrict__ x, const int *__restrict__ vox_xy, int nv, int K, int nx,
                             const float4 *__restrict__ coarse_q, float *__restrict__ xc, float *__restrict__ xd)
{
    const int64_t total = (int64_t)nv * K;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t vi = t / K;
        const int k = (int)(t - vi * K);
        const int xy = vox_xy[vi];
        const float v = x[((int64_t)(xy & 0xffff) + (int64_t)(xy >> 16) * nx) * K + k];
        if (xc) xc[t] = v;
        xd[t] = v * coarse_q[k].z;
    }
}

// Compact -> full grid (the other voxels are left as they are).
__global__ void k_vox_scatter(const float *__restrict__ xc, const int *__restrict__ vox_xy, int nv, int K, int nx,
                              float *__restrict__ x)
{
    const int64_t total = (int64_t)nv * K;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t vi = t / K;
        const int xy = vox_xy[vi];
        x[((int64_t)(xy & 0xffff) + (int64_t)(xy >> 16) * nx) * K + (t - vi * K)] = xc[t];
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

int grid_for(int64_t n, int threads)
{
    int64_t b = (n + threads - 1) / threads;
    if (b > 152 * 32) b = 152 * 32;
    return (int)(b < 1 ? 1 : b);
}

VoxArgs make_args(const VoxOp &op)
{
    VoxArgs a;
    a.P = op.P;
    a.pairs = op.pairs;
    a.energy = op.energy;
    a.rf_win = op.rf_win;
    a.win_lo = op.win_lo;
    a.win_n = op.win_n;
    a.coarse_q = op.coarse_q;
    a.vox_xy = op.vox_xy;
    a.cells = op.cells;
    a.atten_src = op.atten_src;
    a.nv = op.nv;
    a.E = op.P.e_hi - op.P.e_lo + 1;
    a.c = make_f32_consts(op.P);
    return a;
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

template <class F>
cudaError_t allow_dynamic_smem(F *kernel, int max_smem)
{
    // the limit covers static and dynamic shared memory together
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, kernel);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem - (int)fa.sharedSizeBytes);
}

cudaError_t vox_set_attributes(int max_smem)
{
    // the launches stay free of attribute calls, so they can be captured
    cudaError_t e = allow_dynamic_smem(k_vox_fwd<true>, max_smem);
    if (e == cudaSuccess) e = allow_dynamic_smem(k_vox_fwd<false>, max_smem);
    if (e == cudaSuccess) e = allow_dynamic_smem(k_vox_adj, max_smem);
    return e;
}

size_t vox_fwd_static_smem() { return sizeof(PairRec); }

size_t vox_fwd_smem(const DevProblem &P) { return vox_fwd_layout(P, P.e_hi - P.e_lo + 1).total; }

int vox_adj_warps(int K)
{
    // per warp: 32 voxels x K compensated sums, plus the energy rows
    int w = (int)((96 * 1024) / ((size_t)32 * K * sizeof(float2)));
    return w < 1 ? 1 : (w > 4 ? 4 : w);
}

size_t vox_adj_smem(const DevProblem &P, int warps)
{
    const int E = P.e_hi - P.e_lo + 1, K = P.nwt;
    return al16(sizeof(float) * 6 * E) + sizeof(float4) * K + sizeof(float4) * (size_t)warps * E +
           sizeof(float2) * (size_t)warps * 32 * K + sizeof(PairRec) * warps;
}

int vox_adj_groups(const VoxOp &op, int sm_count)
{
    const int chunks = (op.nv + 31) / 32;
    const int64_t npairs = (int64_t)op.P.n_src * op.P.n_det;
    int64_t g = ((int64_t)sm_count * 32 + chunks - 1) / chunks;   // about 32 warps per SM in all
    if (g < 1) g = 1;
    if (g > npairs) g = npairs;
    if (g > 1024) g = 1024;
    return (int)g;
}

cudaError_t launch_vox_forward(const VoxOp &op, const float *xd, float *y, const float *ymeas, const float *cbg,
                               float *what, cudaStream_t s, int64_t *launches)
{
    const VoxArgs a = make_args(op);
    const size_t smem = vox_fwd_smem(op.P);
    dim3 grid(op.P.n_det, op.P.n_src);
    if (what) k_vox_fwd<true><<<grid, kFwdThreads, smem, s>>>(a, xd, nullptr, ymeas, cbg, what);
    else k_vox_fwd<false><<<grid, kFwdThreads, smem, s>>>(a, xd, y, nullptr, nullptr, nullptr);
    if (launches) (*launches)++;
    return cudaGetLastError();
}

cudaError_t launch_vox_wtab(const VoxOp &op, const float *w, float *what, cudaStream_t s, int64_t *launches)
{
    const int E = op.P.e_hi - op.P.e_lo + 1;
    const int64_t n = (int64_t)op.P.n_src * op.P.n_det * E;
    k_vox_wtab<<<grid_for(n, 256), 256, 0, s>>>(op.P, E, op.rf_win, op.win_lo, op.win_n, w, what);
    if (launches) (*launches)++;
    return cudaGetLastError();
}

cudaError_t launch_vox_adjoint(const VoxOp &op, const float *what, float *part, int groups, cudaStream_t s,
                               int64_t *launches)
{
    const VoxArgs a = make_args(op);
    const int warps = vox_adj_warps(op.P.nwt);
    const size_t smem = vox_adj_smem(op.P, warps);
    const int64_t npairs = (int64_t)op.P.n_src * op.P.n_det;
    const int ppg = (int)((npairs + groups - 1) / groups);
    const int chunks = (op.nv + 31) / 32;
    dim3 grid((chunks + warps - 1) / warps, groups);
    k_vox_adj<<<grid, 32 * warps, smem, s>>>(a, what, ppg, part);
    if (launches) (*launches)++;
    return cudaGetLastError();
}

cudaError_t launch_vox_reduce(const VoxOp &op, const float *part, int groups, int mode, double *sens, float *xc,
                              float *xd, float *g, cudaStream_t s, int64_t *launches)
{
    const int64_t n = (int64_t)op.nv * op.P.nwt;
    k_vox_reduce<<<grid_for(n, 256), 256, 0, s>>>(part, groups, op.nv, op.P.nwt, mode, sens, xc, xd, op.coarse_q,
                                                  op.vox_xy, op.P.nx, g);
    if (launches) (*launches)++;
    return cudaGetLastError();
}

cudaError_t launch_vox_gather(const VoxOp &op, const float *x, float *xc, float *xd, cudaStream_t s,
                              int64_t *launches)
{
    const int64_t n = (int64_t)op.nv * op.P.nwt;
    k_vox_gather<<<grid_for(n, 256), 256, 0, s>>>(x, op.vox_xy, op.nv, op.P.nwt, op.P.nx, op.coarse_q, xc, xd);
    if (launches) (*launches)++;
    return cudaGetLastError();
}

cudaError_t launch_vox_scatter(const VoxOp &op, const float *xc, float *x, cudaStream_t s, int64_t *launches)
{
    const int64_t n = (int64_t)op.nv * op.P.nwt;
    k_vox_scatter<<<grid_for(n, 256), 256, 0, s>>>(xc, op.vox_xy, op.nv, op.P.nwt, op.P.nx, x);
    if (launches) (*launches)++;
    return cudaGetLastError();
}

} // namespace xrdt
