// k_ct.cu -- transmission CT sinogram: polychromatic source-to-detector
// transmission through the attenuation map, and the same without the
// phantom (gain0).
//
// The reference declares these outputs (Tphotons and gain0, one value per
// source, detector pixel and energy channel) and the two launches that would
// fill them -- integrate_src2det over (SRC, COL) and polychromatic_src2det --
// only as comments (Forward_XRD.cu:125-140,169-199,263-276); no kernel body
// ships.  The definition used here, restated in the oracle:
//
//   chord: the segment source -> pixel clipped to the region of interest
//          [0,NX] x [0,NY] (slab clipping, FP64); samples at
//          r_in + k DQ u for k DQ <= chord length, bilinear in the (a1, a2)
//          map exactly as the line integrals of attenuator.cu:9-109;
//          (A1, A2) = DQ * sum of the samples
//   Tphotons[src, det, nrg] = sum_{e in window(nrg)} RF[e, nrg] exp(-(A1/ein^3 + A2/KN(ein)))
//   gain0[src, det, nrg]    = sum_{e in window(nrg)} RF[e, nrg]
//
// with the energy window and spectrum weights of find_src_nrg_range.cu and
// the attenuation model of integrate_diffraction.cu:291-296.  Outputs use the
// Nphotons layout, index src + det*SRC + nrg*SRC*DET.  One warp per
// (source, pixel): the chord is walked cooperatively, then lane = energy
// channel forms the two sums.
#include "scatter.cuh"

namespace xrdt {

namespace {

// Slab clipping of (sx,sy) -> (dx,dy) against [0,NX] x [0,NY].  Returns the
// walk of the clipped chord (n = 0 when the segment misses the region).
__device__ void chord_setup(const DevProblem &P, double sx, double sy, double dx, double dy, WalkSetup *w)
{
    const double ex = dsub(dx, sx), ey = dsub(dy, sy);
    double t0 = 0.0, t1 = 1.0;
    const double lo[2] = {0.0, 0.0}, hi[2] = {(double)P.nx, (double)P.ny};
    const double o[2] = {sx, sy}, d[2] = {ex, ey};
    for (int a = 0; a < 2; a++) {
        if (d[a] == 0.0) {
            if (o[a] < lo[a] || o[a] > hi[a]) t1 = -1.0;
            continue;
        }
        double ta = dsub(lo[a], o[a]) / d[a], tb = dsub(hi[a], o[a]) / d[a];
        if (ta > tb) {
            const double t = ta;
            ta = tb;
            tb = t;
        }
        if (ta > t0) t0 = ta;
        if (tb < t1) t1 = tb;
    }
    w->n = 0;
    w->rx = w->ry = w->Lx = w->Ly = 0.f;
    if (!(t1 > t0)) return;
    const double len = sqrt(dadd(dmul(ex, ex), dmul(ey, ey)));
    const double rx = dadd(sx, dmul(t0, ex)), ry = dadd(sy, dmul(t0, ey));
    const double L = dmul(dsub(t1, t0), len);
    long long k = (long long)floor(L / P.DQ);
    while (dmul(P.DQ, (double)(k + 1)) <= L) k++;
    while (k >= 0 && !(dmul(P.DQ, (double)k) <= L)) k--;
    long long n = k + 1;
    if (n > P.kmax) n = P.kmax;
    w->rx = (float)(rx - 1.0);
    w->ry = (float)(ry - 1.0);
    w->Lx = (float)(ex / len * P.DQ);
    w->Ly = (float)(ey / len * P.DQ);
    w->n = (int)n;
}

__global__ void __launch_bounds__(256)
k_ct_sinogram(DevProblem P, const SrcGeom *__restrict__ sg, const float4 *__restrict__ cells,
              const EnergyRow *__restrict__ energy, const float *__restrict__ rf_win, const int *__restrict__ win_lo,
              float *__restrict__ T, float *__restrict__ G0)
{
    const int lane = threadIdx.x & 31;
    const int64_t npairs = (int64_t)P.n_src * P.n_det;
    const int W = 2 * P.dnrg + 1;
    const int64_t wstride = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t p = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); p < npairs; p += wstride) {
        const int src = (int)(p % P.n_src), det = (int)(p / P.n_src);
        const SrcGeom g = sg[src];
        double Rdx, Rdy, Rdz;
        det_position(P, g.sphi, g.cphi, det, &Rdx, &Rdy, &Rdz);
        WalkSetup ws;
        chord_setup(P, g.Rsrc_x, g.Rsrc_y, Rdx, Rdy, &ws);
        const float2 A = walk_coop(cells, P.nx, P.ny, ws, (float)P.DQ, lane);
        for (int n = lane; n < P.nrg_det; n += 32) {
            const int lo = win_lo[n];
            float t = 0.f, g0 = 0.f;
            for (int j = 0; j < W; j++) {
                const EnergyRow r = energy[lo + j];
                const float rf = rf_win[n * W + j];
                t = fmaf(rf, expf(-fmaf(A.x, r.inv_f1, A.y * r.inv_f2)), t);
                g0 += rf;
            }
            const int64_t ray = p + (int64_t)n * npairs;
            T[ray] = t;
            G0[ray] = g0;
        }
    }
}

} // namespace

cudaError_t launch_ct_sinogram(const DevProblem &P, const SrcGeom *sg, const float4 *cells, const EnergyRow *energy,
                               const float *rf_win, const int *win_lo, float *T, float *G0, cudaStream_t s,
                               int64_t *launches)
{
    const int64_t npairs = (int64_t)P.n_src * P.n_det;
    int64_t blocks = (npairs + 7) / 8;
    if (blocks > 64LL * current_sm_count()) blocks = 64LL * current_sm_count();
    k_ct_sinogram<<<(int)blocks, 256, 0, s>>>(P, sg, cells, energy, rf_win, win_lo, T, G0);
    if (launches) (*launches)++;
    return cudaGetLastError();
}

} // namespace xrdt
