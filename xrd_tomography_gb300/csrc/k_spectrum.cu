// k_spectrum.cu -- the spectrum-response matrix of spectrum_builder.m:64-95
// on the GPU: the input spectrum[NS, ND] of the forward projector from a fine
// (e.g. 0.05 keV) source spectrum.
//
//   Ndet[s, d] = sum_h sum_g ws[h, s] wd[g, d] n[h] exp(-(E_h - E_g)^2 / (2 sigma_h^2))
//                / (sqrt(2 pi) sigma_h)
//
// with ws, wd the overlap lengths of fine bin h (g) with coarse source bin s
// (detector bin d) (:87-88).  The reference evaluates every (s, d) as a sum
// over the full fine x fine grid masked by those overlaps, O(NS ND H^2);
// a fine bin overlaps at most two coarse bins, so here one block per (s, d)
// sums only the fine bins of its two ranges: about (H + NS)(H + ND) terms in
// all, some 2 M for the 1440-bin spectrum of the reference, whatever NS and ND.
//
// FP64 throughout: the energies are about 80 keV and the bins 0.05 keV wide,
// so single-precision centres would move the Gaussian exponent by about 1e-5
// relative; the whole build is a fraction of a millisecond at the FP64 rate.
#include "xrdt_device.cuh"

namespace xrdt {

namespace {

constexpr int kSpecThreads = 128;

__global__ void __launch_bounds__(kSpecThreads)
k_spectrum(const SpecFineBin *__restrict__ fb, const SpecCoarseBin *__restrict__ sb,
           const SpecCoarseBin *__restrict__ db, int ns, float *__restrict__ out)
{
    __shared__ double part[kSpecThreads / 32];
    const int s = blockIdx.x, d = blockIdx.y;
    const SpecCoarseBin S = sb[s], D = db[d];
    const int nh = S.h1 - S.h0, ng = D.h1 - D.h0;
    const long long total = (long long)max(nh, 0) * max(ng, 0);
    double acc = 0.0;
    for (long long t = threadIdx.x; t < total; t += kSpecThreads) {
        const int h = S.h0 + (int)(t / ng), g = D.h0 + (int)(t % ng);
        const SpecFineBin a = fb[h], b = fb[g];
        const double ws = fmax(0.0, fmin(S.e2, a.right) - fmax(S.e1, a.left));   // :87
        const double wd = fmax(0.0, fmin(D.e2, b.right) - fmax(D.e1, b.left));   // :88
        const double dE = a.centre - b.centre;
        acc += ws * wd * a.amp * exp(-dE * dE * a.inv_2s2);                      // :75, :91
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double sum = 0.0;
        for (int w = 0; w < kSpecThreads / 32; w++) sum += part[w];
        out[s + (long long)d * ns] = (float)sum;
    }
}

} // namespace

cudaError_t launch_spectrum(const SpecFineBin *fb, const SpecCoarseBin *sb, int ns, const SpecCoarseBin *db, int nd,
                            float *out, cudaStream_t s, int64_t *launches)
{
    if (ns <= 0 || nd <= 0) return cudaSuccess;
    k_spectrum<<<dim3((unsigned)ns, (unsigned)nd), kSpecThreads, 0, s>>>(fb, sb, db, ns, out);
    if (launches) (*launches)++;
    return cudaGetLastError();
}

} // namespace xrdt
