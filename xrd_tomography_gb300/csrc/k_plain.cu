// k_plain.cu -- the plain FP64 forward projector at the reference's launch shape.
//
// One block per ray (src, det, nrg) and NWT threads, one per coarse q bin,
// exactly as Forward_XRD.cu:244-259 launches integrate_diffraction.  Every
// quantity is FP64; the texture fetch is an exact software bilinear of the
// float maps.  This is the denominator path of the throughput comparison
// and an independent GPU cross-check of the fast kernels; it keeps the
// reference's redundancy (each block walks every voxel and recomputes both
// line integrals).  Unlike attenuator.cu:93-101 the shared partial sums are
// protected by a second barrier, so the block has no data race.
#include "xrdt_device.cuh"

namespace xrdt {

namespace {

// Block-wide sum of two doubles; every thread receives the result.
__device__ inline void block_sum2(double &a, double &b, double *red, int nwarps)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    a = warp_sum(a);
    b = warp_sum(b);
    if (lane == 0) {
        red[2 * wid] = a;
        red[2 * wid + 1] = b;
    }
    __syncthreads();
    double sa = 0.0, sb = 0.0;
    for (int w = 0; w < nwarps; w++) {
        sa += red[2 * w];
        sb += red[2 * w + 1];
    }
    __syncthreads();  // partials are reused by the next call
    a = sa;
    b = sb;
}

// attenuator.cu:9-109: cooperative line integral from endpoint e to voxel v.
__device__ inline void attenuate(const DevProblem &P, const float *a1, const float *a2,
                                 double ex, double ey, double vx, double vy, double *red,
                                 int nwarps, double *A1, double *A2)
{
    double rx, ry;
    get_intersection(ex, ey, vx, vy, P.nx, P.ny, &rx, &ry);
    double Lx = vx - rx, Ly = vy - ry;
    const double L2 = dadd(dmul(Lx, Lx), dmul(Ly, Ly));
    const double Lr = sqrt(L2);
    const double rL = 1.0 / sqrt(L2);
    Lx *= rL;
    Ly *= rL;
    double s1 = 0.0, s2 = 0.0;
    for (long long k = threadIdx.x; k < P.kmax; k += blockDim.x) {
        const double qr = dmul(P.DQ, (double)k);
        if (!(qr <= Lr)) break;
        double v1, v2;
        bilinear_f64(a1, a2, P.nx, P.ny, rx + Lx * qr, ry + Ly * qr, &v1, &v2);
        s1 += v1;
        s2 += v2;
    }
    block_sum2(s1, s2, red, nwarps);
    *A1 = s1 * P.DQ;
    *A2 = s2 * P.DQ;
}

__global__ void __launch_bounds__(1024)
k_plain_forward(DevProblem P, int same_grid, const SrcGeom *__restrict__ sg,
                const float *__restrict__ spectrum, const float *__restrict__ Ifine,
                const int32_t *__restrict__ seg, const float *__restrict__ a1,
                const float *__restrict__ a2, const float *__restrict__ S2,
                const double *__restrict__ coarse_q, const int64_t *__restrict__ rays,
                float *__restrict__ Nout, float *__restrict__ Cout, float *__restrict__ Aout)
{
    extern __shared__ double smem[];
    const int NWT = P.nwt, MAT = P.n_mat;
    const int nwarps = (int)(blockDim.x >> 5);
    double *Amodel = smem;                                  // [MAT][NWT]
    double *red = Amodel + (size_t)MAT * NWT;               // [2*nwarps]
    double *spec = red + 2 * nwarps;                        // [2*dnrg+1]
    unsigned char *S2u8 = (unsigned char *)(spec + 2 * P.dnrg + 1);  // [nq*na]

    // the block's ray: the reference grid (src, det, nrg), or entry
    // blockIdx.x of a ray list, whose outputs then go to position blockIdx.x
    int src, det, nrg;
    int64_t out;
    if (rays) {
        const int64_t r = rays[blockIdx.x];
        src = (int)(r % P.n_src);
        det = (int)((r / P.n_src) % P.n_det);
        nrg = (int)(r / ((int64_t)P.n_src * P.n_det));
        out = blockIdx.x;
    } else {
        src = blockIdx.x;
        det = blockIdx.y;
        nrg = blockIdx.z;
        out = (int64_t)src + (int64_t)det * P.n_src + (int64_t)nrg * P.n_src * P.n_det;
    }
    const int nwt = threadIdx.x;

    const double qnow = coarse_q[2 * nwt], dqnow = coarse_q[2 * nwt + 1];
    int lo, hi;
    src_nrg_range(P, same_grid, nrg, &lo, &hi);
    for (int i = nwt; i <= 2 * P.dnrg; i += blockDim.x)
        spec[i] = (double)spectrum[(lo + i) + (int64_t)nrg * P.nrg_src];
    for (int i = nwt; i < P.nq * P.na; i += blockDim.x) {
        int v = floor_to_int((double)S2[i]);
        S2u8[i] = (unsigned char)(v < 0 ? 0 : (v > 255 ? 255 : v));
    }
    for (int m = 0; m < MAT; m++) Amodel[m * NWT + nwt] = 0.0;
    __syncthreads();

    // Scanner geometry, integrate_diffraction.cu:81-128.
    const SrcGeom g = sg[src];
    double Rdet_x, Rdet_y, Rdet_z;
    det_position(P, g.sphi, g.cphi, det, &Rdet_x, &Rdet_y, &Rdet_z);
    const double ndet_x = g.sphi, ndet_y = -g.cphi;
    const double nsrc_x = -g.sphi * P.sta, nsrc_y = g.cphi * P.sta, nsrc_z = -P.cta;
    const double nsrc_xy = sqrt(nsrc_x * nsrc_x + nsrc_y * nsrc_y);
    const double Edet1 = P.e_det_min + (double)nrg * P.dEd;
    const double Edet2 = P.e_det_min + (double)(nrg + 1) * P.dEd;

    double Nnow = 0.0, Cnow = 0.0;
    double Rvox_x = 0.0, Rvox_y = 0.0;
    for (int nx = 0; nx < P.nx; nx++) {
        for (int ny = 0; ny < P.ny; ny++) {
            const int matID = seg[nx + (int64_t)ny * P.nx] - 1;
            if (matID < 0) continue;
            const double cur_x = ((double)nx + 0.5) * P.vox;
            const double cur_y = ((double)ny + 0.5) * P.vox;
            double a1now, a2now;
            if (P.quirk_stale) bilinear_f64(a1, a2, P.nx, P.ny, Rvox_x, Rvox_y, &a1now, &a2now);
            else bilinear_f64(a1, a2, P.nx, P.ny, cur_x, cur_y, &a1now, &a2now);
            int na = floor_to_int((log2(fabs(a1now / a2now)) - P.a_min) / P.da_tab);
            na = na < 0 ? 0 : (na >= P.na ? P.na - 1 : na);
            Rvox_x = cur_x;
            Rvox_y = cur_y;

            const double ax = Rvox_x - g.Rsrc_x, ay = Rvox_y - g.Rsrc_y;
            const double proj = ax * nsrc_x + ay * nsrc_y;
            const double Rvox_z = -proj / nsrc_xy * P.tan_half;
            const double Hvox = proj / nsrc_xy * P.tan_full;
            const double az = Rvox_z;
            const double bx = Rdet_x - Rvox_x, by = Rdet_y - Rvox_y, bz = Rdet_z - Rvox_z;
            const double ab = ax * bx + ay * by + az * bz;
            const double anorm2 = ax * ax + ay * ay + az * az;
            const double bnorm2 = bx * bx + by * by + bz * bz;
            const double costheta = ab * (1.0 / sqrt(anorm2)) * (1.0 / sqrt(bnorm2));
            const double sth = sqrt(fabs(1.0 - costheta) / 2.0);
            const double Sx = bx - ab * ax / anorm2, Sy = by - ab * ay / anorm2, Sz = bz - ab * az / anorm2;
            const double Dx = -ax + ab * bx / bnorm2, Dy = -ay + ab * by / bnorm2, Dz = -az + ab * bz / bnorm2;
            const double Vx = -(Sx + Dx), Vy = -(Sy + Dy), Vz = -(Sz + Dz);
            const double Dndet = Dx * ndet_x + Dy * ndet_y;
            const double Snsrc = Sx * nsrc_x + Sy * nsrc_y + Sz * nsrc_z;
            const double dD2 = (Dx * Dx + Dy * Dy + Dz * Dz - Dndet * Dndet) * P.geomAdet / 12.0;
            const double vV2 = (P.vox * P.vox * (Vx * Vx + Vy * Vy) + Hvox * Hvox * Vz * Vz) / 12.0;
            const double sS2 = (Sx * Sx + Sy * Sy + Sz * Sz - Snsrc * Snsrc) * P.focal * P.focal / 12.0;
            const double Rdotn = -g.sphi * ax + g.cphi * ay;
            const double cospsi = Rdotn * (1.0 / sqrt(ax * ax + ay * ay));
            const double gsv = cospsi * (1.0 / sqrt(anorm2)) * P.tan_full;
            const double gvd = -(ndet_x * bx + ndet_y * by) * (1.0 / sqrt(bnorm2 * bnorm2 * bnorm2));
            const double Rayleigh = (1.0 + costheta * costheta) / 2.0;
            const double gp = gsv * gvd;

            double Ad_x, Ad_y, As_x, As_y;  // :259-260, labels kept as written
            attenuate(P, a1, a2, Rdet_x, Rdet_y, Rvox_x, Rvox_y, red, nwarps, &Ad_x, &Ad_y);
            attenuate(P, a1, a2, g.Rsrc_x, g.Rsrc_y, Rvox_x, Rvox_y, red, nwarps, &As_x, &As_y);

            const float *Im = Ifine + (int64_t)matID * P.nqf;
            for (int e = lo; e <= hi; e++) {
                const double Esrc1 = P.e_src_min + (double)e * P.dEs;
                const double Esrc2 = P.e_src_min + (double)(e + 1) * P.dEs;
                const double Esrc = 0.5 * (Esrc1 + Esrc2);
                const double ein = Esrc / P.mec2;
                const double RF = spec[e - lo];
                const double wvt = 2.0 * Esrc / P.hbarc * sth;
                const double s2 = (2.0 * sth / P.hbarc) * (2.0 * sth / P.hbarc) * P.dEs * P.dEs / 12.0 +
                                  (Esrc / P.hbarc) * (Esrc / P.hbarc) * (sS2 + vV2 + dD2) /
                                      (2.0 * sth) / (2.0 * sth) / anorm2 / bnorm2;
                double f1 = ein * ein * ein;
                double f2 = P.kn0 + P.kn1 * ein + P.kn2 * ein * ein;
                const double Pin = exp(-(Ad_x / f1 + Ad_y / f2));
                const double Pout = exp(-(As_x / f1 + As_y / f2));
                for (int qf = nwt; qf < P.nqf; qf += blockDim.x) {
                    const double qax = P.q_lo + P.dq_fine * (0.5 + (double)qf);
                    const double Rq = RF * exp(-(wvt - qax) * (wvt - qax) / (2.0 * s2)) * P.rsqrt2pi /
                                      sqrt(s2) * P.dq_fine;
                    Nnow += Pin * Pout * gp * Rq * (double)__ldg(Im + qf) * Rayleigh;
                }
                {
                    const double Rq = RF * exp(-(wvt - qnow) * (wvt - qnow) / (2.0 * s2)) * P.rsqrt2pi /
                                      sqrt(s2) * dqnow;
                    Amodel[matID * NWT + nwt] += Pin * Pout * gp * Rq * Rayleigh;
                }
                const double eratio = 1.0 + ein * (1.0 - costheta);
                const double eout = ein / eratio;
                const double Eout1 = Esrc1 / eratio, Eout2 = Esrc2 / eratio;
                const double cm = fmax(0.0, fmin(Eout2, Edet2) - fmax(Eout1, Edet1)) / (Eout2 - Eout1);
                const double w = ein * sth;
                const double l2 = log2(w * sqrt(eratio + w * w) / eratio);
                int nq = floor_to_int((l2 - P.q_min) / P.dq_tab);
                nq = nq < 0 ? 0 : (nq >= P.nq ? P.nq - 1 : nq);
                f1 = eout * eout * eout;
                f2 = P.kn0 + P.kn1 * eout + P.kn2 * eout * eout;
                const double Pc = exp(-(As_x / f1 + As_y / f2));
                const double Cf = eratio * eratio * (eratio + 1.0 / eratio - 1.0 + costheta * costheta) / 2.0;
                Cnow += cm * Pin * Pc * RF * gp * Cf * a2now * (double)S2u8[nq + na * P.nq];
            }
        }
    }

    if (Aout) {
        const int64_t base = out * (int64_t)NWT * MAT;
        for (int m = 0; m < MAT; m++) Aout[base + (int64_t)m * NWT + nwt] = (float)Amodel[m * NWT + nwt];
    }
    double dummy = 0.0;
    block_sum2(Nnow, dummy, red, nwarps);
    if (nwt == 0) {
        Nout[out] = (float)Nnow;
        Cout[out] = (float)Cnow;
    }
}

// The per-voxel model of one ray at the same launch shape, in FP64: thread
// k = coarse bin, every voxel and both line integrals recomputed per block.
// Forward (x != NULL): y[out] = sum_{v,k} Av[ray,v,k] x[v,k].  Adjoint
// (w != NULL): g[v,k] += w[out] Av[ray,v,k], added in FP64 with atomics into
// the full-grid layout (nx + ny*NX)*NWT + k.
__global__ void __launch_bounds__(1024)
k_plain_vox(DevProblem P, int same_grid, const SrcGeom *__restrict__ sg, const float *__restrict__ spectrum,
            const int32_t *__restrict__ seg, const float *__restrict__ a1, const float *__restrict__ a2,
            const double *__restrict__ coarse_q, const int64_t *__restrict__ rays, const float *__restrict__ x,
            float *__restrict__ y, const float *__restrict__ w, double *__restrict__ g)
{
    extern __shared__ double smem[];
    const int NWT = P.nwt;
    const int nwarps = (int)(blockDim.x >> 5);
    double *red = smem;                       // [2*nwarps]
    double *spec = red + 2 * nwarps;          // [2*dnrg+1]
    const int64_t r = rays[blockIdx.x];
    const int src = (int)(r % P.n_src);
    const int det = (int)((r / P.n_src) % P.n_det);
    const int nrg = (int)(r / ((int64_t)P.n_src * P.n_det));
    const int k = threadIdx.x;
    const double qnow = coarse_q[2 * k], dqnow = coarse_q[2 * k + 1];
    int lo, hi;
    src_nrg_range(P, same_grid, nrg, &lo, &hi);
    for (int i = k; i <= 2 * P.dnrg; i += blockDim.x) spec[i] = (double)spectrum[(lo + i) + (int64_t)nrg * P.nrg_src];
    __syncthreads();
    const double wr = w ? (double)w[blockIdx.x] : 0.0;

    const SrcGeom gs = sg[src];
    double Rdet_x, Rdet_y, Rdet_z;
    det_position(P, gs.sphi, gs.cphi, det, &Rdet_x, &Rdet_y, &Rdet_z);
    const double ndet_x = gs.sphi, ndet_y = -gs.cphi;
    const double nsrc_x = -gs.sphi * P.sta, nsrc_y = gs.cphi * P.sta, nsrc_z = -P.cta;
    const double nsrc_xy = sqrt(nsrc_x * nsrc_x + nsrc_y * nsrc_y);
    double acc = 0.0;
    for (int nx = 0; nx < P.nx; nx++) {
        for (int ny = 0; ny < P.ny; ny++) {
            if (seg[nx + (int64_t)ny * P.nx] <= 0) continue;
            const double Rvox_x = ((double)nx + 0.5) * P.vox, Rvox_y = ((double)ny + 0.5) * P.vox;
            const double ax = Rvox_x - gs.Rsrc_x, ay = Rvox_y - gs.Rsrc_y;
            const double proj = ax * nsrc_x + ay * nsrc_y;
            const double az = -proj / nsrc_xy * P.tan_half;
            const double Hvox = proj / nsrc_xy * P.tan_full;
            const double bx = Rdet_x - Rvox_x, by = Rdet_y - Rvox_y, bz = Rdet_z - az;
            const double ab = ax * bx + ay * by + az * bz;
            const double anorm2 = ax * ax + ay * ay + az * az;
            const double bnorm2 = bx * bx + by * by + bz * bz;
            const double costheta = ab * (1.0 / sqrt(anorm2)) * (1.0 / sqrt(bnorm2));
            const double sth = sqrt(fabs(1.0 - costheta) / 2.0);
            const double Sx = bx - ab * ax / anorm2, Sy = by - ab * ay / anorm2, Sz = bz - ab * az / anorm2;
            const double Dx = -ax + ab * bx / bnorm2, Dy = -ay + ab * by / bnorm2, Dz = -az + ab * bz / bnorm2;
            const double Vx = -(Sx + Dx), Vy = -(Sy + Dy), Vz = -(Sz + Dz);
            const double Dndet = Dx * ndet_x + Dy * ndet_y;
            const double Snsrc = Sx * nsrc_x + Sy * nsrc_y + Sz * nsrc_z;
            const double dD2 = (Dx * Dx + Dy * Dy + Dz * Dz - Dndet * Dndet) * P.geomAdet / 12.0;
            const double vV2 = (P.vox * P.vox * (Vx * Vx + Vy * Vy) + Hvox * Hvox * Vz * Vz) / 12.0;
            const double sS2 = (Sx * Sx + Sy * Sy + Sz * Sz - Snsrc * Snsrc) * P.focal * P.focal / 12.0;
            const double Rdotn = -gs.sphi * ax + gs.cphi * ay;
            const double cospsi = Rdotn * (1.0 / sqrt(ax * ax + ay * ay));
            const double gsv = cospsi * (1.0 / sqrt(anorm2)) * P.tan_full;
            const double gvd = -(ndet_x * bx + ndet_y * by) * (1.0 / sqrt(bnorm2 * bnorm2 * bnorm2));
            const double Wg = gsv * gvd * (1.0 + costheta * costheta) / 2.0;
            double Ad_x, Ad_y, As_x, As_y;  // integrate_diffraction.cu:259-260, labels as written
            attenuate(P, a1, a2, Rdet_x, Rdet_y, Rvox_x, Rvox_y, red, nwarps, &Ad_x, &Ad_y);
            attenuate(P, a1, a2, gs.Rsrc_x, gs.Rsrc_y, Rvox_x, Rvox_y, red, nwarps, &As_x, &As_y);
            double t = 0.0;   // sum over the window of this bin's term
            for (int e = lo; e <= hi; e++) {
                const double Esrc1 = P.e_src_min + (double)e * P.dEs, Esrc2 = P.e_src_min + (double)(e + 1) * P.dEs;
                const double Esrc = 0.5 * (Esrc1 + Esrc2);
                const double ein = Esrc / P.mec2;
                const double wvt = 2.0 * Esrc / P.hbarc * sth;
                const double s2 = (2.0 * sth / P.hbarc) * (2.0 * sth / P.hbarc) * P.dEs * P.dEs / 12.0 +
                                  (Esrc / P.hbarc) * (Esrc / P.hbarc) * (sS2 + vV2 + dD2) /
                                      (2.0 * sth) / (2.0 * sth) / anorm2 / bnorm2;
                const double f1 = ein * ein * ein, f2 = P.kn0 + P.kn1 * ein + P.kn2 * ein * ein;
                const double PP = exp(-(Ad_x / f1 + Ad_y / f2)) * exp(-(As_x / f1 + As_y / f2));
                t += spec[e - lo] * PP * exp(-(wvt - qnow) * (wvt - qnow) / (2.0 * s2)) * P.rsqrt2pi / sqrt(s2) * dqnow;
            }
            const int64_t idx = ((int64_t)nx + (int64_t)ny * P.nx) * NWT + k;
            if (x) acc += Wg * t * (double)x[idx];
            if (g) atomicAdd(g + idx, wr * Wg * t);
        }
    }
    if (y) {
        double dummy = 0.0;
        block_sum2(acc, dummy, red, nwarps);
        if (k == 0) y[blockIdx.x] = (float)acc;
    }
}

} // namespace

cudaError_t launch_plain_forward(const DevProblem &P, const SrcGeom *d_src,
                                 const float *spectrum, const float *Ifine, const int32_t *seg,
                                 const float *a1, const float *a2, const float *S2,
                                 const double *d_coarse_q, const int64_t *d_rays, int64_t n_rays,
                                 float *N, float *C, float *A, cudaStream_t s, int64_t *launches)
{
    const int same_grid = (P.nrg_src == P.nrg_det && P.e_src_min == P.e_det_min && P.dEs == P.dEd);
    const int nwarps = P.nwt / 32;
    const size_t smem = sizeof(double) * ((size_t)P.n_mat * P.nwt + 2 * nwarps + 2 * P.dnrg + 1) +
                        (size_t)P.nq * P.na;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_plain_forward, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
    }
    dim3 grid(P.n_src, P.n_det, P.nrg_det);
    if (d_rays) grid = dim3((unsigned)n_rays, 1, 1);
    if (grid.x == 0) return cudaSuccess;
    k_plain_forward<<<grid, P.nwt, smem, s>>>(P, same_grid, d_src, spectrum, Ifine, seg, a1, a2, S2,
                                              d_coarse_q, d_rays, N, C, A);
    if (launches) (*launches)++;
    return cudaGetLastError();
}

cudaError_t launch_plain_vox(const DevProblem &P, const SrcGeom *d_src, const float *spectrum, const int32_t *seg,
                             const float *a1, const float *a2, const double *d_coarse_q, const int64_t *d_rays,
                             int64_t n_rays, const float *x, float *y, const float *w, double *g, cudaStream_t s,
                             int64_t *launches)
{
    if (n_rays == 0) return cudaSuccess;
    const int same_grid = (P.nrg_src == P.nrg_det && P.e_src_min == P.e_det_min && P.dEs == P.dEd);
    const int nwarps = P.nwt / 32;
    const size_t smem = sizeof(double) * (2 * (size_t)nwarps + 2 * P.dnrg + 1);
    k_plain_vox<<<(unsigned)n_rays, P.nwt, smem, s>>>(P, same_grid, d_src, spectrum, seg, a1, a2, d_coarse_q, d_rays,
                                                     x, y, w, g);
    if (launches) (*launches)++;
    return cudaGetLastError();
}

} // namespace xrdt

