// k_decisions.cu -- the integer decisions of the fast forward path, exported
// for bit-exact comparison with the FP64 oracle.
//
// The projector's float outputs hide a one-bin flip of an integer decision
// under their tolerance, so the decisions themselves are compared: for each
// listed ray and each non-empty voxel (in the reference's loop order) this
// kernel makes them with the very device functions the production kernels
// call, on the same inputs:
//
//  * the detector-side walk set-up of k_det_walk (k_walk.cu): FP32 with
//    guard bands, FP64 near a threshold -> ROI edge and sample count
//    (GetIntersection.cu:9-57, attenuator.cu:44-52);
//  * the source-side walk set-up of k_src_atten (k_prep.cu), in FP64;
//  * the Compton table bin nq of k_fwd (k_fwd.cu) for every source energy of
//    the ray's window (integrate_diffraction.cu:331-337).
//
// The window bounds (find_src_nrg_range.cu:8-25), the per-voxel Compton
// column na (integrate_diffraction.cu:177-189) and the u8 table
// (integrate_diffraction.cu:66-74) come out of the production buffers as
// they are (api.cu).  Test infrastructure: nothing on the product path calls
// this kernel.
#include "scatter.cuh"

namespace xrdt {

namespace {

// Block = one ray; threads stride over the voxels.  walk[v] = (det n, det
// edge, src n, src edge); nq[v][j] for source bin lo + j, j < W.
__global__ void k_decisions(DevProblem P, F32Consts c, const SrcGeom *__restrict__ sg,
                            const EnergyRow *__restrict__ energy, const int *__restrict__ win_lo,
                            const int64_t *__restrict__ rays, const int *__restrict__ vox_xy, int nv,
                            int4 *__restrict__ walk, int *__restrict__ nq_out)
{
    const int64_t ray = rays[blockIdx.x];
    const int64_t npairs = (int64_t)P.n_src * P.n_det;
    const int src = (int)(ray % P.n_src);
    const int det = (int)((ray % npairs) / P.n_src);
    const int nrg = (int)(ray / npairs);
    const int W = 2 * P.dnrg + 1;
    const int lo = win_lo[nrg];
    const SrcGeom gs = sg[src];
    double ex, ey, ez;
    det_position(P, gs.sphi, gs.cphi, det, &ex, &ey, &ez);
    const float exf = (float)ex, eyf = (float)ey;
    PairGeom G;
    double Rdx, Rdy;
    pair_geom(P, gs, det, &G, &Rdx, &Rdy);
    const float qmin_t = c.qmin_t, inv_dqt = c.inv_dqt;
    for (int v = threadIdx.x; v < nv; v += blockDim.x) {
        const int xy = vox_xy[v];
        // detector side, as k_det_walk sets it up
        const float vx = ((float)(xy & 0xffff) + 0.5f) * c.vox;
        const float vy = ((float)(xy >> 16) + 0.5f) * c.vox;
        WalkSetup wd;
        wd.n = 0;
        wd.edge = -1;
        if (!walk_setup_f32(P, c, exf, eyf, vx, vy, &wd)) walk_setup_f64(P, ex, ey, (double)vx, (double)vy, &wd);
        // source side, as k_src_atten sets it up
        const double vxd = ((double)(xy & 0xffff) + 0.5) * P.vox;
        const double vyd = ((double)(xy >> 16) + 0.5) * P.vox;
        WalkSetup wsrc;
        walk_setup(P, gs.Rsrc_x, gs.Rsrc_y, vxd, vyd, &wsrc);
        walk[(int64_t)blockIdx.x * nv + v] = make_int4(wd.n, wd.edge, wsrc.n, wsrc.edge);
        // Compton bins, as k_fwd forms them
        const VoxGeom vg = vox_geom<false>(G, vx, vy);
        int *out = nq_out + ((int64_t)blockIdx.x * nv + v) * W;
        for (int j = 0; j < W; j++) {
            const EnergyRow r = energy[lo + j];
            const float ein = r.einf;
            const float eratio = __fadd_rn(1.f, __fmul_rn(ein, vg.omc.hi));   // as k_fwd forms it
            const float inv_er = rcp_approx(eratio);
            out[j] = compton_bin(P, ein, eratio, inv_er, vg.s.hi, vg.omc.hi, vg.omc.lo, r.ein, qmin_t, inv_dqt);
        }
    }
}

} // namespace

cudaError_t launch_decisions(const DevProblem &P, const SrcGeom *sg, const EnergyRow *energy, const int *win_lo,
                             const int64_t *rays, int n_rays, const int *vox_xy, int nv, int4 *walk, int *nq,
                             cudaStream_t s, int64_t *launches)
{
    if (n_rays <= 0 || nv <= 0) return cudaSuccess;
    k_decisions<<<n_rays, 128, 0, s>>>(P, make_f32_consts(P), sg, energy, win_lo, rays, vox_xy, nv, walk, nq);
    if (launches) (*launches)++;
    return cudaGetLastError();
}

} // namespace xrdt
