// xrdt_internal.h -- definitions shared by the host library and its kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "../../include/xrdt.h"

namespace xrdt {

constexpr int kMaxSrc = 1 << 16;
constexpr int kWarp = 32;

// Problem constants in the form the kernels consume: everything the
// reference derives inside integrate_diffraction (:81-168) that does not
// depend on the voxel is derived once on the host, in double.
struct DevProblem {
    int nx, ny, n_src, n_col, n_row, n_det, nrg_src, nrg_det, dnrg;
    int nwt, nqf, n_mat, nq, na;
    int quirk_stale;
    int e_lo, e_hi;        // source bins used by any detector window
    long long kmax;        // maxBatch * NWT: cap on line-integral samples
    double dEs, dEd, e_src_min, e_det_min;
    double q_lo, q_hi, dq0, dq_fine;
    double hbarc, mec2, kn0, kn1, kn2, rsqrt2pi, DQ;
    double cx, cy, r_src, r_det, col_pitch, row_pitch, z0, focal, geomAdet, vox;
    double tan_half, tan_full, sta, cta;
    double q_min, q_max, a_min, a_max, dq_tab, da_tab;
    double dq_grid, da_grid;   // spacing of the tables' grid points (bilinear lookups)
};

// FP32 copies of the problem constants that the FP32 kernels use inside
// their loops, converted once on the host.  A float kernel argument is read
// from the constant bank by the instruction that uses it; a conversion of a
// double argument that the compiler re-derives inside a loop (instead of
// holding it in a register) runs on the FP64 pipe, which on this GPU issues
// at 1/64 of the FP32 rate.
struct F32Consts {
    float vox, DQ, inv_DQ, nxf, nyf, rsqrt2pi;
    float dqf_hi, dqf_lo, inv_dqf, q_lo, q_hi;
    float kn0, kn1, kn2;
    float edmin, inv_dEd, dEd, dEs, inv_dEs;
    float qmin_t, inv_dqt, inv_dqg;
    float qpar_a, qpar_b;   // coarse bin edges: edge(n) = q_lo + qpar_b n + qpar_a n^2
};
F32Consts make_f32_consts(const DevProblem &P);

// Per-source geometry (integrate_diffraction.cu:93-121), host-computed in double.
struct SrcGeom {
    double sphi, cphi;
    double Rsrc_x, Rsrc_y;
};

// Energy-bin table of the source grid (integrate_diffraction.cu:269-292).
struct EnergyRow {
    double Esrc1, Esrc2, Esrc, ein;
    float inv_f1, inv_f2;       // 1/ein^3, 1/KN(ein)
    float wfac_hi, wfac_lo;     // 2*Esrc/hbarc as a float pair
    float sig_c1, sig_c2;       // sigma^2 = c1*s^2 + c2*sg/s^2
    float einf, Esrc1f, Esrc2f;
    float sig_c1_lo, sig_c2_lo; // low parts of c1, c2 as float pairs
    float inv_f1_lo, inv_f2_lo; // low parts of 1/ein^3, 1/KN(ein)
};

std::string fmt(const char *f, ...);

// Per-call tables of the factored kernels, built on the host in double.
struct HostTables {
    std::vector<EnergyRow> energy;  // [nrg_src]
    std::vector<float> rf_win;      // [nrg_det][2*dnrg+1]
    std::vector<int> win_lo;        // [nrg_det]
    std::vector<int> win_n;         // [nrg_src][2]
    int sl = 1;
    std::vector<float> offs_e;      // [nrg_src][sl]
    std::vector<float2> fine_q;     // [nqf]
    std::vector<float4> coarse_q;   // [nwt]
};
// spectrum: host copy [nrg_src][nrg_det] column-major as passed to Forward_XRD.
void build_host_tables(const xrdt_problem *p, const DevProblem &P, const float *spectrum, HostTables *t);

// ---- host-side builders (api.cu) ----
int build_dev_problem(const xrdt_problem *p, float q_min, float q_max, float a_min,
                      float a_max, DevProblem *d, std::string *err);

// ---- kernels (launchers return cudaError_t of the launch) ----
// k_plain.cu: FP64 at the reference launch shape.
cudaError_t launch_plain_forward(const DevProblem &P, const SrcGeom *d_src,
                                 const float *spectrum, const float *Ifine, const int32_t *seg,
                                 const float *a1, const float *a2, const float *S2,
                                 const double *d_coarse_q, const int64_t *d_rays, int64_t n_rays,
                                 float *N, float *C, float *A, cudaStream_t s, int64_t *launches);

// The per-voxel model at the same launch shape (NWT threads, NWT % 32 == 0):
// y[i] = Av[rays[i]] x (x != NULL) and g += sum_i w[i] Av[rays[i]] (w != NULL,
// g in FP64, full-grid layout).
cudaError_t launch_plain_vox(const DevProblem &P, const SrcGeom *d_src, const float *spectrum, const int32_t *seg,
                             const float *a1, const float *a2, const double *d_coarse_q, const int64_t *d_rays,
                             int64_t n_rays, const float *x, float *y, const float *w, double *g, cudaStream_t s,
                             int64_t *launches);

// k_ct.cu: transmission through the map per (source, pixel, energy channel)
// and the same without the phantom, in the Nphotons layout.
cudaError_t launch_ct_sinogram(const DevProblem &P, const SrcGeom *sg, const float4 *cells, const EnergyRow *energy,
                               const float *rf_win, const int *win_lo, float *T, float *G0, cudaStream_t s,
                               int64_t *launches);

// k_basis.cu: I[M x N] = C[M x K] B[K x N] on tcgen05 (3xTF32); err is set
// when the accumulator wait times out.
size_t basis_smem(int K, int N);
cudaError_t launch_basis_expand(const float *C, long long M, int K, const float *B, int N, float *I, unsigned *err,
                                cudaStream_t s, int64_t *launches);

// k_prep.cu
struct PrepBuffers {
    float4 *cells = nullptr;          // [2][(ny+1)*(nx+1)*2] bilinear cells, row- then column-major
    int *vox_xy = nullptr;            // [nx*ny] packed x | y << 16 of non-empty voxels
    int *vox_mat = nullptr;           // [nx*ny]
    int *vox_na = nullptr;            // [nx*ny] Compton table column per voxel
    float *vox_a2 = nullptr;          // [nx*ny] a2 used by the Compton term
    float *vox_ta = nullptr;          // [nx*ny] the same column as a grid coordinate (bilinear lookups), or NULL
    int *counters = nullptr;          // [0] = number of non-empty voxels, [1] = bad material flag
    float2 *atten_src = nullptr;      // [n_src * nv] source-side line integrals
    unsigned char *s2u8 = nullptr;    // [nq*na]
    unsigned char *s1u8 = nullptr;    // [nq*na] the coherent table of the table path, or NULL
};
// S1 (with B.s1u8): the coherent table, quantised like S2.
cudaError_t launch_prep_map(const DevProblem &P, const float *a1, const float *a2,
                            const float *S2, PrepBuffers &B, cudaStream_t s, int64_t *launches,
                            const float *S1 = nullptr);
cudaError_t launch_prep_voxels(const DevProblem &P, const int32_t *seg, const float *a1,
                               const float *a2, PrepBuffers &B, cudaStream_t s, int64_t *launches);
cudaError_t launch_src_atten(const DevProblem &P, const SrcGeom *d_src, int nv, PrepBuffers &B,
                             cudaStream_t s, int64_t *launches);

// k_fwd.cu: factored FP32 forward over (src, det) pairs.
struct FwdTables {
    const EnergyRow *energy;   // [nrg_src]
    const float *rf_win;       // [nrg_det][2*dnrg+1] spectrum window per detector bin
    const float *offs_e;       // [nrg_src][sl] Esrc1(e) - Edet1(win_n(e) + s)
    int sl;                    // slots per source bin: max over e of the number of
                               // detector bins whose window holds e
    const int *win_lo;         // [nrg_det] first source bin of each window
    const int *win_n;          // [nrg_src][2] detector bins whose window holds e
    const float2 *fine_q;      // [nqf] fine q axis as (hi, lo)
    const float4 *coarse_q;    // [nwt] (q_hi, q_lo, dq, 0)
    unsigned long long *work;  // nullable: counts the exp2 evaluations
};
size_t fast_forward_smem(const DevProblem &P, int sl, int e_pass, bool with_n, bool with_a, int tab = 0);
// n_pairs blocks, block b on pair p0 + b: of the list pairs[0 .. n_list)
// when it is given (outputs then go to the compact layout [nrg_det][n_list],
// and [nrg_det][n_list][n_mat*nwt] for A), else of the linear index
// src + det*SRC of the full layout.  walk holds the blocks' detector-side
// integrals, [n_pairs][nv] (launch_det_walk).
cudaError_t launch_fast_forward(const DevProblem &P, const SrcGeom *d_src, const FwdTables &T,
                                const PrepBuffers &B, int nv, const float *Ifine,
                                const int2 *pairs, long long n_list, long long p0, int n_pairs,
                                const float2 *walk, float *N, float *C, float *A, cudaStream_t s,
                                int64_t *launches, int tab = 0);
// k_spectrum.cu: the spectrum-response matrix (spectrum_builder.m:64-95).
// A fine bin: edges, centre, 1/(2 sigma^2) and n/(sqrt(2 pi) sigma); a coarse
// bin: edges and the range [h0, h1) of fine bins that overlap it.
struct SpecFineBin {
    double left, right, centre, inv_2s2, amp;
};
struct SpecCoarseBin {
    double e1, e2;
    int h0, h1;
};
// out[s + d*ns] for every coarse source bin s < ns and detector bin d < nd.
cudaError_t launch_spectrum(const SpecFineBin *fb, const SpecCoarseBin *sb, int ns, const SpecCoarseBin *db, int nd,
                            float *out, cudaStream_t s, int64_t *launches);

// k_walk.cu: tab[item][v] = detector-side line integral of voxel v for the
// pair pairs[item] (or the linear pair p0 + item), item < n_items.  Linear
// pairs come in whole pixels: p0 and n_items multiples of SRC.
cudaError_t launch_det_walk(const DevProblem &P, const SrcGeom *sg, const int2 *pairs, long long p0,
                            long long n_items, const int *vox_xy, int nv, const float4 *cells, float2 *tab,
                            cudaStream_t s, int64_t *launches);
// k_bop.cu: rows of R values per non-empty voxel between the full grid
// [NX*NY][R] and the compact voxel order [nv][R]; the coefficient-space MLEM
// update c <- c g / (s + 1e-7) with the fix-ups of main.m:163,176.
cudaError_t launch_rows_gather(const float *full, const int *vox_xy, int nx, int64_t nv, int R, float *compact,
                               cudaStream_t s, int64_t *launches);
cudaError_t launch_rows_scatter(const float *compact, const int *vox_xy, int nx, int64_t nv, int R, float *full,
                                cudaStream_t s, int64_t *launches);
cudaError_t launch_bop_update(float *c, const float *g, const float *s, int64_t n, cudaStream_t st,
                              int64_t *launches);
cudaError_t launch_to_float(const double *a, int64_t n, float *b, cudaStream_t s, int64_t *launches);
// k_decisions.cu: the integer decisions of the fast path for listed rays
// (test export): walk[i][v] = (detector-side sample count, its ROI edge,
// source-side sample count, its ROI edge); nq[i][v][j] = Compton table bin of
// source bin win_lo[nrg] + j, j < 2*dnrg+1.
cudaError_t launch_decisions(const DevProblem &P, const SrcGeom *sg, const EnergyRow *energy, const int *win_lo,
                             const int64_t *rays, int n_rays, const int *vox_xy, int nv, int4 *walk, int *nq,
                             cudaStream_t s, int64_t *launches);
// out[i] = compact[idx[i]] for N, C and the rows of A (row length mw).
cudaError_t launch_gather_rays(const int64_t *idx, int64_t n, const float *Nc, const float *Cc,
                               const float *Ac, int mw, float *N, float *C, float *A, cudaStream_t s,
                               int64_t *launches);

// k_prep.cu: the current device's SM count, cached per device (152 if the
// query fails); sizes the grids of grid-stride loops.
int current_sm_count();

// k_mlem.cu: MLEM with an explicit model matrix (rows of K floats, K % 4 == 0,
// K <= 1024); partial holds nparts rows of K floats.
int mlem_pass_blocks(int sm_count, int K);
cudaError_t launch_mlem_sensitivity(const float *A, long long rays, int K, float *partial, int nparts,
                                    double *sens, cudaStream_t s, int64_t *launches);
cudaError_t launch_mlem_iteration(const float *A, long long rays, int K, const float *y, const float *c,
                                  float *x, float *partial, int nparts, const double *sens, cudaStream_t s,
                                  int64_t *launches);

// k_vox.cu: the per-voxel-coefficient model (forward, adjoint, MLEM update).
struct PairRec;
size_t pair_rec_bytes();
struct VoxOp {
    DevProblem P;
    int nv;                    // non-empty voxels
    const PairRec *pairs;      // [n_src * n_det]
    const EnergyRow *energy;
    const float *rf_win;
    const int *win_lo, *win_n;
    const float4 *coarse_q;
    const int *vox_xy;
    const float4 *cells;
    const float2 *atten_src;
    const float2 *walk;        // [n_src * n_det][nv] detector-side integrals, or NULL
};
cudaError_t launch_compact_voxels(const DevProblem &P, const int32_t *seg, PrepBuffers &B, cudaStream_t s,
                                  int64_t *launches);
cudaError_t launch_pair_table(const DevProblem &P, const SrcGeom *sg, PairRec *out, cudaStream_t s,
                              int64_t *launches);

// One problem of an operator batch as the kernels read it (device memory):
// its tables, its adjoint split and its buffers.
struct VoxJob {
    VoxOp op;
    F32Consts c;
    int E;                     // source bins in the spectrum windows
    int groups;                // adjoint pair groups (rows of part)
    int ppg;                   // pairs per group
    int chunk_blocks;          // adjoint blocks along the voxel chunks
    float *xd, *xc;            // [nv][nwt] unknowns times dq, unknowns
    float *y;                  // [rays] forward output
    const float *ymeas, *cbg;  // [rays] MLEM counts and background
    float *what;               // [pairs][E] per-energy weights
    float2 *part;              // [groups][nv][nwt] adjoint partial sums, each as a float pair
    double *sens;              // [nv][nwt] sensitivity
    float *g;                  // [nx*ny*nwt] adjoint output
    const float *w;            // [rays] adjoint weights
    const float *xfull;        // [nx*ny*nwt] coefficients to gather
    float *xout;               // [nx*ny*nwt] coefficients to scatter to
    // pairs [pair0, pair1) of the problem that this job covers (all of them,
    // or one tile); op.walk holds their detector-side integrals from row 0
    int64_t pair0, pair1;
    int accumulate;            // adjoint: add to the partial rows instead of writing them
    int pad;
};
// Kernel argument of the batched operator kernels.  off holds five prefix
// sums over the n jobs, each of n + 1 entries: 0 forward items (pairs),
// 1 adjoint items (chunk blocks x groups), 2 unknowns (nv*nwt), 3 full-grid
// entries (nx*ny*nwt), 4 per-energy weights (pairs*E).
struct VoxBatch {
    const VoxJob *jobs;
    const int64_t *off;
    unsigned long long *counters;   // [2] work counters of the two persistent kernels
    int n;
    int adj_warps;
};
// Opts the operator kernels in to max_smem bytes of shared memory per block.
cudaError_t vox_set_attributes(int max_smem);
size_t vox_fwd_static_smem();
size_t vox_adj_static_smem();
size_t vox_fwd_smem(const DevProblem &P);
size_t vox_adj_smem(const DevProblem &P, int warps);
int vox_fwd_blocks_per_sm(size_t smem);
int vox_adj_blocks_per_sm(int warps, size_t smem);
// Persistent kernels: grid blocks take items until the counter passes the total.
cudaError_t launch_vox_forward(const VoxBatch &B, bool mlem, int grid, size_t smem, cudaStream_t s,
                               int64_t *launches);
cudaError_t launch_vox_adjoint(const VoxBatch &B, int grid, size_t smem, cudaStream_t s, int64_t *launches);
// Element-wise kernels over the concatenated ranges (total = the last offset).
cudaError_t launch_vox_wtab(const VoxBatch &B, int64_t total, int mode, cudaStream_t s, int64_t *launches);
cudaError_t launch_vox_reduce(const VoxBatch &B, int64_t total, int mode, cudaStream_t s, int64_t *launches);
cudaError_t launch_vox_gather(const VoxBatch &B, int64_t total, bool with_xc, cudaStream_t s, int64_t *launches);
cudaError_t launch_vox_scatter(const VoxBatch &B, int64_t total, cudaStream_t s, int64_t *launches);

} // namespace xrdt
