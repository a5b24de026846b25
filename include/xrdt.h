/*
 * xrdt.h -- C ABI of the GB300 XRD-tomography projector library (libxrdt.so).
 *
 * The library replaces the `Forward_XRD` MEX call of the reference
 * (Forward_XRD.cu:76-301, a mexcuda build of Forward_projector_kernels/*.cu).
 * Every entry point takes plain pointers and sizes; no C++ or torch types
 * cross this boundary.  All array arguments keep the reference's
 * column-major layouts (first index fastest), so a MATLAB / Python / C
 * caller can hand over the very buffers it would have passed to
 * Forward_XRD.
 *
 * Pointers may be host or device memory: every array pointer is classified
 * with cudaPointerGetAttributes and host arrays are staged through device
 * buffers owned by the context.  Calls return an xrdt_status code and never
 * throw; a human-readable reason for the last failure is available from
 * xrdt_last_error().
 *
 * Compile-time constants of the reference (Forward_XRD.cu:16-53) and the
 * hard-coded scanner (integrate_diffraction.cu:81-143) are runtime fields
 * of xrdt_problem.  xrdt_problem_reference() fills in exactly the values
 * the reference compiles with.
 */
#ifndef XRDT_H
#define XRDT_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define XRDT_ABI_VERSION 1

/* Status codes.  The reference checks no CUDA errors at all
 * (Forward_XRD.cu:210-259); every failure here is reported instead. */
typedef enum xrdt_status {
    XRDT_OK = 0,
    XRDT_ERR_NULL = 1,        /* a required pointer is NULL                    */
    XRDT_ERR_DIMS = 2,        /* a dimension is out of the supported range     */
    XRDT_ERR_GEOMETRY = 3,    /* a source or detector lies inside the phantom  */
    XRDT_ERR_INPUT = 4,       /* bad input values (material id > n_mat, ...)  */
    XRDT_ERR_CUDA = 5,        /* a CUDA runtime call failed                    */
    XRDT_ERR_ALLOC = 6,       /* device or pinned allocation failed            */
    XRDT_ERR_UNSUPPORTED = 7, /* a flag combination that is not implemented    */
    XRDT_ERR_TIMEOUT = 8,     /* a bounded device wait gave up                 */
    XRDT_ERR_IO = 9           /* a file could not be written or read           */
} xrdt_status;

/* Bits of xrdt_problem.quirks: behaviours of the reference kernel that are
 * reproduced on request. */
/* integrate_diffraction.cu:181 samples the (a1,a2) map at the coordinates of
 * the PREVIOUS non-empty voxel (Rvox_x/Rvox_y are assigned only at :192-193,
 * after the fetch); the first non-empty voxel reads them uninitialised.  With
 * this bit set the Compton term uses that stale sample, with (0,0) as the
 * first coordinates; with it clear it uses the current voxel's own value. */
#define XRDT_QUIRK_STALE_VOXEL_A 0x1u

/* Problem description: dimensions, grids, physics constants and scanner
 * geometry.  Lengths are in voxel units (the voxel side is geom vox_side).
 * Field names follow the reference's identifiers. */
typedef struct xrdt_problem {
    int32_t nx, ny;           /* phantom voxels (Forward_XRD.cu:117-119)          */
    int32_t n_src;            /* SRC: source positions (Forward_XRD.cu:17)        */
    int32_t n_col, n_row;     /* COL, ROW: detector pixels (Forward_XRD.cu:18-20) */
    int32_t nrg_src;          /* source energy bins (rows of the spectrum matrix) */
    int32_t nrg_det;          /* NRG: detector energy bins (Forward_XRD.cu:21)    */
    int32_t dnrg;             /* DNRG: window half-width (Forward_XRD.cu:22)      */
    int32_t nwt;              /* NWT: coarse q bins of the model matrix (:23)     */
    int32_t nqf;              /* NQF: fine q bins of Ifine (:24)                  */
    int32_t n_mat;            /* MAT: materials (:25)                             */
    int32_t nq, na;           /* NQ, NA: Compton table size (:47-48)              */
    uint32_t quirks;          /* XRDT_QUIRK_* bits                                */
    int32_t reserved0;        /* must be 0                                        */

    /* Energy grids in keV (integrate_diffraction.cu:138-142): bin i of a grid
     * spans [e_min + i*dE, e_min + (i+1)*dE], dE = (e_max - e_min)/bins. */
    double e_src_min, e_src_max;
    double e_det_min, e_det_max;

    /* q grids in 1/Angstrom (Forward_XRD.cu:39-42; wvt_value.cu:8-22). */
    double q_lo;              /* qmin */
    double q_hi;              /* qmax */
    double dq0;               /* first coarse bin width */

    /* Physics constants (Forward_XRD.cu:34-36,44,51-53; integrate_diffraction.cu:278). */
    double hbarc;             /* keV*Angstrom */
    double mec2;              /* electron rest energy, keV */
    double kn0, kn1, kn2;     /* Klein-Nishina^-1 quadratic fit */
    double rsqrt2pi;          /* 1/sqrt(2 pi) as the reference rounds it */
    double dq_step;           /* DQ: line-integral step in voxels */

    /* Scanner geometry (integrate_diffraction.cu:81-128), voxel units. */
    double cx, cy;            /* rotation centre (Lx/2, Ly/2)                     */
    double r_src, r_det;      /* source / detector trajectory radii              */
    double src_arc;           /* angle spanned by n_src sources (2 pi)           */
    double src_phi0;          /* angle of source 0                               */
    double col_pitch, row_pitch, z0;
    double focal_spot;        /* focal spot size                                 */
    double target_angle;      /* anode target angle, rad                         */
    double wedge_angle;       /* geomphi: fan wedge opening, rad                 */
    double vox_side;          /* geomdvox                                        */
} xrdt_problem;

/* Opaque per-stream context: device buffers, staging, cached tables. */
typedef struct xrdt_ctx xrdt_ctx;

/* Flags of xrdt_forward. */
#define XRDT_FWD_PLAIN_FP64 0x1u  /* run the FP64 kernel at the reference's launch
                                     shape (one block per ray, NWT threads) */
#define XRDT_FWD_NO_SYNC    0x2u  /* return without synchronising the stream; only
                                     valid when every array is device memory */

/* ---- library ---------------------------------------------------------- */
int32_t xrdt_abi_version(void);
const char *xrdt_status_string(int32_t status);

/* ---- problem ---------------------------------------------------------- */
/* Fills *p with the values Forward_XRD.cu compiles with (SRC=32, COL=1024,
 * ROW=1, NRG=64, DNRG=5, NWT=256, NQF=768, MAT=3, NQ=NA=64; Forward_XRD.cu:16-53)
 * and the scanner of integrate_diffraction.cu:81-143 scaled by NX/100, for an
 * nx x ny phantom.  quirks = XRDT_QUIRK_STALE_VOXEL_A. */
int32_t xrdt_problem_reference(xrdt_problem *p, int32_t nx, int32_t ny);
/* Checks dimensions and geometry; XRDT_OK or the first violated rule. */
int32_t xrdt_problem_validate(const xrdt_problem *p);
/* Element counts of the outputs: rays = n_src*n_col*n_row*nrg_det and
 * amatrix = nwt*n_mat*rays (Forward_XRD.cu:143,160). */
int64_t xrdt_problem_rays(const xrdt_problem *p);
int64_t xrdt_problem_amatrix_elems(const xrdt_problem *p);

/* ---- context ---------------------------------------------------------- */
/* stream: a cudaStream_t, or NULL for a stream the context creates. */
int32_t xrdt_ctx_create(xrdt_ctx **ctx, int32_t device, void *stream);
int32_t xrdt_ctx_destroy(xrdt_ctx *ctx);
int32_t xrdt_ctx_synchronize(xrdt_ctx *ctx);
const char *xrdt_last_error(const xrdt_ctx *ctx);
/* Number of kernels this context has launched since creation. */
int64_t xrdt_ctx_launch_count(const xrdt_ctx *ctx);

/* ---- profiling (no counterpart in the reference, which only times the
 * whole MEX call with tic/toc, main.m:55,70) ----------------------------- */
/* Kernel groups reported by xrdt_ctx_kernel_stats. */
#define XRDT_KERNEL_PREP_MAP    0  /* bilinear cell map + Compton table quantisation */
#define XRDT_KERNEL_PREP_VOXELS 1  /* voxel compaction + per-voxel Compton sample    */
#define XRDT_KERNEL_SRC_ATTEN   2  /* source-side line integrals                     */
#define XRDT_KERNEL_FORWARD     3  /* factored forward projector                     */
#define XRDT_KERNEL_PLAIN       4  /* FP64 kernel at the reference launch shape      */
#define XRDT_KERNEL_GATHER      5  /* ray-subset gather                              */
#define XRDT_KERNEL_MLEM        6  /* MLEM passes and updates                        */
#define XRDT_KERNEL_VOX_FORWARD 7  /* per-voxel operator: forward (and MLEM ratios)  */
#define XRDT_KERNEL_VOX_ADJOINT 8  /* per-voxel operator: adjoint                    */
#define XRDT_KERNEL_VOX_UPDATE  9  /* per-voxel operator: sums, update, staging      */
#define XRDT_KERNEL_CT          10 /* transmission sinogram                          */
#define XRDT_KERNEL_BASIS       11 /* basis expansion on the tensor cores            */
#define XRDT_KERNEL_WALK        12 /* detector-side line integrals of the forward    */
#define XRDT_KERNEL_SPECTRUM    13 /* spectrum-response matrix builder               */
#define XRDT_KERNEL_COUNT       14
/* With profiling on, every launch is bracketed by CUDA events on the
 * context's stream and the forward kernel counts the exponentials it
 * evaluates.  Off by default; turning it on or off clears the statistics. */
int32_t xrdt_ctx_set_profiling(xrdt_ctx *ctx, int32_t enable);
/* Launch count, summed device milliseconds, and work units (exp2
 * evaluations, forward kernel only) of one kernel group since profiling was
 * switched on.  Synchronises the context's stream. */
int32_t xrdt_ctx_kernel_stats(xrdt_ctx *ctx, int32_t kernel, int64_t *launches,
                              double *total_ms, int64_t *work);

/* ---- forward projector (replaces mexFunction, Forward_XRD.cu:76-301) -- */
/* Inputs in the order of Forward_XRD's prhs[0..9] (Forward_XRD.cu:82-110):
 *   spectrum  f32 [nrg_src, nrg_det]   detector-smeared source spectrum
 *   Ifine     f32 [nqf * n_mat]        fine-grid XRD pattern per material
 *   seg       i32 [nx, ny]             material id, 1-based, 0 = empty
 *   a1, a2    f32 [nx, ny]             photoelectric / Compton coefficients, 1/voxel
 *   S2        f32 [nq, na]             Compton table scaled to 0..255
 *   q_min, q_max, a_min, a_max         log2 edges of the S2 table axes
 * Outputs (plhs[0..2], Forward_XRD.cu:142-166), caller-owned, fully written:
 *   Nphotons  f32 [n_src, n_col, n_row, nrg_det]   coherent (XRD) counts
 *   Cphotons  f32 [n_src, n_col, n_row, nrg_det]   Compton counts (unscaled)
 *   Amatrix   f32 [nwt, n_mat, n_src, n_col, n_row, nrg_det]  model matrix,
 *             or NULL to skip it.
 * Returns XRDT_ERR_INPUT if a segmentation value exceeds n_mat. */
int32_t xrdt_forward(xrdt_ctx *ctx, const xrdt_problem *p,
                     const float *spectrum, const float *Ifine,
                     const int32_t *seg, const float *a1, const float *a2,
                     const float *S2,
                     float q_min, float q_max, float a_min, float a_max,
                     float *Nphotons, float *Cphotons, float *Amatrix,
                     uint32_t flags);

/* Forward projection of selected rays only.  rays[i] is the linear output
 * index src + det*n_src + nrg*n_src*n_det of Forward_XRD's outputs
 * (integrate_diffraction.cu:404).  Nphotons[i], Cphotons[i] and the model-matrix
 * row A_rows[i][n_mat][nwt] (or NULL) receive what xrdt_forward writes at that
 * index.  No counterpart in the reference, which always computes every ray;
 * used to time and check rays of workloads too large for the FP64 paths. */
int32_t xrdt_forward_rays(xrdt_ctx *ctx, const xrdt_problem *p,
                          const float *spectrum, const float *Ifine,
                          const int32_t *seg, const float *a1, const float *a2,
                          const float *S2,
                          float q_min, float q_max, float a_min, float a_max,
                          const int64_t *rays, int64_t n_rays,
                          float *Nphotons, float *Cphotons, float *A_rows,
                          uint32_t flags);

/* The cross-section table path: the forward model with the coherent
 * (Rayleigh) term read from a tabulated cross-section S1 [NQ, NA] instead of
 * the materials' fine-q patterns -- the form the reference keeps commented
 * out after its kernel (integrate_diffraction.cu:416-418, 479-494, 701-719;
 * tables from XSection_builder.m:93-128):
 *   Nphotons[ray] = sum_v sum_{e in window} RF[e,nrg] Pin Pout geom
 *                   Rayleigh(theta) a2(v) S1[nq, na]
 * with nq the bin of log2(ein sin(theta/2)) on [q_min, q_max) (NQ bins),
 * na the Compton table's column, S1 quantised to u8 by floor and clamp as S2
 * is; Cphotons exactly as xrdt_forward.  XRDT_TAB_BILINEAR reads both tables
 * bilinearly instead, between the grid points q_min + i (q_max - q_min)/(NQ-1)
 * and a_min + j (a_max - a_min)/(NA-1) of XSection_builder.m:121-125
 * (clamped at the ends).  Arguments and layouts as xrdt_forward, with S1 in
 * place of Ifine; the caller scales Nphotons by S1_max/255 as main.m:68
 * scales Cphotons.  Every ray; no model matrix; flags: XRDT_TAB_BILINEAR,
 * XRDT_FWD_NO_SYNC. */
#define XRDT_TAB_BILINEAR 0x4u
int32_t xrdt_forward_tables(xrdt_ctx *ctx, const xrdt_problem *p, const float *spectrum,
                            const int32_t *seg, const float *a1, const float *a2,
                            const float *S1, const float *S2,
                            float q_min, float q_max, float a_min, float a_max,
                            float *Nphotons, float *Cphotons, uint32_t flags);

/* The integer decisions of the fast forward path, for bit-exact comparison
 * with an FP64 restatement (a test export: the float outputs of
 * xrdt_forward would hide a one-bin flip under their tolerance).  For the
 * listed rays (linear indices as in xrdt_forward_rays) and every non-empty
 * voxel v in the reference's loop order (x outer, y inner;
 * integrate_diffraction.cu:173-177), made by the same device functions the
 * production kernels call:
 *   win  [n_rays][2]     source-energy window lo, hi (find_src_nrg_range.cu:8-25)
 *   walk [n_rays][nv][4] detector-side sample count and ROI edge entered, then
 *                        the same for the source side (attenuator.cu:19-52,
 *                        GetIntersection.cu:9-57; edges in its order bottom,
 *                        right, top, left; -1 = missed)
 *   nq   [n_rays][nv][2*dnrg+1]  Compton table bin per window energy
 *                        (integrate_diffraction.cu:331-337)
 *   na   [nv]            Compton table column (integrate_diffraction.cu:177-189)
 *   s2u8 [nq*na]         the quantised table (integrate_diffraction.cu:66-74)
 * nv (the number of voxels with seg > 0) is returned in *nv; the caller sizes
 * walk, nq and na for it.  All lists and outputs are host memory;
 * n_rays <= 65535. */
int32_t xrdt_debug_decisions(xrdt_ctx *ctx, const xrdt_problem *p, const float *spectrum,
                             const int32_t *seg, const float *a1, const float *a2, const float *S2,
                             float q_min, float q_max, float a_min, float a_max,
                             const int64_t *rays, int64_t n_rays, int32_t *win, int32_t *walk,
                             int32_t *na, int32_t *nq, uint8_t *s2u8, int64_t *nv);

/* ---- MLEM with an explicit model matrix (main.m:154-176) --------------- */
/* The spectrum-response matrix of spectrum_builder.m:64-95, the spectrum
 * input of xrdt_forward (prhs[0]).  A fine source spectrum -- bin edges
 * e_hd [n_hd+1] in keV, increasing, and photons per keV n_hd [n_hd]
 * (spectrum_builder.m:22-30) -- is spread over detector energies with a
 * Gaussian of width sigma(E) = sigma0 + sigma1 E (:65; the reference's
 * 0.5 (1.61 + 0.025 E) is sigma0 = 0.805, sigma1 = 0.0125) and integrated
 * over each pair of a coarse source bin (src_edges [ns+1]) and a coarse
 * detector bin (det_edges [nd+1]) with the bins' overlap lengths as weights
 * (:75-91).  spectrum [ns, nd] column-major: (s, d) at s + d*ns.  The
 * reference uses one grid for both axes; separate grids are the same sum.
 * Requires nd <= 65535 and sigma(E) > 0 at every fine bin centre.  Arrays
 * may be host or device memory; FP64 arithmetic, output rounded to float. */
int32_t xrdt_spectrum_build(xrdt_ctx *ctx, const float *e_hd, const float *n_hd, int32_t n_hd_bins,
                            const float *src_edges, int32_t ns, const float *det_edges, int32_t nd,
                            double sigma0, double sigma1, float *spectrum, uint32_t flags);

/* ---- basis expansion on the tensor cores -----------------------------
 * I[M x N] = C[M x K] B[K x N], row-major, FP32 accuracy through 3xTF32 on
 * tcgen05 (FP32 accumulation in tensor memory).  The reference's coarse q
 * basis is point-sampled (wvt_value.cu:8-22, integrate_diffraction.cu:311-315),
 * i.e. diagonal; with a dense basis this expands K coefficients per material
 * (or per voxel) onto the NQF fine q bins, e.g. the Ifine [MAT x NQF] input
 * of xrdt_forward.  K a multiple of 8 in [8, 64], N a multiple of 16 in
 * [16, 256].  XRDT_ERR_TIMEOUT if the accumulator never completed. */
int32_t xrdt_basis_expand(xrdt_ctx *ctx, const float *C, int64_t M, int32_t K,
                          const float *B, int32_t N, float *I, uint32_t flags);

/* ---- transmission CT sinogram ---------------------------------------
 * The reference declares a transmitted-photon output and its no-phantom
 * gain (Tphotons, gain0) and the launches that would fill them,
 * integrate_src2det and polychromatic_src2det, only in comments
 * (Forward_XRD.cu:125-140,169-199,263-276).  Here, per (source, pixel,
 * detector energy bin) in the Nphotons layout [SRC, COL, ROW, NRG]:
 *   Tphotons = sum_{e in window(nrg)} RF[e,nrg] exp(-(A1/ein^3 + A2/KN(ein)))
 *   gain0    = sum_{e in window(nrg)} RF[e,nrg]
 * with (A1, A2) the line integral of the (a1, a2) map along the source ->
 * pixel chord clipped to [0,NX] x [0,NY], sampled every DQ from the entry
 * point as attenuator.cu:9-109 samples.  -log(Tphotons / gain0) is the
 * energy-resolved CT sinogram.  Spectrum, windows and attenuation model as
 * xrdt_forward. */
int32_t xrdt_ct_sinogram(xrdt_ctx *ctx, const xrdt_problem *p, const float *spectrum,
                         const float *a1, const float *a2, float *Tphotons,
                         float *gain0, uint32_t flags);

/* Runs `iters` iterations of
 *     x <- x .* (A' * (y ./ (A*x + c + 1e-20))) ./ (sum(A,1)' + 1e-7)
 *     x(~isfinite(x)) = 0;  x(x < 0) = 0
 * in place on x[K], with A the [rays x K] model matrix stored as rays rows of
 * K contiguous floats -- exactly the Amatrix buffer xrdt_forward writes, K =
 * nwt*n_mat, rays = xrdt_problem_rays (main.m:140 uses its transpose
 * reshape).  y[rays] are measured counts, c[rays] the Compton bias
 * (main.m:162 uses Cphotons(:)).  K must be a multiple of 4, at most 1024;
 * device arrays A and x must be 16-byte aligned (XRDT_ERR_UNSUPPORTED).
 * The iteration body is a fused pass over A (one read of A per iteration)
 * and an FP64 reduction/update, replayed as a CUDA graph. */
int32_t xrdt_mlem_matrix(xrdt_ctx *ctx, const float *A, int64_t rays, int32_t K,
                         const float *y, const float *c, float *x, int32_t iters,
                         uint32_t flags);

/* ---- MLEM checkpoints ------------------------------------------------
 * The state of an MLEM run is its estimate and the number of iterations done
 * (the reference keeps both in MATLAB memory only, main.m:154-176).  write
 * stores x [n] (host or device memory) and iteration in a file at path,
 * replacing it only once the new file is complete; read checks the file's
 * header, element count and checksum (XRDT_ERR_INPUT when the file is not a
 * checkpoint of n elements or is damaged) and fills x (host or device) and
 * *iteration.  An MLEM continued from a checkpoint gives the same estimate as
 * the run that was not interrupted.  XRDT_ERR_IO when the file system fails. */
int32_t xrdt_mlem_checkpoint_write(const char *path, const float *x, int64_t n, int64_t iteration);
int32_t xrdt_mlem_checkpoint_read(const char *path, float *x, int64_t n, int64_t *iteration);

/* ---- per-voxel-coefficient operator: forward, adjoint, MLEM -----------
 * The reference's unknowns are per material: Amatrix[k, m, ray] sums the
 * coarse-q term of integrate_diffraction.cu:311-315 over the voxels of
 * material m (Forward_XRD.cu:160), and main.m:154-176 reconstructs NWT*MAT
 * numbers.  An operator gives every non-empty voxel its own coarse-q
 * pattern, x[k + NWT*(ix + NX*iy)], and computes matrix-free
 *   y[ray] = sum_{v,k} Av[ray, v, k] x[v, k]          (xrdt_op_forward)
 *   g[v,k] = sum_ray  w[ray] Av[ray, v, k]            (xrdt_op_adjoint)
 * where Av is that term for voxel v alone; summing Av over the voxels of a
 * material gives Amatrix.  Rays are ordered as Nphotons, src + det*SRC +
 * nrg*SRC*DET.  The operator is the forward/backward context: creating it
 * stages the attenuation maps, the voxel list, the (source, pixel) pairs and
 * the source-side line integrals once.  The detector-side attenuation of
 * each (pair, voxel) is also walked once and kept ([pairs][voxels] float2)
 * when that table fits in a quarter of the device memory free at creation
 * and the environment variable XRDT_WALK_CACHE is not "0"; otherwise every
 * forward or adjoint walks it again.  Arrays may be host or device memory;
 * calls synchronise the context's stream before they return.  The context
 * must outlive the operator. */
typedef struct xrdt_op xrdt_op;
/* Requires NWT <= 1024, at most 128 source bins in the spectrum windows, and
 * the adjoint's compensated sums of 32 voxels (256 NWT bytes) within one
 * block's shared memory, i.e. NWT up to about 840 on this GPU; otherwise
 * XRDT_ERR_UNSUPPORTED. */
int32_t xrdt_op_create(xrdt_ctx *ctx, const xrdt_problem *p, const float *spectrum,
                       const int32_t *seg, const float *a1, const float *a2,
                       xrdt_op **op);
int32_t xrdt_op_destroy(xrdt_op *op);
/* Number of non-empty voxels (the voxels that carry unknowns), or -1. */
int64_t xrdt_op_voxels(const xrdt_op *op);
/* Bytes of the kept detector-side integrals (0: walked in every call), or
 * -1. */
int64_t xrdt_op_walk_bytes(const xrdt_op *op);
/* y [rays] = Av x; x [NX*NY*NWT] (entries of empty voxels are ignored). */
int32_t xrdt_op_forward(xrdt_op *op, const float *x, float *y, uint32_t flags);
/* g [NX*NY*NWT] = Av^T w; w [rays]; g is 0 at empty voxels. */
int32_t xrdt_op_adjoint(xrdt_op *op, const float *w, float *g, uint32_t flags);
/* iters MLEM updates of main.m:162-176 with per-voxel unknowns:
 *   x <- x .* Av^T(y ./ (Av x + c + 1e-20)) ./ (Av^T 1 + 1e-7),
 * non-finite entries and negatives set to 0.  y, c [rays]; x [NX*NY*NWT] is
 * the starting estimate and receives the result (0 at empty voxels once
 * iters >= 1, where the sensitivity is 0).  Each iteration is one CUDA
 * graph launch of three kernels: forward with the ratios, adjoint, update. */
int32_t xrdt_op_mlem(xrdt_op *op, const float *y, const float *c, float *x,
                     int32_t iters, uint32_t flags);
/* The same model for a host list of rays, computed by the FP64 kernel at the
 * reference's launch shape (one block per ray, NWT threads, every voxel and
 * both line integrals recomputed per block, as integrate_diffraction.cu:33-409
 * is launched by Forward_XRD.cu:244-259): the plain FP64 GPU path the fast
 * operator is measured against.  flags must be XRDT_OP_PLAIN_FP64; NWT must
 * be a multiple of 32, at most 1024.  forward: y[i] = (Av x)[rays[i]];
 * adjoint: g = sum_i w[i] Av[rays[i], :, :] (w and y have n_rays entries). */
#define XRDT_OP_PLAIN_FP64 0x1u
int32_t xrdt_op_forward_rays(xrdt_op *op, const float *x, const int64_t *rays,
                             int64_t n_rays, float *y, uint32_t flags);
int32_t xrdt_op_adjoint_rays(xrdt_op *op, const float *w, const int64_t *rays,
                             int64_t n_rays, float *g, uint32_t flags);

/* ---- the per-voxel operator with a dense q basis -----------------------
 * The reference's coarse q "basis" is point-sampled: bin k of the model row
 * is the Gaussian at the bin centre times its width (wvt_value.cu:8-22,
 * integrate_diffraction.cu:311-315).  With a dense basis B [J][NWT]
 * (row-major, non-negative) the unknowns of a voxel are J coefficients c and
 * its coarse pattern is x[k] = sum_j c[j] B[j][k]: forward(c) = Av (c B),
 * adjoint(w) = (Av^T w) B^T, and MLEM (main.m:162-176) runs on the
 * coefficients.  The expansion and the contraction are GEMMs on the tensor
 * cores (tcgen05, 3xTF32, FP32 accumulation; xrdt_basis_expand).  c and g
 * are [NX*NY*J], voxel index ix + NX*iy, coefficient fastest (0 at empty
 * voxels); y, w, y_meas and c_bg as for the operator.  J and NWT multiples
 * of 16 in [16, 64].  The basis operator uses its operator's buffers: the
 * two take part in one call at a time, and the operator must outlive it. */
typedef struct xrdt_bop xrdt_bop;
int32_t xrdt_bop_create(xrdt_op *op, const float *B, int32_t J, xrdt_bop **bop);
int32_t xrdt_bop_destroy(xrdt_bop *bop);
int32_t xrdt_bop_forward(xrdt_bop *bop, const float *c, float *y, uint32_t flags);
int32_t xrdt_bop_adjoint(xrdt_bop *bop, const float *w, float *g, uint32_t flags);
int32_t xrdt_bop_mlem(xrdt_bop *bop, const float *y_meas, const float *c_bg, float *c, int32_t iters,
                      uint32_t flags);

/* ---- batches: many operators in one launch per kernel ------------------
 * A batch runs the forward, the adjoint and MLEM of several operators
 * (phantoms and scanners of any sizes) together: the forward and the adjoint
 * are persistent kernels whose blocks take work from one queue that holds
 * every problem's (source, pixel) pairs or (voxel chunk, pair group) tiles,
 * so uneven problems fill the GPU together; each MLEM iteration of the whole
 * batch is one CUDA graph launch.  The adjoint's tile shape (warps per block
 * and tiles per block slot) is chosen by timing candidates on the batch on
 * its first MLEM call or on xrdt_batch_tune, and kept in a cache file (one
 * line per GPU and set of problem sizes; the file is $XRDT_TUNE_CACHE, by
 * default $XDG_CACHE_HOME/xrdt/tune.txt or $HOME/.cache/xrdt/tune.txt; an
 * empty XRDT_TUNE_CACHE turns it off).  Arrays are per-problem device
 * pointers in operator order, with each operator's sizes.  A batch uses its
 * operators' buffers: an operator takes part in one call at a time. */
typedef struct xrdt_batch xrdt_batch;
int32_t xrdt_batch_create(xrdt_ctx *ctx, xrdt_op *const *ops, int32_t n,
                          xrdt_batch **batch);
int32_t xrdt_batch_destroy(xrdt_batch *batch);
int32_t xrdt_batch_forward(xrdt_batch *batch, const float *const *x,
                           float *const *y, uint32_t flags);
int32_t xrdt_batch_adjoint(xrdt_batch *batch, const float *const *w,
                           float *const *g, uint32_t flags);
int32_t xrdt_batch_mlem(xrdt_batch *batch, const float *const *y,
                        const float *const *c, float *const *x, int32_t iters,
                        uint32_t flags);
/* Runs the tile-shape search now (once per batch) and reports the choice. */
int32_t xrdt_batch_tune(xrdt_batch *batch, int32_t *adj_warps, int64_t *adj_tiles,
                        int32_t *fwd_grid, int32_t *adj_grid);

/* The same MLEM for callers that cannot allocate device memory (a host
 * framework that owns the device pool, a real-time loop that must not risk
 * an allocation or its implicit synchronisation, an embedder that only hands
 * over buffers).  No counterpart in the reference.  It allocates nothing: its
 * scratch is a fixed 2 MiB + 8 KiB array in the library that every device
 * using it keeps until process exit; K is limited to 1024 as in
 * xrdt_mlem_matrix (larger K: XRDT_ERR_DIMS).  A, y, c and x must be device
 * memory of the current device, with A and x 16-byte aligned (else
 * XRDT_ERR_UNSUPPORTED); work is queued on `stream` (a cudaStream_t, NULL
 * for the default stream) and the call returns after the stream has
 * finished: it synchronises the stream, so it cannot run inside a stream
 * capture.  The first call on a device looks up the scratch address.  All
 * calls share the scratch: calls that overlap on the GPU race. */
int32_t xrdt_mlem_matrix_noalloc(const float *A, int64_t rays, int32_t K,
                                 const float *y, const float *c, float *x,
                                 int32_t iters, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* XRDT_H */
