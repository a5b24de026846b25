/*
 * xrdt_oracle.h -- FP64 CPU restatement of the reference's forward projector.
 *
 * TEST INFRASTRUCTURE ONLY.  This oracle is the checker for the CUDA library;
 * only the tests, the smoke check and the CPU-baseline leg of bench.py may
 * load it.  The product library (libxrdt.so) never links or calls it.
 *
 * It restates Forward_projector_kernels/{integrate_diffraction,attenuator,
 * GetIntersection,find_src_nrg_range,wvt_value}.cu in double precision, one
 * ray (= one CUDA block of the reference, integrate_diffraction.cu:33-35) at a
 * time, with the compile-time constants replaced by xrdt_problem fields.
 * Float-suffixed constants keep their float-rounded values (they are fields
 * of xrdt_problem filled from the reference's literals).  tex2D becomes exact
 * bilinear interpolation with texel centres at i+0.5 and a zero border
 * (Forward_XRD.cu:229-233).  Block reductions become serial sums.
 *
 * Parity pin: tests/golden holds outputs of the reference's own kernel files
 * compiled for the host in FP64 (oracle/ref_emulator.cpp); the oracle is
 * checked against them.
 */
#ifndef XRDT_ORACLE_H
#define XRDT_ORACLE_H

#include <stdint.h>
#include "../include/xrdt.h"

#ifdef __cplusplus
extern "C" {
#endif

/* wvt_value.cu:8-22 on the problem's grid. */
void xrdt_oracle_wvt_value(const xrdt_problem *p, int32_t nwt, double *qnow, double *dqnow);
/* find_src_nrg_range.cu:8-25, generalised to separate source/detector grids. */
void xrdt_oracle_src_nrg_range(const xrdt_problem *p, int32_t nrg, int32_t *lo, int32_t *hi);
/* GetIntersection.cu:9-57; returns 1 and the point, or 0 and NaNs. */
int32_t xrdt_oracle_get_intersection(double x1, double y1, double x2, double y2,
                                     int32_t nx, int32_t ny, double *rx, double *ry);
/* attenuator.cu:9-109 for one endpoint/voxel pair; returns the sample count. */
int64_t xrdt_oracle_attenuator(const xrdt_problem *p, const float *a1, const float *a2,
                               double ex, double ey, double vx, double vy,
                               double *A1, double *A2);

/* Forward projection of selected rays.  rays[i] is the linear output index
 * src + det*n_src + nrg*n_src*n_det (integrate_diffraction.cu:404).
 * N_out, C_out: [n_rays]; A_out: [n_rays][n_mat][nwt] or NULL;
 * Av_out: per-voxel model rows [n_rays][nx*ny][nwt] (voxel index nx+ny*NX),
 * the Amatrix row before it is summed per material, or NULL.
 * Returns 0, or -1 for invalid input (a material id above n_mat). */
int32_t xrdt_oracle_forward_rays(const xrdt_problem *p,
                                 const float *spectrum, const float *Ifine,
                                 const int32_t *seg, const float *a1, const float *a2,
                                 const float *S2,
                                 float q_min, float q_max, float a_min, float a_max,
                                 const int64_t *rays, int64_t n_rays,
                                 double *N_out, double *C_out, double *A_out,
                                 double *Av_out, int32_t n_threads);

/* The per-voxel-coefficient model of the same rays: Av[r][v][k] is the
 * coarse-q model term of integrate_diffraction.cu:311-315 for voxel v alone
 * (the Amatrix row before it is summed per material).  With x [nx*ny][nwt]
 * (voxel index nx+ny*NX) it writes y_out[i] = sum_{v,k} Av[rays[i]][v][k] x[v][k];
 * with w [n_rays] it writes g_out[v][k] = sum_i w[i] Av[rays[i]][v][k].  Either
 * pair may be NULL.  Returns 0, or a negative value for invalid input. */
/* The cross-section table path: the coherent term from the table S1
 * (integrate_diffraction.cu:701-719, code the reference keeps commented out)
 * instead of the fine-q pattern sum, and both tables read by nearest bin or,
 * with bilinear != 0, bilinearly between the grid points of
 * XSection_builder.m:121-125. */
int32_t xrdt_oracle_forward_tables(const xrdt_problem *p, const float *spectrum, const int32_t *seg,
                                   const float *a1, const float *a2, const float *S1, const float *S2,
                                   float q_min, float q_max, float a_min, float a_max, int32_t bilinear,
                                   const int64_t *rays, int64_t n_rays, double *N_out, double *C_out,
                                   int32_t n_threads);
int32_t xrdt_oracle_vox_rays(const xrdt_problem *p, const float *spectrum, const int32_t *seg,
                             const float *a1, const float *a2, const double *x, const double *w,
                             const int64_t *rays, int64_t n_rays, double *y_out, double *g_out,
                             int32_t n_threads);

/* The integer decisions of the FP64 forward for the listed rays and every
 * non-empty voxel in loop order: win [n][2] source-energy window,
 * walk [n][nv][4] (detector-side samples, ROI edge, source-side samples, ROI
 * edge), nq [n][nv][2*dnrg+1] Compton table bins, na [nv] Compton table
 * columns, s2u8 [nq*na] quantised table.  Returns 0, or -1 for a material id
 * above n_mat. */
int32_t xrdt_oracle_decisions(const xrdt_problem *p, const float *spectrum, const float *Ifine,
                              const int32_t *seg, const float *a1, const float *a2, const float *S2,
                              float q_min, float q_max, float a_min, float a_max,
                              const int64_t *rays, int64_t n_rays, int32_t *win, int32_t *walk,
                              int32_t *na, int32_t *nq, uint8_t *s2u8, int32_t n_threads);

/* Transmission through the map per listed ray (Nphotons index) and the
 * same without the phantom: Tphotons and gain0 of the CT sinogram. */
int32_t xrdt_oracle_ct_rays(const xrdt_problem *p, const float *spectrum, const float *a1, const float *a2,
                            const int64_t *rays, int64_t n_rays, double *T_out, double *G_out, int32_t n_threads);

#ifdef __cplusplus
}
#endif
#endif
