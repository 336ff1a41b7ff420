/*
 * oracle.h -- FP64 CPU restatement of curadon's projection operators.
 * Test infrastructure only (see oracle.c); never linked into the product.
 *
 * All shapes are in the reference's internal (x fastest) order:
 *   2D volume W x H (x contiguous), 2D sinogram nangles x det_count;
 *   3D volume X x Y x Z, 3D sinogram nangles x V x U (u contiguous).
 */
#ifndef CURADON_GB300_ORACLE_H
#define CURADON_GB300_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Fan-beam geometry (the arguments of plan_2d, plan.cu:34-56 of the
 * reference's Python extension, after its (y,x) -> (x,y) swap). */
typedef struct {
    int64_t W, H;
    double sx, sy;
    double ox, oy;
    int64_t det_count;
    double det_spacing;
    double det_offset;
    int64_t nangles;
    const float *angles;
    const float *DSO;
    const float *DSD;
} or_fan2d_t;

/* Cone-beam geometry (the arguments of forward_3d / backward_3d,
 * forward.cu:23-75 of the reference's Python extension, after its swaps). */
typedef struct {
    int64_t X, Y, Z;
    double sx, sy, sz;
    double ox, oy, oz;
    int64_t U, V;
    double su, sv;
    double offu, offv;
    double pitch, roll, yaw;
    double DSO, DSD, COR;
    int64_t nangles;
    const float *phi;
    const float *theta;
    const float *psi;
} or_cone3d_t;

void or_fan2d_tables(const or_fan2d_t *g, double *src, double *u0, double *du);
int or_fwd2d(const or_fan2d_t *g, const float *vol, double *sino, int quant, int nthreads);
int or_bwd2d(const or_fan2d_t *g, const float *sino, double *vol, int quant, int nthreads);

/* Vector geometry: vecs is nangles x 6 [S.x, S.y, C.x, C.y, U.x, U.y]; the
 * angles / DSO / DSD / det_offset fields of g are not used, det_spacing must
 * be |U|. */
void or_fan2d_vec_tables(const or_fan2d_t *g, const double *vecs, double *src, double *u0,
                         double *du);
int or_fwd2d_vec(const or_fan2d_t *g, const double *vecs, const float *vol, double *sino,
                 int quant, int nthreads);
int or_bwd2d_vec(const or_fan2d_t *g, const double *vecs, const float *sino, double *vol,
                 int quant, int nthreads);

void or_cone3d_fwd_tables(const or_cone3d_t *g, double *org, double *du, double *dv,
                          double *src);
void or_cone3d_bwd_tables(const or_cone3d_t *g, double *org, double *dx, double *dy,
                          double *dz, double *src);
int or_fwd3d(const or_cone3d_t *g, const float *vol, double *sino, int quant, int nthreads);
int or_bwd3d(const or_cone3d_t *g, const float *sino, double *vol, int quant, int nthreads);

#ifdef __cplusplus
}
#endif

#endif
