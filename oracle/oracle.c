/*
 * oracle.c -- CPU restatement of curadon's projection operators, in FP64.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing on the product path may call, link or
 * load this file: it is imported by tests/, by __graft_entry__.smoke() and by
 * bench.py's CPU-baseline / reference leg, and only as the checker or as the
 * timed CPU baseline.
 *
 * It restates, operation by operation but in double precision and with exact
 * trigonometry, the reference algorithms (paths relative to the reference
 * project root):
 *
 *   2D geometry tables   include/curadon/detail/plan/plan_2d.hpp:50-80,189-241
 *                        include/curadon/detail/rotation.hpp:51-61
 *   2D forward           include/curadon/detail/forward_2d.hpp:52-78
 *                        include/curadon/detail/intersection.h:31-46
 *   2D backprojection    include/curadon/detail/backward_2d.hpp:41-99
 *   3D forward geometry  include/curadon/detail/forward_3d.hpp:117-190
 *                        include/curadon/detail/rotation.hpp:7-48
 *   3D forward           include/curadon/detail/forward_3d.hpp:56-93
 *                        include/curadon/detail/intersection.h:12-28
 *   3D backprojection    include/curadon/detail/backward_3d.hpp:78-94,122-166,218-227
 *   interpolation        include/curadon/detail/texture.hpp:81-87 (linear filter,
 *                        border address mode = 0 outside, unnormalised coords)
 *
 * Interpolation follows the texture-fetch formula of the CUDA programming
 * guide: for coordinate x the texels floor(x-0.5) and floor(x-0.5)+1 are
 * blended with weight frac(x-0.5).  The hardware stores that weight as 9-bit
 * fixed point with 8 fractional bits; `quant` selects exact weights (0),
 * weights rounded to 1/256 (1) or truncated to 1/256 (2) so residuals against
 * the reference's texture unit can be attributed.
 *
 * Parity of this restatement is pinned against outputs of the reference's own
 * CUDA operators (tests/golden/, generated by tests/golden/make_golden.py).
 */
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

/* ---------------------------------------------------------------- threads */

typedef void (*or_body_fn)(void *ctx, int64_t begin, int64_t end);

typedef struct {
    or_body_fn fn;
    void *ctx;
    int64_t begin, end;
} or_task_t;

static void *or_thread_main(void *arg) {
    or_task_t *t = (or_task_t *)arg;
    t->fn(t->ctx, t->begin, t->end);
    return NULL;
}

/* Static block partition of [0, n) over nthreads POSIX threads. */
static void or_parallel_for(int64_t n, int nthreads, or_body_fn fn, void *ctx) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    if ((int64_t)nthreads > n) nthreads = (int)(n > 0 ? n : 1);
    if (nthreads == 1) {
        fn(ctx, 0, n);
        return;
    }
    pthread_t th[256];
    or_task_t task[256];
    int started[256];
    for (int i = 0; i < nthreads; ++i) {
        task[i].fn = fn;
        task[i].ctx = ctx;
        task[i].begin = n * i / nthreads;
        task[i].end = n * (i + 1) / nthreads;
        started[i] = pthread_create(&th[i], NULL, or_thread_main, &task[i]) == 0;
        if (!started[i]) or_thread_main(&task[i]);
    }
    for (int i = 0; i < nthreads; ++i)
        if (started[i]) pthread_join(th[i], NULL);
}

/* ---------------------------------------------------------- interpolation */

static inline double or_weight(double f, int quant) {
    if (quant == 1) return nearbyint(f * 256.0) / 256.0;
    if (quant == 2) return floor(f * 256.0) / 256.0;
    return f;
}

/* Linear filtering of a 1D row of n texels at unnormalised coordinate u. */
static inline double or_lerp1(const float *row, int64_t n, double u, int quant) {
    double ub = u - 0.5;
    double fl = floor(ub);
    double a = or_weight(ub - fl, quant);
    int64_t k = (int64_t)fl;
    double t0 = (k >= 0 && k < n) ? (double)row[k] : 0.0;
    double t1 = (k + 1 >= 0 && k + 1 < n) ? (double)row[k + 1] : 0.0;
    return (1.0 - a) * t0 + a * t1;
}

/* Bilinear filtering of a W x H image (x contiguous) at (x, y). */
static inline double or_lerp2(const float *img, int64_t W, int64_t H, double x, double y,
                              int quant) {
    double xb = x - 0.5, yb = y - 0.5;
    double fx = floor(xb), fy = floor(yb);
    double a = or_weight(xb - fx, quant), b = or_weight(yb - fy, quant);
    int64_t i = (int64_t)fx, j = (int64_t)fy;
    double t[2][2];
    for (int dj = 0; dj < 2; ++dj)
        for (int di = 0; di < 2; ++di) {
            int64_t ii = i + di, jj = j + dj;
            t[dj][di] = (ii >= 0 && ii < W && jj >= 0 && jj < H) ? (double)img[jj * W + ii] : 0.0;
        }
    return (1 - a) * (1 - b) * t[0][0] + a * (1 - b) * t[0][1] + (1 - a) * b * t[1][0] +
           a * b * t[1][1];
}

/* Trilinear filtering of an X x Y x Z volume (x fastest) at (x, y, z). */
static inline double or_lerp3(const float *vol, int64_t X, int64_t Y, int64_t Z, double x,
                              double y, double z, int quant) {
    double xb = x - 0.5, yb = y - 0.5, zb = z - 0.5;
    double fx = floor(xb), fy = floor(yb), fz = floor(zb);
    double a = or_weight(xb - fx, quant), b = or_weight(yb - fy, quant),
           c = or_weight(zb - fz, quant);
    int64_t i = (int64_t)fx, j = (int64_t)fy, k = (int64_t)fz;
    double acc = 0.0;
    for (int dk = 0; dk < 2; ++dk)
        for (int dj = 0; dj < 2; ++dj)
            for (int di = 0; di < 2; ++di) {
                int64_t ii = i + di, jj = j + dj, kk = k + dk;
                if (ii < 0 || ii >= X || jj < 0 || jj >= Y || kk < 0 || kk >= Z) continue;
                double w = (di ? a : 1 - a) * (dj ? b : 1 - b) * (dk ? c : 1 - c);
                acc += w * (double)vol[(kk * Y + jj) * X + ii];
            }
    return acc;
}

/* ------------------------------------------------------------- 2D tables */

/* Per-view source, detector-cell-0 direction and per-cell step, in voxel
 * index units (plan_2d.hpp:189-241).  R(phi) = [[c, s], [-s, c]]. */
void or_fan2d_tables(const or_fan2d_t *g, double *src, double *u0, double *du) {
    const double det_ext = (double)g->det_count * g->det_spacing;
    const double extx = (double)g->W * g->sx, exty = (double)g->H * g->sy;
    for (int64_t i = 0; i < g->nangles; ++i) {
        const double a = g->angles[i], c = cos(a), s = sin(a);
        const double dso = g->DSO[i], dod = (double)g->DSD[i] - dso;
        /* source at (det_offset, DSO), rotated */
        const double swx = g->det_offset * c + dso * s;
        const double swy = -g->det_offset * s + dso * c;
        /* detector cells 0 and 1 at y = -DOD, rotated about the origin then
         * taken relative to the source */
        const double p0x = -det_ext / 2 + g->det_spacing * 0.5, py = -dod;
        const double p1x = -det_ext / 2 + g->det_spacing * 1.5;
        const double c0x = (p0x * c + py * s - swx) / g->sx;
        const double c0y = (-p0x * s + py * c - swy) / g->sy;
        const double c1x = (p1x * c + py * s - swx) / g->sx;
        const double c1y = (-p1x * s + py * c - swy) / g->sy;
        u0[2 * i] = c0x;
        u0[2 * i + 1] = c0y;
        du[2 * i] = c1x - c0x;
        du[2 * i + 1] = c1y - c0y;
        src[2 * i] = (swx - g->ox + 0.5 * extx) / g->sx;
        src[2 * i + 1] = (swy - g->oy + 0.5 * exty) / g->sy;
    }
}

/* ------------------------------------------------------------ 2D forward */

typedef struct {
    const or_fan2d_t *g;
    const float *vol;
    double *sino;
    int quant;
    const double *src, *u0, *du;
} or_fwd2d_ctx;

/* Ray (u, view): slab test against [-1, W] x [-1, H] with tmin starting at
 * FLT_MIN, rint(max|rd|) unit steps along the dominant axis, bilinear sample
 * at each step, sum scaled by the physical step length (forward_2d.hpp:52-78,
 * intersection.h:31-46). */
static double or_fwd2d_ray(const or_fwd2d_ctx *c, int64_t view, int64_t u) {
    const or_fan2d_t *g = c->g;
    const double sx = c->src[2 * view], sy = c->src[2 * view + 1];
    const double dx = c->u0[2 * view] + (double)u * c->du[2 * view];
    const double dy = c->u0[2 * view + 1] + (double)u * c->du[2 * view + 1];
    double tmin = FLT_MIN, tmax = FLT_MAX;
    const double ro[2] = {sx, sy}, rd[2] = {dx, dy}, bmax[2] = {(double)g->W, (double)g->H};
    for (int d = 0; d < 2; ++d) {
        double t1 = (-1.0 - ro[d]) / rd[d];
        double t2 = (bmax[d] - ro[d]) / rd[d];
        tmin = fmin(fmax(t1, tmin), fmax(t2, tmin));
        tmax = fmax(fmin(t1, tmax), fmin(t2, tmax));
    }
    if (tmin > tmax - 1e-6) return 0.0;
    const double ox = sx + tmin * dx, oy = sy + tmin * dy;
    const double rx = dx * (tmax - tmin), ry = dy * (tmax - tmin);
    const double m = fmax(fabs(rx), fabs(ry));
    const int64_t n = (int64_t)nearbyint(m);
    const double vx = rx / m, vy = ry / m;
    double acc = 0.0;
    for (int64_t j = 0; j < n; ++j)
        acc += or_lerp2(c->vol, g->W, g->H, ox + (double)j * vx, oy + (double)j * vy, c->quant);
    return acc * hypot(vx * g->sx, vy * g->sy);
}

static void or_fwd2d_body(void *ctx, int64_t b, int64_t e) {
    or_fwd2d_ctx *c = (or_fwd2d_ctx *)ctx;
    const int64_t det = c->g->det_count;
    for (int64_t r = b; r < e; ++r) {
        const int64_t view = r / det, u = r % det;
        c->sino[r] = or_fwd2d_ray(c, view, u);
    }
}

int or_fwd2d(const or_fan2d_t *g, const float *vol, double *sino, int quant, int nthreads) {
    const int64_t n = g->nangles;
    double *tab = (double *)malloc(sizeof(double) * 6 * (size_t)(n > 0 ? n : 1));
    if (!tab) return -1;
    or_fan2d_tables(g, tab, tab + 2 * n, tab + 4 * n);
    or_fwd2d_ctx c = {g, vol, sino, quant, tab, tab + 2 * n, tab + 4 * n};
    or_parallel_for(n * g->det_count, nthreads, or_fwd2d_body, &c);
    free(tab);
    return 0;
}

/* ------------------------------------------------- 2D vector geometry */

/* Per-view vectors [S.x, S.y, C.x, C.y, U.x, U.y] (source, detector centre,
 * step between detector cell centres) in the circular plan's world frame,
 * the layout of FanGeometry.to_vec (geometry.py:54-80).  Forward tables as
 * plan_2d::precompute defines them: the source in voxel index units, the
 * direction from it to the centre of cell 0, C - (det - 1)/2 U, and the
 * per-cell step, both divided by the voxel spacing. */
void or_fan2d_vec_tables(const or_fan2d_t *g, const double *vecs, double *src, double *u0,
                         double *du) {
    for (int64_t i = 0; i < g->nangles; ++i) {
        const double *v = vecs + 6 * i;
        const double d0x = v[2] - 0.5 * (double)(g->det_count - 1) * v[4];
        const double d0y = v[3] - 0.5 * (double)(g->det_count - 1) * v[5];
        src[2 * i] = (v[0] - g->ox) / g->sx + 0.5 * (double)g->W;
        src[2 * i + 1] = (v[1] - g->oy) / g->sy + 0.5 * (double)g->H;
        u0[2 * i] = (d0x - v[0]) / g->sx;
        u0[2 * i + 1] = (d0y - v[1]) / g->sy;
        du[2 * i] = v[4] / g->sx;
        du[2 * i + 1] = v[5] / g->sy;
    }
}

int or_fwd2d_vec(const or_fan2d_t *g, const double *vecs, const float *vol, double *sino,
                 int quant, int nthreads) {
    const int64_t n = g->nangles;
    double *tab = (double *)malloc(sizeof(double) * 6 * (size_t)(n > 0 ? n : 1));
    if (!tab) return -1;
    or_fan2d_vec_tables(g, vecs, tab, tab + 2 * n, tab + 4 * n);
    or_fwd2d_ctx c = {g, vol, sino, quant, tab, tab + 2 * n, tab + 4 * n};
    or_parallel_for(n * g->det_count, nthreads, or_fwd2d_body, &c);
    free(tab);
    return 0;
}

typedef struct {
    const or_fan2d_t *g;
    const double *vecs;
    const float *sino;
    double *vol;
    int quant;
} or_bwd2d_vec_ctx;

/* Pixel P (the backprojector's world position, unscaled +1/2 as in
 * backward_2d.hpp:41-44): per view the ray S + s (P - S) meets the detector
 * line C + t U where [P - S, -U] (s, t)^T = C - S (Cramer's rule); the sample
 * of the view's row at t + det/2 is weighted by the magnification s, which is
 * DSD / (x' + DSO) for a circular view; the sum times 1/|U| is added. */
static void or_bwd2d_vec_body(void *ctx, int64_t b, int64_t e) {
    or_bwd2d_vec_ctx *c = (or_bwd2d_vec_ctx *)ctx;
    const or_fan2d_t *g = c->g;
    const double inv = 1.0 / g->det_spacing;
    const double half_det = (double)g->det_count / 2.0;
    for (int64_t p = b; p < e; ++p) {
        const int64_t ix = p % g->W, iy = p / g->W;
        const double X = ((double)ix - (double)g->W / 2.0) * g->sx + g->ox + 0.5;
        const double Y = ((double)iy - (double)g->H / 2.0) * g->sy + g->oy + 0.5;
        double acc = 0.0;
        for (int64_t v = 0; v < g->nangles; ++v) {
            const double *q = c->vecs + 6 * v;
            const double a11 = X - q[0], a21 = Y - q[1], a12 = -q[4], a22 = -q[5];
            const double b1 = q[2] - q[0], b2 = q[3] - q[1];
            const double det = a11 * a22 - a12 * a21;
            const double s = (b1 * a22 - a12 * b2) / det;
            const double t = (a11 * b2 - b1 * a21) / det;
            acc += or_lerp1(c->sino + v * g->det_count, g->det_count, t + half_det, c->quant) * s;
        }
        c->vol[p] += acc * inv;
    }
}

int or_bwd2d_vec(const or_fan2d_t *g, const double *vecs, const float *sino, double *vol,
                 int quant, int nthreads) {
    or_bwd2d_vec_ctx c = {g, vecs, sino, vol, quant};
    or_parallel_for(g->W * g->H, nthreads, or_bwd2d_vec_body, &c);
    return 0;
}

/* ------------------------------------------------------- 2D backprojection */

typedef struct {
    const or_fan2d_t *g;
    const float *sino;
    double *vol;
    int quant;
    const double *sn, *cs; /* -sin, cos per view */
} or_bwd2d_ctx;

/* Pixel (x, y): world position with the unscaled +1/2 shift, per view the
 * rotated coordinates x' = -s X - c Y, weight DSD / (x' + DSO), detector
 * coordinate u = w (c X - s Y) / ds + det / 2, linear sample of the view's
 * row times w; the sum times 1/ds is added to the volume
 * (backward_2d.hpp:41-99; det_offset is not used there). */
static void or_bwd2d_body(void *ctx, int64_t b, int64_t e) {
    or_bwd2d_ctx *c = (or_bwd2d_ctx *)ctx;
    const or_fan2d_t *g = c->g;
    const double inv = 1.0 / g->det_spacing;
    const double half_det = (double)g->det_count / 2.0;
    for (int64_t p = b; p < e; ++p) {
        const int64_t ix = p % g->W, iy = p / g->W;
        const double X = ((double)ix - (double)g->W / 2.0) * g->sx + g->ox + 0.5;
        const double Y = ((double)iy - (double)g->H / 2.0) * g->sy + g->oy + 0.5;
        double acc = 0.0;
        for (int64_t v = 0; v < g->nangles; ++v) {
            const double s = c->sn[v], co = c->cs[v];
            const double xi = s * X - co * Y;
            const double yi = co * X * inv + s * Y * inv;
            const double w = (double)g->DSD[v] / (xi + (double)g->DSO[v]);
            const double u = w * yi + half_det;
            acc += or_lerp1(c->sino + v * g->det_count, g->det_count, u, c->quant) * w;
        }
        c->vol[p] += acc * inv;
    }
}

int or_bwd2d(const or_fan2d_t *g, const float *sino, double *vol, int quant, int nthreads) {
    const int64_t n = g->nangles;
    double *tab = (double *)malloc(sizeof(double) * 2 * (size_t)(n > 0 ? n : 1));
    if (!tab) return -1;
    for (int64_t v = 0; v < n; ++v) {
        tab[v] = -sin((double)g->angles[v]);
        tab[n + v] = cos((double)g->angles[v]);
    }
    or_bwd2d_ctx c = {g, sino, vol, quant, tab, tab + n};
    or_parallel_for(g->W * g->H, nthreads, or_bwd2d_body, &c);
    free(tab);
    return 0;
}

/* -------------------------------------------------------- 3D rotations */

/* Combined Y-Z-Y Euler rotation (rotation.hpp:7-28). */
static void or_rot_yzy(double v[3], double phi, double theta, double psi) {
    const double cph = cos(phi), sph = sin(phi), cth = cos(theta), sth = sin(theta);
    const double cps = cos(psi), sps = sin(psi);
    const double x = v[0], y = v[1], z = v[2];
    v[0] = x * (cph * cps * cth - sph * sps) - y * sth * cph + z * (sph * cps + sps * cph * cth);
    v[1] = x * (sth * cps) + y * cth + z * sps * sth;
    v[2] = x * (-sph * cps * cth - sps * cph) + y * sph * sth + z * (-sph * sps * cth + cps * cph);
}

/* Roll-pitch-yaw rotation of the detector (rotation.hpp:31-48). */
static void or_rot_rpy(double v[3], double roll, double pitch, double yaw) {
    const double cr = cos(roll), sr = sin(roll), cp = cos(pitch), sp = sin(pitch);
    const double sy = sin(yaw), cy = cos(yaw);
    const double x = v[0], y = v[1], z = v[2];
    v[0] = cr * cp * x + (cr * sp * sy - sr * cy) * y + (cr * sp * cy + sr * sy) * z;
    v[1] = sr * cp * x + (sr * sp * sy + cr * cy) * y + (sr * sp * cy - cr * sy) * z;
    v[2] = -sp * x + cp * sy * y + cp * cy * z;
}

/* ------------------------------------------------------- 3D forward tables */

/* Per view: detector origin, u step, v step and source in voxel-index
 * coordinates whose voxel centres sit on integers (forward_3d.hpp:117-190). */
void or_cone3d_fwd_tables(const or_cone3d_t *g, double *org, double *du, double *dv,
                          double *src) {
    const double dod = g->DSD - g->DSO;
    const double ext[3] = {(double)g->X * g->sx, (double)g->Y * g->sy, (double)g->Z * g->sz};
    const double sp[3] = {g->sx, g->sy, g->sz}, off[3] = {g->ox, g->oy, g->oz};
    for (int64_t i = 0; i < g->nangles; ++i) {
        double s[3] = {0, 0, -g->DSO};
        double o[3] = {-g->su * ((double)g->U / 2.0) + g->su * 0.5,
                       -g->sv * ((double)g->V / 2.0) + g->sv * 0.5, 0.0};
        double pu[3] = {o[0] + g->su, o[1], o[2]};
        double pv[3] = {o[0], o[1] + g->sv, o[2]};
        or_rot_rpy(o, g->roll, g->pitch, g->yaw);
        or_rot_rpy(pu, g->roll, g->pitch, g->yaw);
        or_rot_rpy(pv, g->roll, g->pitch, g->yaw);
        o[2] += dod;
        pu[2] += dod;
        pv[2] += dod;
        const double ph = g->phi[i], th = g->theta[i], ps = g->psi[i];
        or_rot_yzy(o, ph, th, ps);
        or_rot_yzy(pu, ph, th, ps);
        or_rot_yzy(pv, ph, th, ps);
        or_rot_yzy(s, ph, th, ps);
        for (int d = 0; d < 3; ++d) {
            const double tr = ext[d] / 2.0 - sp[d] / 2.0;
            o[d] = (o[d] - off[d] + tr) / sp[d];
            pu[d] = (pu[d] - off[d] + tr) / sp[d];
            pv[d] = (pv[d] - off[d] + tr) / sp[d];
            s[d] = (s[d] - off[d] + tr) / sp[d];
        }
        const double cx = g->COR * sin(ph) / g->sx, cz = g->COR * cos(ph) / g->sz;
        o[0] += cx, o[2] += cz, pu[0] += cx, pu[2] += cz;
        pv[0] += cx, pv[2] += cz, s[0] += cx, s[2] += cz;
        for (int d = 0; d < 3; ++d) {
            org[3 * i + d] = o[d];
            du[3 * i + d] = pu[d] - o[d];
            dv[3 * i + d] = pv[d] - o[d];
            src[3 * i + d] = s[d];
        }
    }
}

/* ------------------------------------------------------------ 3D forward */

typedef struct {
    const or_cone3d_t *g;
    const float *vol;
    double *sino;
    int quant;
    const double *org, *du, *dv, *src;
} or_fwd3d_ctx;

/* Ray (u, v, view): slab test against [-1, N+1]^3 (tmin from FLT_MIN);
 * nothing is written on a miss.  nsteps = ceil((tmax - tmin) ceil(|dir|)),
 * samples at t = tmin + k h for t <= tmax, trilinear at p + 1/2, the sum is
 * not scaled by the step length (forward_3d.hpp:56-93). */
static void or_fwd3d_body(void *ctx, int64_t b, int64_t e) {
    or_fwd3d_ctx *c = (or_fwd3d_ctx *)ctx;
    const or_cone3d_t *g = c->g;
    const int64_t per_view = g->U * g->V;
    const double bmax[3] = {(double)g->X + 1, (double)g->Y + 1, (double)g->Z + 1};
    for (int64_t r = b; r < e; ++r) {
        const int64_t view = r / per_view, rem = r % per_view;
        const int64_t iv = rem / g->U, iu = rem % g->U;
        const double *o = c->org + 3 * view, *du = c->du + 3 * view, *dv = c->dv + 3 * view;
        const double *s = c->src + 3 * view;
        double dir[3];
        for (int d = 0; d < 3; ++d) dir[d] = o[d] + (double)iu * du[d] + (double)iv * dv[d] - s[d];
        const double len = sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
        const double ns = ceil(len);
        double tmin = FLT_MIN, tmax = FLT_MAX;
        for (int d = 0; d < 3; ++d) {
            double t1 = (-1.0 - s[d]) / dir[d];
            double t2 = (bmax[d] - s[d]) / dir[d];
            tmin = fmin(fmax(t1, tmin), fmax(t2, tmin));
            tmax = fmax(fmin(t1, tmax), fmin(t2, tmax));
        }
        if (!(tmin <= tmax)) continue;
        const double nsteps = ceil((tmax - tmin) * ns);
        const double h = (tmax - tmin) / nsteps;
        /* In exact arithmetic t_k = tmin + k h reaches tmax at k = nsteps; the
         * end samples lie on the box faces at -1 / N+1 where every texel of the
         * footprint is border (0), so nsteps vs nsteps+1 samples is immaterial. */
        double acc = 0.0;
        for (int64_t k = 0; k <= (int64_t)nsteps; ++k) {
            const double t = tmin + (double)k * h;
            acc += or_lerp3(c->vol, g->X, g->Y, g->Z, dir[0] * t + s[0] + 0.5,
                            dir[1] * t + s[1] + 0.5, dir[2] * t + s[2] + 0.5, c->quant);
        }
        c->sino[r] = acc;
    }
}

int or_fwd3d(const or_cone3d_t *g, const float *vol, double *sino, int quant, int nthreads) {
    const int64_t n = g->nangles;
    double *tab = (double *)malloc(sizeof(double) * 12 * (size_t)(n > 0 ? n : 1));
    if (!tab) return -1;
    or_cone3d_fwd_tables(g, tab, tab + 3 * n, tab + 6 * n, tab + 9 * n);
    or_fwd3d_ctx c = {g, vol, sino, quant, tab, tab + 3 * n, tab + 6 * n, tab + 9 * n};
    or_parallel_for(n * g->U * g->V, nthreads, or_fwd3d_body, &c);
    free(tab);
    return 0;
}

/* ----------------------------------------------------- 3D backprojection */

/* Per view: world position of voxel (0,0,0) and the x/y/z voxel steps,
 * each rotated by YZY, shifted by the detector offset and rotated by
 * roll-pitch-yaw about z = DOD (backward_3d.hpp:122-166); the source is
 * (-off_u, -off_v, -DSO) under the same roll-pitch-yaw (:218-227). */
void or_cone3d_bwd_tables(const or_cone3d_t *g, double *org, double *dx, double *dy,
                          double *dz, double *src) {
    const double dod = g->DSD - g->DSO;
    const double ext[3] = {(double)g->X * g->sx, (double)g->Y * g->sy, (double)g->Z * g->sz};
    const double sp[3] = {g->sx, g->sy, g->sz}, off[3] = {g->ox, g->oy, g->oz};
    double o0[3];
    for (int d = 0; d < 3; ++d) o0[d] = -ext[d] / 2.0 + sp[d] / 2.0 + off[d];
    for (int64_t i = 0; i < g->nangles; ++i) {
        double pts[4][3];
        for (int k = 0; k < 4; ++k) {
            for (int d = 0; d < 3; ++d) pts[k][d] = o0[d];
            if (k > 0) pts[k][k - 1] += sp[k - 1];
            or_rot_yzy(pts[k], g->phi[i], g->theta[i], g->psi[i]);
            pts[k][0] += g->offu;
            pts[k][1] += g->offv;
            pts[k][2] -= dod;
            or_rot_rpy(pts[k], g->roll, g->pitch, g->yaw);
            pts[k][2] += dod;
        }
        for (int d = 0; d < 3; ++d) {
            org[3 * i + d] = pts[0][d];
            dx[3 * i + d] = pts[1][d] - pts[0][d];
            dy[3 * i + d] = pts[2][d] - pts[0][d];
            dz[3 * i + d] = pts[3][d] - pts[0][d];
        }
    }
    double s[3] = {-g->offu, -g->offv, -g->DSO};
    s[2] -= dod;
    or_rot_rpy(s, g->roll, g->pitch, g->yaw);
    s[2] += dod;
    for (int d = 0; d < 3; ++d) src[d] = s[d];
}

typedef struct {
    const or_cone3d_t *g;
    const float *sino;
    double *vol;
    int quant;
    const double *org, *dx, *dy, *dz, *src;
} or_bwd3d_ctx;

/* Voxel (x, y, z): P = o + x dx + y dy + z dz, ray from the source through
 * P meets the plane z = DSO - DSD at u = dir.x t + s.x + floor(U/2),
 * v = dir.y t + s.y + floor(V/2) (no detector spacing, no distance weight);
 * bilinear sample of that view, summed into the volume (backward_3d.hpp:78-94). */
static void or_bwd3d_body(void *ctx, int64_t b, int64_t e) {
    or_bwd3d_ctx *c = (or_bwd3d_ctx *)ctx;
    const or_cone3d_t *g = c->g;
    const double *s = c->src;
    const double hu = (double)(g->U / 2), hv = (double)(g->V / 2);
    const double zplane = g->DSO - g->DSD;
    for (int64_t p = b; p < e; ++p) {
        const int64_t ix = p % g->X, iy = (p / g->X) % g->Y, iz = p / (g->X * g->Y);
        double acc = 0.0;
        for (int64_t v = 0; v < g->nangles; ++v) {
            const double *o = c->org + 3 * v, *dx = c->dx + 3 * v, *dy = c->dy + 3 * v,
                         *dz = c->dz + 3 * v;
            double dir[3];
            for (int d = 0; d < 3; ++d)
                dir[d] = o[d] + (double)ix * dx[d] + (double)iy * dy[d] + (double)iz * dz[d] - s[d];
            const double t = (zplane - s[2]) / dir[2];
            const double u = dir[0] * t + s[0] + hu;
            const double w = dir[1] * t + s[1] + hv;
            acc += or_lerp2(c->sino + v * g->U * g->V, g->U, g->V, u, w, c->quant);
        }
        c->vol[p] += acc;
    }
}

int or_bwd3d(const or_cone3d_t *g, const float *sino, double *vol, int quant, int nthreads) {
    const int64_t n = g->nangles;
    double *tab = (double *)malloc(sizeof(double) * (12 * (size_t)(n > 0 ? n : 1) + 3));
    if (!tab) return -1;
    or_cone3d_bwd_tables(g, tab, tab + 3 * n, tab + 6 * n, tab + 9 * n, tab + 12 * n);
    or_bwd3d_ctx c = {g, sino, vol, quant, tab, tab + 3 * n, tab + 6 * n, tab + 9 * n, tab + 12 * n};
    or_parallel_for(g->X * g->Y * g->Z, nthreads, or_bwd3d_body, &c);
    free(tab);
    return 0;
}
