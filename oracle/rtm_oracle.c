/*
 * CPU oracle for the RTM hot path of caixh90/RTM_GPU.
 *
 * TEST INFRASTRUCTURE ONLY: tests, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg are the only code that loads this library.  The product
 * (rtm_gpu_gb300) never links or calls it.
 *
 * Contents
 *   - wavefield kernels, FP32 and FP64 (rtm_oracle_body.h)
 *   - per-shot driver loops (rtm_driver_body.h)
 *   - model preparation: velocity padding (GPU_velocity_real.cpp:6-118),
 *     velocity binning (kernel.cu:704-742), Ricker wavelet (kernel.cu:1261-1266)
 *   - per-shot image finishing (kernel.cu:935-990) and the stack
 *     (kernel.cu:992-1059), plus a compensated (Kahan) stack
 * The coefficient optimiser lives in lsm_oracle.c.
 *
 * Floating-point: built with -ffp-contract=off so that no multiply-add is
 * fused; with that, the FP32 path reproduces the reference's rounding
 * sequence operation for operation (checked bit for bit against the
 * reference's own kernel bodies run on the CPU).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "rtm_oracle.h"

void or_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int or_get_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

#define REAL float
#define SFX(n) n##_f32
#include "rtm_oracle_body.h"
#undef REAL
#undef SFX
#define REAL double
#define SFX(n) n##_f64
#include "rtm_oracle_body.h"
#undef REAL
#undef SFX

/* ---- drivers: bind the loop of rtm_driver_body.h to the restated kernels */
#define K_EQUAL(lf, rt, up, dw, a0, a1) SFX(or_equal)(lf, rt, up, dw, a0, a1, P->NZ, P->NX, P->N2, P->M)
#define K_ADD(a2, a0, a1, wv)                                                                    \
    SFX(or_add)(v, a2, a0, a1, c, idx, P->adaptive, P->tao2, P->h2, P->vmin, P->dv, P->M, P->NZ, \
                P->NX, P->r_u, P->r_x, wv, P->hzx2_1)
#define K_HYB1(a1, a0, a2, bb) \
    SFX(or_hybrid1)(a1, a0, a2, bb, v, r1, P->NZ, P->NX, P->N2, P->taoh, P->taoh2, P->quirk)
#define K_HYB2(a1, a0, a2, bb) SFX(or_hybrid2)(a2, bb, w, P->NZ, P->NX, P->N2)
#define K_BKHYB1 K_HYB1
#define K_BKHYB2 K_HYB2
#define K_HYB3(a1, a0, a2, bb, kk) SFX(or_ring_save)(lf, rt, up, dw, a2, P->NZ, P->NX, P->N2, P->M, kk)
#define K_DELIVER(a1, a0, a2) SFX(or_deliver)(a1, a0, a2, P->NZ, P->NX, P->N2, 0)
#define K_BKEQUAL(a1, kk) SFX(or_bkequal)(lf, rt, up, dw, a1, P->NZ, P->NX, P->N2, P->M, kk)
#define K_BKADD_EFF(a2, a0, a1, wv)                                                              \
    SFX(or_bkadd_eff)(v, a2, a0, a1, c, idx, P->adaptive, P->tao2, P->h2, P->vmin, P->dv, P->M,  \
                      P->N2, P->NZ, P->NX, P->r_u, P->r_x, wv, P->hzx2_1)
#define K_DELIVER_EFF(a1, a0, a2) SFX(or_deliver)(a1, a0, a2, P->NZ, P->NX, P->N2, 1)
#define K_BKADD(a2, a1, a0, sd)                                                                  \
    SFX(or_bkadd)(v, a2, a1, a0, c, idx, P->adaptive, sd, P->tao2, P->h2, P->vmin, P->dv, P->M,  \
                  P->NZ, P->NX, P->s_l, P->s_r, P->s_z, P->ds, P->hzx2_1)
#define K_REL(S, R, SA, RA, q1, q2) SFX(or_rel)(S, R, SA, RA, q1, q2, P->NZ, P->NX, P->compen)

#define REAL float
#define SFX(n) n##_f32
#define DRV_NAME(n) or_##n##_f32
#include "rtm_driver_body.h"
#undef REAL
#undef SFX
#undef DRV_NAME
#define REAL double
#define SFX(n) n##_f64
#define DRV_NAME(n) or_##n##_f64
#include "rtm_driver_body.h"
#undef REAL
#undef SFX
#undef DRV_NAME

/* ---- model preparation ------------------------------------------------- */

#define OR_PI 3.1415926535898 /* the reference's value of pi (kernel.cu:16) */

/* Ricker wavelet of kernel.cu:1261-1266, delay t0 = 1/f0, evaluated in
 * double and rounded to float as the reference does. */
float or_ricker(float t1, float f0)
{
    float t00 = 1 / f0;
    double a = OR_PI * f0 * (t1 - t00);
    return (float)((1 - 2 * pow(a, 2)) * exp(-pow(a, 2)));
}

/* Wavelet table wav[i] = f(i*tao) for i = 0..n-1 (the reference forms the
 * time as an int times a float, kernel.cu:812). */
void or_wavelet_table(float *wav, int n, float tao, float f0)
{
    for (int i = 0; i < n; ++i) wav[i] = or_ricker(i * tao, f0);
}

/* GPU_velocity_real.cpp:6-118 from an in-memory interior model.
 * vin is the interior model as stored in the reference's velocity file:
 * column-major, nx columns of nz samples.  Fills the padded grid v (NZ*NX)
 * by edge extension, optionally flips left/right (choice==1), and derives
 * r = v*tao/h and r_1 = sqrt(r^2/2). */
void or_pad_velocity(const float *vin, float *v, float *r1, int NZ, int NX, int N2,
                     float tao, float h, int choice)
{
    int nz = NZ - 2 * N2, nx = NX - 2 * N2;
    for (int xi = 0; xi < nx; ++xi)
        for (int zi = 0; zi < nz; ++zi) v[(long)(N2 + zi) * NX + N2 + xi] = vin[(long)xi * nz + zi];
    for (int z = 0; z < NZ; ++z)
        for (int x = 0; x < NX; ++x) {
            int zc = z < N2 ? N2 : (z >= NZ - N2 ? NZ - N2 - 1 : z);
            int xc = x < N2 ? N2 : (x >= NX - N2 ? NX - N2 - 1 : x);
            if (zc != z || xc != x) v[(long)z * NX + x] = v[(long)zc * NX + xc];
        }
    if (choice == 1)
        for (int z = 0; z < NZ; ++z)
            for (int x = 0; x < NX / 2; ++x) {
                float t = v[(long)z * NX + x];
                v[(long)z * NX + x] = v[(long)z * NX + NX - 1 - x];
                v[(long)z * NX + NX - 1 - x] = t;
            }
    for (long i = 0; i < (long)NZ * NX; ++i) {
        float r = v[i] * tao / h;
        float r2 = (float)(pow(r, 2) / 2);
        r1[i] = (float)sqrt(r2);
    }
}

/* Velocity range and bin bookkeeping of kernel.cu:704-742: vmin/vmax are
 * snapped outward to multiples of dv, nvel = int((vmax-vmin)/dv+1.5), and
 * need[k]=1 for every bin k = int((v-vmin)/dv+0.5) that occurs.
 * need must hold at least nvel ints; call with need=NULL to get nvel. */
int or_bin_velocity(const float *v, long ncell, float dv, float *vmin_out, float *vmax_out,
                    int *need, int need_cap)
{
    float vmin = v[0], vmax = v[0], vel;
    for (long i = 0; i < ncell; ++i) {
        if (v[i] < vmin) vmin = v[i];
        if (v[i] > vmax) vmax = v[i];
    }
    vel = ((int)(vmin / dv)) * dv;
    vmin = (vel > vmin) ? vel - dv : vel;
    vel = ((int)(vmax / dv)) * dv;
    vmax = (vel < vmax) ? vel + dv : vel;
    int nvel = (int)((vmax - vmin) / dv + 1.5);
    *vmin_out = vmin;
    *vmax_out = vmax;
    if (need) {
        if (need_cap < nvel) return -1;
        for (int k = 0; k < nvel; ++k) need[k] = 0;
        for (long i = 0; i < ncell; ++i) need[(int)((v[i] - vmin) / dv + 0.5)] = 1;
    }
    return nvel;
}

/* ---- per-shot image finishing (kernel.cu:935-990) ------------------------
 * up   = -(Laplacian of rel1)*v^2/vmax^2 on the interior, with even
 *        reflection at the interior edges;
 * down = rel2 + whitecoe*max|rel2| on the interior.
 * Both are written column-major (nx columns of nz), as the reference writes
 * its per-shot files. rel1/rel2 are full padded grids (FP32). */
void or_finish_shot_f32(const float *rel1, const float *rel2, const float *v, int NZ, int NX,
                        int N2, float vmax, float whitecoe, float *up, float *down)
{
    int nz = NZ - 2 * N2, nx = NX - 2 * N2;
    for (int j = N2; j < NX - N2; ++j)
        for (int i = N2; i < NZ - N2; ++i) {
            int i1 = i - 1, i2 = i + 1, j1 = j - 1, j2 = j + 1;
            if (i1 < N2) i1 = 2 * N2 - i1;
            if (j1 < N2) j1 = 2 * N2 - j1;
            if (i2 >= NZ - N2) i2 = 2 * (NZ - N2 - 1) - i2;
            if (j2 >= NX - N2) j2 = 2 * (NX - N2 - 1) - j2;
            float s = rel1[(long)i * NX + j2] + rel1[(long)i * NX + j1] + rel1[(long)i2 * NX + j] +
                      rel1[(long)i1 * NX + j] - 4 * rel1[(long)i * NX + j];
            float vv = v[(long)i * NX + j];
            up[(long)(j - N2) * nz + (i - N2)] = (float)(-1.0 * s * vv * vv / (vmax * vmax));
        }
    float mx = 0.0f;
    for (int j = N2; j < NX - N2; ++j)
        for (int i = N2; i < NZ - N2; ++i)
            if (fabs(rel2[(long)i * NX + j]) > mx) mx = (float)fabs(rel2[(long)i * NX + j]);
    float stable = mx * whitecoe;
    for (int j = N2; j < NX - N2; ++j)
        for (int i = N2; i < NZ - N2; ++i)
            down[(long)(j - N2) * nz + (i - N2)] = rel2[(long)i * NX + j] + stable;
    (void)nx;
}

/* FP64 version of the finishing step (the FP64 oracle's image). */
void or_finish_shot_f64(const double *rel1, const double *rel2, const float *v, int NZ, int NX,
                        int N2, float vmax, float whitecoe, double *up, double *down)
{
    int nz = NZ - 2 * N2;
    for (int j = N2; j < NX - N2; ++j)
        for (int i = N2; i < NZ - N2; ++i) {
            int i1 = i - 1, i2 = i + 1, j1 = j - 1, j2 = j + 1;
            if (i1 < N2) i1 = 2 * N2 - i1;
            if (j1 < N2) j1 = 2 * N2 - j1;
            if (i2 >= NZ - N2) i2 = 2 * (NZ - N2 - 1) - i2;
            if (j2 >= NX - N2) j2 = 2 * (NX - N2 - 1) - j2;
            double s = rel1[(long)i * NX + j2] + rel1[(long)i * NX + j1] +
                       rel1[(long)i2 * NX + j] + rel1[(long)i1 * NX + j] - 4 * rel1[(long)i * NX + j];
            double vv = v[(long)i * NX + j];
            up[(long)(j - N2) * nz + (i - N2)] = -1.0 * s * vv * vv / ((double)vmax * vmax);
        }
    double mx = 0.0;
    for (int j = N2; j < NX - N2; ++j)
        for (int i = N2; i < NZ - N2; ++i)
            if (fabs(rel2[(long)i * NX + j]) > mx) mx = fabs(rel2[(long)i * NX + j]);
    double stable = mx * whitecoe;
    for (int j = N2; j < NX - N2; ++j)
        for (int i = N2; i < NZ - N2; ++i)
            down[(long)(j - N2) * nz + (i - N2)] = rel2[(long)i * NX + j] + stable;
}

/* ---- stack (kernel.cu:992-1059) ------------------------------------------
 * ups/downs hold nshot per-shot images of ncell values each.  The reference
 * sums them in shot order in float, divides by nrec and, when inorm, divides
 * the image by the stacked illumination.  kahan=1 replaces the plain float
 * sums by compensated sums (same order, same final divisions). */
void or_stack_f32(const float *ups, const float *downs, int nshot, long ncell, int nrec,
                  int inorm, int kahan, float *img, float *illum)
{
    for (long i = 0; i < ncell; ++i) {
        float s1 = 0, s2 = 0, c1 = 0, c2 = 0;
        for (int m = 0; m < nshot; ++m) {
            float a = ups[(long)m * ncell + i], b = downs[(long)m * ncell + i];
            if (kahan) {
                float y1 = a - c1, t1 = s1 + y1;
                c1 = (t1 - s1) - y1;
                s1 = t1;
                float y2 = b - c2, t2 = s2 + y2;
                c2 = (t2 - s2) - y2;
                s2 = t2;
            } else {
                s1 += a;
                s2 += b;
            }
        }
        float g1 = s1 / nrec, g2 = s2 / nrec;
        if (inorm) g1 = g1 / g2;
        img[i] = g1;
        illum[i] = g2;
    }
}

void or_stack_f64(const double *ups, const double *downs, int nshot, long ncell, int nrec,
                  int inorm, double *img, double *illum)
{
    for (long i = 0; i < ncell; ++i) {
        double s1 = 0, s2 = 0;
        for (int m = 0; m < nshot; ++m) {
            s1 += ups[(long)m * ncell + i];
            s2 += downs[(long)m * ncell + i];
        }
        double g1 = s1 / nrec, g2 = s2 / nrec;
        if (inorm) g1 = g1 / g2;
        img[i] = g1;
        illum[i] = g2;
    }
}
