/*
 * Runs the reference's own code for the RTM hot path on the CPU, to pin the
 * oracle.  TEST INFRASTRUCTURE ONLY.
 *
 * build_ref.py compiles this file into oracle/_ref/libref_rtm.so together
 * with the __global__ kernel bodies of kernel.cu (the block from
 * "#define BLOCKSIZE 16" up to the Ricker prototype, kernel.cu:15-517) and
 * the Ricker function f (kernel.cu:1261-1266), which build_ref.py copies
 * verbatim from a caixh90/RTM_GPU checkout into oracle/_ref/ (never into the
 * repository).  The reference's host routines are in ref_host_shim.cpp.
 * Each kernel runs as a plain function over the reference's own launch
 * shape (16x16 blocks over ceil(NZ/16) x ceil(NX/16)), with blockIdx and
 * threadIdx provided as thread-local variables.  The per-shot loop is the
 * shared restatement in rtm_driver_body.h.
 */
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

struct ref_uint3 {
    unsigned x, y, z;
};
static thread_local ref_uint3 blockIdx, threadIdx;
#define __global__

#include "ref_kernels.inc" /* generated from kernel.cu */
#include "ref_ricker.inc"  /* generated from kernel.cu */

extern "C" float ref_ricker(float t, float f0) { return f(t, f0); }

extern "C" {
#include "rtm_oracle.h"
}

template <class F>
static void grid_run(int NZ, int NX, F body)
{
    int gx = (NZ + BLOCKSIZE - 1) / BLOCKSIZE, gy = (NX + BLOCKSIZE - 1) / BLOCKSIZE;
#pragma omp parallel for collapse(2) schedule(static)
    for (int bx = 0; bx < gx; ++bx)
        for (int by = 0; by < gy; ++by) {
            blockIdx.x = bx;
            blockIdx.y = by;
            blockIdx.z = 0;
            for (int tx = 0; tx < BLOCKSIZE; ++tx)
                for (int ty = 0; ty < BLOCKSIZE; ++ty) {
                    threadIdx.x = tx;
                    threadIdx.y = ty;
                    threadIdx.z = 0;
                    body();
                }
        }
}

extern "C" {

/* ---- single kernels, reference argument lists ---- */
void ref_k_Equal(float *Dlf, float *Drt, float *Dup, float *Ddw, float *DFW0, float *DFW1, int NZ,
                 int NX, int N2, int nfdmax)
{
    grid_run(NZ, NX, [&] { Equal(Dlf, Drt, Dup, Ddw, DFW0, DFW1, NZ, NX, N2, nfdmax); });
}
void ref_k_Add(float *Dv, float *DFW2, float *DFW0, float *DFW1, float *Dc, int *DIndex, float tao2,
               float h2, float vmin, float dv, int nfdmax, int NZ, int NX, int NXZ, int r_u,
               int r_x, float wavelet, float hzx2_1)
{
    grid_run(NZ, NX, [&] {
        Add(Dv, DFW2, DFW0, DFW1, Dc, DIndex, tao2, h2, vmin, dv, nfdmax, NZ, NX, NXZ, r_u, r_x,
            wavelet, hzx2_1);
    });
}
void ref_k_Add_Con(float *Dv, float *DFW2, float *DFW0, float *DFW1, float *Dc, float tao2, float h2,
                   int nfdmax, int NZ, int NX, int NXZ, int r_u, int r_x, float wavelet, float hzx2_1)
{
    grid_run(NZ, NX, [&] {
        Add_Con(Dv, DFW2, DFW0, DFW1, Dc, tao2, h2, nfdmax, NZ, NX, NXZ, r_u, r_x, wavelet, hzx2_1);
    });
}
void ref_k_Hybrid1(float *DFW1, float *DFW0, float *DFW2, float *DFWb, float *Dlf, float *Drt,
                   float *Dup, float *Ddw, float *Dv, float *Dr_1, float *Dw, int NZ, int NX, int N2,
                   int nfdmax, int k, float taoh, float taoh2)
{
    grid_run(NZ, NX, [&] {
        Hybrid1(DFW1, DFW0, DFW2, DFWb, Dlf, Drt, Dup, Ddw, Dv, Dr_1, Dw, NZ, NX, N2, nfdmax, k,
                taoh, taoh2);
    });
}
void ref_k_Hybrid2(float *DFW1, float *DFW0, float *DFW2, float *DFWb, float *Dlf, float *Drt,
                   float *Dup, float *Ddw, float *Dv, float *Dr_1, float *Dw, int NZ, int NX, int N2,
                   int nfdmax, int k, float taoh, float taoh2)
{
    grid_run(NZ, NX, [&] {
        Hybrid2(DFW1, DFW0, DFW2, DFWb, Dlf, Drt, Dup, Ddw, Dv, Dr_1, Dw, NZ, NX, N2, nfdmax, k,
                taoh, taoh2);
    });
}
void ref_k_Hybrid3(float *DFW1, float *DFW0, float *DFW2, float *DFWb, float *Dlf, float *Drt,
                   float *Dup, float *Ddw, float *Dv, float *Dr_1, float *Dw, int NZ, int NX, int N2,
                   int nfdmax, int k, float taoh, float taoh2)
{
    grid_run(NZ, NX, [&] {
        Hybrid3(DFW1, DFW0, DFW2, DFWb, Dlf, Drt, Dup, Ddw, Dv, Dr_1, Dw, NZ, NX, N2, nfdmax, k,
                taoh, taoh2);
    });
}
void ref_k_Deliver(float *DFW1, float *DFW0, float *DFW2, int NZ, int NX)
{
    grid_run(NZ, NX, [&] { Deliver(DFW1, DFW0, DFW2, NZ, NX); });
}
void ref_k_BKEqual(float *Dlf, float *Drt, float *Dup, float *Ddw, float *DFW1, int NZ, int NX,
                   int N2, int nfdmax, int k)
{
    grid_run(NZ, NX, [&] { BKEqual(Dlf, Drt, Dup, Ddw, DFW1, NZ, NX, N2, nfdmax, k); });
}
void ref_k_BKAdd_EFF(float *Dv, float *DFW2, float *DFW0, float *DFW1, float *Dc, int *DIndex,
                     float tao2, float h2, float vmin, float dv, int N2, int NZ, int NX, int NXZ,
                     int r_u, int r_x, float wavelet, float hzx2_1)
{
    grid_run(NZ, NX, [&] {
        BKAdd_EFF(Dv, DFW2, DFW0, DFW1, Dc, DIndex, tao2, h2, vmin, dv, N2, NZ, NX, NXZ, r_u, r_x,
                  wavelet, hzx2_1);
    });
}
void ref_k_BKAdd_EFF_Con(float *Dv, float *DFW2, float *DFW0, float *DFW1, float *Dc, float tao2,
                         float h2, int N2, int NZ, int NX, int NXZ, int r_u, int r_x, int nfdmax,
                         float wavelet, float hzx2_1)
{
    grid_run(NZ, NX, [&] {
        BKAdd_EFF_Con(Dv, DFW2, DFW0, DFW1, Dc, tao2, h2, N2, NZ, NX, NXZ, r_u, r_x, nfdmax, wavelet,
                      hzx2_1);
    });
}
void ref_k_Deliver_EFF(float *DFW1, float *DFW0, float *DFW2, int N2, int NZ, int NX)
{
    grid_run(NZ, NX, [&] { Deliver_EFF(DFW1, DFW0, DFW2, N2, NZ, NX); });
}
void ref_k_BKAdd(float *Dv, float *DBW2, float *DBW1, float *DBW0, float *Dc, int *DIndex,
                 float *Dseis, float tao2, float h2, float vmin, float dv, int nfdmax, int NZ,
                 int NX, int NXZ, int s_l, int s_r, int s_z, int ds, float hzx2_1)
{
    grid_run(NZ, NX, [&] {
        BKAdd(Dv, DBW2, DBW1, DBW0, Dc, DIndex, Dseis, tao2, h2, vmin, dv, nfdmax, NZ, NX, NXZ, s_l,
              s_r, s_z, ds, hzx2_1);
    });
}
void ref_k_BKAdd_Con(float *Dv, float *DBW2, float *DBW1, float *DBW0, float *Dc, float *Dseis,
                     float tao2, float h2, int nfdmax, int NZ, int NX, int NXZ, int s_l, int s_r,
                     int s_z, int ds, float hzx2_1)
{
    grid_run(NZ, NX, [&] {
        BKAdd_Con(Dv, DBW2, DBW1, DBW0, Dc, Dseis, tao2, h2, nfdmax, NZ, NX, NXZ, s_l, s_r, s_z, ds,
                  hzx2_1);
    });
}
void ref_k_BKHybrid1(float *DFW1, float *DFW0, float *DFW2, float *DFWb, float *Dv, float *Dr_1,
                     float *Dw, int NZ, int NX, int N2, float taoh, float taoh2)
{
    grid_run(NZ, NX, [&] { BKHybrid1(DFW1, DFW0, DFW2, DFWb, Dv, Dr_1, Dw, NZ, NX, N2, taoh, taoh2); });
}
void ref_k_BKHybrid2(float *DFW1, float *DFW0, float *DFW2, float *DFWb, float *Dv, float *Dr_1,
                     float *Dw, int NZ, int NX, int N2, float taoh, float taoh2)
{
    grid_run(NZ, NX, [&] { BKHybrid2(DFW1, DFW0, DFW2, DFWb, Dv, Dr_1, Dw, NZ, NX, N2, taoh, taoh2); });
}
void ref_k_Rel_NonCompen(float *DBW2, float *DFW2, float *Drel1, float *Drel2, int NZ, int NX)
{
    grid_run(NZ, NX, [&] { Rel_NonCompen(DBW2, DFW2, Drel1, Drel2, NZ, NX); });
}
void ref_k_Rel_Compen(float *DBW2, float *DFW2, float *DBWADD, float *DFWADD, float *Drel1,
                      float *Drel2, int NZ, int NX)
{
    grid_run(NZ, NX, [&] { Rel_Compen(DBW2, DFW2, DBWADD, DFWADD, Drel1, Drel2, NZ, NX); });
}

/* ---- per-shot loop over the reference kernels ---- */
#define REAL float
#define DRV_NAME(n) ref_##n
#define K_EQUAL(lf_, rt_, up_, dw_, a0, a1) \
    grid_run(P->NZ, P->NX, [&] { Equal(lf_, rt_, up_, dw_, a0, a1, P->NZ, P->NX, P->N2, P->M); })
#define K_ADD(a2, a0, a1, wv)                                                                        \
    grid_run(P->NZ, P->NX, [&] {                                                                     \
        if (P->adaptive)                                                                             \
            Add((float *)v, a2, a0, a1, (float *)c, (int *)idx, P->tao2, P->h2, P->vmin, P->dv, P->M, \
                P->NZ, P->NX, P->NZ * P->NX, P->r_u, P->r_x, wv, P->hzx2_1);                         \
        else                                                                                         \
            Add_Con((float *)v, a2, a0, a1, (float *)c, P->tao2, P->h2, P->M, P->NZ, P->NX,          \
                    P->NZ * P->NX, P->r_u, P->r_x, wv, P->hzx2_1);                                   \
    })
#define K_HYB1(a1, a0, a2, bb)                                                                      \
    grid_run(P->NZ, P->NX, [&] {                                                                    \
        Hybrid1(a1, a0, a2, bb, lf, rt, up, dw, (float *)v, (float *)r1, (float *)w, P->NZ, P->NX, \
                P->N2, P->M, 0, P->taoh, P->taoh2);                                                 \
    })
#define K_HYB2(a1, a0, a2, bb)                                                                      \
    grid_run(P->NZ, P->NX, [&] {                                                                    \
        Hybrid2(a1, a0, a2, bb, lf, rt, up, dw, (float *)v, (float *)r1, (float *)w, P->NZ, P->NX, \
                P->N2, P->M, 0, P->taoh, P->taoh2);                                                 \
    })
#define K_HYB3(a1, a0, a2, bb, kk)                                                                  \
    grid_run(P->NZ, P->NX, [&] {                                                                    \
        Hybrid3(a1, a0, a2, bb, lf, rt, up, dw, (float *)v, (float *)r1, (float *)w, P->NZ, P->NX, \
                P->N2, P->M, kk, P->taoh, P->taoh2);                                                \
    })
#define K_DELIVER(a1, a0, a2) grid_run(P->NZ, P->NX, [&] { Deliver(a1, a0, a2, P->NZ, P->NX); })
#define K_BKEQUAL(a1, kk) \
    grid_run(P->NZ, P->NX, [&] { BKEqual(lf, rt, up, dw, a1, P->NZ, P->NX, P->N2, P->M, kk); })
#define K_BKADD_EFF(a2, a0, a1, wv)                                                                  \
    grid_run(P->NZ, P->NX, [&] {                                                                     \
        if (P->adaptive)                                                                             \
            BKAdd_EFF((float *)v, a2, a0, a1, (float *)c, (int *)idx, P->tao2, P->h2, P->vmin, P->dv, \
                      P->N2, P->NZ, P->NX, P->NZ * P->NX, P->r_u, P->r_x, wv, P->hzx2_1);            \
        else                                                                                         \
            BKAdd_EFF_Con((float *)v, a2, a0, a1, (float *)c, P->tao2, P->h2, P->N2, P->NZ, P->NX,   \
                          P->NZ * P->NX, P->r_u, P->r_x, P->M, wv, P->hzx2_1);                       \
    })
#define K_DELIVER_EFF(a1, a0, a2) \
    grid_run(P->NZ, P->NX, [&] { Deliver_EFF(a1, a0, a2, P->N2, P->NZ, P->NX); })
#define K_BKADD(a2, a1, a0, sd)                                                                       \
    grid_run(P->NZ, P->NX, [&] {                                                                      \
        if (P->adaptive)                                                                              \
            BKAdd((float *)v, a2, a1, a0, (float *)c, (int *)idx, sd, P->tao2, P->h2, P->vmin, P->dv, \
                  P->M, P->NZ, P->NX, P->NZ * P->NX, P->s_l, P->s_r, P->s_z, P->ds, P->hzx2_1);       \
        else                                                                                          \
            BKAdd_Con((float *)v, a2, a1, a0, (float *)c, sd, P->tao2, P->h2, P->M, P->NZ, P->NX,     \
                      P->NZ * P->NX, P->s_l, P->s_r, P->s_z, P->ds, P->hzx2_1);                       \
    })
#define K_BKHYB1(a1, a0, a2, bb)                                                              \
    grid_run(P->NZ, P->NX, [&] {                                                              \
        BKHybrid1(a1, a0, a2, bb, (float *)v, (float *)r1, (float *)w, P->NZ, P->NX, P->N2,   \
                  P->taoh, P->taoh2);                                                         \
    })
#define K_BKHYB2(a1, a0, a2, bb)                                                              \
    grid_run(P->NZ, P->NX, [&] {                                                              \
        BKHybrid2(a1, a0, a2, bb, (float *)v, (float *)r1, (float *)w, P->NZ, P->NX, P->N2,   \
                  P->taoh, P->taoh2);                                                         \
    })
#define K_REL(S, R, SA, RA, q1, q2)                                                 \
    grid_run(P->NZ, P->NX, [&] {                                                    \
        if (P->compen)                                                              \
            Rel_Compen(R, S, RA, SA, q1, q2, P->NZ, P->NX);                         \
        else                                                                        \
            Rel_NonCompen(R, S, q1, q2, P->NZ, P->NX);                              \
    })
#include "rtm_driver_body.h"

} /* extern "C" */
