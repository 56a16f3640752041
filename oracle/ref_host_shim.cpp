/*
 * Host routines of the reference used by the oracle's pin tests, compiled
 * from a caixh90/RTM_GPU checkout by build_ref.py into
 * oracle/_ref/libref_host.so.  TEST INFRASTRUCTURE ONLY.
 *   - LSMOrCon_rec_2D.cpp (least-squares FD coefficients, Taylor order())
 *   - GPU_velocity_real.cpp (velocity file reader and ABC padding)
 *   - Resample.cpp (trace resampling, 8-point sinc interpolation)
 * All are included in place, unmodified, from the checkout's directory.
 */
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "LSMOrCon_rec_2D.cpp"
#include "GPU_velocity_real.cpp"
#include "Resample.cpp"

extern "C" {

/* ---- host routines of the reference ---- */
void ref_order(int N, float *c) { order(N, c); }

void ref_cal2dfdcoe(double *c, double r, double bb, int M, double hzx) { CAL2DFDCOE_LSM(c, r, bb, M, hzx); }

int ref_callenfd(int nfdmin, int nfdmax, double vel, double tao, double h, double df, int nfre,
                 int nthita, double eps, double hzx)
{
    double *hk = (double *)malloc(sizeof(double) * nfre);
    double *de = (double *)malloc(sizeof(double) * nfre);
    int len = 0;
    callenfd2d_ls(hk, de, nfre, nfdmin, nfdmax, vel, tao, h, df, nthita, eps, &len, 0, hzx);
    free(hk);
    free(de);
    return len;
}

/* funMandC with caller-provided outputs: M[nvel], Index[nvel+1]; returns NC
 * and copies the float table into c (capacity ccap). */
int ref_funMandC(int nthita, int nfdmax, int nfdmin, int nvel, double tao, double h, double df,
                 double eps, double fmax, double vmin, double vmax, double dv, int *need, int *M,
                 int *Index, float *c, int ccap, double hzx)
{
    float *cc = nullptr;
    int NC = funMandC(nthita, nfdmax, nfdmin, nvel, tao, h, df, eps, fmax, vmin, vmax, dv, need, M,
                      Index, 0, &cc, hzx);
    if (NC <= ccap) memcpy(c, cc, sizeof(float) * NC);
    free(cc);
    return NC;
}

void ref_velocity(char *path, float *v, float *v_2, float *r, float *r_1, float *r_2, int NZ, int NX,
                  int N2, float tao, float h, int choice)
{
    velocity(path, v, v_2, r, r_1, r_2, NZ, NX, NZ * NX, N2, tao, h, choice);
}

void ref_resample(int nxin, float dxin, float *yin, int nxout, float dxout, float *yout)
{
    resample(nxin, dxin, yin, nxout, dxout, yout);
}

} /* extern "C" */
