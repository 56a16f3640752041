/*
 * Least-squares optimal finite-difference coefficients with adaptive
 * operator length, restated from LSMOrCon_rec_2D.cpp (FP64, CPU).
 *
 * TEST INFRASTRUCTURE ONLY (part of the CPU oracle; see rtm_oracle.c).  The
 * product computes the same tables on the GPU (rtm_gpu_gb300/csrc/
 * rtm_coeffs.cu); this file is the checker for it.
 *
 * The arithmetic follows the reference operation for operation (same
 * quadrature nodes and accumulation order, same elimination order) so the
 * results match its CPU build bit for bit when both are compiled without
 * multiply-add contraction.
 */
#include <math.h>
#include <stdlib.h>

#define LS_PI 3.1415926535898 /* LSMOrCon_rec_2D.cpp:4 */

/* 5-point Gauss-Legendre nodes and weights as tabulated (10 digits) in
 * LSMOrCon_rec_2D.cpp:142-145. */
static const double GL_T[5] = {-0.9061798459, -0.5384693101, 0.0, 0.5384693101, 0.9061798459};
static const double GL_W[5] = {0.2369268851, 0.4786286705, 0.5688888889, 0.4786286705, 0.2369268851};

/* Normal-equation integrand of LSMOrCon_rec_2D.cpp:216-233: with
 * g_l(th,kh) = ((1+1/hzx^2) - cos(l*kh*cos th) - cos(hzx*l*kh*sin th)/hzx^2)
 *              / (r^-2 (1-cos(r*kh))),
 * returns g_i*g_j (prod=1) or g_i (prod=0). */
static double ls_integrand(double th, double kh, int ai, int aj, double r, int prod, double hzx)
{
    double hzx2 = hzx * hzx;
    double c = cos(th), s = sin(th);
    double p = pow(r, -2);
    double car = cos(r * kh);
    double f1 = ((1 + 1 / hzx2) - cos(ai * kh * c) - cos(hzx * ai * kh * s) / hzx2) / (p * (1 - car));
    if (!prod) return f1;
    double f2 = ((1 + 1 / hzx2) - cos(aj * kh * c) - cos(hzx * aj * kh * s) / hzx2) / (p * (1 - car));
    return f1 * f2;
}

/* Composite Gauss-Legendre rule over th in [0,2pi] (outer) and kh in [0,bb]
 * (inner), 4 panels x 5 nodes per axis (fgaus with js={4,4},
 * LSMOrCon_rec_2D.cpp:139-214).  The panel centres advance by repeated
 * addition and the sums are accumulated node by node in the same order as
 * the reference, so the rounding matches. */
double ls_quad(int ai, int aj, double bb, double r, int prod, double hzx)
{
    const int npan = 4;
    double h0 = 0.5 * (2 * LS_PI - 0.0) / npan;
    double b0 = h0 + 0.0;
    double outer = 0.0;
    for (int p0 = 0; p0 < npan; ++p0) {
        if (p0 > 0) b0 = b0 + h0 * 2.0;
        for (int n0 = 0; n0 < 5; ++n0) {
            double th = h0 * GL_T[n0] + b0;
            double h1 = 0.5 * (bb - 0.0) / npan;
            double b1 = h1 + 0.0;
            double inner = 0.0;
            for (int p1 = 0; p1 < npan; ++p1) {
                if (p1 > 0) b1 = b1 + h1 * 2.0;
                for (int n1 = 0; n1 < 5; ++n1) {
                    double kh = h1 * GL_T[n1] + b1;
                    double f = ls_integrand(th, kh, ai, aj, r, prod, hzx);
                    inner = 1.0 * 1.0 * f * GL_W[n1] + inner;
                }
            }
            outer = inner * h1 * 1.0 * GL_W[n0] + outer;
        }
    }
    return outer * h0;
}

/* Row-scaled Gaussian elimination with partial pivoting
 * (LSMOrCon_rec_2D.cpp:74-137).  A is n*n row-major and is overwritten.
 * Returns 0 if a row is numerically zero. */
int ls_gauss(double *A, int n, double *b, double *x)
{
    for (int i = 0; i < n; ++i) {
        double mx = A[i * n + 0];
        for (int j = 0; j < n; ++j)
            if (fabs(A[i * n + j]) > fabs(mx)) mx = A[i * n + j];
        if (fabs(mx) < 1e-10) return 0;
        for (int j = 0; j < n; ++j) A[i * n + j] = A[i * n + j] / mx;
        b[i] = b[i] / mx;
    }
    for (int i = 0; i < n - 1; ++i) {
        int k = i;
        for (int j = i; j < n; ++j)
            if (fabs(A[j * n + i]) > fabs(A[k * n + i])) k = j;
        if (k != i) {
            double t = b[i];
            b[i] = b[k];
            b[k] = t;
            for (int j = i; j < n; ++j) {
                t = A[i * n + j];
                A[i * n + j] = A[k * n + j];
                A[k * n + j] = t;
            }
        }
        for (int p = i + 1; p < n; ++p) {
            double m = A[p * n + i] / A[i * n + i];
            b[p] = b[p] - m * b[i];
            for (int j = i; j < n; ++j) A[p * n + j] = A[p * n + j] - m * A[i * n + j];
        }
    }
    x[n - 1] = b[n - 1] / A[(n - 1) * n + n - 1];
    for (int i = n - 2; i >= 0; --i) {
        double m = 0.0;
        for (int j = i + 1; j < n; ++j) m = m + A[i * n + j] * x[j];
        x[i] = (b[i] - m) / A[i * n + i];
    }
    return 1;
}

/* LS coefficients c[0..M] for Courant number r and band limit bb = kmax*h
 * (CAL2DFDCOE_LSM, LSMOrCon_rec_2D.cpp:236-287): A_ij = int g_i g_j,
 * b_i = int g_i, solve, c[0] = -2*sum c_l. */
void ls_coefs(double *c, double r, double bb, int M, double hzx)
{
    double *A = (double *)malloc(sizeof(double) * M * M);
    double *b = (double *)malloc(sizeof(double) * M);
    double *x = (double *)malloc(sizeof(double) * M);
    for (int i = 0; i < M; ++i) {
        for (int j = i; j < M; ++j) A[i * M + j] = ls_quad(i + 1, j + 1, bb, r, 1, hzx);
        b[i] = ls_quad(i + 1, M + 1, bb, r, 0, hzx);
    }
    for (int i = 0; i < M; ++i)
        for (int j = 0; j < i; ++j) A[i * M + j] = A[j * M + i];
    ls_gauss(A, M, b, x);
    double s = 0.0;
    for (int i = 1; i <= M; ++i) {
        c[i] = x[i - 1];
        s += c[i];
    }
    c[0] = -2.0 * s;
    free(A);
    free(b);
    free(x);
}

/* Dispersion test of one operator length (the body of the M loop of
 * callenfd2d_ls, LSMOrCon_rec_2D.cpp:321-337).  Returns 1 when the length
 * passes.  Quirks kept: a failure found only at the last angle (n == nthita)
 * does not count, and a NaN error never fails. */
int ls_len_passes(const double *c, int M, double r, const double *hk, int nfre, int nthita,
                  double eps, double ra, double hzx)
{
    double hzx2 = hzx * hzx;
    int k;
    for (k = 1; k < nfre; ++k) {
        double rat = 2 / (r * hk[k]);
        int n;
        for (n = 0; n <= nthita; ++n) {
            double nth = n * LS_PI / (4 * nthita);
            double mid = 0;
            for (int l = 1; l <= M; ++l)
                mid = mid + c[l] * (pow(sin(l * hzx * hk[k] * sin(nth) / 2), 2) / hzx2 +
                                    pow(sin(l * hk[k] * cos(nth) / 2), 2));
            double e = rat * asin(sqrt(r * r * mid));
            e = fabs(ra * (1.0 / e - 1.0));
            if (e > eps) break;
        }
        if (n < nthita) break;
    }
    return k == nfre;
}

/* Shortest operator length >= lstart meeting the dispersion bound at
 * velocity vel (callenfd2d_ls, LSMOrCon_rec_2D.cpp:293-346); nfdmax when
 * none does. */
int ls_min_len(int lstart, int nfdmax, double vel, double tao, double h, double df, int nfre,
               int nthita, double eps, double hzx)
{
    double *hk = (double *)malloc(sizeof(double) * nfre);
    double *c = (double *)calloc(nfdmax + 1, sizeof(double));
    double b = 2.0 * LS_PI * df * h / vel;
    for (int i = 0; i < nfre; ++i) hk[i] = b * i;
    double r = vel * tao / h;
    b = 2 * LS_PI * df * (nfre - 1) * tao / r;
    double ra = h / vel;
    int len = 0;
    for (int j = lstart; j <= nfdmax; ++j) {
        ls_coefs(c, r, b, j, hzx);
        len = j;
        if (ls_len_passes(c, j, r, hk, nfre, nthita, eps, ra, hzx)) break;
    }
    free(hk);
    free(c);
    return len;
}

/* Adaptive operator length for every velocity bin (calfdlen_ls,
 * LSMOrCon_rec_2D.cpp:347-524): a bisection over the bins that assumes the
 * length does not grow with velocity and evaluates only the bins it needs.
 * len[i] is the length of bin i (velocity vmin + i*dv).  Returns the number
 * of bins evaluated, or -1 when an evaluation yields length 0. */
int ls_len_table(int *len, int nvel, int nfdmin, int nfdmax, double tao, double h, double df,
                 int nfre, int nthita, double eps, double vmin, double dv, double hzx)
{
#define EVAL(bin1, start) ls_min_len((start), nfdmax, vmin + ((bin1) - 1) * dv, tao, h, df, nfre, nthita, eps, hzx)
    int ibeg = 1, iend = nvel, num = 0, flag = 0;
    int i1, i2, i3 = 0, i4, l1, l2, l3 = 0, l4, lbeg;
    i1 = ibeg;
    l1 = EVAL(i1, nfdmin); ++num;
    if (l1 == 0) return -1;
    lbeg = l1;
    len[i1 - 1] = l1;
    i2 = iend;
    l2 = EVAL(i2, nfdmin); ++num;
    if (l2 == 0) return -1;
    len[i2 - 1] = l2;
    if (l1 == l2) {
        for (int i = ibeg + 1; i <= iend; ++i) len[i - 1] = l1;
        return num;
    }
    int inc = (iend - ibeg) / (2 * (l1 - l2));
    if (inc < 1) inc = 1;
    for (;;) { /* label a100 */
        i1 = i2 - inc;
        if (i1 < ibeg) {
            i1 = ibeg;
            l1 = lbeg;
            if (i1 == i2) return num;
        } else {
            l1 = EVAL(i1, l2); ++num;
            if (l1 == 0) return -1;
        }
        for (;;) { /* label a200 */
            if (l1 == l2) {
                for (int i = i1; i <= i2 - 1; ++i) len[i - 1] = l1;
                i2 = i1;
                l2 = l1;
            } else if (i1 == i2 - 1) {
                len[i1 - 1] = l1;
                i2 = i1;
                l2 = l1;
            } else {
                i4 = (i1 + i2) / 2;
                if (flag == 0) {
                    flag = 1;
                    i3 = i1;
                    l3 = l1;
                }
                l4 = EVAL(i4, l2); ++num;
                if (l4 == 0) return -1;
                if (l4 == l2) {
                    for (int i = i4; i <= i2 - 1; ++i) len[i - 1] = l2;
                    i2 = i4;
                    l2 = l4;
                } else {
                    i1 = i4;
                    l1 = l4;
                }
                continue; /* goto a200 */
            }
            if (flag == 1) {
                flag = 0;
                if (l3 == l2) {
                    for (int i = i3; i <= i2 - 1; ++i) len[i - 1] = l2;
                    i2 = i3;
                    l2 = l3;
                    break; /* goto a100 */
                }
                i1 = i3;
                l1 = l3;
                continue; /* goto a200 */
            }
            if (l2 == lbeg) {
                for (int i = ibeg; i <= i2 - 1; ++i) len[i - 1] = l2;
                return num;
            }
            break; /* goto a100 */
        }
    }
#undef EVAL
}

/* Coefficient table of funMandC (LSMOrCon_rec_2D.cpp:22-73).
 * Inputs: velocity bins (vmin, dv, nvel), the bins in use need[], the
 * optimiser settings.  Outputs: len[nvel] (operator length, -1 for unused
 * bins), idx[nvel+1] (prefix offsets: bin i owns c[idx[i] .. idx[i+1]-1]),
 * and c[] (float, capacity ccap).  Returns NC = idx[nvel], or -1.
 * Quirk kept: the coefficients of bin i are designed at velocity vmin + i
 * (LSMOrCon_rec_2D.cpp:58), which equals vmin + i*dv only for dv = 1. */
int ls_fun_m_and_c(int nthita, int nfdmax, int nfdmin, int nvel, double tao, double h,
                   double df, double eps, double fmax, double vmin, double dv, const int *need,
                   int *len, int *idx, float *c, int ccap, double hzx)
{
    int nfre = (int)(fmax / df) + 1;
    if (ls_len_table(len, nvel, nfdmin, nfdmax, tao, h, df, nfre, nthita, eps, vmin, dv, hzx) < 0)
        return -1;
    for (int i = 0; i < nvel; ++i)
        if (need[i] == 0) len[i] = -1;
    idx[0] = 0;
    for (int i = 1; i <= nvel; ++i) idx[i] = idx[i - 1] + len[i - 1] + 1;
    int NC = idx[nvel];
    if (!c) return NC;
    if (ccap < NC) return -1;
    double rat = tao / h, ra = 2.0 * LS_PI * fmax * tao;
    /* bins are independent: spread over the host threads (same results) */
#pragma omp parallel
    {
        double *cd = (double *)malloc(sizeof(double) * (nfdmax + 1));
#pragma omp for schedule(dynamic, 8)
        for (int i = 0; i < nvel; ++i)
            if (need[i] == 1) {
                double r = (vmin + i) * rat;
                double b = ra / r;
                ls_coefs(cd, r, b, len[i], hzx);
                for (int l = 0; l <= len[i]; ++l) c[l + idx[i]] = (float)cd[l];
            }
        free(cd);
    }
    return NC;
}

/* Conventional (Taylor) coefficients of order N = 2M (order(),
 * LSMOrCon_rec_2D.cpp:526-551), in float as the reference computes them. */
void ls_taylor(int N, float *c)
{
    int M = N / 2;
    float *x = (float *)malloc(sizeof(float) * (M + 1));
    c[0] = 0.0f;
    for (int i = 0; i <= M; ++i) x[i] = 1.0f;
    for (int i = 1; i <= M; ++i) {
        for (int j = 1; j <= M; ++j)
            if (j != i) x[i] = x[i] * fabs(pow(j, 2) / (pow(j, 2) - pow(i, 2)));
        c[i] = pow(-1, i + 1) / pow(i, 2) * x[i];
        c[0] = (c[0] - 2 * c[i]);
    }
    free(x);
}
