/*
 * Trace resampling as the reference does it when the data sample interval
 * differs from the modelling step (kernel.cu:839-845 calling resample(),
 * Resample.cpp:193-225).  TEST INFRASTRUCTURE ONLY.
 *
 * The reference's routine is Seismic Unix's 8-point least-squares sinc
 * interpolator (CWP/SU, D. Hale: resample -> intt8r with a 513-row table of
 * mksinc() filters, each the solution of a symmetric Toeplitz system by
 * Levinson recursion).  Restated here step by step in the same floating
 * point order, so the oracle reproduces the reference's output bit for bit:
 *   table row j (0 < j < 512): the 8 taps for fractional shift d = j/512;
 *     fmax = min(0.066 + 0.265 ln 8, 1), autocorrelation a_k = sinc(fmax k),
 *     crosscorrelation c_k = sinc(fmax (3 - k + d)), taps = a^-1 c (double,
 *     stored as float); rows 0 and 512 are unit impulses at taps 3 and 4;
 *   output sample i at x = i*dxout: u = 8 + x/dxin, m = int(u), taps of row
 *     int(frac(u)*512 + 0.5) applied to inputs m-11 .. m-4 (zero outside).
 */
#include <math.h>

#define RS_TAPS 8
#define RS_ROWS 513

static double rs_sinc(double x)
{
    if (x == 0.0) return 1.0;
    const double px = 3.1415926535898 * x;
    return sin(px) / px;
}

/* Levinson recursion for the symmetric Toeplitz system T f = g with first
 * row t (Claerbout, FGDP p. 57); w is scratch for the prediction filter. */
static void rs_levinson(int n, const double *t, const double *g, double *f, double *w)
{
    if (t[0] == 0.0) return;
    w[0] = 1.0;
    double v = t[0];
    f[0] = g[0] / t[0];
    for (int j = 1; j < n; ++j) {
        w[j] = 0.0;
        f[j] = 0.0;
        double e = 0.0;
        for (int i = 0; i < j; ++i) e += w[i] * t[j - i];
        double k = e / v;
        v -= k * e;
        for (int i = 0; i <= j / 2; ++i) {
            const double hi = w[j - i] - k * w[i];
            w[i] -= k * w[j - i];
            w[j - i] = hi;
        }
        double q = 0.0;
        for (int i = 0; i < j; ++i) q += f[i] * t[j - i];
        k = (q - g[j]) / v;
        for (int i = 0; i <= j; ++i) f[i] -= k * w[j - i];
    }
}

static void rs_filter(float d, float *taps)
{
    double a[RS_TAPS], c[RS_TAPS], s[RS_TAPS], w[RS_TAPS];
    double fmax = 0.066 + 0.265 * log((double)RS_TAPS);
    if (fmax > 1.0) fmax = 1.0;
    for (int k = 0; k < RS_TAPS; ++k) {
        a[k] = rs_sinc(fmax * k);
        /* the shift is formed in float (int + float), as the reference does */
        const float sh = (float)(RS_TAPS / 2 - k - 1) + d;
        c[k] = rs_sinc(fmax * sh);
    }
    rs_levinson(RS_TAPS, a, c, s, w);
    for (int k = 0; k < RS_TAPS; ++k) taps[k] = (float)s[k];
}

/* The 513 x 8 filter table. */
void rs_table(float *tab)
{
    for (int j = 1; j < RS_ROWS - 1; ++j) rs_filter((float)j / (float)(RS_ROWS - 1), tab + j * RS_TAPS);
    for (int k = 0; k < RS_TAPS; ++k) {
        tab[k] = 0.0f;
        tab[(RS_ROWS - 1) * RS_TAPS + k] = 0.0f;
    }
    tab[RS_TAPS / 2 - 1] = 1.0f;
    tab[(RS_ROWS - 1) * RS_TAPS + RS_TAPS / 2] = 1.0f;
}

/* One trace: nxin samples at dxin -> nxout samples at dxout. */
void or_resample(int nxin, float dxin, const float *yin, int nxout, float dxout, float *yout)
{
    static float tab[RS_ROWS * RS_TAPS];
    static int ready = 0;
    if (!ready) {
        rs_table(tab);
        ready = 1;
    }
    const float inv = 1.0 / dxin;          /* double quotient, stored as float */
    const float u0 = 8.0 - 0.0f * inv;     /* first input sample at x = 0 */
    const float rows = (float)(RS_ROWS - 1);
    for (int i = 0; i < nxout; ++i) {
        const float x = i * dxout;
        const float u = u0 + x * inv;
        const int m = (int)u;
        const float fr = u - (float)m;
        const int row = fr >= 0.0 ? (int)(fr * rows + 0.5) : (int)((fr + 1.0) * rows - 0.5);
        const float *t = tab + row * RS_TAPS;
        int k = m - 11;
        float sum = 0.0f;
        for (int j = 0; j < RS_TAPS; ++j, ++k) {
            const float y = (k < 0 || k >= nxin) ? 0.0f : yin[k];
            sum += y * t[j];
        }
        yout[i] = sum;
    }
}
