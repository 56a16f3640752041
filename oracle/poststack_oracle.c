/*
 * The reference's post-stack display chain, restated in C for the oracle.
 * TEST INFRASTRUCTURE ONLY.
 *
 *   or_d2t   DisToTimeAndTimeToDis1D.cpp:120-180 (D2T): two-way time of every
 *            depth sample, t_j = sum_{i=1..j} 2 dz / v_i (t_0 = 0), then the
 *            trace linearly interpolated onto a regular time grid;
 *   or_t2d   DisToTimeAndTimeToDis1D.cpp:30-118 (T2D): depth of every time
 *            sample, z_j = sum dt v(int(z)/dz)/2 with the velocity index
 *            clamped, then interpolated onto a regular depth grid;
 *   or_phase phase_correction_ricker_decon.cpp:160-224 (phase_correction):
 *            every trace's spectrum rotated by a constant angle.
 *
 * Same floating-point order as the reference, so the outputs match it bit
 * for bit (phase rotation: up to the last bit of libm's atan / cos / sin).
 * The reference leaves the first entry of its time/depth table
 * uninitialised; large allocations come back zeroed, and that is what is
 * taken here (t_0 = 0).
 */
#include <math.h>
#include <stdlib.h>

/* DisToTimeAndTimeToDis1D.cpp:7-26 (interpolate): out[0] = y[0]; sample j of
 * the regular grid (spacing d) from the segment i with k(i-1) < j <= k(i),
 * k(i) = int(x_i/d); samples beyond the last segment keep their value. */
static void pt_interp(float *out, const float *x, const float *y, int nout, int nin, float d)
{
    int k1 = 0;
    out[0] = y[0];
    for (int i = 1; i < nin; ++i) {
        const int k2 = (int)(x[i] / d);
        for (int j = k1 + 1; j <= k2; ++j) {
            if (j == nout) continue;
            out[j] = y[i - 1] + (j * d - x[i - 1]) / (x[i] - x[i - 1]) * (y[i] - y[i - 1]);
        }
        k1 = k2;
    }
}

/* v, img: [ntr][nz]; out: [ntr][nt] with nt returned (cap: capacity; out may
 * be NULL to query). */
int or_d2t(const float *v, const float *img, int ntr, int nz, float dz, float dt, float *out,
           long cap)
{
    float *t = (float *)calloc((size_t)ntr * nz, sizeof(float));
    float tmax = 0;
    for (int i = 0; i < ntr; ++i) {
        float acc = 0;
        for (int j = 1; j < nz; ++j) {
            acc += 2 * dz / v[(size_t)i * nz + j];
            t[(size_t)i * nz + j] = acc;
        }
        if (tmax < acc) tmax = acc;
    }
    const int nt = (int)(tmax / dt);
    if (out) {
        if ((long)nt * ntr > cap) {
            free(t);
            return -1;
        }
        for (long q = 0; q < (long)nt * ntr; ++q) out[q] = 0.0f;
        for (int i = 0; i < ntr; ++i)
            pt_interp(out + (size_t)i * nt, t + (size_t)i * nz, img + (size_t)i * nz, nt, nz, dt);
    }
    free(t);
    return nt;
}

/* v: [ntr][nzv] depth velocities; img: [ntr][nt] time traces at dt; out:
 * [ntr][nz] at dz with nz returned. */
int or_t2d(const float *v, int nzv, const float *img, int ntr, int nt, float dt, float dz, float *out,
           long cap)
{
    float *z = (float *)calloc((size_t)ntr * nt, sizeof(float));
    float zmax = 0;
    for (int i = 0; i < ntr; ++i) {
        float acc = 0;
        for (int j = 1; j < nt; ++j) {
            int jv = (int)((int)acc / dz);
            if (jv >= nzv) jv = nzv - 1;
            acc += dt * v[(size_t)i * nzv + jv] / 2;
            z[(size_t)i * nt + j] = acc;
        }
        if (zmax < acc) zmax = acc;
    }
    const int nz = (int)(zmax / dz);
    if (out) {
        if ((long)nz * ntr > cap) {
            free(z);
            return -1;
        }
        for (long q = 0; q < (long)nz * ntr; ++q) out[q] = 0.0f;
        for (int i = 0; i < ntr; ++i)
            pt_interp(out + (size_t)i * nz, z + (size_t)i * nt, img + (size_t)i * nt, nz, nt, dz);
    }
    free(z);
    return nz;
}

/* Radix-2 FFT of n = 2^k points in the reference's formulation
 * (phase_correction_ricker_decon.cpp:326-389, the published "kbfft"
 * routine): bit-reversed copy into (fr, fi), twiddles w_i by the recurrence
 * w_i = w_{i-1} w_1 with the three-multiply complex product and
 * w_1 = exp(-+2 pi i / n) using 6.283185306 for 2 pi, radix-2 stages,
 * 1/n scaling for the inverse (inv != 0), and with amp != 0 the amplitude
 * |F|/(n/2) and phase (degrees +-90 when the real part is negligible,
 * radians otherwise) left in (pr, pi). */
void or_fft(double *pr, double *pi, int n, int k, double *fr, double *fi, int inv, int amp)
{
    for (int it = 0; it < n; ++it) {
        int m = it, is = 0;
        for (int i = 0; i < k; ++i) {
            const int j = m / 2;
            is = 2 * is + (m - 2 * j);
            m = j;
        }
        fr[it] = pr[is];
        fi[it] = pi[is];
    }
    pr[0] = 1.0;
    pi[0] = 0.0;
    double p = 6.283185306 / (1.0 * n);
    pr[1] = cos(p);
    pi[1] = -sin(p);
    if (inv) pi[1] = -pi[1];
    for (int i = 2; i < n; ++i) {
        const double a = pr[i - 1] * pr[1], b = pi[i - 1] * pi[1];
        const double c = (pr[i - 1] + pi[i - 1]) * (pr[1] + pi[1]);
        pr[i] = a - b;
        pi[i] = c - a - b;
    }
    for (int it = 0; it < n - 1; it += 2) {
        const double vr = fr[it], vi = fi[it];
        fr[it] = vr + fr[it + 1];
        fi[it] = vi + fi[it + 1];
        fr[it + 1] = vr - fr[it + 1];
        fi[it + 1] = vi - fi[it + 1];
    }
    int m = n / 2, nv = 2;
    for (int l0 = k - 2; l0 >= 0; --l0) {
        m /= 2;
        nv *= 2;
        for (int it = 0; it <= (m - 1) * nv; it += nv)
            for (int j = 0; j < nv / 2; ++j) {
                const int h = it + j + nv / 2;
                const double a = pr[m * j] * fr[h], b = pi[m * j] * fi[h];
                double c = pr[m * j] + pi[m * j];
                c = c * (fr[h] + fi[h]);
                const double dr = a - b, di = c - a - b;
                fr[h] = fr[it + j] - dr;
                fi[h] = fi[it + j] - di;
                fr[it + j] = fr[it + j] + dr;
                fi[it + j] = fi[it + j] + di;
            }
    }
    if (inv)
        for (int i = 0; i < n; ++i) {
            fr[i] = fr[i] / (1.0 * n);
            fi[i] = fi[i] / (1.0 * n);
        }
    if (amp)
        for (int i = 0; i < n; ++i) {
            pr[i] = sqrt(fr[i] * fr[i] + fi[i] * fi[i]);
            pr[i] = pr[i] / (n / 2);
            if (fabs(fr[i]) < 0.000001 * fabs(fi[i]))
                pi[i] = (fi[i] * fr[i] > 0) ? 90.0 : -90.0;
            else
                pi[i] = atan(fi[i] / fr[i]);
        }
}

/* din, dout: [ntr][nt]; angle in degrees. */
void or_phase(const float *din, float *dout, int ntr, int nt, float angle)
{
    const double theta = angle * 3.1415926535898 / 180;
    int n = 2, k = 1;
    while (n < nt) {
        n *= 2;
        ++k;
    }
    const double cs = cos(theta), sn = sin(theta);
    const int h = n / 2;
    double *pr = (double *)malloc(sizeof(double) * n), *pi = (double *)malloc(sizeof(double) * n);
    double *fr = (double *)malloc(sizeof(double) * n), *fi = (double *)malloc(sizeof(double) * n);
    for (int tr = 0; tr < ntr; ++tr) {
        for (int i = 0; i < n; ++i) {
            pr[i] = i < nt ? din[(size_t)tr * nt + i] : 0.0;
            pi[i] = 0.0;
        }
        or_fft(pr, pi, n, k, fr, fi, 0, 1);
        for (int i = 1; i < h; ++i) {
            pr[i] = fr[i] * cs - fi[i] * sn;
            pi[i] = fi[i] * cs + fr[i] * sn;
        }
        for (int i = n - 1; i > h; --i) {
            pr[i] = pr[n - i];
            pi[i] = -pi[n - i];
        }
        or_fft(pr, pi, n, k, fr, fi, 1, 0);
        for (int i = 0; i < nt; ++i) dout[(size_t)tr * nt + i] = (float)fr[i];
    }
    free(pr);
    free(pi);
    free(fr);
    free(fi);
}
