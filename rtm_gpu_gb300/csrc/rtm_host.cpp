// Host-side set-up of the RTM engine (replaces the reference's host set-up
// code) and the library's error reporting.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "../../include/rtm_gb300.h"

static thread_local std::string g_last_error;

void rtm_set_last_error(const char *msg) { g_last_error = msg ? msg : ""; }

extern "C" {

const char *rtm_last_error(void) { return g_last_error.c_str(); }

int rtm_version(void) { return 10000; }

// GPU_velocity_real.cpp:6-118.  The interior model arrives column-major (the
// reference's file order); pad cells copy the nearest interior cell (the
// reference extends the edges and then the corners, which is the same map);
// flip==1 mirrors the padded grid left/right; r_1 = sqrt((v*tao/h)^2/2) with
// the square and root in double, rounded to float.
int rtm_prep_velocity(const float *vin, int nz, int nx, int N2, float tao, float h, int flip,
                      float *v, float *r1)
{
    if (!vin || !v || !r1 || nz < 1 || nx < 1 || N2 < 0) {
        rtm_set_last_error("rtm_prep_velocity: bad argument");
        return RTM_ERR_ARG;
    }
    const int NZ = nz + 2 * N2, NX = nx + 2 * N2;
    for (int z = 0; z < NZ; ++z) {
        const int zi = std::min(std::max(z - N2, 0), nz - 1);
        for (int x = 0; x < NX; ++x) {
            const int xi = std::min(std::max(x - N2, 0), nx - 1);
            v[(long)z * NX + x] = vin[(long)xi * nz + zi];
        }
    }
    if (flip)
        for (int z = 0; z < NZ; ++z)
            for (int x = 0; x < NX / 2; ++x) std::swap(v[(long)z * NX + x], v[(long)z * NX + NX - 1 - x]);
    for (long i = 0; i < (long)NZ * NX; ++i) {
        const float r = v[i] * tao / h;
        const float r2 = (float)(std::pow((double)r, 2) / 2);
        r1[i] = (float)std::sqrt((double)r2);
    }
    return RTM_OK;
}

// kernel.cu:704-742: the velocity range is snapped outward to multiples of
// dv; bins are int((v-vmin)/dv+0.5).
int rtm_prep_bins(const float *v, long ncell, float dv, float *vmin_out, float *vmax_out,
                  int *nvel_out, int *need, int need_cap)
{
    if (!v || ncell < 1 || !(dv > 0) || !vmin_out || !vmax_out || !nvel_out) {
        rtm_set_last_error("rtm_prep_bins: bad argument");
        return RTM_ERR_ARG;
    }
    float vmin = v[0], vmax = v[0];
    for (long i = 0; i < ncell; ++i) {
        vmin = std::min(vmin, v[i]);
        vmax = std::max(vmax, v[i]);
    }
    float vel = ((int)(vmin / dv)) * dv;
    vmin = (vel > vmin) ? vel - dv : vel;
    vel = ((int)(vmax / dv)) * dv;
    vmax = (vel < vmax) ? vel + dv : vel;
    const int nvel = (int)((vmax - vmin) / dv + 1.5);
    *vmin_out = vmin;
    *vmax_out = vmax;
    *nvel_out = nvel;
    if (need) {
        if (need_cap < nvel) {
            rtm_set_last_error("rtm_prep_bins: need[] too small");
            return RTM_ERR_ARG;
        }
        std::memset(need, 0, sizeof(int) * nvel);
        for (long i = 0; i < ncell; ++i) need[(int)((v[i] - vmin) / dv + 0.5)] = 1;
    }
    return RTM_OK;
}

// kernel.cu:1261-1266: Ricker wavelet with delay 1/f0, evaluated in double
// and rounded to float; the sample time is an int times a float.
int rtm_prep_wavelet(float *wav, int n, float tao, float f0)
{
    if (!wav || n < 0 || !(f0 > 0)) return RTM_ERR_ARG;
    const double kPi = 3.1415926535898;  // the reference's constant
    for (int i = 0; i < n; ++i) {
        const float t1 = i * tao;
        const float t00 = 1 / f0;
        const double a = kPi * f0 * (t1 - t00);
        wav[i] = (float)((1 - 2 * std::pow(a, 2)) * std::exp(-std::pow(a, 2)));
    }
    return RTM_OK;
}

// LSMOrCon_rec_2D.cpp:526-551: 2M-order Taylor coefficients,
// c_i = (-1)^(i+1)/i^2 * prod_{j!=i} |j^2/(j^2-i^2)|, c_0 = -2*sum c_i,
// accumulated in float as the reference does.
int rtm_prep_taylor(int N, float *c)
{
    if (!c || N < 2) return RTM_ERR_ARG;
    const int M = N / 2;
    c[0] = 0.0f;
    for (int i = 1; i <= M; ++i) {
        float x = 1.0f;
        for (int j = 1; j <= M; ++j)
            if (j != i) x = x * std::fabs(std::pow(j, 2) / (std::pow(j, 2) - std::pow(i, 2)));
        c[i] = std::pow(-1, i + 1) / std::pow(i, 2) * x;
        c[0] = c[0] - 2 * c[i];
    }
    return RTM_OK;
}

}  // extern "C"
