// Post-stack display chain of the reference on the GPU, and a SEG-Y writer.
//
//   rtm_depth_to_time   DisToTimeAndTimeToDis1D.cpp:120-180 (D2T)
//   rtm_time_to_depth   DisToTimeAndTimeToDis1D.cpp:30-118 (T2D)
//   rtm_phase_rotate    phase_correction_ricker_decon.cpp:160-224
//                       (phase_correction) with its radix-2 FFT (:326-389)
//   rtm_write_segy      SGYWrite.cpp:3-55 (WriteSGY), written from the SEG-Y
//                       rev 1 layout (big-endian headers, IBM or IEEE samples)
//
// Every trace is independent: the time/depth tables are one thread per trace
// (a running sum, in the reference's order), the interpolation one thread
// per output sample, the phase rotation one CTA per trace with the spectrum
// in shared memory (FP64, as the reference).  Results match the reference
// bit for bit except the phase rotation, whose two special bins take libm's
// atan on the CPU and CUDA's on the GPU (a difference in the last bit of a
// double, below float resolution in almost every sample).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "rtm_common.cuh"

namespace {

// ---- depth <-> time tables ------------------------------------------------

// t[tr][j] = sum_{i=1..j} 2 dz / v[tr][i] (t[tr][0] = 0); tmax[tr] = t[tr][nz-1]
__global__ void k_d2t_table(const float *__restrict__ v, int ntr, int nz, float dz,
                            float *__restrict__ t, float *__restrict__ tmax)
{
    const int tr = blockIdx.x * blockDim.x + threadIdx.x;
    if (tr >= ntr) return;
    const float *vv = v + (long)tr * nz;
    float *tt = t + (long)tr * nz;
    const float two_dz = 2 * dz;
    float acc = 0.0f;
    tt[0] = 0.0f;
    for (int j = 1; j < nz; ++j) {
        acc = __fadd_rn(acc, __fdiv_rn(two_dz, vv[j]));
        tt[j] = acc;
    }
    tmax[tr] = acc;
}

// z[tr][j]: z += dt * v[tr][min(int(int(z)/dz), nzv-1)] / 2 per time sample
__global__ void k_t2d_table(const float *__restrict__ v, int nzv, int ntr, int nt, float dt, float dz,
                            float *__restrict__ z, float *__restrict__ zmax)
{
    const int tr = blockIdx.x * blockDim.x + threadIdx.x;
    if (tr >= ntr) return;
    const float *vv = v + (long)tr * nzv;
    float *zz = z + (long)tr * nt;
    float acc = 0.0f;
    zz[0] = 0.0f;
    for (int j = 1; j < nt; ++j) {
        int jv = (int)__fdiv_rn((float)(int)acc, dz);
        if (jv >= nzv) jv = nzv - 1;
        acc = __fadd_rn(acc, __fdiv_rn(__fmul_rn(dt, vv[jv]), 2.0f));
        zz[j] = acc;
    }
    zmax[tr] = acc;
}

// Linear interpolation onto a regular grid (DisToTimeAndTimeToDis1D.cpp:7-26):
// out[0] = y[0]; sample j >= 1 comes from the first segment i with
// int(x[i]/d) >= j; samples past the last segment are 0.
__global__ void k_interp(const float *__restrict__ x, const float *__restrict__ y, int nin,
                         int nout, float d, float *__restrict__ out)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const long tr = blockIdx.y;
    if (j >= nout) return;
    const float *xx = x + tr * nin, *yy = y + tr * nin;
    float r = 0.0f;
    if (j == 0) {
        r = yy[0];
    } else {
        int lo = 1, hi = nin;  // smallest i in [1, nin) with int(x[i]/d) >= j (nin: none)
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if ((int)__fdiv_rn(xx[mid], d) >= j) hi = mid; else lo = mid + 1;
        }
        if (lo < nin) {
            const float x0 = xx[lo - 1], x1 = xx[lo], y0 = yy[lo - 1], y1 = yy[lo];
            const float q = __fdiv_rn(__fsub_rn(__fmul_rn((float)j, d), x0), __fsub_rn(x1, x0));
            r = __fadd_rn(y0, __fmul_rn(q, __fsub_rn(y1, y0)));
        }
    }
    out[tr * nout + j] = r;
}

// ---- phase rotation ----------------------------------------------------------

constexpr int PH_THREADS = 512;
constexpr int PH_MAXN = 8192;  // 2 x 8 x 8192 bytes of spectrum in shared memory

__device__ __forceinline__ int bitrev(int i, int k)
{
    return (int)(__brev((unsigned)i) >> (32 - k));
}

// Radix-2 stages on (fr, fi) in shared memory (the reference's stage order:
// pairs first, then spans 4, 8, ...); twiddles (wr, wi) of the direction.
__device__ void fft_stages(double *fr, double *fi, int n, int k, const double *__restrict__ wr,
                           const double *__restrict__ wi)
{
    for (int it = 2 * threadIdx.x; it < n; it += 2 * PH_THREADS) {
        const double vr = fr[it], vi = fi[it];
        const double ar = fr[it + 1], ai = fi[it + 1];
        fr[it] = __dadd_rn(vr, ar);
        fi[it] = __dadd_rn(vi, ai);
        fr[it + 1] = __dsub_rn(vr, ar);
        fi[it + 1] = __dsub_rn(vi, ai);
    }
    __syncthreads();
    int m = n / 2, nv = 2;
    for (int l0 = k - 2; l0 >= 0; --l0) {
        m /= 2;
        nv *= 2;
        const int half = nv / 2;
        for (int b = threadIdx.x; b < n / 2; b += PH_THREADS) {
            const int it = (b / half) * nv, j = b % half, h = it + j + half;
            const double tr_ = __ldg(wr + m * j), ti_ = __ldg(wi + m * j);
            const double a = __dmul_rn(tr_, fr[h]), c0 = __dmul_rn(ti_, fi[h]);
            const double s = __dmul_rn(__dadd_rn(tr_, ti_), __dadd_rn(fr[h], fi[h]));
            const double dr = __dsub_rn(a, c0), di = __dsub_rn(__dsub_rn(s, a), c0);
            const double er = fr[it + j], ei = fi[it + j];
            fr[h] = __dsub_rn(er, dr);
            fi[h] = __dsub_rn(ei, di);
            fr[it + j] = __dadd_rn(er, dr);
            fi[it + j] = __dadd_rn(ei, di);
        }
        __syncthreads();
    }
}

// amplitude / phase entry of the forward transform (kept by the reference at
// the DC and Nyquist bins of the rotated spectrum)
__device__ __forceinline__ void amp_phase(double fr, double fi, int n, double &pr, double &pi)
{
    pr = __ddiv_rn(__dsqrt_rn(__dadd_rn(__dmul_rn(fr, fr), __dmul_rn(fi, fi))), (double)(n / 2));
    if (fabs(fr) < __dmul_rn(0.000001, fabs(fi)))
        pi = (__dmul_rn(fi, fr) > 0) ? 90.0 : -90.0;
    else
        pi = atan(__ddiv_rn(fi, fr));
}

// One CTA per trace: forward FFT, rotation of bins 1..n/2-1 by (cs, sn),
// conjugate mirror, inverse FFT with 1/n scaling, real part out.
__global__ void __launch_bounds__(PH_THREADS) k_phase(const float *__restrict__ din, float *__restrict__ dout,
                                                      int nt, int n, int k, double cs, double sn,
                                                      const double *__restrict__ wfr, const double *__restrict__ wfi,
                                                      const double *__restrict__ wir, const double *__restrict__ wii)
{
    extern __shared__ double sm[];
    double *fr = sm, *fi = sm + n;
    const long tr = blockIdx.x;
    const float *x = din + tr * nt;
    for (int it = threadIdx.x; it < n; it += PH_THREADS) {
        const int is = bitrev(it, k);
        fr[it] = is < nt ? (double)x[is] : 0.0;
        fi[it] = 0.0;
    }
    __syncthreads();
    fft_stages(fr, fi, n, k, wfr, wfi);
    // rotated spectrum, gathered in registers, then written bit-reversed for
    // the inverse transform
    constexpr int PER = PH_MAXN / PH_THREADS;
    double gr[PER], gi[PER];
    const int h = n / 2;
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const int i = threadIdx.x + q * PH_THREADS;
        if (i >= n) continue;
        double pr, pi;
        if (i == 0 || i == h) {
            amp_phase(fr[i], fi[i], n, pr, pi);
        } else {
            const int s = i < h ? i : n - i;  // mirror: conjugate of bin n-i
            const double a = fr[s], b = fi[s];
            pr = __dsub_rn(__dmul_rn(a, cs), __dmul_rn(b, sn));
            pi = __dadd_rn(__dmul_rn(b, cs), __dmul_rn(a, sn));
            if (i > h) pi = -pi;
        }
        gr[q] = pr;
        gi[q] = pi;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const int i = threadIdx.x + q * PH_THREADS;
        if (i >= n) continue;
        const int d = bitrev(i, k);  // the inverse transform's input order
        fr[d] = gr[q];
        fi[d] = gi[q];
    }
    __syncthreads();
    fft_stages(fr, fi, n, k, wir, wii);
    for (int i = threadIdx.x; i < nt; i += PH_THREADS)
        dout[tr * nt + i] = (float)__ddiv_rn(fr[i], 1.0 * n);
}

// Twiddles w_i = w_{i-1} w_1 of the reference's FFT (w_1 = exp(-+2 pi i/n)
// with 2 pi taken as 6.283185306, three-multiply complex product), in the
// same double operations on the host.
void twiddles(int n, bool inverse, std::vector<double> &wr, std::vector<double> &wi)
{
    wr.assign(n, 0.0);
    wi.assign(n, 0.0);
    wr[0] = 1.0;
    wi[0] = 0.0;
    if (n < 2) return;
    const double p = 6.283185306 / (1.0 * n);
    wr[1] = std::cos(p);
    wi[1] = -std::sin(p);
    if (inverse) wi[1] = -wi[1];
    for (int i = 2; i < n; ++i) {
        const double a = wr[i - 1] * wr[1], b = wi[i - 1] * wi[1];
        const double c = (wr[i - 1] + wi[i - 1]) * (wr[1] + wi[1]);
        wr[i] = a - b;
        wi[i] = c - a - b;
    }
}

// ---- device buffers ----------------------------------------------------------

template <class T>
struct Buf {
    T *p = nullptr;
    ~Buf() { cudaFree(p); }
    bool alloc(size_t n) { return cudaMalloc(&p, sizeof(T) * std::max<size_t>(n, 1)) == cudaSuccess; }
};

// A device view of a caller buffer: the buffer itself (RTM_DEVICE_PTRS) or a
// device copy.
int stage_in(const float *src, size_t n, bool dev, Buf<float> &tmp, const float *&out)
{
    if (dev) {
        out = src;
        return RTM_OK;
    }
    if (!tmp.alloc(n)) return RTM_ERR_NOMEM;
    if (cudaMemcpy(tmp.p, src, sizeof(float) * n, cudaMemcpyHostToDevice) != cudaSuccess) return RTM_ERR_CUDA;
    out = tmp.p;
    return RTM_OK;
}

int finish_out(float *dst, const float *dsrc, size_t n, bool dev)
{
    if (dev) return cudaDeviceSynchronize() == cudaSuccess ? RTM_OK : RTM_ERR_CUDA;
    return cudaMemcpy(dst, dsrc, sizeof(float) * n, cudaMemcpyDeviceToHost) == cudaSuccess ? RTM_OK
                                                                                          : RTM_ERR_CUDA;
}

// Table pass + interpolation shared by the two conversions.
int convert(bool d2t, const float *v, int nzv, const float *img, int ntr, int nin, float step_in,
            float step_out, float *out, long cap, int *nout_p, int flags)
{
    const bool dev = flags & RTM_DEVICE_PTRS;
    const float *dv, *di;
    Buf<float> tv, ti, tab, tmax, tout;
    int rc;
    if ((rc = stage_in(v, (size_t)ntr * nzv, dev, tv, dv)) || (rc = stage_in(img, (size_t)ntr * nin, dev, ti, di)))
        return rc;
    if (!tab.alloc((size_t)ntr * nin) || !tmax.alloc(ntr)) return RTM_ERR_NOMEM;
    if (d2t)
        k_d2t_table<<<(ntr + 127) / 128, 128>>>(dv, ntr, nin, step_in, tab.p, tmax.p);
    else
        k_t2d_table<<<(ntr + 127) / 128, 128>>>(dv, nzv, ntr, nin, step_in, step_out, tab.p, tmax.p);
    std::vector<float> hm(ntr);
    if (cudaMemcpy(hm.data(), tmax.p, sizeof(float) * ntr, cudaMemcpyDeviceToHost) != cudaSuccess)
        return RTM_ERR_CUDA;
    float mx = 0.0f;
    for (float m : hm)
        if (mx < m) mx = m;
    const int nout = (int)(mx / step_out);
    if (nout_p) *nout_p = nout;
    if (!out) return RTM_OK;  // size query
    if (nout < 1) return RTM_OK;
    if ((long)nout * ntr > cap) {
        rtm_set_last_error("output capacity too small");
        return RTM_ERR_ARG;
    }
    float *dout = out;
    if (!dev) {
        if (!tout.alloc((size_t)ntr * nout)) return RTM_ERR_NOMEM;
        dout = tout.p;
    }
    for (int t0 = 0; t0 < ntr; t0 += 65535) {
        const int nt_ = std::min(65535, ntr - t0);
        k_interp<<<dim3((nout + 255) / 256, nt_), 256>>>(tab.p + (size_t)t0 * nin, di + (size_t)t0 * nin, nin,
                                                       nout, step_out, dout + (size_t)t0 * nout);
    }
    if (cudaGetLastError() != cudaSuccess) return RTM_ERR_CUDA;
    return finish_out(out, dout, (size_t)ntr * nout, dev);
}

// ---- SEG-Y -------------------------------------------------------------------

void put2(unsigned char *b, int v)
{
    b[0] = (unsigned char)((v >> 8) & 0xff);
    b[1] = (unsigned char)(v & 0xff);
}

void put4(unsigned char *b, unsigned v)
{
    b[0] = (unsigned char)(v >> 24);
    b[1] = (unsigned char)(v >> 16);
    b[2] = (unsigned char)(v >> 8);
    b[3] = (unsigned char)v;
}

int get2(const unsigned char *b) { return (short)((b[0] << 8) | b[1]); }

// IEEE single -> IBM hexadecimal single: the 24-bit significand (hidden bit
// restored) shifted so the base-2 exponent becomes a multiple of 4, then
// normalised to at most 24 bits; truncation, no rounding; overflow saturates
// to the largest magnitude, underflow gives a signed zero.
unsigned ieee_to_ibm(float y)
{
    unsigned x;
    std::memcpy(&x, &y, 4);
    if ((x & 0x7fffffffu) == 0) return x;
    unsigned s = x & 0x80000000u;
    int e = (int)((x >> 23) & 0xff) - 127;
    unsigned f = ((x & 0x007fffffu) << 1) | 0x01000000u;
    if (e >= 0) {
        f <<= (e & 3);
        e >>= 2;
    } else {
        f >>= ((-e) & 3);
        e = -((-e) >> 2);
    }
    if (f & 0x0f000000u) {
        f >>= 4;
        e += 1;
    }
    e += 64;
    if (e > 127) return s | 0x7fffffffu;
    if (e >= 0) return s | ((unsigned)e << 24) | f;
    return s;
}

}  // namespace

extern "C" {

int rtm_depth_to_time(const float *v, const float *img, int ntr, int nz, float dz, float dt, float *out,
                      long cap, int *nt, int flags)
{
    if (!v || !img || !nt || ntr < 1 || nz < 2 || !(dz > 0.0f) || !(dt > 0.0f)) return RTM_ERR_ARG;
    return convert(true, v, nz, img, ntr, nz, dz, dt, out, cap, nt, flags);
}

int rtm_time_to_depth(const float *v, int nzv, const float *img, int ntr, int nt, float dt, float dz,
                      float *out, long cap, int *nz, int flags)
{
    if (!v || !img || !nz || ntr < 1 || nt < 2 || nzv < 1 || !(dz > 0.0f) || !(dt > 0.0f)) return RTM_ERR_ARG;
    return convert(false, v, nzv, img, ntr, nt, dt, dz, out, cap, nz, flags);
}

int rtm_phase_rotate(const float *din, float *dout, int ntr, int nt, float angle, int flags)
{
    if (!din || !dout || ntr < 1 || nt < 1) return RTM_ERR_ARG;
    int n = 2, k = 1;
    while (n < nt) {
        n *= 2;
        ++k;
    }
    if (n > PH_MAXN) {
        rtm_set_last_error("phase rotation: traces longer than 8192 samples");
        return RTM_ERR_UNSUPPORTED;
    }
    const bool dev = flags & RTM_DEVICE_PTRS;
    const double theta = angle * 3.1415926535898 / 180;
    const double cs = std::cos(theta), sn = std::sin(theta);
    std::vector<double> fwr, fwi, iwr, iwi;
    twiddles(n, false, fwr, fwi);
    twiddles(n, true, iwr, iwi);
    Buf<double> tw;
    if (!tw.alloc((size_t)4 * n)) return RTM_ERR_NOMEM;
    for (int q = 0; q < 4; ++q) {
        const std::vector<double> &src = q == 0 ? fwr : q == 1 ? fwi : q == 2 ? iwr : iwi;
        if (cudaMemcpy(tw.p + (size_t)q * n, src.data(), sizeof(double) * n, cudaMemcpyHostToDevice) != cudaSuccess)
            return RTM_ERR_CUDA;
    }
    const float *di;
    Buf<float> tin, tout;
    int rc;
    if ((rc = stage_in(din, (size_t)ntr * nt, dev, tin, di))) return rc;
    float *dd = dout;
    if (!dev) {
        if (!tout.alloc((size_t)ntr * nt)) return RTM_ERR_NOMEM;
        dd = tout.p;
    }
    const int smem = (int)(2 * sizeof(double) * n);
    if (cudaFuncSetAttribute(k_phase, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
        return RTM_ERR_CUDA;
    k_phase<<<ntr, PH_THREADS, smem>>>(di, dd, nt, n, k, cs, sn, tw.p, tw.p + n, tw.p + 2 * n, tw.p + 3 * n);
    if (cudaGetLastError() != cudaSuccess) return RTM_ERR_CUDA;
    return finish_out(dout, dd, (size_t)ntr * nt, dev);
}

int rtm_write_segy(const char *path, const char *template_path, const float *data, int ntr, int ns,
                   float dt, const float *sx, const float *sy, float gx, float gy, const float *offset)
{
    if (!path || !data || ntr < 1 || ns < 1 || ns > 32767) return RTM_ERR_ARG;
    unsigned char text[3200], bin[400], th[240];
    std::memset(text, 0x40, sizeof(text));  // EBCDIC blanks
    std::memset(bin, 0, sizeof(bin));
    std::memset(th, 0, sizeof(th));
    int format = 5;  // IEEE
    if (template_path) {
        FILE *t = std::fopen(template_path, "rb");
        if (!t) {
            rtm_set_last_error("cannot open the SEG-Y template");
            return RTM_ERR_IO;
        }
        const bool ok = std::fread(text, 1, 3200, t) == 3200 && std::fread(bin, 1, 400, t) == 400 &&
                        std::fread(th, 1, 240, t) == 240;
        std::fclose(t);
        if (!ok) {
            rtm_set_last_error("SEG-Y template shorter than its headers");
            return RTM_ERR_IO;
        }
        format = get2(bin + 24);
    } else {
        put2(bin + 24, format);
        put2(bin + 28, 1);  // trace sorting: as recorded
    }
    if (format != 1 && format != 5) {
        rtm_set_last_error("SEG-Y sample format other than IBM (1) or IEEE (5)");
        return RTM_ERR_UNSUPPORTED;
    }
    // sample interval: seconds (< 1) or milliseconds, stored in microseconds
    const float scale = dt < 1.0f ? 1000000.f : 1000.f;
    put2(bin + 16, (int)(scale * dt));
    put2(bin + 20, ns);
    FILE *o = std::fopen(path, "wb");
    if (!o) {
        rtm_set_last_error("cannot create the SEG-Y file");
        return RTM_ERR_IO;
    }
    bool ok = std::fwrite(text, 1, 3200, o) == 3200 && std::fwrite(bin, 1, 400, o) == 400;
    std::vector<unsigned char> tb((size_t)4 * ns);
    for (int i = 0; i < ntr && ok; ++i) {
        unsigned char h[240];
        std::memcpy(h, th, 240);
        if (offset) put4(h + 36, (unsigned)(int)offset[i]);
        if (sx) put4(h + 72, (unsigned)(int)sx[i]);
        if (sy) put4(h + 76, (unsigned)(int)sy[i]);
        put4(h + 80, (unsigned)(int)gx);
        put4(h + 84, (unsigned)(int)gy);
        if (!template_path) put2(h + 114, ns);
        for (int s = 0; s < ns; ++s) {
            const float y = data[(size_t)i * ns + s];
            unsigned w;
            if (format == 1)
                w = ieee_to_ibm(y);
            else
                std::memcpy(&w, &y, 4);
            put4(&tb[(size_t)4 * s], w);
        }
        ok = std::fwrite(h, 1, 240, o) == 240 && std::fwrite(tb.data(), 1, tb.size(), o) == tb.size();
    }
    ok = (std::fclose(o) == 0) && ok;
    if (!ok) {
        rtm_set_last_error("SEG-Y write failed");
        return RTM_ERR_IO;
    }
    return RTM_OK;
}

}  // extern "C"
