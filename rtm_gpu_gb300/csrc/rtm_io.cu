// Shot-level file flow of the reference and trace resampling.
//
//   rtm_resample     kernel.cu:839-845 / Resample.cpp:193-225: every trace
//                    resampled from dxin to dxout by the 8-point
//                    least-squares sinc interpolator of Seismic Unix (CWP,
//                    D. Hale), one GPU thread per output sample.
//   rtm_run_config   kernel.cu:542-1098 up to the stacked image: reads the
//                    reference's run file (2D_Real_RVSP_RTM.txt layout), its
//                    parameter file, the source-depth list, the velocity file
//                    and one gather file per shot; migrates all shots on the
//                    batched engine; writes the per-shot up/down images, the
//                    stacked image and the velocity window in the reference's
//                    file names and layouts.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "rtm_common.cuh"

namespace {

// ---------------------------------------------------------------------------
// 8-point sinc table: row j (0 < j < 512) holds the least-squares filter for
// a fractional shift j/512: with fmax = min(0.066 + 0.265 ln 8, 1), the
// autocorrelation a_k = sinc(fmax k) and crosscorrelation
// c_k = sinc(fmax (3 - k + d)) (the shift formed in float), taps = a^-1 c by
// Levinson recursion in double, stored as float.  Rows 0 and 512 are unit
// impulses at taps 3 and 4.  Same operation order as the reference, so the
// table (and every output) matches it bit for bit.
constexpr int RS_TAPS = 8, RS_ROWS = 513;

double rs_sinc(double x)
{
    if (x == 0.0) return 1.0;
    const double px = 3.1415926535898 * x;
    return std::sin(px) / px;
}

void rs_levinson(int n, const double *t, const double *g, double *f, double *w)
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

void rs_table(float *tab)
{
    double fmax = 0.066 + 0.265 * std::log((double)RS_TAPS);
    if (fmax > 1.0) fmax = 1.0;
    for (int j = 1; j < RS_ROWS - 1; ++j) {
        const float d = (float)j / (float)(RS_ROWS - 1);
        double a[RS_TAPS], c[RS_TAPS], s[RS_TAPS], w[RS_TAPS];
        for (int k = 0; k < RS_TAPS; ++k) {
            a[k] = rs_sinc(fmax * k);
            const float sh = (float)(RS_TAPS / 2 - k - 1) + d;
            c[k] = rs_sinc(fmax * sh);
        }
        rs_levinson(RS_TAPS, a, c, s, w);
        for (int k = 0; k < RS_TAPS; ++k) tab[j * RS_TAPS + k] = (float)s[k];
    }
    for (int k = 0; k < RS_TAPS; ++k) {
        tab[k] = 0.0f;
        tab[(RS_ROWS - 1) * RS_TAPS + k] = 0.0f;
    }
    tab[RS_TAPS / 2 - 1] = 1.0f;
    tab[(RS_ROWS - 1) * RS_TAPS + RS_TAPS / 2] = 1.0f;
}

// Output sample i of trace blockIdx.y: u = 8 + (i*dxout)/dxin (inv = 1/dxin
// rounded to float), inputs m-11 .. m-4 of m = int(u) against table row
// int(frac(u)*512 + 0.5); products summed left to right, no contraction.
__global__ void k_resample(const float *__restrict__ yin, int nxin, float inv, float dxout,
                           const float *__restrict__ tab, float *__restrict__ yout, int nxout)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nxout) return;
    const float *y = yin + (long)blockIdx.y * nxin;
    const float x = __fmul_rn((float)i, dxout);
    const float u = __fadd_rn(8.0f, __fmul_rn(x, inv));
    const int m = (int)u;
    const float fr = __fsub_rn(u, (float)m);
    const float fs = __fmul_rn(fr, (float)(RS_ROWS - 1));
    const int row = (int)((double)fs + 0.5);  // fr >= 0 here (u >= 8)
    const float *t = tab + row * RS_TAPS;
    float sum = 0.0f;
#pragma unroll
    for (int j = 0; j < RS_TAPS; ++j) {
        const int k = m - 11 + j;
        const float v = (k < 0 || k >= nxin) ? 0.0f : __ldg(y + k);
        sum = __fadd_rn(sum, __fmul_rn(v, __ldg(t + j)));
    }
    yout[(long)blockIdx.y * nxout + i] = sum;
}

// ---------------------------------------------------------------------------
// Reading the reference's text files the way its fscanf calls do: a label
// line ("%[^\n]\n": the rest of the line after leading whitespace) followed
// by a value token ("%d\n", "%f\n", "%s\n").

struct Scanner {
    std::string text;
    size_t pos = 0;
    bool ok = true;
    void skip_ws()
    {
        while (pos < text.size() && std::isspace((unsigned char)text[pos])) ++pos;
    }
    std::string line()
    {
        skip_ws();
        const size_t e = text.find('\n', pos);
        std::string s = text.substr(pos, e == std::string::npos ? std::string::npos : e - pos);
        pos = e == std::string::npos ? text.size() : e;
        if (s.empty()) ok = false;
        return s;
    }
    std::string token()
    {
        skip_ws();
        const size_t b = pos;
        while (pos < text.size() && !std::isspace((unsigned char)text[pos])) ++pos;
        if (pos == b) ok = false;
        return text.substr(b, pos - b);
    }
    int i() { return (int)std::strtol(token().c_str(), nullptr, 10); }
    float f() { return std::strtof(token().c_str(), nullptr); }
};

bool read_file(const std::string &path, std::string &out)
{
    FILE *fh = std::fopen(path.c_str(), "rb");
    if (!fh) return false;
    char buf[1 << 16];
    size_t n;
    out.clear();
    while ((n = std::fread(buf, 1, sizeof(buf), fh)) > 0) out.append(buf, n);
    std::fclose(fh);
    return true;
}

bool read_floats(const std::string &path, float *dst, size_t n)
{
    FILE *fh = std::fopen(path.c_str(), "rb");
    if (!fh) return false;
    const size_t got = std::fread(dst, sizeof(float), n, fh);
    std::fclose(fh);
    return got == n;
}

bool write_floats(const std::string &path, const float *src, size_t n)
{
    FILE *fh = std::fopen(path.c_str(), "wb");
    if (!fh) return false;
    const size_t put = std::fwrite(src, sizeof(float), n, fh);
    return std::fclose(fh) == 0 && put == n;
}

int fail(const std::string &msg, int code = RTM_ERR_ARG)
{
    rtm_set_last_error(msg.c_str());
    return code;
}

}  // namespace

extern "C" {

int rtm_resample(const float *yin, int ntrace, int nxin, float dxin, float *yout, int nxout,
                 float dxout, int flags)
{
    if (!yin || !yout || ntrace < 0 || nxin < 1 || nxout < 1 || !(dxin > 0.0f) || !(dxout > 0.0f))
        return RTM_ERR_ARG;
    if (ntrace == 0) return RTM_OK;
    static const std::vector<float> htab = [] {
        std::vector<float> t(RS_ROWS * RS_TAPS);
        rs_table(t.data());
        return t;
    }();
    const bool dev = flags & RTM_DEVICE_PTRS;
    float *dtab = nullptr, *din = nullptr, *dout = nullptr;
    const size_t nin = (size_t)ntrace * nxin, nout = (size_t)ntrace * nxout;
    int rc = RTM_OK;
    auto done = [&](int r) {
        cudaFree(dtab);
        if (!dev) {
            cudaFree(din);
            cudaFree(dout);
        }
        return r;
    };
    if (cudaMalloc(&dtab, sizeof(float) * htab.size()) != cudaSuccess) return done(RTM_ERR_NOMEM);
    if (dev) {
        din = const_cast<float *>(yin);
        dout = yout;
    } else if (cudaMalloc(&din, sizeof(float) * nin) != cudaSuccess ||
               cudaMalloc(&dout, sizeof(float) * nout) != cudaSuccess) {
        return done(RTM_ERR_NOMEM);
    }
    if (cudaMemcpy(dtab, htab.data(), sizeof(float) * htab.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
        (!dev && cudaMemcpy(din, yin, sizeof(float) * nin, cudaMemcpyHostToDevice) != cudaSuccess))
        return done(RTM_ERR_CUDA);
    const float inv = (float)(1.0 / dxin);
    for (int t0 = 0; t0 < ntrace; t0 += 65535) {  // grid y limit
        const int nt = std::min(65535, ntrace - t0);
        k_resample<<<dim3((nxout + 127) / 128, nt), 128>>>(din + (size_t)t0 * nxin, nxin, inv, dxout,
                                                           dtab, dout + (size_t)t0 * nxout, nxout);
    }
    if (cudaGetLastError() != cudaSuccess) return done(RTM_ERR_CUDA);
    if (!dev && cudaMemcpy(yout, dout, sizeof(float) * nout, cudaMemcpyDeviceToHost) != cudaSuccess)
        rc = RTM_ERR_CUDA;
    if (dev && cudaDeviceSynchronize() != cudaSuccess) rc = RTM_ERR_CUDA;
    return done(rc);
}

int rtm_run_config(const char *run_file, int max_batch)
{
    if (!run_file) return RTM_ERR_ARG;
    // ---- run file (kernel.cu:542-601)
    Scanner sc;
    if (!read_file(run_file, sc.text)) return fail(std::string("cannot open ") + run_file, RTM_ERR_IO);
    int nfdmax, nfdmin, N2, nthita, iLSTE, ifv, iNorm, iCompen, Nsmooth, NX_BG, NX_ED, NZ_BG, NZ_ED;
    float f0, fmax, df, eps, dv, whitecoe, hz, tao, wthite_phase, angle;
    std::string seis_prefix, vp_file, dpr_file, para_file, result;
    sc.line(); nfdmax = sc.i();
    sc.line(); nfdmin = sc.i();
    sc.line(); N2 = sc.i();
    sc.line(); f0 = sc.f();
    sc.line(); fmax = sc.f();
    sc.line(); df = sc.f();
    sc.line(); nthita = sc.i();
    sc.line(); eps = sc.f();
    sc.line(); dv = sc.f();
    sc.line(); iLSTE = sc.i();
    sc.line(); ifv = sc.i();
    sc.line(); whitecoe = sc.f();
    sc.line(); hz = sc.f();
    sc.line(); tao = sc.f();
    sc.line(); iNorm = sc.i();
    sc.line(); iCompen = sc.i();
    sc.line(); Nsmooth = sc.i();
    sc.line(); wthite_phase = sc.f();
    sc.line(); angle = sc.f();
    sc.line(); NX_BG = sc.i();
    sc.line(); NX_ED = sc.i();
    sc.line(); NZ_BG = sc.i();
    sc.line(); NZ_ED = sc.i();
    sc.line(); seis_prefix = sc.token();
    sc.line(); vp_file = sc.token();
    sc.line(); dpr_file = sc.token();
    sc.line(); para_file = sc.token();
    sc.line(); result = sc.token();
    (void)Nsmooth; (void)wthite_phase;  // read by the reference, not used by its chain
    if (!sc.ok) return fail("run file: missing entries");
    // ---- parameter file (kernel.cu:603-605)
    Scanner ps;
    if (!read_file(para_file, ps.text)) return fail("cannot open " + para_file, RTM_ERR_IO);
    const float h = ps.f(), tao1 = ps.f();
    const int mod_NZ = ps.i(), mod_NX = ps.i(), NT1 = ps.i();
    int s_l = ps.i(), s_z = ps.i();
    const int n = ps.i(), ds = ps.i();
    int r_x = ps.i();
    const int nrec = ps.i(), dr = ps.i();
    (void)dr;
    if (!ps.ok) return fail("parameter file: missing entries");
    if (nfdmax < 1 || nfdmax > 12 || nfdmin < 1 || nfdmin > nfdmax || N2 < nfdmax || mod_NZ < 2 ||
        mod_NX < 2 || NT1 < 4 || n < 1 || nrec < 1 || !(tao > 0.0f) || !(tao1 > 0.0f) || !(h > 0.0f))
        return fail("run/parameter file: values out of range");
    // kernel.cu:608-631 (float arithmetic as there)
    s_l = s_l + N2 - 1;
    r_x = r_x + N2 - 1;
    s_z = s_z + N2 - 1;
    const int NZ = mod_NZ + 2 * N2, NX = mod_NX + 2 * N2;
    const int NT = (int)((NT1 - 1) * tao1 / tao + 1.5);
    const float taoh = tao / h;
    const float tao2 = (float)std::pow(tao, 2);
    const float h2 = (float)(1 / std::pow(h, 2));
    const float taoh2 = tao2 * h2 / 2;
    const int NT2 = int(2.0 / (f0 * tao)) + 1;
    const float hzx = hz / h;
    const float hzx2_1 = 1 / (hzx * hzx);
    if (s_l < 0 || s_z < 0 || s_z >= NZ || (n - 1) * ds + s_l >= NX || r_x < 0 || r_x >= NX || NT < 4)
        return fail("geometry outside the grid");
    // the output window must lie in the image (the reference would read
    // whatever its work array held outside it)
    if (NX_BG < 0 || NZ_BG < 0 || NX_BG >= NX_ED || NZ_BG >= NZ_ED || NZ_ED > mod_NZ ||
        (ifv == 1 ? NX_ED >= mod_NX : NX_ED > mod_NX))
        return fail("output window outside the image");
    // ---- source depths (kernel.cu:686-691)
    Scanner ds_;
    if (!read_file(dpr_file, ds_.text)) return fail("cannot open " + dpr_file, RTM_ERR_IO);
    std::vector<float> inre(nrec);
    for (int i = 0; i < nrec; ++i) inre[i] = ds_.f();
    if (!ds_.ok) return fail("source-depth file: fewer than nrec entries");
    // ---- velocity (GPU_velocity_real.cpp: x-major interior) and bins
    std::vector<float> vin((size_t)mod_NX * mod_NZ);
    if (!read_floats(vp_file, vin.data(), vin.size())) return fail("cannot read " + vp_file, RTM_ERR_IO);
    std::vector<float> v((size_t)NZ * NX), r1((size_t)NZ * NX);
    int rc;
    if ((rc = rtm_prep_velocity(vin.data(), mod_NZ, mod_NX, N2, tao, h, ifv, v.data(), r1.data())))
        return rc;
    float vmin, vmax;
    int nvel;
    if ((rc = rtm_prep_bins(v.data(), (long)NZ * NX, dv, &vmin, &vmax, &nvel, nullptr, 0))) return rc;
    std::vector<int> need(nvel);
    if ((rc = rtm_prep_bins(v.data(), (long)NZ * NX, dv, &vmin, &vmax, &nvel, need.data(), nvel)))
        return rc;
    // ---- coefficients (kernel.cu:744-754)
    std::vector<int> len(nvel), index(nvel + 1);
    std::vector<float> coef;
    if (iLSTE == 0) {
        rtm_ls_settings s{nthita, nfdmax, nfdmin, tao, h, df, eps, fmax, hzx};
        int nc = 0;
        if ((rc = rtm_coeffs_optimise_fp64(&s, vmin, dv, nvel, need.data(), len.data(), index.data(),
                                           nullptr, 0, &nc)))
            return rc;
        coef.resize(std::max(nc, 1));
        if ((rc = rtm_coeffs_optimise_fp64(&s, vmin, dv, nvel, need.data(), len.data(), index.data(),
                                           coef.data(), nc, &nc)))
            return rc;
    } else {
        coef.resize(nfdmax + 1);
        if ((rc = rtm_prep_taylor(2 * nfdmax, coef.data()))) return rc;
    }
    // ---- wavelet table and the problem
    std::vector<float> wav(NT + 1);
    if ((rc = rtm_prep_wavelet(wav.data(), NT + 1, tao, f0))) return rc;
    std::vector<float> w(N2 + 1);
    for (int i = 0; i <= N2; ++i) w[i] = (float)((1.0 * i) / (1.0 * N2));  // kernel.cu:677-681
    rtm_problem p{};
    p.nz = mod_NZ; p.nx = mod_NX; p.N2 = N2; p.M = nfdmax; p.NT = NT; p.NT2 = NT2;
    p.adaptive = iLSTE == 0; p.compen = iCompen; p.quirk = 1; p.nbins = iLSTE == 0 ? nvel : 0;
    p.tao2 = tao2; p.h2 = h2; p.taoh = taoh; p.taoh2 = taoh2;
    p.vmin = vmin; p.dv = dv; p.hzx2_1 = hzx2_1; p.spike = wav[0] / 2;
    p.v = v.data(); p.r1 = r1.data(); p.w = w.data(); p.coef = coef.data();
    p.index = iLSTE == 0 ? index.data() : nullptr; p.wav = wav.data();
    p.rz0 = s_z; p.rx0 = s_l; p.rdz = 0; p.rdx = ds; p.nrec = n;
    p.ring_precision = RTM_RING_F32;
    // ---- sources (kernel.cu:793-795) and gathers (kernel.cu:827-852)
    std::vector<int> src(nrec);
    std::vector<float> seis((size_t)nrec * n * NT);
    std::vector<float> raw((size_t)n * NT1);
    for (int m = 0; m < nrec; ++m) {
        const int N = int(inre[m]);
        const int r_u = (int)(std::fabs(N / hz) + N2 - 1);
        if (r_u < 0 || r_u >= NZ) return fail("source depth outside the grid");
        src[m] = r_u * NX + r_x;
        char name[64];
        std::snprintf(name, sizeof(name), "NEW_L10-1932-X_%d.dat", N);
        const std::string path = seis_prefix + name;
        if (!read_floats(path, raw.data(), raw.size())) return fail("cannot read " + path, RTM_ERR_IO);
        float *dst = seis.data() + (size_t)m * n * NT;
        if (NT != NT1) {
            if ((rc = rtm_resample(raw.data(), n, NT1, tao1, dst, NT, tao, 0))) return rc;
        } else {
            std::memcpy(dst, raw.data(), sizeof(float) * raw.size());
        }
    }
    // ---- migration, per-shot finishing and the stack on the engine
    rtm_ctx *ctx = nullptr;
    const int B = std::max(1, std::min(max_batch > 0 ? max_batch : 16, nrec));
    if ((rc = rtm_ctx_create(&ctx, &p, B, nullptr))) return rc;
    const size_t ncell = (size_t)mod_NZ * mod_NX;
    std::vector<float> ups(ncell * nrec), downs(ncell * nrec), img(ncell), ill(ncell);
    rc = rtm_migrate_stack(ctx, nrec, src.data(), seis.data(), whitecoe, nrec, iNorm, img.data(),
                           ill.data(), ups.data(), downs.data(), 0);
    rtm_ctx_destroy(ctx);
    if (rc) return rc;
    // ---- per-shot files (kernel.cu:949-990): interior, x-major
    std::vector<float> col(ncell);
    auto xmajor = [&](const float *zmaj) {
        for (int j = 0; j < mod_NX; ++j)
            for (int i = 0; i < mod_NZ; ++i) col[(size_t)j * mod_NZ + i] = zmaj[(size_t)i * mod_NX + j];
    };
    for (int m = 0; m < nrec; ++m) {
        char name[64];
        std::snprintf(name, sizeof(name), "RVSP_RTM_up_%d.dat", m + 1);
        xmajor(ups.data() + (size_t)m * ncell);
        if (!write_floats(result + name, col.data(), ncell)) return fail("cannot write " + result + name, RTM_ERR_IO);
        std::snprintf(name, sizeof(name), "RVSP_RTM_down_%d.dat", m + 1);
        xmajor(downs.data() + (size_t)m * ncell);
        if (!write_floats(result + name, col.data(), ncell)) return fail("cannot write " + result + name, RTM_ERR_IO);
    }
    // ---- stacked image and velocity window (kernel.cu:1059-1108).  The
    // reference holds the stack in an NX-pitched array indexed from 0 by
    // interior (i, j); the velocity window reads the padded model.
    auto mig = [&](int i, int j) -> float {
        return (i < mod_NZ && j < mod_NX) ? img[(size_t)i * mod_NX + j] : 0.0f;
    };
    std::vector<float> out;
    std::vector<float> vout;
    if (ifv == 1) {
        for (int j = NX_ED; j > NX_BG; --j)
            for (int i = NZ_BG; i < NZ_ED; ++i) out.push_back(mig(i, j));
        for (int j = NX_ED + N2; j > NX_BG + N2; --j)
            for (int i = NZ_BG + N2; i < NZ_ED + N2; ++i)
                vout.push_back(i < NZ && j < NX ? v[(size_t)i * NX + j] : 0.0f);
    } else {
        for (int j = NX_BG; j < NX_ED; ++j)
            for (int i = NZ_BG; i < NZ_ED; ++i) out.push_back(mig(i, j));
        for (int j = NX_BG + N2; j < NX_ED + N2; ++j)
            for (int i = NZ_BG; i < NZ_ED + N2; ++i)
                vout.push_back(i < NZ && j < NX ? v[(size_t)i * NX + j] : 0.0f);
    }
    if (!write_floats(result + "RVSP_Migration_Real_new2.dat", out.data(), out.size()) ||
        !write_floats(result + "vnew.dat", vout.data(), vout.size()))
        return fail("cannot write the stacked image", RTM_ERR_IO);
    // ---- post-stack display chain (kernel.cu:1108-1196).  The reference
    // reads the two files back as NX_ED-NX_BG traces of mod_NZ samples each
    // (a flat read, whatever their row count); it only makes sense, and is
    // only run here, for a full-depth window.
    if (NZ_BG != 0 || NZ_ED != mod_NZ) return RTM_OK;
    const int ntr = NX_ED - NX_BG;
    std::vector<float> img2((size_t)ntr * mod_NZ, 0.0f), vdt((size_t)ntr * mod_NZ, 0.0f);
    std::memcpy(img2.data(), out.data(), sizeof(float) * std::min(out.size(), img2.size()));
    std::memcpy(vdt.data(), vout.data(), sizeof(float) * std::min(vout.size(), vdt.size()));
    for (float x : vdt)
        if (!(x > 0.0f)) return fail("velocity window of the post-stack chain is not positive");
    int nt = 0;
    if ((rc = rtm_depth_to_time(vdt.data(), img2.data(), ntr, mod_NZ, hz, tao, nullptr, 0, &nt, 0))) return rc;
    std::vector<float> mt((size_t)ntr * nt), mtp((size_t)ntr * nt);
    if ((rc = rtm_depth_to_time(vdt.data(), img2.data(), ntr, mod_NZ, hz, tao, mt.data(), (long)mt.size(), &nt, 0)))
        return rc;
    if (!write_floats(result + "RVSP_Migration_Real_T.dat", mt.data(), mt.size()))
        return fail("cannot write the time image", RTM_ERR_IO);
    if ((rc = rtm_phase_rotate(mt.data(), mtp.data(), ntr, nt, angle, 0))) return rc;
    if (!write_floats(result + "RVSP_Migration_Real_T_phase.dat", mtp.data(), mtp.size()))
        return fail("cannot write the phase-rotated image", RTM_ERR_IO);
    int nzd = 0;
    if ((rc = rtm_time_to_depth(vdt.data(), mod_NZ, mtp.data(), ntr, nt, tao, hz, nullptr, 0, &nzd, 0)))
        return rc;
    std::vector<float> md((size_t)ntr * std::max(nzd, 1));
    if ((rc = rtm_time_to_depth(vdt.data(), mod_NZ, mtp.data(), ntr, nt, tao, hz, md.data(), (long)md.size(),
                                &nzd, 0)))
        return rc;
    if (!write_floats(result + "RVSP_Migration_Real_D.dat", md.data(), (size_t)ntr * nzd))
        return fail("cannot write the depth image", RTM_ERR_IO);
    // SEG-Y of the stacked depth image (SGYWrite.cpp, called at kernel.cu:1190)
    std::vector<float> sx(ntr), sy(ntr), dsr(ntr);
    for (int i = 0; i < ntr; ++i) {
        sx[i] = 1.0f * i * 10;
        sy[i] = -1.0f * i * 10;
        dsr[i] = 1000 - i;
    }
    FILE *tp = std::fopen("SGY_Model.sgy", "rb");
    if (tp) std::fclose(tp);
    return rtm_write_segy((result + "RVSP_migration_Real.sgy").c_str(), tp ? "SGY_Model.sgy" : nullptr,
                          img2.data(), ntr, mod_NZ, (float)(int)hz, sx.data(), sy.data(), 1.0f, 1.0f, dsr.data());
}

}  // extern "C"
