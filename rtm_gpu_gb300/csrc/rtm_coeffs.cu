// FP64 least-squares optimal finite-difference coefficients on the GPU, with
// the adaptive operator length of LSMOrCon_rec_2D.cpp (funMandC, :22-73).
//
// For a velocity v (Courant number r = v*tao/h) and a band limit
// bb = kmax*h, the coefficients c_1..c_M minimise the time-space dispersion
// misfit: the normal equations A_ij = int g_i g_j, b_i = int g_i over
// theta in [0,2pi], kh in [0,bb] with
//   g_l = ((1+1/hzx^2) - cos(l kh cos th) - cos(hzx l kh sin th)/hzx^2)
//         / (r^-2 (1-cos(r kh)))
// are integrated by a composite 5-point Gauss-Legendre rule (4 panels per
// axis), solved by row-scaled Gaussian elimination with partial pivoting, and
// c_0 = -2 sum c_l (LSMOrCon_rec_2D.cpp:236-287).  The operator length per
// velocity is the shortest M whose dispersion error stays below eps over the
// frequency band and propagation angles (LSMOrCon_rec_2D.cpp:293-346); the
// lengths of all velocity bins follow from the reference's bisection over
// the bins (LSMOrCon_rec_2D.cpp:347-524), replayed here on the host from a
// table of pass/fail flags that the GPU computes for every (bin, M) pair.
//
// Each matrix entry is accumulated by one thread in the reference's order
// and this file is compiled without multiply-add contraction (-fmad=false),
// so the arithmetic matches the reference's CPU build except where the
// device's cos/sin/asin differ from the host's in the last bit.
#include <cmath>
#include <cstring>
#include <vector>

#include "rtm_common.cuh"

namespace {

constexpr double kPi = 3.1415926535898;  // LSMOrCon_rec_2D.cpp:4
constexpr int kMaxM = 16;  // rtm_ls_coefs_fp64 writes c[i*(kMaxM+1) + l]
constexpr int kThreads = 128;

__constant__ double c_gl_t[5] = {-0.9061798459, -0.5384693101, 0.0, 0.5384693101, 0.9061798459};
__constant__ double c_gl_w[5] = {0.2369268851, 0.4786286705, 0.5688888889, 0.4786286705,
                                 0.2369268851};

struct LsCase {
    double r;      // Courant number
    double bb;     // band limit kmax*h
    double pinv2;  // r^-2 (host pow)
    int M;
};

__device__ double integrand(double th, double kh, int ai, int aj, const LsCase &q, int prod,
                            double hzx)
{
    const double hzx2 = hzx * hzx;
    const double c = cos(th), s = sin(th);
    const double car = cos(q.r * kh);
    const double f1 =
        ((1 + 1 / hzx2) - cos(ai * kh * c) - cos(hzx * ai * kh * s) / hzx2) / (q.pinv2 * (1 - car));
    if (!prod) return f1;
    const double f2 =
        ((1 + 1 / hzx2) - cos(aj * kh * c) - cos(hzx * aj * kh * s) / hzx2) / (q.pinv2 * (1 - car));
    return f1 * f2;
}

// One normal-equation entry, accumulated node by node as the reference does.
__device__ double quad_entry(int ai, int aj, const LsCase &q, int prod, double hzx)
{
    const int npan = 4;
    const double h0 = 0.5 * (2 * kPi - 0.0) / npan;
    double b0 = h0 + 0.0;
    double outer = 0.0;
    for (int p0 = 0; p0 < npan; ++p0) {
        if (p0 > 0) b0 = b0 + h0 * 2.0;
        for (int n0 = 0; n0 < 5; ++n0) {
            const double th = h0 * c_gl_t[n0] + b0;
            const double h1 = 0.5 * (q.bb - 0.0) / npan;
            double b1 = h1 + 0.0;
            double inner = 0.0;
            for (int p1 = 0; p1 < npan; ++p1) {
                if (p1 > 0) b1 = b1 + h1 * 2.0;
                for (int n1 = 0; n1 < 5; ++n1) {
                    const double kh = h1 * c_gl_t[n1] + b1;
                    const double f = integrand(th, kh, ai, aj, q, prod, hzx);
                    inner = 1.0 * 1.0 * f * c_gl_w[n1] + inner;
                }
            }
            outer = inner * h1 * 1.0 * c_gl_w[n0] + outer;
        }
    }
    return outer * h0;
}

// Row-scaled Gaussian elimination with partial pivoting (one thread).
__device__ void gauss_solve(double *A, int n, double *b, double *x)
{
    for (int i = 0; i < n; ++i) {
        double mx = A[i * n];
        for (int j = 0; j < n; ++j)
            if (fabs(A[i * n + j]) > fabs(mx)) mx = A[i * n + j];
        if (fabs(mx) < 1e-10) {
            for (int k = 0; k < n; ++k) x[k] = 0.0;
            return;
        }
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
            const double m = A[p * n + i] / A[i * n + i];
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
}

// Block-wide LS solve: c[0..M] in shared memory on return.
__device__ void block_solve(const LsCase &q, double hzx, double *sA, double *sb, double *sx,
                            double *c)
{
    const int M = q.M;
    const int nA = M * (M + 1) / 2;
    for (int t = threadIdx.x; t < nA + M; t += blockDim.x) {
        if (t < nA) {
            int i = 0, rem = t;
            while (rem >= M - i) {
                rem -= M - i;
                ++i;
            }
            const int j = i + rem;
            sA[i * M + j] = quad_entry(i + 1, j + 1, q, 1, hzx);
        } else {
            const int i = t - nA;
            sb[i] = quad_entry(i + 1, M + 1, q, 0, hzx);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 0; i < M; ++i)
            for (int j = 0; j < i; ++j) sA[i * M + j] = sA[j * M + i];
        gauss_solve(sA, M, sb, sx);
        double s = 0.0;
        for (int i = 1; i <= M; ++i) {
            c[i] = sx[i - 1];
            s += c[i];
        }
        c[0] = -2.0 * s;
    }
    __syncthreads();
}

struct PassArgs {
    double vmin, dv, tao, h, df, eps, hzx;
    int nfre, nthita, nfdmin, nfdmax, nvel;
    const double *pinv2;  // [nvel] r^-2 of each bin's velocity (host pow)
    unsigned char *pass;  // [nvel][nfdmax+1]
};

// Pass/fail of operator length M at the velocity of bin i
// (callenfd2d_ls, LSMOrCon_rec_2D.cpp:306-344): one block per (bin, M).
__global__ void __launch_bounds__(kThreads) k_len_pass(PassArgs a)
{
    __shared__ double sA[kMaxM * kMaxM], sb[kMaxM], sx[kMaxM], c[kMaxM + 1];
    __shared__ int fail;
    const int nj = a.nfdmax - a.nfdmin + 1;
    const int bin = blockIdx.x / nj;
    const int M = a.nfdmin + blockIdx.x % nj;
    const double vel = a.vmin + bin * a.dv;  // vmin+(i-1)*dv with i = bin+1
    const double r = vel * a.tao / a.h;
    LsCase q;
    q.r = r;
    q.bb = 2 * kPi * a.df * (a.nfre - 1) * a.tao / r;
    q.pinv2 = a.pinv2[bin];
    q.M = M;
    block_solve(q, a.hzx, sA, sb, sx, c);
    if (threadIdx.x == 0) fail = 0;
    __syncthreads();
    const double bk = 2.0 * kPi * a.df * a.h / vel;
    const double ra = a.h / vel;
    const double hzx2 = a.hzx * a.hzx;
    const long total = (long)(a.nfre - 1) * a.nthita;  // angles n < nthita decide
    for (long t = threadIdx.x; t < total; t += blockDim.x) {
        if (*(volatile int *)&fail) break;
        const int k = 1 + (int)(t / a.nthita), n = (int)(t % a.nthita);
        const double hk = bk * k;
        const double rat = 2 / (r * hk);
        const double nth = n * kPi / (4 * a.nthita);
        double mid = 0;
        for (int l = 1; l <= M; ++l) {
            const double s1 = sin(l * a.hzx * hk * sin(nth) / 2);
            const double s2 = sin(l * hk * cos(nth) / 2);
            mid = mid + c[l] * (s1 * s1 / hzx2 + s2 * s2);
        }
        double e = rat * asin(sqrt(r * r * mid));
        e = fabs(ra * (1.0 / e - 1.0));
        if (e > a.eps) atomicExch(&fail, 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) a.pass[(long)bin * (a.nfdmax + 1) + M] = fail ? 0 : 1;
}

struct CoefArgs {
    const double *r;      // [n] Courant number of each case
    const double *bb;     // [n] band limit kmax*h
    const double *pinv2;  // [n] r^-2 (host pow)
    const int *M;         // [n] operator length
    double hzx;
    double *out;          // [n][kMaxM+1]
};

// Coefficients of a batch of (r, bb, M) cases, one block each (for the
// coefficient table: the needed bins at velocity vmin+i, bb = 2pi fmax tao/r,
// funMandC, LSMOrCon_rec_2D.cpp:52-66).
__global__ void __launch_bounds__(kThreads) k_coef(CoefArgs a)
{
    __shared__ double sA[kMaxM * kMaxM], sb[kMaxM], sx[kMaxM], c[kMaxM + 1];
    LsCase q;
    q.r = a.r[blockIdx.x];
    q.bb = a.bb[blockIdx.x];
    q.pinv2 = a.pinv2[blockIdx.x];
    q.M = a.M[blockIdx.x];
    block_solve(q, a.hzx, sA, sb, sx, c);
    if (threadIdx.x <= q.M) a.out[(long)blockIdx.x * (kMaxM + 1) + threadIdx.x] = c[threadIdx.x];
}

// Solves n cases on the device; c receives [n][kMaxM+1].
int solve_cases(const std::vector<double> &r, const std::vector<double> &bb,
                const std::vector<int> &M, double hzx, std::vector<double> &c);

// Bisection of calfdlen_ls over the bins, with the per-velocity search
// "shortest passing length >= start" answered from the pass table.
struct LenSearch {
    const std::vector<unsigned char> &pass;
    int nfdmax;
    int eval(int bin1, int start) const
    {
        int len = 0;
        for (int j = start; j <= nfdmax; ++j) {
            len = j;
            if (pass[(size_t)(bin1 - 1) * (nfdmax + 1) + j]) break;
        }
        return len;
    }
};

int len_table(const LenSearch &S, int *len, int nvel, int nfdmin)
{
    int ibeg = 1, iend = nvel, flag = 0;
    int i1, i2, i3 = 0, i4, l1, l2, l3 = 0, l4, lbeg;
    i1 = ibeg;
    l1 = S.eval(i1, nfdmin);
    if (l1 == 0) return -1;
    lbeg = l1;
    len[i1 - 1] = l1;
    i2 = iend;
    l2 = S.eval(i2, nfdmin);
    if (l2 == 0) return -1;
    len[i2 - 1] = l2;
    if (l1 == l2) {
        for (int i = ibeg + 1; i <= iend; ++i) len[i - 1] = l1;
        return 0;
    }
    int inc = (iend - ibeg) / (2 * (l1 - l2));
    if (inc < 1) inc = 1;
    for (;;) {
        i1 = i2 - inc;
        if (i1 < ibeg) {
            i1 = ibeg;
            l1 = lbeg;
            if (i1 == i2) return 0;
        } else {
            l1 = S.eval(i1, l2);
            if (l1 == 0) return -1;
        }
        for (;;) {
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
                l4 = S.eval(i4, l2);
                if (l4 == 0) return -1;
                if (l4 == l2) {
                    for (int i = i4; i <= i2 - 1; ++i) len[i - 1] = l2;
                    i2 = i4;
                    l2 = l4;
                } else {
                    i1 = i4;
                    l1 = l4;
                }
                continue;
            }
            if (flag == 1) {
                flag = 0;
                if (l3 == l2) {
                    for (int i = i3; i <= i2 - 1; ++i) len[i - 1] = l2;
                    i2 = i3;
                    l2 = l3;
                    break;
                }
                i1 = i3;
                l1 = l3;
                continue;
            }
            if (l2 == lbeg) {
                for (int i = ibeg; i <= i2 - 1; ++i) len[i - 1] = l2;
                return 0;
            }
            break;
        }
    }
}

template <class T>
struct DevBuf {
    T *p = nullptr;
    ~DevBuf()
    {
        if (p) cudaFree(p);
    }
    cudaError_t alloc(size_t n) { return cudaMalloc(&p, sizeof(T) * (n ? n : 1)); }
};

int solve_cases(const std::vector<double> &r, const std::vector<double> &bb,
                const std::vector<int> &M, double hzx, std::vector<double> &c)
{
    const int n = (int)r.size();
    std::vector<double> pp(n);
    for (int i = 0; i < n; ++i) pp[i] = std::pow(r[i], -2);
    DevBuf<double> dr, dbb, dp, dout;
    DevBuf<int> dm;
    RTM_CUDA_TRY(dr.alloc(n));
    RTM_CUDA_TRY(dbb.alloc(n));
    RTM_CUDA_TRY(dp.alloc(n));
    RTM_CUDA_TRY(dm.alloc(n));
    RTM_CUDA_TRY(dout.alloc((size_t)n * (kMaxM + 1)));
    RTM_CUDA_TRY(cudaMemcpy(dr.p, r.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
    RTM_CUDA_TRY(cudaMemcpy(dbb.p, bb.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
    RTM_CUDA_TRY(cudaMemcpy(dp.p, pp.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
    RTM_CUDA_TRY(cudaMemcpy(dm.p, M.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    RTM_CUDA_TRY(cudaMemset(dout.p, 0, sizeof(double) * n * (kMaxM + 1)));
    CoefArgs ca;
    ca.r = dr.p; ca.bb = dbb.p; ca.pinv2 = dp.p; ca.M = dm.p; ca.hzx = hzx; ca.out = dout.p;
    k_coef<<<n, kThreads>>>(ca);
    RTM_LAUNCH_CHECK();
    c.assign((size_t)n * (kMaxM + 1), 0.0);
    RTM_CUDA_TRY(cudaMemcpy(c.data(), dout.p, sizeof(double) * c.size(), cudaMemcpyDeviceToHost));
    return RTM_OK;
}

}  // namespace

extern "C" {

int rtm_coeffs_optimise_fp64(const rtm_ls_settings *s, double vmin, double dv, int nvel,
                             const int *need, int *len, int *index, float *coef, int ccap,
                             int *nc_out)
{
    if (!s || nvel < 1 || !need || !len || !index || !nc_out || s->nfdmin < 1 ||
        s->nfdmax < s->nfdmin || s->nfdmax > kMaxM || s->nthita < 1 || !(s->df > 0) ||
        !(s->fmax > 0)) {
        rtm_set_last_error("rtm_coeffs_optimise_fp64: bad argument");
        return RTM_ERR_ARG;
    }
    const int nfre = (int)(s->fmax / s->df) + 1;
    const int nj = s->nfdmax - s->nfdmin + 1;
    std::vector<double> pinv(nvel);
    for (int i = 0; i < nvel; ++i) {
        const double vel = vmin + i * dv;
        pinv[i] = std::pow(vel * s->tao / s->h, -2);
    }
    DevBuf<double> dpinv;
    DevBuf<unsigned char> dpass;
    RTM_CUDA_TRY(dpinv.alloc(nvel));
    RTM_CUDA_TRY(dpass.alloc((size_t)nvel * (s->nfdmax + 1)));
    RTM_CUDA_TRY(cudaMemcpy(dpinv.p, pinv.data(), sizeof(double) * nvel, cudaMemcpyHostToDevice));
    RTM_CUDA_TRY(cudaMemset(dpass.p, 0, (size_t)nvel * (s->nfdmax + 1)));
    PassArgs pa;
    pa.vmin = vmin; pa.dv = dv; pa.tao = s->tao; pa.h = s->h; pa.df = s->df; pa.eps = s->eps;
    pa.hzx = s->hzx; pa.nfre = nfre; pa.nthita = s->nthita; pa.nfdmin = s->nfdmin;
    pa.nfdmax = s->nfdmax; pa.nvel = nvel; pa.pinv2 = dpinv.p; pa.pass = dpass.p;
    k_len_pass<<<(unsigned)(nvel * nj), kThreads>>>(pa);
    RTM_LAUNCH_CHECK();
    std::vector<unsigned char> pass((size_t)nvel * (s->nfdmax + 1));
    RTM_CUDA_TRY(cudaMemcpy(pass.data(), dpass.p, pass.size(), cudaMemcpyDeviceToHost));
    LenSearch S{pass, s->nfdmax};
    if (len_table(S, len, nvel, s->nfdmin) < 0) {
        rtm_set_last_error("operator length search failed (fmax or eps too large)");
        return RTM_ERR_ARG;
    }
    for (int i = 0; i < nvel; ++i)
        if (need[i] == 0) len[i] = -1;
    index[0] = 0;
    for (int i = 1; i <= nvel; ++i) index[i] = index[i - 1] + len[i - 1] + 1;
    *nc_out = index[nvel];
    if (!coef) return RTM_OK;
    if (ccap < index[nvel]) {
        rtm_set_last_error("coefficient buffer too small");
        return RTM_ERR_ARG;
    }
    std::vector<int> bins, mm;
    std::vector<double> rr, bbv;
    const double rat = s->tao / s->h, ra = 2.0 * kPi * s->fmax * s->tao;
    for (int i = 0; i < nvel; ++i)
        if (need[i] == 1) {
            bins.push_back(i);
            const double r = (vmin + i) * rat;  // velocity vmin+i (LSMOrCon_rec_2D.cpp:58)
            rr.push_back(r);
            bbv.push_back(ra / r);
            mm.push_back(len[i]);
        }
    if (bins.empty()) return RTM_OK;
    std::vector<double> out;
    if (int rc = solve_cases(rr, bbv, mm, s->hzx, out)) return rc;
    for (size_t q = 0; q < bins.size(); ++q) {
        const int i = bins[q];
        for (int l = 0; l <= len[i]; ++l) coef[index[i] + l] = (float)out[q * (kMaxM + 1) + l];
    }
    return RTM_OK;
}

int rtm_ls_coefs_fp64(const double *r, const double *bb, const int *M, int n, double hzx,
                      double *c)
{
    if (!r || !bb || !M || !c || n < 1) return RTM_ERR_ARG;
    for (int i = 0; i < n; ++i)
        if (M[i] < 1 || M[i] > kMaxM) return RTM_ERR_ARG;
    std::vector<double> out;
    if (int rc = solve_cases(std::vector<double>(r, r + n), std::vector<double>(bb, bb + n),
                             std::vector<int>(M, M + n), hzx, out))
        return rc;
    for (int i = 0; i < n; ++i)
        for (int l = 0; l <= M[i]; ++l) c[(size_t)i * (kMaxM + 1) + l] = out[(size_t)i * (kMaxM + 1) + l];
    return RTM_OK;
}

}  // extern "C"
