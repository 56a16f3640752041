// Learned finite-difference coefficients: a 3-layer MLP (3 -> 64 -> 64 -> 16,
// tanh hidden layers, FP32) that maps (r = v*tao/h, band limit kmax*h, M) to
// the M spatial coefficients c_1..c_M of the least-squares optimal operator
// (c_0 = -2*sum c_l as the optimiser sets it, LSMOrCon_rec_2D.cpp:274-279).
// Trained on the GPU against coefficient sets the FP64 optimiser produces
// (rtm_ls_coefs_fp64) by matching their operators (FD symbols, see
// k_mlp_delta), with hand-written forward / backward / Adam kernels.
// A coefficient table built with it is judged per velocity bin by the
// dispersion error; bins that miss the tolerance fall back to the optimiser.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "rtm_common.cuh"

namespace {

constexpr int NI = 3, NH = 64, NO = 16;  // outputs c_1..c_16 (M <= 16; unused ones masked)
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + NH * NI, OFF_W2 = OFF_B1 + NH, OFF_B2 = OFF_W2 + NH * NH,
              OFF_W3 = OFF_B2 + NH, OFF_B3 = OFF_W3 + NO * NH, NPARAM = OFF_B3 + NO;

struct Norm {
    float in_mean[NI], in_scale[NI];
    float out_mean[NO], out_scale[NO];
};

// x: [n][3] raw inputs (r, kh, M); h1, h2: [n][64]; y: [n][16] (normalised outputs)
__global__ void k_mlp_forward(const float *__restrict__ P, Norm nm, const float *__restrict__ x,
                              int n, float *__restrict__ h1o, float *__restrict__ h2o,
                              float *__restrict__ y)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    float xi[NI];
#pragma unroll
    for (int k = 0; k < NI; ++k) xi[k] = (x[b * NI + k] - nm.in_mean[k]) / nm.in_scale[k];
    float h1[NH];
#pragma unroll
    for (int i = 0; i < NH; ++i) {
        float a = P[OFF_B1 + i];
#pragma unroll
        for (int k = 0; k < NI; ++k) a = fmaf(P[OFF_W1 + i * NI + k], xi[k], a);
        h1[i] = tanhf(a);
        if (h1o) h1o[(long)b * NH + i] = h1[i];
    }
    float out[NO];
#pragma unroll
    for (int o = 0; o < NO; ++o) out[o] = P[OFF_B3 + o];
    for (int i = 0; i < NH; ++i) {
        float a = P[OFF_B2 + i];
#pragma unroll
        for (int j = 0; j < NH; ++j) a = fmaf(P[OFF_W2 + i * NH + j], h1[j], a);
        const float h = tanhf(a);
        if (h2o) h2o[(long)b * NH + i] = h;
#pragma unroll
        for (int o = 0; o < NO; ++o) out[o] = fmaf(P[OFF_W3 + o * NH + i], h, out[o]);
    }
#pragma unroll
    for (int o = 0; o < NO; ++o) y[(long)b * NO + o] = out[o];
}

// Training loss in operator space.  For a coefficient set c the 2-D FD
// symbol at wavenumber k (kh = u*bb) and angle th is
//   S(u, th) = sum_{l<=M} c_l g_l,  g_l = sin^2(l kh cos th/2) + sin^2(l kh sin th/2),
// and the exact symbol is (kh)^2/4, so S_net - S_opt relative to (kh)^2/4 is
// (to first order) the dispersion difference of the two operators.  The loss
// is the mean over samples and over an 8 x 4 grid of (u, th) of that squared
// relative difference; it is insensitive to the ill-conditioned directions in
// which the optimiser's coefficients move without changing the operator.
// Also back-propagates dz2 = (W3^T dy)*(1-h2^2), dz1 = (W2^T dz2)*(1-h1^2).
constexpr int NU = 8, NT_ = 4;

__global__ void k_mlp_delta(const float *__restrict__ P, Norm nm, const float *__restrict__ x,
                            const float *__restrict__ t, const float *__restrict__ y,
                            const float *__restrict__ h1, const float *__restrict__ h2, int n,
                            float inv_n, float *__restrict__ dy, float *__restrict__ dz1,
                            float *__restrict__ dz2, float *__restrict__ loss)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    const int M = min((int)x[b * NI + 2], NO);
    const float bb = x[b * NI + 1];
    float dc[NO];  // c_net - c_opt (raw units)
#pragma unroll
    for (int o = 0; o < NO; ++o)
        dc[o] = (o < M) ? (y[(long)b * NO + o] - t[(long)b * NO + o]) * nm.out_scale[o] : 0.0f;
    float gsum[NO];
#pragma unroll
    for (int o = 0; o < NO; ++o) gsum[o] = 0.0f;
    float l2 = 0.0f;
    const float wnorm = 1.0f / (NU * NT_);
    for (int iu = 1; iu <= NU; ++iu) {
        const float kh = bb * iu / NU;
        const float w = 4.0f / (kh * kh);
        for (int it = 0; it < NT_; ++it) {
            const float th = it * (0.78539816f / (NT_ - 1));
            const float cs = cosf(th) * kh * 0.5f, sn = sinf(th) * kh * 0.5f;
            float g[NO];
            float e = 0.0f;
#pragma unroll
            for (int o = 0; o < NO; ++o) {
                const float s1 = sinf((o + 1) * cs), s2 = sinf((o + 1) * sn);
                g[o] = (o < M) ? s1 * s1 + s2 * s2 : 0.0f;
                e = fmaf(dc[o], g[o], e);
            }
            const float r = w * e;
            l2 = fmaf(r, r, l2);
#pragma unroll
            for (int o = 0; o < NO; ++o) gsum[o] = fmaf(r * w, g[o], gsum[o]);
        }
    }
    atomicAdd(loss, l2 * wnorm * inv_n);
    float d[NO];
#pragma unroll
    for (int o = 0; o < NO; ++o) {
        d[o] = 2.0f * gsum[o] * wnorm * inv_n * nm.out_scale[o];
        dy[(long)b * NO + o] = d[o];
    }
    float g2[NH];
#pragma unroll
    for (int i = 0; i < NH; ++i) {
        float a = 0.0f;
#pragma unroll
        for (int o = 0; o < NO; ++o) a = fmaf(P[OFF_W3 + o * NH + i], d[o], a);
        const float h = h2[(long)b * NH + i];
        g2[i] = a * (1.0f - h * h);
        dz2[(long)b * NH + i] = g2[i];
    }
    for (int j = 0; j < NH; ++j) {
        float a = 0.0f;
#pragma unroll
        for (int i = 0; i < NH; ++i) a = fmaf(P[OFF_W2 + i * NH + j], g2[i], a);
        const float h = h1[(long)b * NH + j];
        dz1[(long)b * NH + j] = a * (1.0f - h * h);
    }
}

// Parameter gradients: one thread per parameter, summing over the batch.
__global__ void k_mlp_grad(Norm nm, const float *__restrict__ x, const float *__restrict__ h1,
                           const float *__restrict__ h2, const float *__restrict__ dy,
                           const float *__restrict__ dz1, const float *__restrict__ dz2, int n,
                           float *__restrict__ G)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= NPARAM) return;
    float g = 0.0f;
    if (p < OFF_B1) {
        const int i = p / NI, k = p % NI;
        for (int b = 0; b < n; ++b)
            g = fmaf(dz1[(long)b * NH + i], (x[b * NI + k] - nm.in_mean[k]) / nm.in_scale[k], g);
    } else if (p < OFF_W2) {
        const int i = p - OFF_B1;
        for (int b = 0; b < n; ++b) g += dz1[(long)b * NH + i];
    } else if (p < OFF_B2) {
        const int i = (p - OFF_W2) / NH, j = (p - OFF_W2) % NH;
        for (int b = 0; b < n; ++b) g = fmaf(dz2[(long)b * NH + i], h1[(long)b * NH + j], g);
    } else if (p < OFF_W3) {
        const int i = p - OFF_B2;
        for (int b = 0; b < n; ++b) g += dz2[(long)b * NH + i];
    } else if (p < OFF_B3) {
        const int o = (p - OFF_W3) / NH, i = (p - OFF_W3) % NH;
        for (int b = 0; b < n; ++b) g = fmaf(dy[(long)b * NO + o], h2[(long)b * NH + i], g);
    } else {
        const int o = p - OFF_B3;
        for (int b = 0; b < n; ++b) g += dy[(long)b * NO + o];
    }
    G[p] = g;
}

__global__ void k_adam(float *P, const float *G, float *m1, float *m2, float lr, float b1, float b2,
                       float eps, float c1, float c2)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= NPARAM) return;
    const float g = G[p];
    const float a = b1 * m1[p] + (1.0f - b1) * g;
    const float v = b2 * m2[p] + (1.0f - b2) * g * g;
    m1[p] = a;
    m2[p] = v;
    P[p] -= lr * (a / c1) / (sqrtf(v / c2) + eps);
}

// Gathers a minibatch of samples by index.
__global__ void k_gather(const float *x, const float *t, const int *idx, int n, float *xb, float *tb)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    const int s = idx[b];
#pragma unroll
    for (int k = 0; k < NI; ++k) xb[b * NI + k] = x[s * NI + k];
#pragma unroll
    for (int o = 0; o < NO; ++o) tb[(long)b * NO + o] = t[(long)s * NO + o];
}

// Largest relative phase-velocity error |v_FD/v - 1| of each coefficient set
// over kh in (0, bb] (nk samples) and propagation angles theta in [0, pi/4]
// (nth+1 samples), for the 2-D operator with hz = hzx*h:
//   v_FD/v = 2/(r kh) asin( r sqrt( sum_l c_l (sin^2(l kh cos th/2)
//                                        + sin^2(l hzx kh sin th/2)/hzx^2) ) )
// One block per set.
__global__ void k_disp_err(const double *c, int cstride, const int *M, const double *r,
                           const double *bb, int nk, int nth, double hzx, int metric, double tao,
                           double *err)
{
    const int s = blockIdx.x;
    const int m = M[s];
    const double rr = r[s], kmax = bb[s];
    double worst = 0.0;
    for (int t = threadIdx.x; t < nk * (nth + 1); t += blockDim.x) {
        const int k = 1 + t / (nth + 1), n = t % (nth + 1);
        const double kh = kmax * k / nk;
        const double th = n * (M_PI / 4) / nth;
        double mid = 0.0;
        for (int l = 1; l <= m; ++l) {
            const double s1 = sin(l * hzx * kh * sin(th) / 2), s2 = sin(l * kh * cos(th) / 2);
            mid += c[(long)s * cstride + l] * (s1 * s1 / (hzx * hzx) + s2 * s2);
        }
        const double arg = rr * sqrt(fmax(mid, 0.0));
        double e;
        if (arg > 1.0 || !(arg > 0.0)) {
            e = 1.0;  // no real phase velocity: the operator is unstable here
        } else {
            const double ratio = 2.0 / (rr * kh) * asin(arg);  // v_FD / v
            // metric 1: the reference's measure (h/v) |v/v_FD - 1|, h/v = tao/r
            e = metric ? fabs(1.0 / ratio - 1.0) * (tao / rr) : fabs(ratio - 1.0);
        }
        worst = fmax(worst, e);
    }
    __shared__ double red[256];
    red[threadIdx.x] = worst;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) err[s] = red[0];
}

template <class T>
struct DBuf {
    T *p = nullptr;
    size_t n = 0;
    ~DBuf()
    {
        if (p) cudaFree(p);
    }
    int ensure(size_t k)
    {
        if (k <= n) return RTM_OK;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        if (cudaMalloc(&p, sizeof(T) * (k ? k : 1)) != cudaSuccess) {
            cudaGetLastError();
            rtm_set_last_error("cudaMalloc failed");
            return RTM_ERR_NOMEM;
        }
        n = k;
        return RTM_OK;
    }
};

inline unsigned cdiv(long a, long b) { return (unsigned)((a + b - 1) / b); }

}  // namespace

struct rtm_mlp {
    Norm nm{};
    DBuf<float> P, G, m1, m2;
    DBuf<float> x, t, xb, tb, h1, h2, y, dy, dz1, dz2, loss;
    DBuf<int> idx;
    long step = 0;
    unsigned seed = 0;
};

extern "C" {

int rtm_mlp_create(rtm_mlp **out, unsigned seed)
{
    if (!out) return RTM_ERR_ARG;
    rtm_mlp *m = new rtm_mlp();
    m->seed = seed;
    for (int k = 0; k < NI; ++k) {
        m->nm.in_mean[k] = 0.0f;
        m->nm.in_scale[k] = 1.0f;
    }
    for (int o = 0; o < NO; ++o) {
        m->nm.out_mean[o] = 0.0f;
        m->nm.out_scale[o] = 1.0f;
    }
    int rc;
    if ((rc = m->P.ensure(NPARAM)) || (rc = m->G.ensure(NPARAM)) || (rc = m->m1.ensure(NPARAM)) ||
        (rc = m->m2.ensure(NPARAM))) {
        delete m;
        return rc;
    }
    // Xavier-uniform weights, zero biases
    std::mt19937 rng(seed);
    std::vector<float> P(NPARAM, 0.0f);
    auto fill = [&](int off, int fan_out, int fan_in) {
        std::uniform_real_distribution<float> u(-1.0f, 1.0f);
        const float a = std::sqrt(6.0f / (fan_in + fan_out));
        for (int i = 0; i < fan_out * fan_in; ++i) P[off + i] = a * u(rng);
    };
    fill(OFF_W1, NH, NI);
    fill(OFF_W2, NH, NH);
    fill(OFF_W3, NO, NH);
    if (cudaMemcpy(m->P.p, P.data(), sizeof(float) * NPARAM, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(m->m1.p, 0, sizeof(float) * NPARAM) != cudaSuccess ||
        cudaMemset(m->m2.p, 0, sizeof(float) * NPARAM) != cudaSuccess) {
        delete m;
        rtm_set_last_error("upload failed");
        return RTM_ERR_CUDA;
    }
    *out = m;
    return RTM_OK;
}

int rtm_mlp_destroy(rtm_mlp *m)
{
    delete m;
    return RTM_OK;
}

int rtm_mlp_nparams(void) { return NPARAM; }

int rtm_mlp_get_params(const rtm_mlp *m, float *params)
{
    if (!m || !params) return RTM_ERR_ARG;
    RTM_CUDA_TRY(cudaMemcpy(params, m->P.p, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost));
    return RTM_OK;
}

int rtm_mlp_set_params(rtm_mlp *m, const float *params)
{
    if (!m || !params) return RTM_ERR_ARG;
    RTM_CUDA_TRY(cudaMemcpy(m->P.p, params, sizeof(float) * NPARAM, cudaMemcpyHostToDevice));
    return RTM_OK;
}

// norm: in_mean[3], in_scale[3], out_mean[16], out_scale[16]
int rtm_mlp_set_norm(rtm_mlp *m, const float *norm)
{
    if (!m || !norm) return RTM_ERR_ARG;
    std::memcpy(&m->nm, norm, sizeof(Norm));
    return RTM_OK;
}

int rtm_mlp_get_norm(const rtm_mlp *m, float *norm)
{
    if (!m || !norm) return RTM_ERR_ARG;
    std::memcpy(norm, &m->nm, sizeof(Norm));
    return RTM_OK;
}

static int upload_samples(rtm_mlp *m, const float *x, const float *c, int n)
{
    // targets: normalised coefficients
    std::vector<float> t((size_t)n * NO, 0.0f);
    for (int b = 0; b < n; ++b)
        for (int o = 0; o < NO; ++o)
            t[(size_t)b * NO + o] = (c[(size_t)b * NO + o] - m->nm.out_mean[o]) / m->nm.out_scale[o];
    int rc;
    if ((rc = m->x.ensure((size_t)n * NI)) || (rc = m->t.ensure((size_t)n * NO))) return rc;
    RTM_CUDA_TRY(cudaMemcpy(m->x.p, x, sizeof(float) * n * NI, cudaMemcpyHostToDevice));
    RTM_CUDA_TRY(cudaMemcpy(m->t.p, t.data(), sizeof(float) * t.size(), cudaMemcpyHostToDevice));
    return RTM_OK;
}

static int ensure_batch(rtm_mlp *m, int nb)
{
    int rc;
    if ((rc = m->xb.ensure((size_t)nb * NI)) || (rc = m->tb.ensure((size_t)nb * NO)) ||
        (rc = m->h1.ensure((size_t)nb * NH)) || (rc = m->h2.ensure((size_t)nb * NH)) ||
        (rc = m->y.ensure((size_t)nb * NO)) || (rc = m->dy.ensure((size_t)nb * NO)) ||
        (rc = m->dz1.ensure((size_t)nb * NH)) || (rc = m->dz2.ensure((size_t)nb * NH)) ||
        (rc = m->loss.ensure(1)) || (rc = m->idx.ensure(nb)))
        return rc;
    return RTM_OK;
}

// Loss and parameter gradient on one batch given as arrays (x [n][3] with
// x[:,2] = M; c [n][16] raw coefficients, unused entries ignored).
int rtm_mlp_grad(rtm_mlp *m, const float *x, const float *c, int n, float *grad, float *loss)
{
    if (!m || !x || !c || n < 1) return RTM_ERR_ARG;
    int rc;
    if ((rc = upload_samples(m, x, c, n)) || (rc = ensure_batch(m, n))) return rc;
    const float inv = 1.0f / (float)n;
    RTM_CUDA_TRY(cudaMemset(m->loss.p, 0, sizeof(float)));
    k_mlp_forward<<<cdiv(n, 128), 128>>>(m->P.p, m->nm, m->x.p, n, m->h1.p, m->h2.p, m->y.p);
    k_mlp_delta<<<cdiv(n, 128), 128>>>(m->P.p, m->nm, m->x.p, m->t.p, m->y.p, m->h1.p, m->h2.p, n, inv,
                                       m->dy.p, m->dz1.p, m->dz2.p, m->loss.p);
    k_mlp_grad<<<cdiv(NPARAM, 128), 128>>>(m->nm, m->x.p, m->h1.p, m->h2.p, m->dy.p, m->dz1.p,
                                           m->dz2.p, n, m->G.p);
    RTM_LAUNCH_CHECK();
    if (grad) RTM_CUDA_TRY(cudaMemcpy(grad, m->G.p, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost));
    if (loss) RTM_CUDA_TRY(cudaMemcpy(loss, m->loss.p, sizeof(float), cudaMemcpyDeviceToHost));
    return RTM_OK;
}

// Minibatch Adam training on n samples for `epochs` passes.
int rtm_mlp_train(rtm_mlp *m, const float *x, const float *c, int n, int epochs, int batch, float lr,
                  float *final_loss)
{
    if (!m || !x || !c || n < 1 || epochs < 0 || batch < 1) return RTM_ERR_ARG;
    int rc;
    if ((rc = upload_samples(m, x, c, n)) || (rc = ensure_batch(m, batch))) return rc;
    std::mt19937 rng(m->seed * 7919u + 17u);
    std::vector<int> perm(n);
    for (int i = 0; i < n; ++i) perm[i] = i;
    float last = 0.0f;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int e = 0; e < epochs; ++e) {
        // cosine decay from lr to lr/20 over the run
        const float lre = lr * (0.05f + 0.475f * (1.0f + std::cos(3.14159265f * e / epochs)));
        std::shuffle(perm.begin(), perm.end(), rng);
        RTM_CUDA_TRY(cudaMemset(m->loss.p, 0, sizeof(float)));
        int nbat = 0;
        for (int s0 = 0; s0 < n; s0 += batch, ++nbat) {
            const int nb = std::min(batch, n - s0);
            const float inv = 1.0f / (float)nb;
            RTM_CUDA_TRY(cudaMemcpyAsync(m->idx.p, perm.data() + s0, sizeof(int) * nb,
                                         cudaMemcpyHostToDevice, 0));
            k_gather<<<cdiv(nb, 128), 128>>>(m->x.p, m->t.p, m->idx.p, nb, m->xb.p, m->tb.p);
            k_mlp_forward<<<cdiv(nb, 128), 128>>>(m->P.p, m->nm, m->xb.p, nb, m->h1.p, m->h2.p, m->y.p);
            k_mlp_delta<<<cdiv(nb, 128), 128>>>(m->P.p, m->nm, m->xb.p, m->tb.p, m->y.p, m->h1.p, m->h2.p, nb,
                                                inv, m->dy.p, m->dz1.p, m->dz2.p, m->loss.p);
            k_mlp_grad<<<cdiv(NPARAM, 128), 128>>>(m->nm, m->xb.p, m->h1.p, m->h2.p, m->dy.p,
                                                   m->dz1.p, m->dz2.p, nb, m->G.p);
            ++m->step;
            k_adam<<<cdiv(NPARAM, 128), 128>>>(m->P.p, m->G.p, m->m1.p, m->m2.p, lre, b1, b2, eps,
                                               1.0f - std::pow(b1, (float)m->step),
                                               1.0f - std::pow(b2, (float)m->step));
        }
        RTM_LAUNCH_CHECK();
        float l = 0.0f;
        RTM_CUDA_TRY(cudaMemcpy(&l, m->loss.p, sizeof(float), cudaMemcpyDeviceToHost));
        last = l / nbat;
    }
    if (final_loss) *final_loss = last;
    return RTM_OK;
}

// Raw coefficients c_1..c_16 [n][16] predicted for inputs x [n][3].
int rtm_mlp_predict(rtm_mlp *m, const float *x, int n, float *c)
{
    if (!m || !x || !c || n < 1) return RTM_ERR_ARG;
    int rc;
    if ((rc = m->xb.ensure((size_t)n * NI)) || (rc = m->y.ensure((size_t)n * NO))) return rc;
    RTM_CUDA_TRY(cudaMemcpy(m->xb.p, x, sizeof(float) * n * NI, cudaMemcpyHostToDevice));
    k_mlp_forward<<<cdiv(n, 128), 128>>>(m->P.p, m->nm, m->xb.p, n, nullptr, nullptr, m->y.p);
    RTM_LAUNCH_CHECK();
    RTM_CUDA_TRY(cudaMemcpy(c, m->y.p, sizeof(float) * n * NO, cudaMemcpyDeviceToHost));
    for (int b = 0; b < n; ++b)
        for (int o = 0; o < NO; ++o)
            c[(size_t)b * NO + o] = c[(size_t)b * NO + o] * m->nm.out_scale[o] + m->nm.out_mean[o];
    return RTM_OK;
}

// Largest phase-velocity error of n coefficient sets c[n][cstride] (c_0..c_M
// in FP64) at Courant numbers r and band limits bb, in the measure `metric`
// (RTM_DISP_RELATIVE or RTM_DISP_REFERENCE; tao is the time step of the
// latter's h/v = tao/r).
int rtm_disp_error_fp64(const double *c, int cstride, const int *M, const double *r,
                        const double *bb, int n, int nk, int nth, double hzx, int metric, double tao,
                        double *err)
{
    if (!c || !M || !r || !bb || !err || n < 1 || nk < 1 || nth < 1 ||
        (metric != RTM_DISP_RELATIVE && metric != RTM_DISP_REFERENCE) || (metric && !(tao > 0)))
        return RTM_ERR_ARG;
    DBuf<double> dc, dr, dbb, de;
    DBuf<int> dm;
    int rc;
    if ((rc = dc.ensure((size_t)n * cstride)) || (rc = dr.ensure(n)) || (rc = dbb.ensure(n)) ||
        (rc = de.ensure(n)) || (rc = dm.ensure(n)))
        return rc;
    RTM_CUDA_TRY(cudaMemcpy(dc.p, c, sizeof(double) * n * cstride, cudaMemcpyHostToDevice));
    RTM_CUDA_TRY(cudaMemcpy(dr.p, r, sizeof(double) * n, cudaMemcpyHostToDevice));
    RTM_CUDA_TRY(cudaMemcpy(dbb.p, bb, sizeof(double) * n, cudaMemcpyHostToDevice));
    RTM_CUDA_TRY(cudaMemcpy(dm.p, M, sizeof(int) * n, cudaMemcpyHostToDevice));
    k_disp_err<<<n, 256>>>(dc.p, cstride, dm.p, dr.p, dbb.p, nk, nth, hzx, metric, tao, de.p);
    RTM_LAUNCH_CHECK();
    RTM_CUDA_TRY(cudaMemcpy(err, de.p, sizeof(double) * n, cudaMemcpyDeviceToHost));
    return RTM_OK;
}


int rtm_ls_coefs_fp64(const double *r, const double *bb, const int *M, int n, double hzx, double *c);

// Coefficient table (the layout of funMandC, LSMOrCon_rec_2D.cpp:45-66) from
// the network: every needed bin i (velocity vmin + i, band limit
// bb = 2 pi fmax tao / r as funMandC designs it) gets operator length M and
// the network's coefficients when their largest phase-velocity error (in the
// measure `metric`) is <= tol.  For the other bins the FP64 optimiser designs
// the set too, and the bin keeps whichever of the two sets has the lower
// error (*nfallback counts the bins that keep the optimiser's), so no bin's
// error is above the network's or the optimiser's.  err_net[nvel] /
// err_used[nvel] (optional) receive the errors of the network's set and of
// the set kept (-1 for bins not needed).
int rtm_coeffs_mlp(rtm_mlp *m, const rtm_ls_settings *s, double vmin, int nvel, const int *need,
                   int M, double tol, int metric, int *len, int *index, float *coef, int ccap,
                   int *nc, int *nfallback, double *err_net, double *err_used)
{
    if (!m || !s || nvel < 1 || !need || !len || !index || !nc || M < 1 || M > NO ||
        (metric != RTM_DISP_RELATIVE && metric != RTM_DISP_REFERENCE))
        return RTM_ERR_ARG;
    index[0] = 0;
    for (int i = 0; i < nvel; ++i) {
        len[i] = need[i] ? M : -1;
        index[i + 1] = index[i] + len[i] + 1;
    }
    *nc = index[nvel];
    if (!coef) return RTM_OK;
    if (ccap < *nc) return RTM_ERR_ARG;
    std::vector<int> bins;
    std::vector<float> x;
    std::vector<double> rr, bbv;
    const double rat = s->tao / s->h, ra = 2.0 * 3.1415926535898 * s->fmax * s->tao;
    for (int i = 0; i < nvel; ++i)
        if (need[i]) {
            const double r = (vmin + i) * rat;
            bins.push_back(i);
            rr.push_back(r);
            bbv.push_back(ra / r);
            x.push_back((float)r);
            x.push_back((float)(ra / r));
            x.push_back((float)M);
        }
    const int nb = (int)bins.size();
    if (err_net)
        for (int i = 0; i < nvel; ++i) err_net[i] = -1.0;
    if (err_used)
        for (int i = 0; i < nvel; ++i) err_used[i] = -1.0;
    if (nfallback) *nfallback = 0;
    if (nb == 0) return RTM_OK;
    std::vector<float> pc((size_t)nb * NO);
    if (int rc = rtm_mlp_predict(m, x.data(), nb, pc.data())) return rc;
    const int CS = NO + 1;
    std::vector<double> cd((size_t)nb * CS, 0.0);
    std::vector<int> mm(nb, M);
    for (int q = 0; q < nb; ++q) {
        double sum = 0.0;
        for (int l = 1; l <= M; ++l) {
            cd[(size_t)q * CS + l] = pc[(size_t)q * NO + l - 1];
            sum += cd[(size_t)q * CS + l];
        }
        cd[(size_t)q * CS] = -2.0 * sum;
    }
    const int nk = std::max(8, (int)(s->fmax / s->df));
    std::vector<double> err(nb);
    if (int rc = rtm_disp_error_fp64(cd.data(), CS, mm.data(), rr.data(), bbv.data(), nb, nk, 32,
                                     s->hzx, metric, s->tao, err.data()))
        return rc;
    std::vector<int> fb;
    for (int q = 0; q < nb; ++q)
        if (!(err[q] <= tol)) fb.push_back(q);
    std::vector<double> used_err(err);
    int nopt = 0;
    if (!fb.empty()) {
        std::vector<double> fr, fbb, fc((size_t)fb.size() * CS);
        std::vector<int> fm(fb.size(), M);
        for (int q : fb) {
            fr.push_back(rr[q]);
            fbb.push_back(bbv[q]);
        }
        if (int rc = rtm_ls_coefs_fp64(fr.data(), fbb.data(), fm.data(), (int)fb.size(), s->hzx, fc.data()))
            return rc;
        std::vector<double> ferr(fb.size());
        if (int rc = rtm_disp_error_fp64(fc.data(), CS, fm.data(), fr.data(), fbb.data(), (int)fb.size(),
                                         nk, 32, s->hzx, metric, s->tao, ferr.data()))
            return rc;
        for (size_t k = 0; k < fb.size(); ++k) {
            // the lower-error set of the two (a NaN error never wins)
            if (!(ferr[k] < err[fb[k]]) && err[fb[k]] == err[fb[k]]) continue;
            std::copy(fc.begin() + k * CS, fc.begin() + (k + 1) * CS, cd.begin() + (size_t)fb[k] * CS);
            used_err[fb[k]] = ferr[k];
            ++nopt;
        }
    }
    if (nfallback) *nfallback = nopt;
    for (int q = 0; q < nb; ++q) {
        const int i = bins[q];
        for (int l = 0; l <= M; ++l) coef[index[i] + l] = (float)cd[(size_t)q * CS + l];
        if (err_net) err_net[i] = err[q];
        if (err_used) err_used[i] = used_err[q];
    }
    return RTM_OK;
}

}  // extern "C"
