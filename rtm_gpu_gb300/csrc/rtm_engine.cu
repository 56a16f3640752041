// Shot-level engine: context, batched forward / backward time loops captured
// in CUDA graphs, per-shot finishing and the compensated stack.
//
// Per shot (kernel.cu:791-990), for a batch of shots advancing together:
//   forward  k = 2..NT-1 : k_step<FWD> ; k_pad (blend, ring save, record)
//   hand-off            : k_img_init (accumulator initialisation)
//   backward k = NT-3..0 : k_step<BWD> (source reconstruction + receiver
//                          propagation + imaging) ; k_pad (receiver blend,
//                          ring restore of the source field)
// Levels rotate through three buffers by index (level k lives in buffer
// k % 3), so the reference's copy kernels (Deliver, Deliver_EFF) disappear.
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "rtm_engine_kernels.cuh"

namespace {

PFN_cuTensorMapEncodeTiled_v12000 get_encode()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        void *p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

int make_map(CUtensorMap *m, float *base, int NX, int NZ, int B, int P, int bw, int bh)
{
    auto enc = get_encode();
    if (!enc) {
        rtm_set_last_error("cuTensorMapEncodeTiled unavailable");
        return RTM_ERR_CUDA;
    }
    cuuint64_t dims[3] = {(cuuint64_t)NX, (cuuint64_t)NZ, (cuuint64_t)B};
    cuuint64_t strides[2] = {(cuuint64_t)P * 4, (cuuint64_t)P * 4 * NZ};
    cuuint32_t box[3] = {(cuuint32_t)bw, (cuuint32_t)bh, 1};
    cuuint32_t es[3] = {1, 1, 1};
    CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        rtm_set_last_error("cuTensorMapEncodeTiled failed");
        return RTM_ERR_CUDA;
    }
    return RTM_OK;
}

inline unsigned cdiv(long a, long b) { return (unsigned)((a + b - 1) / b); }

}  // namespace

struct rtm_ctx {
    rtm_problem p{};
    int NZ = 0, NX = 0, P = 0, nz = 0, nx = 0, N2 = 0, M = 0, MM = 0, B = 0, NT = 0, nrec = 0;
    long long ss = 0;       // floats per shot grid
    long ringsz = 0;        // cells per ring slot
    cudaStream_t st = nullptr;
    bool own_stream = false;  // created by the context (graphs cannot capture the legacy stream)
    cudaStream_t st2 = nullptr;           // second half-batch stream (RTM_KERNEL_SPLIT)
    cudaEvent_t evf[2] = {nullptr, nullptr};  // fork / join of the two streams
    cudaEvent_t evc[2] = {nullptr, nullptr};  // data upload on st2: may start / done
    std::vector<float> wav; // host wavelet table
    float vmax = 0.f;
    int nbins = 1;
    // device
    float *v = nullptr, *r1 = nullptr, *w = nullptr, *ctab = nullptr;
    float4 *ctab4 = nullptr;  // adaptive table in float4 groups
    int *blen = nullptr;      // operator length of each bin (adaptive)
    int4 *pad_meta = nullptr;
    float4 *pad_fac = nullptr;
    float *S[3] = {nullptr, nullptr, nullptr}, *R[3] = {nullptr, nullptr, nullptr};
    float *pre = nullptr, *rel1 = nullptr, *rel2 = nullptr, *sacc = nullptr, *racc = nullptr;
    float *ring = nullptr, *data = nullptr, *rec = nullptr, *stage = nullptr;
    // 16-bit ring store (ring_precision BF16 / F16)
    uint16_t *ring16 = nullptr;
    float *rstage = nullptr, *rscale = nullptr;  // [2][B][ringsz], [B][NT]
    unsigned *ramax = nullptr;                    // [B][NT]
    int *src = nullptr;
    unsigned *imax = nullptr;
    float *ups = nullptr, *downs = nullptr;                       // per-batch finished images
    float *ks1 = nullptr, *kc1 = nullptr, *ks2 = nullptr, *kc2 = nullptr;  // Kahan state
    float *img = nullptr, *ill = nullptr;
    CUtensorMap mapS[3], mapR[3];      // halo boxes of the rotating levels
    CUtensorMap flatS[3], flatR[3];    // flat tiles of the same buffers
    // per-cell model factors (v^2 tao^2/h^2 and velocity bin) of the model
    // shared by the batch, and of the per-shot window models
    float *mvv = nullptr, *mvvs = nullptr;
    int *mbin = nullptr, *mbins = nullptr;
    eng::ModelMaps mmaps, mmaps_s;
    // per-shot geometry of the current batch (device): padded width, window
    // start column in the survey interior, receiver start column
    int *gnx = nullptr, *gxa = nullptr, *grx0 = nullptr;
    int *gitem = nullptr;              // [B+1] first tile item of each shot (persistent kernel)
    std::vector<int> hnx, hxa;         // host copies for the current batch
    // stencil kernel form (fwd, bwd): the forms the autotuner picks on the
    // batched workloads, until it or rtm_ctx_set_kernel sets others
    int kv[2] = {RTM_KERNEL_X2_SPLIT, RTM_KERNEL_TILED};
    int nbl = 0;                           // shots per launch (<= B)
    int kstop = 0;                         // autotuning: time steps per phase (0: all)
    bool windowed = false;             // current batch uses per-shot models
    float *vs = nullptr, *r1s = nullptr;          // [B][NZ][P] window models
    int4 *meta_s = nullptr;
    float4 *fac_s = nullptr;                      // [B][nabc] window pad tables
    eng::ImgMaps imaps;                // flat tiles of the imaging accumulators
    // source snapshots (rtm_ctx_set_snapshots): every snap_every-th step
    // (0: off) the forward run stores the source field's interior and its
    // running sum (RTM_RING_* storage, per-(shot, slot) scales for 16-bit
    // codes); the backward run then advances the receiver field alone and
    // images at the snapshot steps
    int snap_every = 0, snap_prec = 0, snap_nslots = 0, snap_off = 0, snap_pitch = 0;
    void *snapS = nullptr;                      // [B][nslots][nz][snap_pitch] source field
    float *snapQ = nullptr;                     // the same for its running sum (fp32)
    float *pacc = nullptr;                      // [B][NZ][P] running sum of the source field
    float *snap_scale = nullptr;                // [B][nslots] scale of the 16-bit codes
    unsigned *snap_amax = nullptr;              // [B][nslots] max |S| (float bits)
    // cells around the receiver line, imaged at every step: their source
    // field and running sum at every step k <= NT-3 ([B][NT-2][zn*xn], fp32)
    eng::SnapBand band{};
    float *bandS = nullptr, *bandP = nullptr;
    size_t snap_bytes = 0;                      // device bytes of the above
    eng::SnapMaps smaps_f{}, smaps_b{};         // running sums: pacc (forward), racc (backward)
    size_t bytes = 0;
    // graphs keyed by (phase, batch)
    std::map<std::pair<int, int>, cudaGraphExec_t> graphs;
    // timing
    bool timing = false;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    double ms_stencil = 0, ms_pad = 0, ms_bwd = 0;
    long n_stencil = 0, n_pad = 0, n_bwd = 0;
    // kernels launched (graph replays count their kernels)
    long launches = 0;
    std::map<std::pair<int, int>, long> graph_kernels;
};

namespace {

template <class T>
int dalloc(rtm_ctx *c, T **p, size_t n)
{
    if (n == 0) n = 1;
    if (cudaMalloc(p, n * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        rtm_set_last_error("cudaMalloc failed");
        return RTM_ERR_NOMEM;
    }
    c->bytes += n * sizeof(T);
    if (cudaMemset(*p, 0, n * sizeof(T)) != cudaSuccess) return RTM_ERR_CUDA;
    return RTM_OK;
}

void free_snapshots(rtm_ctx *c)
{
    for (void *q : {c->snapS, (void *)c->snapQ, (void *)c->pacc, (void *)c->snap_scale, (void *)c->snap_amax,
                    (void *)c->bandS, (void *)c->bandP})
        if (q) cudaFree(q);
    c->snapS = nullptr;
    c->snapQ = c->pacc = c->snap_scale = c->bandS = c->bandP = nullptr;
    c->band = eng::SnapBand{};
    c->snap_amax = nullptr;
    c->snap_every = c->snap_nslots = 0;
    c->bytes -= c->snap_bytes;
    c->snap_bytes = 0;
}

void free_all(rtm_ctx *c)
{
    free_snapshots(c);
    if (c->st2) cudaStreamDestroy(c->st2);
    c->st2 = nullptr;
    for (cudaEvent_t *ev : {&c->evf[0], &c->evf[1], &c->evc[0], &c->evc[1]})
        if (*ev) {
            cudaEventDestroy(*ev);
            *ev = nullptr;
        }
    for (auto &kv : c->graphs) cudaGraphExecDestroy(kv.second);
    c->graphs.clear();
    float *fl[] = {c->mvv, c->mvvs, c->v, c->r1, c->w, c->ctab, c->S[0], c->S[1], c->S[2], c->R[0], c->R[1], c->R[2],
                   c->pre, c->rel1, c->rel2, c->sacc, c->racc, c->ring, c->data, c->rec, c->stage,
                   c->ups, c->downs, c->ks1, c->kc1, c->ks2, c->kc2, c->img, c->ill};
    for (float *p : fl)
        if (p) cudaFree(p);
    if (c->src) cudaFree(c->src);
    if (c->ctab4) cudaFree(c->ctab4);
    if (c->blen) cudaFree(c->blen);
    for (int *q : {c->gnx, c->gxa, c->grx0, c->gitem, c->mbin, c->mbins})
        if (q) cudaFree(q);
    if (c->vs) cudaFree(c->vs);
    if (c->r1s) cudaFree(c->r1s);
    if (c->meta_s) cudaFree(c->meta_s);
    if (c->fac_s) cudaFree(c->fac_s);
    if (c->ring16) cudaFree(c->ring16);
    if (c->rstage) cudaFree(c->rstage);
    if (c->rscale) cudaFree(c->rscale);
    if (c->ramax) cudaFree(c->ramax);
    if (c->pad_meta) cudaFree(c->pad_meta);
    if (c->pad_fac) cudaFree(c->pad_fac);
    if (c->imax) cudaFree(c->imax);
    for (auto &e : c->ev)
        if (e) cudaEventDestroy(e);
    if (c->own_stream && c->st) {
        cudaStreamDestroy(c->st);
        c->st = nullptr;
    }
}

// ---------------------------------------------------------------------------
// launch helpers

struct StepMaps {
    const CUtensorMap *A, *S, *A0, *S0;
};

// grid of the persistent stencil kernel: resident CTAs per SM x SMs
template <int MMAX, bool AD, int MODE>
int &pipe_grid()
{
    static int g = 0;
    return g;
}

template <int MMAX, bool AD, int MODE>
int launch_step_t(rtm_ctx *c, const StepMaps &m, const eng::StepArgs &a, int nb, cudaStream_t st)
{
    const eng::ModelMaps &fv = c->windowed ? c->mmaps_s : c->mmaps;
    constexpr int KI = eng::fwd_mode(MODE) ? 0 : 1;  // kernel-form slot of the step
    // (the snapshot steps run in the tiled form, in one stream or two halves)
    if constexpr (MODE == eng::MODE_FWD || MODE == eng::MODE_BWD) {
        if (c->kv[KI] == RTM_KERNEL_PERSISTENT) {
            const unsigned smem = eng::PipeSmem<MMAX, MODE>::BYTES;
            eng::k_step_pipe<MMAX, AD, MODE><<<pipe_grid<MMAX, AD, MODE>(), eng::NTHREADS, smem, c->st>>>(
                *m.A, *m.S, *m.A0, *m.S0, fv, c->imaps, a, c->gitem, nb);
            return RTM_OK;
        }
    }
    const unsigned smem = eng::Smem<MMAX, MODE>::BYTES;
    dim3 grid(cdiv(c->NX, eng::TX), cdiv(c->NZ, eng::TZ), nb);
    eng::StepArgs la = a;
    if (c->windowed) {
        // narrowest grid among the launch's shots
        int mn = c->NX;
        for (int i = a.shot0; i < a.shot0 + nb && i < (int)c->hnx.size(); ++i) mn = std::min(mn, c->hnx[i]);
        la.min_nx = mn;
    }
    if constexpr (MODE == eng::MODE_FWD) {
        if (c->kv[KI] == RTM_KERNEL_X2 || c->kv[KI] == RTM_KERNEL_X2_SPLIT) {
            eng::k_step_x2<MMAX, AD><<<grid, eng::X2_THREADS, smem, st>>>(*m.A, *m.S, *m.A0, *m.S0, fv,
                                                                         c->imaps, la);
            return RTM_OK;
        }
    }
    eng::k_step<MMAX, AD, MODE><<<grid, eng::NTHREADS, smem, st>>>(
        *m.A, *m.S, *m.A0, *m.S0, fv, c->imaps, MODE == eng::MODE_BWDS ? c->smaps_b : c->smaps_f, la);
    return RTM_OK;
}

template <int MMAX, bool AD, int MODE>
void set_attr_t()
{
    const int smem = (int)eng::Smem<MMAX, MODE>::BYTES;
    cudaFuncSetAttribute(eng::k_step<MMAX, AD, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if constexpr (MODE == eng::MODE_FWDS || MODE == eng::MODE_BWDS) return;
    if constexpr (MODE == eng::MODE_FWD)
        cudaFuncSetAttribute(eng::k_step_x2<MMAX, AD>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    const int psmem = (int)eng::PipeSmem<MMAX, MODE>::BYTES;
    cudaFuncSetAttribute(eng::k_step_pipe<MMAX, AD, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, psmem);
    int dev = 0, sms = 0, occ = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, eng::k_step_pipe<MMAX, AD, MODE>, eng::NTHREADS, psmem);
    pipe_grid<MMAX, AD, MODE>() = std::max(1, occ) * std::max(1, sms);
}

template <int MMAX>
void set_attr_m()
{
    set_attr_t<MMAX, true, eng::MODE_FWD>();
    set_attr_t<MMAX, false, eng::MODE_FWD>();
    set_attr_t<MMAX, true, eng::MODE_BWD>();
    set_attr_t<MMAX, false, eng::MODE_BWD>();
    set_attr_t<MMAX, true, eng::MODE_FWDS>();
    set_attr_t<MMAX, false, eng::MODE_FWDS>();
    set_attr_t<MMAX, true, eng::MODE_BWDS>();
    set_attr_t<MMAX, false, eng::MODE_BWDS>();
}

void init_step_attrs()
{
    static std::once_flag once;
    std::call_once(once, [] {
        set_attr_m<4>();
        set_attr_m<8>();
        set_attr_m<12>();
    });
}

template <int MMAX>
int launch_step_m(rtm_ctx *c, int mode, const StepMaps &m, const eng::StepArgs &a, int nb, cudaStream_t st)
{
    const bool ad = c->p.adaptive != 0;
    switch (mode) {
    case eng::MODE_FWD:
        return ad ? launch_step_t<MMAX, true, eng::MODE_FWD>(c, m, a, nb, st)
                  : launch_step_t<MMAX, false, eng::MODE_FWD>(c, m, a, nb, st);
    case eng::MODE_BWD:
        return ad ? launch_step_t<MMAX, true, eng::MODE_BWD>(c, m, a, nb, st)
                  : launch_step_t<MMAX, false, eng::MODE_BWD>(c, m, a, nb, st);
    case eng::MODE_FWDS:
        return ad ? launch_step_t<MMAX, true, eng::MODE_FWDS>(c, m, a, nb, st)
                  : launch_step_t<MMAX, false, eng::MODE_FWDS>(c, m, a, nb, st);
    default:
        return ad ? launch_step_t<MMAX, true, eng::MODE_BWDS>(c, m, a, nb, st)
                  : launch_step_t<MMAX, false, eng::MODE_BWDS>(c, m, a, nb, st);
    }
}

int launch_step(rtm_ctx *c, int mode, const StepMaps &m, const eng::StepArgs &a, int nb, cudaStream_t st)
{
    switch (c->MM) {
    case 4: return launch_step_m<4>(c, mode, m, a, nb, st);
    case 8: return launch_step_m<8>(c, mode, m, a, nb, st);
    case 12: return launch_step_m<12>(c, mode, m, a, nb, st);
    default: rtm_set_last_error("unsupported operator length"); return RTM_ERR_UNSUPPORTED;
    }
}

eng::StepArgs base_step(rtm_ctx *c)
{
    eng::StepArgs a{};
    a.NZ = c->NZ; a.NX = c->NX; a.P = c->P; a.N2 = c->N2; a.nbins = c->nbins;
    a.ss = c->ss;
    a.vmin = c->p.vmin; a.dv = c->p.dv; a.tao2 = c->p.tao2; a.h2 = c->p.h2;
    a.k0 = (float)(1.0 + (double)c->p.hzx2_1);
    a.hzx2_1 = c->p.hzx2_1;
    a.v = c->v; a.ctab = c->ctab; a.ctab4 = c->ctab4; a.src = c->src; a.compen = c->p.compen;
    a.rz0 = c->p.rz0; a.rx0 = c->p.rx0; a.rdz = c->p.rdz; a.rdx = c->p.rdx; a.nrec = 0;
    a.rel1 = c->rel1; a.rel2 = c->rel2; a.sacc = c->sacc; a.racc = c->racc;
    a.nxs = c->gnx; a.rx0s = c->grx0; a.vshot = c->windowed ? 1 : 0;
    a.gbin = c->windowed ? c->mbins : c->mbin;
    a.gbin_ss = c->windowed ? c->ss : 0;
    a.xas = c->gxa;
    a.gsbin = c->mbin;
    a.min_nx = c->NX;
    return a;
}

// Snapshot steps of a backward run over k = 0..N (N = NT-3) with snapshots
// every K steps: the start levels 0 and 1 (level 1 is the start-up spike of a
// single cell, level 0 is zero: both enter with weight 1), then k = 2, 2+K,
// .., 2+KJ (J = (N-2) / K).  snap_slot gives the slot of a snapshot step (-1
// at other steps); snap_weight the step's imaging weight in the time sum --
// on the sampled steps the trapezoidal rule with step K, the rectangle sum's
// end terms, the first end's derivative term of the Euler-Maclaurin formula
// (the running sums are largest there) and the last sample standing for the
// N-2-KJ steps above it.  The weights add up to N + 1; with K = 1 every
// weight is 1.
int snap_slot(int k, int K)
{
    if (k <= 1) return k;
    return (k - 2) % K ? -1 : 2 + (k - 2) / K;
}

int snap_slots(int N, int K) { return 3 + (N - 2) / K; }

double snap_weight(int k, int K, int N)
{
    if (k <= 1) return 1.0;
    if ((k - 2) % K) return 0.0;
    const int J = (N - 2) / K, j = (k - 2) / K;
    if (J == 0) return N - 1.0;
    const double e = (double(K) * K - 1.0) / (12.0 * K);
    double w = K;
    if (j == 0) w = (K + 1) / 2.0 - e;
    if (j == J) w = (K + 1) / 2.0 + (N - 2 - K * J);
    if (j == 1) w += e;
    return w;
}

// The receiver band's part of the pad launches of a migration with
// snapshots: mode 1 stores the band cells of forward step k, mode 2 images
// them at backward step k (0: none).  Returns the extra threads per shot.
long pad_band(rtm_ctx *c, eng::PadArgs &pa, int mode, int k)
{
    pa.band_mode = c->band.zn ? mode : 0;
    if (!pa.band_mode) return 0;
    pa.band = c->band;
    pa.band_k = k;
    pa.band_steps = c->NT - 2;
    pa.band_qzero = 0;
    pa.bandS = c->bandS;
    pa.bandP = c->bandP;
    pa.sum = c->pacc;
    pa.racc = c->racc;
    pa.rel1 = c->rel1;
    pa.rel2 = c->rel2;
    pa.compen = c->p.compen;
    return (long)c->band.zn * c->band.xn;
}

// Stores the snapshot of step k of n shots from the source level `lev` (its
// interior; the running sum is c->pacc): max pass for 16-bit codes, then the
// store.
void snap_store(rtm_ctx *c, const float *lev, int k, int qzero, int shot0, int n, cudaStream_t st)
{
    const int slot = snap_slot(k, c->snap_every);
    const dim3 grid(cdiv((long)c->nz * c->nx, 256), n);
    if (c->snap_prec) {
        eng::k_snap_max<<<grid, 256, 0, st>>>(lev, c->ss, c->NZ, c->P, c->N2, c->gnx, c->snap_amax,
                                              c->snap_nslots, slot, shot0);
        c->launches++;
    }
    eng::k_snap_store<<<grid, 256, 0, st>>>(lev, c->pacc, c->ss, c->NZ, c->P, c->N2, c->gnx, c->snap_amax,
                                            c->snap_scale, c->snap_nslots, slot, qzero, c->snap_prec,
                                            c->snap_pitch, c->snap_off, c->snapS, c->snapQ, shot0);
    c->launches++;
}

eng::PadArgs base_pad(rtm_ctx *c)
{
    eng::PadArgs a{};
    a.NZ = c->NZ; a.P = c->P; a.N2 = c->N2; a.M = c->M;
    a.ss = c->ss; a.nabc = abc_count(c->NZ, c->NX, c->N2);
    a.nxs = c->gnx; a.rx0s = c->grx0;
    a.meta = c->windowed ? c->meta_s : c->pad_meta;
    a.fac = c->windowed ? c->fac_s : c->pad_fac;
    a.tab_ss = c->windowed ? a.nabc : 0;
    a.pre = c->pre;
    a.ring_prec = c->p.ring_precision;
    a.ringsz = c->ringsz;
    a.slots = c->NT;
    a.ring16 = c->ring16;
    a.amax = c->ramax;
    a.scale = c->rscale;
    a.qslot = -1;
    a.ring_ss = (long long)c->NT * c->ringsz;
    a.rz0 = c->p.rz0; a.rx0 = c->p.rx0; a.rdz = c->p.rdz; a.rdx = c->p.rdx; a.nrec = c->nrec;
    return a;
}

void tic(rtm_ctx *c)
{
    if (c->timing) cudaEventRecord(c->ev[0], c->st);
}
// kind: 0 forward stencil, 1 backward stencil, 2 pad kernel
void toc(rtm_ctx *c, int kind)
{
    c->launches++;
    if (!c->timing) return;
    cudaEventRecord(c->ev[1], c->st);
    cudaEventSynchronize(c->ev[1]);
    float ms = 0;
    cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]);
    if (kind == 0) { c->ms_stencil += ms; c->n_stencil++; }
    else if (kind == 1) { c->ms_bwd += ms; c->n_bwd++; }
    else { c->ms_pad += ms; c->n_pad++; }
}

// Kernel form RTM_KERNEL_SPLIT: the two halves of a batch run their time
// loops on two streams.  Their shots are independent, so the latency-bound
// pad launches of one half overlap the other half's stencil launches (the
// backward stencil leaves room for a pad CTA on every SM).
struct Half {
    int shot0, n;
    cudaStream_t st;
};

int halves(rtm_ctx *c, int mode, int nb, Half h[2])
{
    const bool split = c->kv[mode] == RTM_KERNEL_SPLIT || c->kv[mode] == RTM_KERNEL_X2_SPLIT;
    if (split && nb >= 2 && !c->timing && c->st2) {
        h[0] = Half{0, nb / 2, c->st};
        h[1] = Half{nb / 2, nb - nb / 2, c->st2};
        cudaEventRecord(c->evf[0], c->st);
        cudaStreamWaitEvent(c->st2, c->evf[0], 0);
        return 2;
    }
    h[0] = Half{0, nb, c->st};
    return 1;
}

void join(rtm_ctx *c, int nh)
{
    if (nh < 2) return;
    cudaEventRecord(c->evf[1], c->st2);
    cudaStreamWaitEvent(c->st, c->evf[1], 0);
}

// Pad update of a launch of n shots; `extra` threads record receivers and
// quantise the previous step's 16-bit ring.
void launch_pad(rtm_ctx *c, const eng::PadArgs &pa, int n, long extra, cudaStream_t st)
{
    const long npad = cdiv(abc_count(c->NZ, c->NX, c->N2), eng::PAD_CPT) + extra;
    eng::k_pad<<<dim3(cdiv(npad, 256), n), 256, 0, st>>>(pa);
}

// Forward run of nb shots (sources already in c->src).  rec_on: record the
// receivers into c->rec (time-major [shot][NT][nrec]).
int enqueue_forward(rtm_ctx *c, int nb, bool rec_on)
{
    const long long ss = c->ss;
    const int NT = c->NT;
    eng::k_shot_init<<<dim3(cdiv(ss, 256), nb), 256, 0, c->st>>>(c->S[0], c->S[1], c->S[2], c->pre,
                                                                 c->src, c->gnx, c->p.spike, ss, c->P);
    c->launches++;
    // a migration with source snapshots saves no rings (its backward run
    // does not reconstruct the source field)
    const bool snap = c->snap_every > 0 && !rec_on;
    const bool r16 = c->p.ring_precision != RTM_RING_F32 && !snap;
    const long long bstage = (long long)c->B * c->ringsz;  // floats of one stage parity
    if (r16 && c->M > 0)
        RTM_CUDA_TRY(cudaMemsetAsync(c->ramax, 0, sizeof(unsigned) * (size_t)c->B * NT, c->st));
    if (snap) {
        // running sum of levels 0 and 1 (the start spike), and the slots of
        // those two levels (level 0 is zero)
        RTM_CUDA_TRY(cudaMemcpyAsync(c->pacc, c->S[1], sizeof(float) * (size_t)ss * nb, cudaMemcpyDeviceToDevice,
                                     c->st));
        RTM_CUDA_TRY(cudaMemsetAsync(c->snap_amax, 0, sizeof(unsigned) * (size_t)nb * c->snap_nslots, c->st));
        snap_store(c, c->S[0], 0, 1, 0, nb, c->st);
        snap_store(c, c->S[1], 1, 0, 0, nb, c->st);
        if (c->band.zn) {
            eng::k_band_start<<<dim3(cdiv((long)c->band.zn * c->band.xn, 256), nb), 256, 0, c->st>>>(
                c->S[1], ss, c->P, c->N2, c->gnx, c->grx0, c->band, NT - 2, c->bandS, c->bandP);
            c->launches++;
        }
    }
    if (c->M > 0 && !snap) {
        if (r16)
            eng::k_ring_fill<<<dim3(cdiv(abc_count(c->NZ, c->NX, c->N2), 256), nb), 256, 0, c->st>>>(
                c->S[1], c->rstage + 1 * bstage, ss, c->ringsz, c->NZ, c->gnx, c->P, c->N2, c->M,
                c->ramax + 1, NT);
        else
            eng::k_ring_fill<<<dim3(cdiv(abc_count(c->NZ, c->NX, c->N2), 256), nb), 256, 0, c->st>>>(
                c->S[1], c->ring + c->ringsz, ss, (long long)NT * c->ringsz, c->NZ, c->gnx, c->P, c->N2,
                c->M, nullptr, 0);
    }
    c->launches += (c->M > 0 && !snap);
    const long long rss = (long long)NT * c->nrec;
    if (rec_on && c->nrec > 0) {
        eng::k_record<<<dim3(cdiv(c->nrec, 128), nb), 128, 0, c->st>>>(
            c->S[0], c->rec, ss, rss, c->P, c->p.rz0, c->grx0, c->p.rdz, c->p.rdx, c->nrec);
        c->launches++;
    }
    RTM_LAUNCH_CHECK();
    eng::StepArgs sa = base_step(c);
    eng::PadArgs pa = base_pad(c);
    const long extra = (rec_on ? c->nrec : 0) + (r16 ? c->ringsz : 0);
    const int kend = c->kstop ? std::min(c->kstop, NT) : NT;  // kstop-2 steps when tuning
    const int mode = snap ? eng::MODE_FWDS : eng::MODE_FWD;
    if (snap) sa.pacc = c->pacc;
    Half hv[2];
    const int nh = halves(c, eng::MODE_FWD, nb, hv);
    for (int k = 2; k < kend; ++k) {
        float *a0 = c->S[(k - 2) % 3], *a1 = c->S[(k - 1) % 3], *a2 = c->S[k % 3];
        sa.a0 = a0; sa.a2 = a2; sa.pre = c->pre;
        sa.wavelet = (k < c->p.NT2) ? c->wav[k - 1] : 0.0f;
        const StepMaps sm{&c->mapS[(k - 1) % 3], &c->mapS[(k - 1) % 3], &c->flatS[(k - 2) % 3],
                          &c->flatS[(k - 2) % 3]};
        pa.a0 = a0; pa.a1 = a1; pa.a2 = a2;
        pa.ring_mode = c->M > 0 && !snap ? 1 : 0;
        pa.ring = c->ring ? c->ring + (long long)k * c->ringsz : nullptr;
        if (r16) {
            pa.slot = k;
            pa.qslot = k - 1;
            pa.stage = c->rstage + (k & 1) * bstage;
            pa.qstage = c->rstage + ((k - 1) & 1) * bstage;
        }
        pa.rec = rec_on ? c->rec + (long long)(k - 1) * c->nrec : nullptr;
        pa.rec_ss = rss;
        const long bextra = pad_band(c, pa, snap && k <= NT - 3 ? 1 : 0, k);
        for (int h = 0; h < nh; ++h) {
            sa.shot0 = pa.shot0 = hv[h].shot0;
            tic(c);
            if (int rc = launch_step(c, mode, sm, sa, hv[h].n, hv[h].st)) return rc;
            toc(c, 0);
            tic(c);
            launch_pad(c, pa, hv[h].n, extra + bextra, hv[h].st);
            toc(c, 2);
            if (snap && k <= NT - 3 && snap_slot(k, c->snap_every) >= 0)  // the backward run images k <= NT-3
                snap_store(c, a2, k, 0, hv[h].shot0, hv[h].n, hv[h].st);
        }
    }
    join(c, nh);
    if (rec_on && c->nrec > 0)
        eng::k_record<<<dim3(cdiv(c->nrec, 128), nb), 128, 0, c->st>>>(
            c->S[(NT - 1) % 3], c->rec + (long long)(NT - 1) * c->nrec, ss, rss, c->P, c->p.rz0,
            c->grx0, c->p.rdz, c->p.rdx, c->nrec);
    c->launches += (rec_on && c->nrec > 0);
    RTM_LAUNCH_CHECK();
    return RTM_OK;
}

// Backward pass of nb shots (after enqueue_forward; observed data in c->data
// time-major [shot][NT][nrec]).
int enqueue_backward(rtm_ctx *c, int nb)
{
    const long long ss = c->ss;
    const int NT = c->NT;
    float *F1 = c->S[(NT - 1) % 3], *F0 = c->S[(NT - 2) % 3];
    eng::k_img_init<<<dim3(cdiv(ss, 256), nb), 256, 0, c->st>>>(
        F1, F0, c->R[0], c->R[1], c->R[2], c->rel1, c->rel2, c->sacc, c->racc, c->src, c->gnx,
        c->p.spike, c->p.compen, ss, c->P);
    c->launches++;
    RTM_LAUNCH_CHECK();
    eng::StepArgs sa = base_step(c);
    sa.nrec = c->nrec;
    sa.dstride = (long long)NT * c->nrec;
    eng::PadArgs pa = base_pad(c);
    const int kend = c->kstop ? std::max(NT - c->kstop, 0) : 0;  // kstop-2 steps when tuning
    const bool snap = c->snap_every > 0;
    const int mode = snap ? eng::MODE_BWDS : eng::MODE_BWD;
    Half hv[2];
    const int nh = halves(c, eng::MODE_BWD, nb, hv);
    for (int k = NT - 3; k >= kend; --k) {
        const int i2 = k % 3, i1 = (k + 1) % 3, i0 = (k + 2) % 3;
        sa.a0 = c->R[i0]; sa.a2 = c->R[i2]; sa.pre = c->pre;
        sa.s0 = c->S[i0]; sa.s2 = c->S[i2];
        sa.wavelet = (k < c->p.NT2) ? c->wav[k + 1] : 0.0f;
        sa.dinj = c->data + (long long)(k + 1) * c->nrec;
        const StepMaps sm{&c->mapR[i1], &c->mapS[i1], &c->flatR[i0], &c->flatS[i0]};
        pa.a0 = c->R[i0]; pa.a1 = c->R[i1]; pa.a2 = c->R[i2];
        pa.ring_mode = c->M > 0 && !snap ? 2 : 0;
        if (snap) sa.pacc = c->racc;
        const long bextra = pad_band(c, pa, snap ? 2 : 0, k);
        const float w = snap ? (float)snap_weight(k, c->snap_every, NT - 3) : 0.0f;

        pa.ring = c->ring ? c->ring + (long long)k * c->ringsz : nullptr;
        pa.slot = k;
        pa.s2 = c->S[i2];
        pa.rec = nullptr;
        for (int h = 0; h < nh; ++h) {
            sa.shot0 = pa.shot0 = hv[h].shot0;
            tic(c);
            if (int rc = launch_step(c, mode, sm, sa, hv[h].n, hv[h].st)) return rc;
            toc(c, 1);
            if (w != 0.0f) {
                eng::k_snap_image<<<dim3(cdiv((long)c->nz * c->nx, 256), hv[h].n), 256, 0, hv[h].st>>>(
                    c->R[i2], c->racc, c->pacc, c->snapS, c->snapQ, c->snap_scale, c->rel1, c->rel2, c->ss,
                    c->NZ, c->P, c->N2, c->gnx, c->grx0, c->band, c->snap_nslots, snap_slot(k, c->snap_every),
                    c->snap_prec, c->snap_pitch, c->snap_off, w, c->p.compen, hv[h].shot0);
                c->launches++;
            }
            tic(c);
            launch_pad(c, pa, hv[h].n, bextra, hv[h].st);
            toc(c, 2);
        }
    }
    join(c, nh);
    RTM_LAUNCH_CHECK();
    return RTM_OK;
}

// Runs phase (0 forward+record, 1 forward+backward) for nb shots, through a
// cached CUDA graph unless timing is on or RTM_NO_GRAPH is given.
int run_phase(rtm_ctx *c, int phase, int nb, int flags)
{
    const bool use_graph = !(flags & RTM_NO_GRAPH) && !c->timing;
    // phase 0: forward run with receiver recording; 1: forward + backward;
    // 2: forward run of a migration; 3: its backward run
    auto body = [&]() -> int {
        if (phase == 0) return enqueue_forward(c, nb, true);
        if (phase == 2) return enqueue_forward(c, nb, false);
        if (phase == 3) return enqueue_backward(c, nb);
        if (int rc = enqueue_forward(c, nb, false)) return rc;
        return enqueue_backward(c, nb);
    };
    if (!use_graph) return body();
    auto key = std::make_pair(phase * 2 + (c->windowed ? 1 : 0), nb);
    auto it = c->graphs.find(key);
    if (it == c->graphs.end()) {
        cudaGraph_t g;
        RTM_CUDA_TRY(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
        const long before = c->launches;
        int rc = body();
        c->graph_kernels[key] = c->launches - before;
        c->launches = before;
        cudaError_t e = cudaStreamEndCapture(c->st, &g);
        if (rc) {
            if (e == cudaSuccess) cudaGraphDestroy(g);
            return rc;
        }
        RTM_CUDA_TRY(e);
        cudaGraphExec_t ge;
        e = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        RTM_CUDA_TRY(e);
        it = c->graphs.emplace(key, ge).first;
    }
    RTM_CUDA_TRY(cudaGraphLaunch(it->second, c->st));
    c->launches += c->graph_kernels[key];
    return RTM_OK;
}

// Per-cell vv and bin of ncell model cells (kernel.cu's v*v*tao2*h2 and
// int((v-vmin)/dv+0.5), formed once instead of at every step).
void model_prep(rtm_ctx *c, const float *v, long long ncell, float *vv, int *bin)
{
    eng::k_model_prep<<<(unsigned)cdiv(ncell, 256), 256, 0, c->st>>>(
        v, ncell, c->p.tao2, c->p.h2, c->p.vmin, c->p.dv, std::max(c->nbins, 1), c->blen, vv,
        c->p.adaptive ? bin : nullptr);
}

// Sets the per-shot geometry of the next batch: window start column xa and
// interior width nx of each shot (NULL: the whole survey grid), sources in
// each shot's own padded grid.  Windowed batches get their models and pad
// tables built on the device.
int set_batch(rtm_ctx *c, int nb, const int *src_cells, const int *xa, const int *nx)
{
    c->hnx.assign(nb, c->NX);
    c->hxa.assign(nb, 0);
    std::vector<int> rx0(nb, c->p.rx0);
    bool windowed = false;
    for (int i = 0; i < nb; ++i) {
        if (xa && nx) {
            if (nx[i] < 2 * c->MM + 2 || xa[i] < 0 || xa[i] + nx[i] > c->nx) {
                rtm_set_last_error("aperture window outside the survey");
                return RTM_ERR_ARG;
            }
            c->hxa[i] = xa[i];
            c->hnx[i] = nx[i] + 2 * c->N2;
            rx0[i] = c->p.rx0 - xa[i];
            windowed = windowed || xa[i] != 0 || nx[i] != c->nx;
        }
        const int NXi = c->hnx[i];
        if (src_cells[i] < 0 || src_cells[i] >= c->NZ * NXi) {
            rtm_set_last_error("source cell outside the shot's grid");
            return RTM_ERR_ARG;
        }
        for (int j = 0; j < c->nrec; j += std::max(1, c->nrec - 1)) {
            const int x = rx0[i] + j * c->p.rdx;
            if (x < 0 || x >= NXi) {
                rtm_set_last_error("receivers outside the shot's aperture window");
                return RTM_ERR_ARG;
            }
        }
    }
    std::vector<int> hn(c->hnx);
    std::vector<int> items(nb + 1, 0);  // tile items per shot: tile rows x tile columns
    for (int i = 0; i < nb; ++i)
        items[i + 1] = items[i] + cdiv(c->NZ, eng::TZ) * cdiv(c->hnx[i], eng::TX);
    RTM_CUDA_TRY(cudaMemcpyAsync(c->gitem, items.data(), sizeof(int) * (nb + 1), cudaMemcpyHostToDevice, c->st));
    RTM_CUDA_TRY(cudaMemcpyAsync(c->src, src_cells, sizeof(int) * nb, cudaMemcpyHostToDevice, c->st));
    RTM_CUDA_TRY(cudaMemcpyAsync(c->gnx, hn.data(), sizeof(int) * nb, cudaMemcpyHostToDevice, c->st));
    RTM_CUDA_TRY(cudaMemcpyAsync(c->gxa, c->hxa.data(), sizeof(int) * nb, cudaMemcpyHostToDevice, c->st));
    RTM_CUDA_TRY(cudaMemcpyAsync(c->grx0, rx0.data(), sizeof(int) * nb, cudaMemcpyHostToDevice, c->st));
    // the host vectors must outlive the async copies
    RTM_CUDA_TRY(cudaStreamSynchronize(c->st));
    c->windowed = windowed;
    if (!windowed) return RTM_OK;
    if (!c->vs) {
        const size_t bgrid = (size_t)c->ss * c->B;
        const long nabc = abc_count(c->NZ, c->NX, c->N2);
        if (int rc = dalloc(c, &c->vs, bgrid)) return rc;
        if (int rc = dalloc(c, &c->r1s, bgrid)) return rc;
        if (int rc = dalloc(c, &c->meta_s, (size_t)nabc * c->B)) return rc;
        if (int rc = dalloc(c, &c->fac_s, (size_t)nabc * c->B)) return rc;
        if (int rc = dalloc(c, &c->mvvs, bgrid)) return rc;
        if (int rc = make_map(&c->mmaps_s.vv, c->mvvs, c->NX, c->NZ, c->B, c->P, eng::TX, eng::TZ)) return rc;
        // window-interior tiles read the survey's grid (tile_on_survey)
        c->mmaps_s.svv = c->mmaps.vv;
        c->mmaps_s.sbin = c->mmaps.bin;
        if (c->p.adaptive) {
            if (int rc = dalloc(c, &c->mbins, bgrid)) return rc;
            if (int rc = make_map(&c->mmaps_s.bin, reinterpret_cast<float *>(c->mbins), c->NX, c->NZ, c->B,
                                  c->P, eng::TX, eng::TZ))
                return rc;
        }
    }
    const long nabc = abc_count(c->NZ, c->NX, c->N2);
    eng::k_window_model<<<dim3(cdiv(c->ss, 256), nb), 256, 0, c->st>>>(
        c->v, c->r1, c->P, c->gxa, c->gnx, c->vs, c->r1s, c->ss, c->NZ, c->P, c->N2);
    eng::k_pad_tables<<<dim3(cdiv(nabc, 256), nb), 256, 0, c->st>>>(
        c->vs, c->r1s, c->w, c->gnx, c->ss, nabc, c->NZ, c->P, c->N2, c->M, c->p.taoh, c->p.taoh2,
        c->p.quirk, c->meta_s, c->fac_s);
    model_prep(c, c->vs, (long long)c->ss * nb, c->mvvs, c->mbins);
    c->launches += 3;
    RTM_LAUNCH_CHECK();
    return RTM_OK;
}

// [nb][nrec][NT] (trace-major) <-> [nb][NT][nrec] (time-major)
__global__ void k_transpose(const float *in, float *out, int rows, int cols, long long per)
{
    __shared__ float t[32][33];
    const int shot = blockIdx.z;
    const float *I = in + shot * per;
    float *O = out + shot * per;
    int c = blockIdx.x * 32 + threadIdx.x, r = blockIdx.y * 32 + threadIdx.y;
    for (int j = 0; j < 32; j += 8)
        if (r + j < rows && c < cols) t[threadIdx.y + j][threadIdx.x] = I[(long)(r + j) * cols + c];
    __syncthreads();
    c = blockIdx.y * 32 + threadIdx.x;
    r = blockIdx.x * 32 + threadIdx.y;
    for (int j = 0; j < 32; j += 8)
        if (r + j < cols && c < rows) O[(long)(r + j) * rows + c] = t[threadIdx.x][threadIdx.y + j];
}

void transpose(rtm_ctx *c, const float *in, float *out, int rows, int cols, int nb, cudaStream_t st)
{
    dim3 g(cdiv(cols, 32), cdiv(rows, 32), nb);
    k_transpose<<<g, dim3(32, 8), 0, st>>>(in, out, rows, cols, (long long)rows * cols);
    c->launches++;
}

// full padded grid [nb][NZ][P] -> [nb][NZ][NX]
int copy_grid_out(rtm_ctx *c, const float *dsrc, float *dst, int nb, bool dev)
{
    RTM_CUDA_TRY(cudaMemcpy2DAsync(dst, sizeof(float) * c->NX, dsrc, sizeof(float) * c->P,
                                   sizeof(float) * c->NX, (size_t)c->NZ * nb,
                                   dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, c->st));
    return RTM_OK;
}

}  // namespace

extern "C" {

// Self-test of the bounded waits: one CTA waits on an mbarrier that nothing
// completes, for `polls` polls; every thread gives up, records the timeout in
// the device error word and returns.
__global__ void k_wait_selftest(unsigned polls)
{
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_barrier_init();
    }
    __syncthreads();
    mbar_wait_bounded(&bar, 0, &g_rtm_dev_error, polls);
}

int rtm_selftest_wait_timeout(unsigned polls, unsigned int *code)
{
    if (!code || polls < 1 || polls > (1u << 20)) return RTM_ERR_ARG;
    unsigned z = 0;
    RTM_CUDA_TRY(cudaMemcpyToSymbol(g_rtm_dev_error, &z, sizeof(z)));
    k_wait_selftest<<<1, 64>>>(polls);
    RTM_CUDA_TRY(cudaGetLastError());
    RTM_CUDA_TRY(cudaDeviceSynchronize());
    return rtm_device_error(code);
}

int rtm_device_error(unsigned int *code)
{
    unsigned v = 0, z = 0;
    RTM_CUDA_TRY(cudaMemcpyFromSymbol(&v, g_rtm_dev_error, sizeof(v)));
    RTM_CUDA_TRY(cudaMemcpyToSymbol(g_rtm_dev_error, &z, sizeof(z)));
    if (code) *code = v;
    return RTM_OK;
}

int rtm_ctx_create(rtm_ctx **out, const rtm_problem *p, int max_batch, rtm_stream_t stream)
{
    if (!out || !p || max_batch < 1) return RTM_ERR_ARG;
    *out = nullptr;
    if (p->nz < 1 || p->nx < 1 || p->N2 < 2 || p->M < 0 || p->M > p->N2 || p->NT < 4 || !p->v ||
        !p->r1 || !p->w || !p->coef || !p->wav || (p->adaptive && (!p->index || p->nbins < 1)) ||
        p->ring_precision < RTM_RING_F32 || p->ring_precision > RTM_RING_I16) {
        rtm_set_last_error("rtm_ctx_create: invalid problem");
        return RTM_ERR_ARG;
    }
    if (p->nrec > 0 && p->rdz == 0 && p->rdx == 0) {
        rtm_set_last_error("rtm_ctx_create: receiver step is zero");
        return RTM_ERR_ARG;
    }
    rtm_ctx *c = new rtm_ctx();
    c->p = *p;
    c->nz = p->nz; c->nx = p->nx; c->N2 = p->N2; c->M = p->M; c->NT = p->NT;
    c->NZ = p->nz + 2 * p->N2; c->NX = p->nx + 2 * p->N2;
    c->P = (c->NX + eng::TX - 1) / eng::TX * eng::TX;
    c->B = max_batch;
    c->nbl = max_batch;
    c->nrec = p->nrec;
    c->ss = (long long)c->NZ * c->P;
    c->ringsz = 2L * c->M * (c->nx + c->nz);
    for (int j = 0; j < p->nrec; ++j) {
        const int z = p->rz0 + j * p->rdz, x = p->rx0 + j * p->rdx;
        if (z < 0 || z >= c->NZ || x < 0 || x >= c->NX) {
            rtm_set_last_error("receiver outside the grid");
            delete c;
            return RTM_ERR_ARG;
        }
    }
    // operator length of the kernels: every bin's length padded to MM
    int mlen = p->M;
    std::vector<float> tab;
    if (p->adaptive) {
        mlen = 0;
        for (int b = 0; b < p->nbins; ++b) mlen = std::max(mlen, p->index[b + 1] - p->index[b] - 1);
    }
    c->MM = mlen <= 4 ? 4 : (mlen <= 8 ? 8 : (mlen <= 12 ? 12 : 0));
    if (c->MM == 0 || mlen > p->N2) {
        rtm_set_last_error("operator length above 12 or above the pad width");
        delete c;
        return RTM_ERR_UNSUPPORTED;
    }
    if (c->NZ < 2 * c->MM + 2 || c->NX < 2 * c->MM + 2) {
        rtm_set_last_error("grid smaller than the operator");
        delete c;
        return RTM_ERR_ARG;
    }
    init_step_attrs();
    if (stream) {
        c->st = stream;
    } else if (cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) != cudaSuccess) {
        rtm_set_last_error("cudaStreamCreate failed");
        delete c;
        return RTM_ERR_CUDA;
    } else {
        c->own_stream = true;
    }
    if (cudaStreamCreateWithFlags(&c->st2, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->evf[0], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->evf[1], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->evc[0], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->evc[1], cudaEventDisableTiming) != cudaSuccess) {
        rtm_set_last_error("cudaStreamCreate failed");
        free_all(c);
        delete c;
        return RTM_ERR_CUDA;
    }
    if (p->adaptive && p->nbins >= (1 << eng::BIN_BITS)) {
        rtm_set_last_error("rtm_ctx_create: too many velocity bins");
        free_all(c);
        delete c;
        return RTM_ERR_ARG;
    }
    if (p->adaptive) {
        c->nbins = p->nbins;
        tab.assign((size_t)(c->MM + 1) * c->nbins, 0.0f);
        for (int b = 0; b < p->nbins; ++b)
            for (int l = 0; l < p->index[b + 1] - p->index[b]; ++l)
                tab[(size_t)l * c->nbins + b] = p->coef[p->index[b] + l];
    } else {
        c->nbins = 1;
        tab.assign(c->MM + 1, 0.0f);
        for (int l = 0; l <= p->M; ++l) tab[l] = p->coef[l];
    }
    c->wav.assign(p->wav, p->wav + p->NT + 1);
    int rc = RTM_OK;
    const size_t grid = (size_t)c->ss;
    const size_t bgrid = grid * c->B;
#define TRY(x)                     \
    do {                           \
        if ((rc = (x)) != RTM_OK) { \
            free_all(c);           \
            delete c;              \
            return rc;             \
        }                          \
    } while (0)
    TRY(dalloc(c, &c->v, grid));
    TRY(dalloc(c, &c->r1, grid));
    TRY(dalloc(c, &c->w, (size_t)c->N2 + 1));
    TRY(dalloc(c, &c->ctab, tab.size()));
    if (p->adaptive) {
        // float4 groups (c_{4q..4q+3} of a bin) in the kernels' table layout
        const int Q = eng::tab_groups(c->MM);
        std::vector<float4> t4((size_t)eng::tab_pitch(c->MM) * c->nbins, make_float4(0.f, 0.f, 0.f, 0.f));
        for (int q = 0; q < Q; ++q)
            for (int b = 0; b < c->nbins; ++b) {
                float g[4];
                for (int k = 0; k < 4; ++k) {
                    const int l = 4 * q + k;
                    g[k] = l <= c->MM ? tab[(size_t)l * c->nbins + b] : 0.0f;
                }
                t4[eng::tab_index(q, b, c->nbins, c->MM)] = make_float4(g[0], g[1], g[2], g[3]);
            }
        // each bin's operator length (unused bins: 0, their coefficients are zero)
        std::vector<int> bl(c->nbins);
        for (int b = 0; b < c->nbins; ++b) bl[b] = std::max(p->index[b + 1] - p->index[b] - 1, 0);
        TRY(dalloc(c, &c->ctab4, t4.size()));
        TRY(dalloc(c, &c->blen, bl.size()));
        if (cudaMemcpy(c->ctab4, t4.data(), sizeof(float4) * t4.size(), cudaMemcpyHostToDevice) !=
                cudaSuccess ||
            cudaMemcpy(c->blen, bl.data(), sizeof(int) * bl.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
            rtm_set_last_error("upload failed");
            free_all(c);
            delete c;
            return RTM_ERR_CUDA;
        }
    }
    for (int i = 0; i < 3; ++i) {
        TRY(dalloc(c, &c->S[i], bgrid));
        TRY(dalloc(c, &c->R[i], bgrid));
    }
    TRY(dalloc(c, &c->pre, bgrid));
    TRY(dalloc(c, &c->rel1, bgrid));
    TRY(dalloc(c, &c->rel2, bgrid));
    TRY(dalloc(c, &c->sacc, bgrid));
    TRY(dalloc(c, &c->racc, bgrid));
    if (p->ring_precision == RTM_RING_F32) {
        TRY(dalloc(c, &c->ring, (size_t)c->B * c->NT * std::max<long>(c->ringsz, 1)));
    } else {
        TRY(dalloc(c, &c->ring16, (size_t)c->B * c->NT * std::max<long>(c->ringsz, 1)));
        TRY(dalloc(c, &c->rstage, (size_t)2 * c->B * std::max<long>(c->ringsz, 1)));
        TRY(dalloc(c, &c->rscale, (size_t)c->B * c->NT));
        TRY(dalloc(c, &c->ramax, (size_t)c->B * c->NT));
    }
    TRY(dalloc(c, &c->data, (size_t)c->B * c->NT * std::max(c->nrec, 1)));
    TRY(dalloc(c, &c->rec, (size_t)c->B * c->NT * std::max(c->nrec, 1)));
    TRY(dalloc(c, &c->stage, (size_t)c->B * c->NT * std::max(c->nrec, 1)));
    TRY(dalloc(c, &c->src, (size_t)c->B));
    TRY(dalloc(c, &c->gnx, (size_t)c->B));
    TRY(dalloc(c, &c->gitem, (size_t)c->B + 1));
    TRY(dalloc(c, &c->gxa, (size_t)c->B));
    TRY(dalloc(c, &c->grx0, (size_t)c->B));
    TRY(dalloc(c, &c->imax, (size_t)c->B));
    TRY(dalloc(c, &c->ups, (size_t)c->B * c->nz * c->nx));
    TRY(dalloc(c, &c->downs, (size_t)c->B * c->nz * c->nx));
    for (float **q : {&c->ks1, &c->kc1, &c->ks2, &c->kc2, &c->img, &c->ill})
        TRY(dalloc(c, q, (size_t)c->nz * c->nx));
    // model: padded rows, pad columns of each row hold the row's last value so
    // that bins computed there stay in range
    {
        std::vector<float> hv((size_t)grid), hr((size_t)grid);
        for (int z = 0; z < c->NZ; ++z)
            for (int x = 0; x < c->P; ++x) {
                const int xs = std::min(x, c->NX - 1);
                hv[(size_t)z * c->P + x] = p->v[(size_t)z * c->NX + xs];
                hr[(size_t)z * c->P + x] = p->r1[(size_t)z * c->NX + xs];
            }
        // the per-shot finishing scales by vmax snapped outward to the bin
        // grid, as kernel.cu:717-720 leaves it before kernel.cu:947 uses it
        float vmx = p->v[0];
        for (long i = 0; i < (long)c->NZ * c->NX; ++i) vmx = std::max(vmx, p->v[i]);
        if (p->dv > 0.0f) {
            const float vel = (float)((int)(vmx / p->dv)) * p->dv;
            vmx = (vel < vmx) ? vel + p->dv : vel;
        }
        c->vmax = vmx;
        if (cudaMemcpy(c->v, hv.data(), grid * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(c->r1, hr.data(), grid * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(c->w, p->w, (c->N2 + 1) * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(c->ctab, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess) {
            rtm_set_last_error("upload failed");
            free_all(c);
            delete c;
            return RTM_ERR_CUDA;
        }
    }
    // per-pad-cell classification and model factors (shared by every shot)
    {
        const long nabc = abc_count(c->NZ, c->NX, c->N2);
        std::vector<int4> meta(nabc);
        std::vector<float4> fac(nabc);
        const int NZ = c->NZ, NX = c->NX, N2 = c->N2;
        const float taoh = p->taoh, taoh2 = p->taoh2;
        for (long t = 0; t < nabc; ++t) {
            const AbcCell cc = abc_cell(t, NZ, NX, N2);
            const int z = cc.z, x = cc.x;
            const int a = std::min(z, NZ - 1 - z), e = std::min(x, NX - 1 - x);
            const int dz = (z < NZ - 1 - z) ? 1 : -1, dx = (x < NX - 1 - x) ? 1 : -1;
            int kind;
            long q = (long)z * NX + x;  // flat index of the lateral-term velocity
            if (e >= a + 2) {
                kind = eng::PAD_ROWEDGE;
                if (p->quirk && dz < 0) q = (long)(NZ - 1 - z) * NX + x;
            } else if (a >= e + 2) {
                kind = eng::PAD_COLEDGE;
                if (p->quirk) q = (dx > 0) ? (long)x * NX + z : (long)(NX - 1 - x) * NX + z;
            } else {
                kind = eng::PAD_CORNER;
            }
            const long ci = (long)z * NX + x;
            const float wj = p->w[blend_index(z, x, NZ, NX, N2)];
            if (kind == eng::PAD_CORNER) {
                const float rr = p->r1[ci];
                fac[t] = make_float4(rr, 1.0f / (2.0f * rr + 1.0f), 0.0f, wj);
            } else {
                const float vc = p->v[ci], vq = p->v[q];
                fac[t] = make_float4(taoh * vc, 1.0f / (taoh * vc + 1.0f), taoh2 * vq * vq, wj);
            }
            meta[t] = eng::pad_meta(t, NZ, NX, c->P, N2, c->M);
        }
        TRY(dalloc(c, &c->pad_meta, (size_t)nabc));
        TRY(dalloc(c, &c->pad_fac, (size_t)nabc));
        if (cudaMemcpy(c->pad_meta, meta.data(), sizeof(int4) * nabc, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(c->pad_fac, fac.data(), sizeof(float4) * nabc, cudaMemcpyHostToDevice) != cudaSuccess) {
            rtm_set_last_error("upload failed");
            free_all(c);
            delete c;
            return RTM_ERR_CUDA;
        }
    }
    int bw = 0, bh = 0;
    switch (c->MM) {
    case 4: bw = eng::Shape<4>::BW; bh = eng::Shape<4>::BH; break;
    case 8: bw = eng::Shape<8>::BW; bh = eng::Shape<8>::BH; break;
    default: bw = eng::Shape<12>::BW; bh = eng::Shape<12>::BH; break;
    }
    for (int i = 0; i < 3; ++i) {
        TRY(make_map(&c->mapS[i], c->S[i], c->NX, c->NZ, c->B, c->P, bw, bh));
        TRY(make_map(&c->mapR[i], c->R[i], c->NX, c->NZ, c->B, c->P, bw, bh));
        TRY(make_map(&c->flatS[i], c->S[i], c->NX, c->NZ, c->B, c->P, eng::TX, eng::TZ));
        TRY(make_map(&c->flatR[i], c->R[i], c->NX, c->NZ, c->B, c->P, eng::TX, eng::TZ));
    }
    TRY(dalloc(c, &c->mvv, (size_t)c->ss));
    TRY(make_map(&c->mmaps.vv, c->mvv, c->NX, c->NZ, 1, c->P, eng::TX, eng::TZ));
    if (c->p.adaptive) {
        TRY(dalloc(c, &c->mbin, (size_t)c->ss));
        TRY(make_map(&c->mmaps.bin, reinterpret_cast<float *>(c->mbin), c->NX, c->NZ, 1, c->P, eng::TX, eng::TZ));
    }
    model_prep(c, c->v, c->ss, c->mvv, c->mbin);
    if (cudaStreamSynchronize(c->st) != cudaSuccess) {
        rtm_set_last_error("model preparation failed");
        free_all(c);
        delete c;
        return RTM_ERR_CUDA;
    }
    TRY(make_map(&c->imaps.rel1, c->rel1, c->NX, c->NZ, c->B, c->P, eng::TX, eng::TZ));
    TRY(make_map(&c->imaps.rel2, c->rel2, c->NX, c->NZ, c->B, c->P, eng::TX, eng::TZ));
    TRY(make_map(&c->imaps.sacc, c->sacc, c->NX, c->NZ, c->B, c->P, eng::TX, eng::TZ));
    TRY(make_map(&c->imaps.racc, c->racc, c->NX, c->NZ, c->B, c->P, eng::TX, eng::TZ));
#undef TRY
    cudaEventCreate(&c->ev[0]);
    cudaEventCreate(&c->ev[1]);
    *out = c;
    return RTM_OK;
}

int rtm_ctx_destroy(rtm_ctx *c)
{
    if (!c) return RTM_OK;
    cudaStreamSynchronize(c->st);
    free_all(c);
    delete c;
    return RTM_OK;
}

int rtm_ctx_bytes(const rtm_ctx *c, size_t *bytes)
{
    if (!c || !bytes) return RTM_ERR_ARG;
    *bytes = c->bytes;
    return RTM_OK;
}

int rtm_ctx_set_timing(rtm_ctx *c, int enable)
{
    if (!c) return RTM_ERR_ARG;
    c->timing = enable != 0;
    c->ms_stencil = c->ms_pad = c->ms_bwd = 0;
    c->n_stencil = c->n_pad = c->n_bwd = 0;
    return RTM_OK;
}

int rtm_ctx_timing(const rtm_ctx *c, double ms[3], long n[3])
{
    if (!c || !ms || !n) return RTM_ERR_ARG;
    ms[0] = c->ms_stencil; ms[1] = c->ms_bwd; ms[2] = c->ms_pad;
    n[0] = c->n_stencil; n[1] = c->n_bwd; n[2] = c->n_pad;
    return RTM_OK;
}

int rtm_ctx_set_kernel(rtm_ctx *c, int fwd_variant, int bwd_variant, int shots_per_launch)
{
    auto ok = [](int v) { return v == RTM_KERNEL_TILED || v == RTM_KERNEL_PERSISTENT || v == RTM_KERNEL_SPLIT; };
    const bool fwd_only = fwd_variant == RTM_KERNEL_X2 || fwd_variant == RTM_KERNEL_X2_SPLIT;
    if (!c || !(ok(fwd_variant) || fwd_only) || !ok(bwd_variant) || shots_per_launch < 0 ||
        shots_per_launch > c->B)
        return RTM_ERR_ARG;
    if (fwd_variant != c->kv[0] || bwd_variant != c->kv[1]) {
        // captured graphs embed the old kernels
        for (auto &kv : c->graphs) cudaGraphExecDestroy(kv.second);
        c->graphs.clear();
        c->graph_kernels.clear();
    }
    c->kv[0] = fwd_variant;
    c->kv[1] = bwd_variant;
    c->nbl = shots_per_launch ? shots_per_launch : c->B;
    return RTM_OK;
}

int rtm_ctx_set_snapshots(rtm_ctx *c, int every, int precision)
{
    if (!c || every < 0 || precision < RTM_RING_F32 || precision > RTM_RING_I16) return RTM_ERR_ARG;
    if (c->NT < 5 && every > 0) return RTM_ERR_ARG;
    // the captured time loops change with the mode
    for (auto &kv : c->graphs) cudaGraphExecDestroy(kv.second);
    c->graphs.clear();
    RTM_CUDA_TRY(cudaStreamSynchronize(c->st));
    free_snapshots(c);
    if (every == 0) return RTM_OK;
    const int nslots = snap_slots(c->NT - 3, every);  // steps 0, 1, 2, 2+K, .. <= NT-3
    // column offset of the stored interior: a plane row from x0 - N2 + off =
    // x0 - 8*floor(N2/8) on (x0 a multiple of 8) starts on 16 bytes
    const int off = c->N2 % 8;
    const int pitch = (c->nx + off + 7) / 8 * 8;
    const size_t es = precision == RTM_RING_F32 ? 4 : 2;
    const size_t plane = (size_t)c->nz * pitch;
    const long long planes = (long long)c->B * nslots;
    int rc = RTM_OK;
    auto balloc = [&](void **q, size_t bytes) {
        if (rc) return;
        if (cudaMalloc(q, bytes) != cudaSuccess) {
            cudaGetLastError();
            *q = nullptr;
            rtm_set_last_error("cudaMalloc failed (source snapshots)");
            rc = RTM_ERR_NOMEM;
            return;
        }
        c->bytes += bytes;
        c->snap_bytes += bytes;
    };
    balloc(&c->snapS, plane * planes * es);
    if (c->p.compen) balloc(reinterpret_cast<void **>(&c->snapQ), plane * planes * sizeof(float));
    balloc(reinterpret_cast<void **>(&c->pacc), sizeof(float) * (size_t)c->B * c->ss);
    balloc(reinterpret_cast<void **>(&c->snap_scale), sizeof(float) * (size_t)planes);
    balloc(reinterpret_cast<void **>(&c->snap_amax), sizeof(unsigned) * (size_t)planes);
    // receiver band: SNAP_BAND cells on each side of the receiver line
    eng::SnapBand b{};
    if (c->nrec > 0) {
        constexpr int SNAP_BAND = 24;
        const int zl = std::min(c->p.rz0, c->p.rz0 + (c->nrec - 1) * c->p.rdz);
        const int zh = std::max(c->p.rz0, c->p.rz0 + (c->nrec - 1) * c->p.rdz);
        const int xl = std::min(0, (c->nrec - 1) * c->p.rdx), xh = std::max(0, (c->nrec - 1) * c->p.rdx);
        b.z0 = std::max(c->N2, zl - SNAP_BAND);
        b.zn = std::max(0, std::min(c->NZ - c->N2 - 1, zh + SNAP_BAND) - b.z0 + 1);
        b.xoff = xl - SNAP_BAND;
        b.xn = xh - xl + 2 * SNAP_BAND + 1;
    }
    if (b.zn) {
        const size_t bcells = (size_t)c->B * (c->NT - 2) * b.zn * b.xn;
        balloc(reinterpret_cast<void **>(&c->bandS), sizeof(float) * bcells);
        if (c->p.compen) balloc(reinterpret_cast<void **>(&c->bandP), sizeof(float) * bcells);
    }
    if (!rc) {
        c->snap_every = every;
        c->snap_prec = precision;
        c->snap_nslots = nslots;
        c->snap_off = off;
        c->snap_pitch = pitch;
        c->band = b;
        rc = make_map(&c->smaps_f.sum, c->pacc, c->NX, c->NZ, c->B, c->P, eng::TX, eng::TZ);
        c->smaps_b.sum = c->imaps.racc;
    }
    if (rc) free_snapshots(c);
    return rc;
}

int rtm_ctx_get_snapshots(const rtm_ctx *c, int *every, int *precision, size_t *bytes)
{
    if (!c) return RTM_ERR_ARG;
    if (every) *every = c->snap_every;
    if (precision) *precision = c->snap_prec;
    if (bytes)
        *bytes = c->snap_every ? (size_t)c->B * c->snap_nslots * c->nz * c->snap_pitch *
                                         ((c->snap_prec ? 2 : 4) + (c->snapQ ? 4 : 0)) +
                                     (size_t)c->B * (c->NT - 2) * c->band.zn * c->band.xn *
                                         ((c->bandS ? 4 : 0) + (c->bandP ? 4 : 0))
                               : 0;
    return RTM_OK;
}

int rtm_ctx_get_kernel(const rtm_ctx *c, int *fwd_variant, int *bwd_variant, int *shots_per_launch)
{
    if (!c || !fwd_variant || !bwd_variant || !shots_per_launch) return RTM_ERR_ARG;
    *fwd_variant = c->kv[0];
    *bwd_variant = c->kv[1];
    *shots_per_launch = c->nbl;
    return RTM_OK;
}

int rtm_ctx_autotune(rtm_ctx *c, int nshot, const int *src_cells, const int *win_x0, const int *win_nx,
                     int nsteps, double *gcells_per_s)
{
    if (!c || nshot < 1 || !src_cells || nsteps < 1 || (!win_x0) != (!win_nx)) return RTM_ERR_ARG;
    nsteps = std::min(nsteps, c->NT - 3);  // both loops stay inside their step ranges
    if (nsteps < 1) return RTM_ERR_ARG;
    const bool was_timing = c->timing;
    c->timing = false;
    cudaEvent_t e[3];
    for (auto &x : e) RTM_CUDA_TRY(cudaEventCreate(&x));
    double best = -1.0;
    int bf = c->kv[0], bb = c->kv[1], bn = c->nbl;
    int rc = RTM_OK;
    for (int nb = std::min(c->B, nshot); nb >= 1 && rc == RTM_OK; nb = nb > 4 ? nb / 2 : 0) {
        if ((rc = set_batch(c, nb, src_cells, win_x0, win_nx))) break;
        double cells = 0;  // cell updates of one forward + one backward step of the batch
        for (int i = 0; i < nb; ++i)
            cells += (double)c->NZ * c->hnx[i] + (double)c->nz * (c->hnx[i] - 2 * c->N2);
        // tiled, persistent, tiled in two stream halves, two columns per
        // lane, two columns per lane in two stream halves (the last two
        // forward only: the backward form is timed as tiled / split there);
        // every form timed twice, interleaved, keeping its faster run
        constexpr int NV = 5, REPS = 2;
        double fwd_ms[NV], bwd_ms[NV];
        for (int v = 0; v < NV; ++v) fwd_ms[v] = bwd_ms[v] = 1e30;
        for (int rep = 0; rep < REPS && rc == RTM_OK; ++rep)
            for (int v = 0; v < NV && rc == RTM_OK; ++v) {
                c->kv[0] = v;
                c->kv[1] = v == RTM_KERNEL_X2 ? RTM_KERNEL_TILED : v == RTM_KERNEL_X2_SPLIT ? RTM_KERNEL_SPLIT : v;
                c->kstop = 2 + 1;  // warm-up: one step of each phase
                if ((rc = enqueue_forward(c, nb, false)) || (rc = enqueue_backward(c, nb))) break;
                c->kstop = 2 + nsteps;
                cudaEventRecord(e[0], c->st);
                if ((rc = enqueue_forward(c, nb, false))) break;
                cudaEventRecord(e[1], c->st);
                if ((rc = enqueue_backward(c, nb))) break;
                cudaEventRecord(e[2], c->st);
                if (cudaEventSynchronize(e[2]) != cudaSuccess) { rc = RTM_ERR_CUDA; break; }
                float a = 0, b = 0;
                cudaEventElapsedTime(&a, e[0], e[1]);
                cudaEventElapsedTime(&b, e[1], e[2]);
                fwd_ms[v] = std::min(fwd_ms[v], (double)a);
                bwd_ms[v] = std::min(bwd_ms[v], (double)b);
            }
        if (rc) break;
        int vf = 0, vb = 0;
        for (int v = 1; v < NV; ++v) {
            if (fwd_ms[v] < fwd_ms[vf]) vf = v;
            if (v != RTM_KERNEL_X2 && v != RTM_KERNEL_X2_SPLIT && bwd_ms[v] < bwd_ms[vb]) vb = v;
        }
        const double rate = cells * nsteps / ((fwd_ms[vf] + bwd_ms[vb]) * 1e-3) / 1e9;
        if (rate > best) {
            best = rate;
            bf = vf; bb = vb; bn = nb;
        }
    }
    c->kstop = 0;
    c->timing = was_timing;
    for (auto &x : e) cudaEventDestroy(x);
    if (rc) return rc;
    unsigned derr = 0;
    rtm_device_error(&derr);
    if (derr) {
        rtm_set_last_error("device-side wait timed out");
        return RTM_ERR_DEVICE;
    }
    if (gcells_per_s) *gcells_per_s = best;
    return rtm_ctx_set_kernel(c, bf, bb, bn);
}

int rtm_ctx_launches(rtm_ctx *c, long *count, int reset)
{
    if (!c || !count) return RTM_ERR_ARG;
    *count = c->launches;
    if (reset) c->launches = 0;
    return RTM_OK;
}

int rtm_model_batch(rtm_ctx *c, int nshot, const int *src_cells, float *rec, int flags)
{
    if (!c || nshot < 0 || (nshot > 0 && (!src_cells || !rec))) return RTM_ERR_ARG;
    const bool dev = flags & RTM_DEVICE_PTRS;
    const long long per = (long long)c->NT * c->nrec;
    for (int s0 = 0; s0 < nshot; s0 += c->nbl) {
        const int nb = std::min(c->nbl, nshot - s0);
        if (int rc = set_batch(c, nb, src_cells + s0, nullptr, nullptr)) return rc;
        if (int rc = run_phase(c, 0, nb, flags)) return rc;
        if (c->nrec > 0) {
            transpose(c, c->rec, c->stage, c->NT, c->nrec, nb, c->st);
            RTM_CUDA_TRY(cudaMemcpyAsync(rec + (long long)s0 * per, c->stage, sizeof(float) * per * nb,
                                         dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, c->st));
        }
    }
    RTM_CUDA_TRY(cudaStreamSynchronize(c->st));
    unsigned e = 0;
    rtm_device_error(&e);
    if (e) {
        rtm_set_last_error("device-side wait timed out");
        return RTM_ERR_DEVICE;
    }
    return RTM_OK;
}

static int migrate_group(rtm_ctx *c, int s0, int nb, const int *src_cells, const int *xa,
                         const int *nx, const float *seis, int flags)
{
    const bool dev = flags & RTM_DEVICE_PTRS;
    const long long per = (long long)c->NT * c->nrec;
    if (int rc = set_batch(c, nb, src_cells + s0, xa ? xa + s0 : nullptr, nx ? nx + s0 : nullptr))
        return rc;
    if (c->nrec == 0) return run_phase(c, 1, nb, flags);
    // The observed data are only read by the backward run: their upload and
    // transpose go to the second stream and overlap the forward run.
    RTM_CUDA_TRY(cudaEventRecord(c->evc[0], c->st));  // earlier users of data / stage are done
    RTM_CUDA_TRY(cudaStreamWaitEvent(c->st2, c->evc[0], 0));
    RTM_CUDA_TRY(cudaMemcpyAsync(c->stage, seis + (long long)s0 * per, sizeof(float) * per * nb,
                                 dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, c->st2));
    transpose(c, c->stage, c->data, c->nrec, c->NT, nb, c->st2);
    RTM_CUDA_TRY(cudaEventRecord(c->evc[1], c->st2));
    if (int rc = run_phase(c, 2, nb, flags)) return rc;
    RTM_CUDA_TRY(cudaStreamWaitEvent(c->st, c->evc[1], 0));
    return run_phase(c, 3, nb, flags);
}

int rtm_migrate_batch(rtm_ctx *c, int nshot, const int *src_cells, const float *seis, float *rel1,
                      float *rel2, int flags)
{
    if (!c || nshot < 0 || (nshot > 0 && (!src_cells || (!seis && c->nrec > 0)))) return RTM_ERR_ARG;
    const bool dev = flags & RTM_DEVICE_PTRS;
    const long long gsz = (long long)c->NZ * c->NX;
    for (int s0 = 0; s0 < nshot; s0 += c->nbl) {
        const int nb = std::min(c->nbl, nshot - s0);
        if (int rc = migrate_group(c, s0, nb, src_cells, nullptr, nullptr, seis, flags)) return rc;
        if (rel1)
            if (int rc = copy_grid_out(c, c->rel1, rel1 + s0 * gsz, nb, dev)) return rc;
        if (rel2)
            if (int rc = copy_grid_out(c, c->rel2, rel2 + s0 * gsz, nb, dev)) return rc;
    }
    RTM_CUDA_TRY(cudaStreamSynchronize(c->st));
    unsigned e = 0;
    rtm_device_error(&e);
    if (e) {
        rtm_set_last_error("device-side wait timed out");
        return RTM_ERR_DEVICE;
    }
    return RTM_OK;
}

static int migrate_stack_impl(rtm_ctx *c, int nshot, const int *src_cells, const int *xa,
                              const int *nx, const float *seis, float whitecoe, int nrec_div,
                              int inorm, float *image, float *illum, float *ups, float *downs,
                              int flags)
{
    if (!c || nshot < 1 || !src_cells || (!seis && c->nrec > 0) || nrec_div < 1) return RTM_ERR_ARG;
    const bool dev = flags & RTM_DEVICE_PTRS;
    const long ncell = (long)c->nz * c->nx;  // survey interior
    for (float *q : {c->ks1, c->kc1, c->ks2, c->kc2})
        RTM_CUDA_TRY(cudaMemsetAsync(q, 0, sizeof(float) * ncell, c->st));
    for (int s0 = 0; s0 < nshot; s0 += c->nbl) {
        const int nb = std::min(c->nbl, nshot - s0);
        if (int rc = migrate_group(c, s0, nb, src_cells, xa, nx, seis, flags)) return rc;
        RTM_CUDA_TRY(cudaMemsetAsync(c->imax, 0, sizeof(unsigned) * nb, c->st));
        eng::k_illum_max<<<dim3(64, nb), 256, 0, c->st>>>(c->rel2, c->imax, c->ss, c->NZ, c->gnx,
                                                          c->P, c->N2);
        eng::k_finish<<<dim3(cdiv(ncell, 256), nb), 256, 0, c->st>>>(
            c->rel1, c->rel2, c->windowed ? c->vs : c->v, c->windowed ? c->ss : 0, c->imax, c->ups,
            c->downs, c->ss, c->NZ, c->gnx, c->P, c->N2, c->nx, c->vmax, whitecoe);
        eng::k_stack_kahan<<<cdiv(ncell, 256), 256, 0, c->st>>>(c->ups, c->downs, nb, c->nz, c->nx,
                                                               c->nx, c->gxa, c->gnx, c->N2, c->ks1,
                                                               c->kc1, c->ks2, c->kc2);
        c->launches += 3;
        RTM_LAUNCH_CHECK();
        const auto kind = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
        if (ups)
            RTM_CUDA_TRY(cudaMemcpyAsync(ups + (long long)s0 * ncell, c->ups, sizeof(float) * ncell * nb,
                                         kind, c->st));
        if (downs)
            RTM_CUDA_TRY(cudaMemcpyAsync(downs + (long long)s0 * ncell, c->downs,
                                         sizeof(float) * ncell * nb, kind, c->st));
    }
    eng::k_stack_final<<<cdiv(ncell, 256), 256, 0, c->st>>>(c->ks1, c->ks2, c->img, c->ill, ncell,
                                                            nrec_div, inorm);
    c->launches++;
    RTM_LAUNCH_CHECK();
    const auto kind = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (image) RTM_CUDA_TRY(cudaMemcpyAsync(image, c->img, sizeof(float) * ncell, kind, c->st));
    if (illum) RTM_CUDA_TRY(cudaMemcpyAsync(illum, c->ill, sizeof(float) * ncell, kind, c->st));
    RTM_CUDA_TRY(cudaStreamSynchronize(c->st));
    unsigned e = 0;
    rtm_device_error(&e);
    if (e) {
        rtm_set_last_error("device-side wait timed out");
        return RTM_ERR_DEVICE;
    }
    return RTM_OK;
}

int rtm_migrate_stack(rtm_ctx *c, int nshot, const int *src_cells, const float *seis,
                      float whitecoe, int nrec_div, int inorm, float *image, float *illum,
                      float *ups, float *downs, int flags)
{
    return migrate_stack_impl(c, nshot, src_cells, nullptr, nullptr, seis, whitecoe, nrec_div,
                              inorm, image, illum, ups, downs, flags);
}

int rtm_migrate_stack_windows(rtm_ctx *c, int nshot, const int *src_cells, const int *win_x0,
                              const int *win_nx, const float *seis, float whitecoe, int nrec_div,
                              int inorm, float *image, float *illum, int flags)
{
    if (!win_x0 || !win_nx) return RTM_ERR_ARG;
    return migrate_stack_impl(c, nshot, src_cells, win_x0, win_nx, seis, whitecoe, nrec_div, inorm,
                              image, illum, nullptr, nullptr, flags);
}

}  // extern "C"
