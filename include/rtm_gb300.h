/*
 * rtm_gb300.h -- C ABI of the GB300 (sm_103a) engine for the 2-D acoustic
 * reverse-time-migration path of caixh90/RTM_GPU.
 *
 * Two levels:
 *
 *  1. Kernel level (rtm_k_*): one entry point per __global__ kernel of the
 *     reference's kernel.cu, with the same argument list, units and
 *     [iz*NX + ix] row-major layout, plus a trailing stream.  A copy of the
 *     reference's main() whose "Name<<<gridDim,blockDim>>>(" launches are
 *     rewritten to "rtm_k_Name(" runs unchanged in logic on these kernels.
 *     Buffers are caller-owned device pointers; nothing is allocated.
 *
 *  2. Shot level (rtm_ctx_*, rtm_model_*, rtm_migrate_*, ...): a context owns
 *     the device copies of the model and the per-shot wavefields, and advances
 *     a batch of shots together through fused, TMA-staged kernels (captured in
 *     CUDA graphs).  Host buffers are caller-owned; device buffers are
 *     context-owned.  A context is thread-compatible (not thread-safe).
 *
 * Every function returns RTM_OK (0) or a negative status; rtm_last_error()
 * gives a message for the calling thread's last failure.
 */
#ifndef RTM_GB300_H
#define RTM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *rtm_stream_t; /* a cudaStream_t; NULL = legacy default stream */

enum {
    RTM_OK = 0,
    RTM_ERR_ARG = -1,       /* invalid argument or size                         */
    RTM_ERR_CUDA = -2,      /* CUDA runtime error (message in rtm_last_error)   */
    RTM_ERR_NOMEM = -3,     /* device or host allocation failed                 */
    RTM_ERR_DEVICE = -4,    /* a kernel reported a device-side error            */
    RTM_ERR_UNSUPPORTED = -5,
    RTM_ERR_IO = -6         /* a file could not be read or written              */
};

const char *rtm_last_error(void);
int rtm_version(void);
/* Device-side error word (bit 0: a bounded TMA wait gave up); cleared on read. */
int rtm_device_error(unsigned int *code);

/* ======================================================================
 * 1. Kernel level: drop-in replacements for kernel.cu's kernels.
 *    Each cites the reference kernel it replaces.
 * ====================================================================== */

/* kernel.cu:18-45 Equal */
int rtm_k_Equal(float *Dlf, float *Drt, float *Dup, float *Ddw, float *DFW0, float *DFW1, int NZ,
                int NX, int N2, int nfdmax, rtm_stream_t s);
/* kernel.cu:46-80 Add */
int rtm_k_Add(float *Dv, float *DFW2, float *DFW0, float *DFW1, float *Dc, int *DIndex, float tao2,
              float h2, float vmin, float dv, int nfdmax, int NZ, int NX, int NXZ, int r_u, int r_x,
              float wavelet, float hzx2_1, rtm_stream_t s);
/* kernel.cu:82-114 Add_Con */
int rtm_k_Add_Con(float *Dv, float *DFW2, float *DFW0, float *DFW1, float *Dc, float tao2, float h2,
                  int nfdmax, int NZ, int NX, int NXZ, int r_u, int r_x, float wavelet,
                  float hzx2_1, rtm_stream_t s);
/* kernel.cu:116-158 Hybrid1 */
int rtm_k_Hybrid1(float *DFW1, float *DFW0, float *DFW2, float *DFWb, float *Dlf, float *Drt,
                  float *Dup, float *Ddw, float *Dv, float *Dr_1, float *Dw, int NZ, int NX, int N2,
                  int nfdmax, int k, float taoh, float taoh2, rtm_stream_t s);
/* kernel.cu:160-183 Hybrid2 */
int rtm_k_Hybrid2(float *DFW1, float *DFW0, float *DFW2, float *DFWb, float *Dlf, float *Drt,
                  float *Dup, float *Ddw, float *Dv, float *Dr_1, float *Dw, int NZ, int NX, int N2,
                  int nfdmax, int k, float taoh, float taoh2, rtm_stream_t s);
/* kernel.cu:184-208 Hybrid3 */
int rtm_k_Hybrid3(float *DFW1, float *DFW0, float *DFW2, float *DFWb, float *Dlf, float *Drt,
                  float *Dup, float *Ddw, float *Dv, float *Dr_1, float *Dw, int NZ, int NX, int N2,
                  int nfdmax, int k, float taoh, float taoh2, rtm_stream_t s);
/* kernel.cu:210-221 Deliver */
int rtm_k_Deliver(float *DFW1, float *DFW0, float *DFW2, int NZ, int NX, rtm_stream_t s);
/* kernel.cu:222-245 BKEqual */
int rtm_k_BKEqual(float *Dlf, float *Drt, float *Dup, float *Ddw, float *DFW1, int NZ, int NX,
                  int N2, int nfdmax, int k, rtm_stream_t s);
/* kernel.cu:246-283 BKAdd_EFF */
int rtm_k_BKAdd_EFF(float *Dv, float *DFW2, float *DFW0, float *DFW1, float *Dc, int *DIndex,
                    float tao2, float h2, float vmin, float dv, int N2, int NZ, int NX, int NXZ,
                    int r_u, int r_x, float wavelet, float hzx2_1, rtm_stream_t s);
/* kernel.cu:286-320 BKAdd_EFF_Con */
int rtm_k_BKAdd_EFF_Con(float *Dv, float *DFW2, float *DFW0, float *DFW1, float *Dc, float tao2,
                        float h2, int N2, int NZ, int NX, int NXZ, int r_u, int r_x, int nfdmax,
                        float wavelet, float hzx2_1, rtm_stream_t s);
/* kernel.cu:323-337 Deliver_EFF */
int rtm_k_Deliver_EFF(float *DFW1, float *DFW0, float *DFW2, int N2, int NZ, int NX,
                      rtm_stream_t s);
/* kernel.cu:339-380 BKAdd */
int rtm_k_BKAdd(float *Dv, float *DBW2, float *DBW1, float *DBW0, float *Dc, int *DIndex,
                float *Dseis, float tao2, float h2, float vmin, float dv, int nfdmax, int NZ,
                int NX, int NXZ, int s_l, int s_r, int s_z, int ds, float hzx2_1, rtm_stream_t s);
/* kernel.cu:381-418 BKAdd_Con */
int rtm_k_BKAdd_Con(float *Dv, float *DBW2, float *DBW1, float *DBW0, float *Dc, float *Dseis,
                    float tao2, float h2, int nfdmax, int NZ, int NX, int NXZ, int s_l, int s_r,
                    int s_z, int ds, float hzx2_1, rtm_stream_t s);
/* kernel.cu:421-463 BKHybrid1 */
int rtm_k_BKHybrid1(float *DFW1, float *DFW0, float *DFW2, float *DFWb, float *Dv, float *Dr_1,
                    float *Dw, int NZ, int NX, int N2, float taoh, float taoh2, rtm_stream_t s);
/* kernel.cu:464-487 BKHybrid2 */
int rtm_k_BKHybrid2(float *DFW1, float *DFW0, float *DFW2, float *DFWb, float *Dv, float *Dr_1,
                    float *Dw, int NZ, int NX, int N2, float taoh, float taoh2, rtm_stream_t s);
/* kernel.cu:489-501 Rel_NonCompen */
int rtm_k_Rel_NonCompen(float *DBW2, float *DFW2, float *Drel1, float *Drel2, int NZ, int NX,
                        rtm_stream_t s);
/* kernel.cu:503-517 Rel_Compen */
int rtm_k_Rel_Compen(float *DBW2, float *DFW2, float *DBWADD, float *DFWADD, float *Drel1,
                     float *Drel2, int NZ, int NX, rtm_stream_t s);

/* No counterpart in the reference.  The same update as rtm_k_Hybrid1 followed
 * by rtm_k_Hybrid2 (or the BK pair), for callers that cannot allocate device
 * memory where they step the wavefield (their device memory belongs to their
 * own pool, or their time loop must not call cudaMalloc): the one-way scratch
 * lives in a fixed 1,048,576-value device array inside this library instead of
 * a caller DFWb buffer.  Pads with more cells are rejected (RTM_ERR_ARG).  All
 * calls share that array, so calls overlapping on the GPU race; the first call
 * on each device, and the first after the device's context was re-created
 * (cudaDeviceReset), looks the array up and should come before any stream
 * capture. */
int rtm_k_HybridStatic(float *DFW1, float *DFW0, float *DFW2, float *Dv, float *Dr_1, float *Dw,
                       int NZ, int NX, int N2, float taoh, float taoh2, rtm_stream_t s);

/* ======================================================================
 * 2. Host preparation (replaces the reference's host set-up code).
 * ====================================================================== */

/* GPU_velocity_real.cpp:6-118 (velocity): vin is the interior model as the
 * reference's velocity file stores it (column-major, nx columns of nz).
 * Fills the padded v[NZ*NX] (edge extension, optional left/right flip) and
 * r_1[NZ*NX] = sqrt((v*tao/h)^2/2). */
int rtm_prep_velocity(const float *vin, int nz, int nx, int N2, float tao, float h, int flip,
                      float *v, float *r1);
/* kernel.cu:704-742: snapped vmin/vmax, nvel, and need[nvel] (may be NULL to
 * query nvel; need_cap is its capacity). */
int rtm_prep_bins(const float *v, long ncell, float dv, float *vmin, float *vmax, int *nvel,
                  int *need, int need_cap);
/* kernel.cu:1261-1266 (f): wav[i] = Ricker(i*tao, f0), i < n. */
int rtm_prep_wavelet(float *wav, int n, float tao, float f0);
/* LSMOrCon_rec_2D.cpp:526-551 (order): Taylor coefficients c[0..N/2]. */
int rtm_prep_taylor(int N, float *c);

/* Least-squares optimiser settings (the reference's parameter file:
 * nthita, nfdmax, nfdmin, df, eps, fmax; hzx = hz/h). */
typedef struct rtm_ls_settings {
    int nthita, nfdmax, nfdmin;
    double tao, h, df, eps, fmax, hzx;
} rtm_ls_settings;

/* LSMOrCon_rec_2D.cpp:22-73 (funMandC) in FP64 on the GPU: operator length
 * len[nvel] (-1 for bins not in need[]), prefix offsets index[nvel+1] and the
 * float coefficient table coef[index[nvel]] (coef may be NULL to query the
 * size, returned in *nc).  Bin i is velocity vmin + i*dv. */
int rtm_coeffs_optimise_fp64(const rtm_ls_settings *s, double vmin, double dv, int nvel,
                             const int *need, int *len, int *index, float *coef, int ccap,
                             int *nc);
/* LSMOrCon_rec_2D.cpp:236-287 (CAL2DFDCOE_LSM) for n cases on the GPU:
 * c[i*17 + l], l <= M[i] (M[i] <= 16). */
int rtm_ls_coefs_fp64(const double *r, const double *bb, const int *M, int n, double hzx,
                      double *c);

/* Learned coefficients: a 3-layer MLP (3 -> 64 -> 64 -> 16, tanh, FP32)
 * mapping (r = v*tao/h, band limit kmax*h, M) to c_1..c_M, trained on the GPU
 * by its own forward/backward/Adam kernels on sets the FP64 optimiser makes.
 * Parameters are a flat array of rtm_mlp_nparams() floats; the normalisation
 * block is in_mean[3], in_scale[3], out_mean[16], out_scale[16].  Samples:
 * x[n][3] = (r, kh, M), c[n][16] = c_1..c_16 (entries >= M ignored).  The
 * training loss (rtm_mlp_grad, rtm_mlp_train) is the mean squared relative
 * difference of the FD symbols of the network's and the sample's coefficients
 * on 8 wavenumbers (kh/8 .. kh) x 4 angles (0 .. pi/4). */
typedef struct rtm_mlp rtm_mlp;
int rtm_mlp_create(rtm_mlp **m, unsigned seed);
int rtm_mlp_destroy(rtm_mlp *m);
int rtm_mlp_nparams(void);
int rtm_mlp_get_params(const rtm_mlp *m, float *params);
int rtm_mlp_set_params(rtm_mlp *m, const float *params);
int rtm_mlp_set_norm(rtm_mlp *m, const float *norm);
int rtm_mlp_get_norm(const rtm_mlp *m, float *norm);
int rtm_mlp_grad(rtm_mlp *m, const float *x, const float *c, int n, float *grad, float *loss);
int rtm_mlp_train(rtm_mlp *m, const float *x, const float *c, int n, int epochs, int batch,
                  float lr, float *final_loss);
int rtm_mlp_predict(rtm_mlp *m, const float *x, int n, float *c);
/* Dispersion measures: the relative phase-velocity error |v_FD/v - 1|, or
 * the reference's own measure (h/v) |v/v_FD - 1| that its operator-length
 * test compares with `eps` (LSMOrCon_rec_2D.cpp:321-337; h/v = tao/r). */
#define RTM_DISP_RELATIVE 0
#define RTM_DISP_REFERENCE 1
/* Largest dispersion error (in the measure `metric`) of n coefficient sets
 * c[n][cstride] over kh in (0,bb] (nk samples) and angles [0,pi/4] (nth+1);
 * tao (the time step) is used by RTM_DISP_REFERENCE. */
int rtm_disp_error_fp64(const double *c, int cstride, const int *M, const double *r,
                        const double *bb, int n, int nk, int nth, double hzx, int metric, double tao,
                        double *err);
/* Coefficient table (funMandC layout) from the network with length M for
 * every needed bin, judged by the FP64 dispersion error in the measure
 * `metric`; for the bins whose network set misses `tol` the FP64 optimiser
 * designs the set too and the bin keeps the lower-error set of the two
 * (*nfallback counts the bins that keep the optimiser's). */
int rtm_coeffs_mlp(rtm_mlp *m, const rtm_ls_settings *s, double vmin, int nvel, const int *need,
                   int M, double tol, int metric, int *len, int *index, float *coef, int ccap,
                   int *nc, int *nfallback, double *err_net, double *err_used);

/* ======================================================================
 * 3. Shot level.
 * ====================================================================== */

/* One model grid shared by a batch of shots.  Host pointers; copied at
 * rtm_ctx_create.  Coordinates are 0-based cells of the padded grid. */
typedef struct rtm_problem {
    int nz, nx, N2;     /* interior size and pad width (NZ = nz+2*N2, ...)      */
    int M;              /* nfdmax: ring width and longest operator              */
    int NT, NT2;        /* time steps; wavelet injected while step < NT2        */
    int adaptive;       /* 1: per-velocity-bin coefficients (iLSTE=0)           */
    int compen;         /* iCompen                                              */
    int quirk;          /* 1: the reference's velocity indexing in the ABC      */
    int nbins;          /* nvel (adaptive) ; ignored otherwise                  */
    float tao2, h2, taoh, taoh2, vmin, dv, hzx2_1, spike;
    const float *v;     /* [NZ*NX] padded velocity                               */
    const float *r1;    /* [NZ*NX] r_1                                           */
    const float *w;     /* [N2+1] blend weights                                  */
    const float *coef;  /* adaptive: reference table c[Index[b] .. Index[b+1]-1];
                           fixed: c[0..M]                                        */
    const int *index;   /* [nbins+1] (adaptive)                                  */
    const float *wav;   /* [NT+1] wav[i] = f(i*tao)                              */
    /* receivers: cells (rz0 + j*rdz, rx0 + j*rdx), j < nrec (a surface line,
       a vertical well, ...); both steps 0 is invalid */
    int rz0, rx0, rdz, rdx, nrec;
    int ring_precision; /* RTM_RING_F32 / _BF16 / _F16 / _I16                   */
} rtm_problem;

/* Storage of the saved boundary rings (the stencil and imaging arithmetic
 * stay FP32): FP32, or 16 bits with one FP32 scale per shot and step -- BF16
 * or FP16 values scaled so the step's max |value| is 16384, or int16
 * fractions of the step's max |value| (RTM_RING_I16: fixed point, the
 * finest absolute rounding at the values that dominate the field). */
enum { RTM_RING_F32 = 0, RTM_RING_BF16 = 1, RTM_RING_F16 = 2, RTM_RING_I16 = 3 };

/* flags for rtm_model_batch / rtm_migrate_batch */
enum {
    RTM_DEVICE_PTRS = 1, /* data/result pointers are device pointers            */
    RTM_NO_GRAPH = 2     /* launch step by step instead of replaying a graph    */
};

typedef struct rtm_ctx rtm_ctx;

/* max_batch: shots advanced together (device memory is sized for it). */
int rtm_ctx_create(rtm_ctx **ctx, const rtm_problem *p, int max_batch, rtm_stream_t stream);
int rtm_ctx_destroy(rtm_ctx *ctx);
/* Device bytes held by the context. */
int rtm_ctx_bytes(const rtm_ctx *ctx, size_t *bytes);

/* Forward modelling with receiver recording (new relative to the reference,
 * which reads recorded gathers from files).  src_cells[nshot] are flat
 * padded-grid indices z*NX+x of the sources (host).  rec is trace-major
 * [nshot][nrec][NT]. */
int rtm_model_batch(rtm_ctx *ctx, int nshot, const int *src_cells, float *rec, int flags);

/* Migration of nshot shots (kernel.cu:798-933 per shot): forward source run,
 * boundary-ring reconstruction, receiver back-propagation with Dirichlet
 * injection of the gathers seis [nshot][nrec][NT] (trace-major), imaging.
 * rel1/rel2 receive the full padded cross-correlation / illumination grids
 * [nshot][NZ][NX] (either may be NULL). */
int rtm_migrate_batch(rtm_ctx *ctx, int nshot, const int *src_cells, const float *seis,
                      float *rel1, float *rel2, int flags);

/* Migration plus per-shot finishing (kernel.cu:935-990) and a compensated
 * (Kahan) stack over the shots (kernel.cu:992-1059): image and illum are the
 * interior [nz][nx] stacked results (image divided by nrec_div and, when
 * inorm, by the stacked illumination).  ups/downs (may be NULL) receive the
 * per-shot interior images [nshot][nz][nx]. */
int rtm_migrate_stack(rtm_ctx *ctx, int nshot, const int *src_cells, const float *seis,
                      float whitecoe, int nrec_div, int inorm, float *image, float *illum,
                      float *ups, float *downs, int flags);

/* Uneven aperture windows (reverse-VSP and other geometries where each shot
 * sees its own part of the survey): the context's model is the whole survey
 * (nz x nx interior); shot i migrates on interior columns
 * [win_x0[i], win_x0[i]+win_nx[i]) padded by edge extension as the reference
 * pads a model it reads (GPU_velocity_real.cpp:20-80).  src_cells[i] is the
 * flat index z*NX_i + x in the shot's own padded grid (NX_i = win_nx[i]+2*N2);
 * the context's receiver line moves with the window (columns rx0 - win_x0[i])
 * and must lie inside it.  Shots of a batch advance together; images are
 * finished per shot and stacked (Kahan) into the survey frame [nz][nx]. */
int rtm_migrate_stack_windows(rtm_ctx *ctx, int nshot, const int *src_cells, const int *win_x0,
                              const int *win_nx, const float *seis, float whitecoe, int nrec_div,
                              int inorm, float *image, float *illum, int flags);

/* The reference's per-shot loop (kernel.cu:798-933) on the rtm_k_* kernels
 * (legacy stream, one synchronous copy of the trace samples per backward
 * step, device buffers allocated inside): the plain single-shot drop-in.
 * Receivers must form the reference's surface line (rdz == 0).  seis is
 * trace-major [nrec][NT]; rel1/rel2 receive the padded grids [NZ][NX]. */
int rtm_plain_migrate_shot(const rtm_problem *p, int src_cell, const float *seis, float *rel1,
                           float *rel2);

/* Per-launch timing: with timing enabled, launches go one by one (no graph)
 * with CUDA events around each kernel; rtm_ctx_timing returns the summed
 * milliseconds and launch counts of [0] forward stencil, [1] backward
 * stencil (source + receiver + imaging), [2] pad kernels. */
int rtm_ctx_set_timing(rtm_ctx *ctx, int enable);
int rtm_ctx_timing(const rtm_ctx *ctx, double ms[3], long n[3]);
/* Kernels this context has launched (graph replays count their kernels). */
int rtm_ctx_launches(rtm_ctx *ctx, long *count, int reset);

/* Stencil kernel form and shots per launch (no reference counterpart: the
 * reference launches one shot at a time).  RTM_KERNEL_TILED (the backward
 * default): one CTA per 128 x 16 tile of every shot; RTM_KERNEL_PERSISTENT:
 * a fixed grid of resident CTAs walks the batch's tiles with a two-stage TMA
 * pipeline;
 * RTM_KERNEL_SPLIT: the tiled kernel with the two halves of a batch on two
 * streams, so one half's pad launches overlap the other's stencil launches;
 * RTM_KERNEL_X2 (forward only): the tiled kernel with two columns per lane;
 * RTM_KERNEL_X2_SPLIT (forward only; the forward default): RTM_KERNEL_X2 on
 * the two stream halves.  All forms give bit-identical results.
 * Set separately for the forward and the backward stencil; shots_per_launch
 * in 1..max_batch (0: max_batch). */
enum {
    RTM_KERNEL_TILED = 0,
    RTM_KERNEL_PERSISTENT = 1,
    RTM_KERNEL_SPLIT = 2,
    RTM_KERNEL_X2 = 3,
    RTM_KERNEL_X2_SPLIT = 4
};
int rtm_ctx_set_kernel(rtm_ctx *ctx, int fwd_variant, int bwd_variant, int shots_per_launch);
int rtm_ctx_get_kernel(const rtm_ctx *ctx, int *fwd_variant, int *bwd_variant,
                       int *shots_per_launch);

/* Source snapshots (no reference counterpart: the reference reconstructs the
 * source field from its boundary rings at every backward step,
 * kernel.cu:892-901).  With every = K > 0, a migration's forward run stores
 * the source field's interior at steps 0, 1 (the start levels), 2, 2+K,
 * 2+2K, .. <= NT-3 and, for
 * compensated imaging, the running sum of the source field before each of
 * those steps; the source field as RTM_RING_* storage (16-bit codes with one
 * scale per shot and slot, the slot's max |value|; or fp32), the running sum
 * as fp32 (it changes slowly from slot to slot, so its rounding would not
 * average out and the image's Laplacian filter would show it); it saves no
 * rings.
 * Its backward run advances the receiver field alone (no source
 * reconstruction) and applies the imaging condition at the snapshot steps
 * only, each weighted by its share of the time sum (levels 0 and 1 with
 * weight 1, the others by the trapezoidal rule with step K plus end
 * corrections: every weight is 1 when K = 1), the source's running
 * sum being the forward total minus the stored prefix -- except on the band
 * of cells within 24 of the receiver line, where the receiver field is held
 * to the recorded data, whose content reaches far above the sampled steps'
 * rate: those cells are stored (fp32) and imaged at every step.  The image
 * therefore differs from the reference's per-step imaging by the remaining
 * time-sampling error and the storage rounding (measured at K = 4 against
 * FP64: 1.4e-4 of the finished image on a 201x401, 2000-step shot, 5.7e-4
 * on a 401x1201, 4000-step shot whose ring-scheme image is 5.5e-4 away).
 * Storage per shot: 3 + (NT-5)/K slots x nz x nx values of 2 or 4 bytes,
 * plus as many of 4 bytes with compensated imaging, plus the band's cells at
 * NT-2 steps in 4 bytes (8 compensated).  every = 0 turns snapshots
 * off (the default).  Returns RTM_ERR_NOMEM, snapshots off, when the device
 * cannot hold them.  Snapshot steps always run the tiled stencil forms (one
 * stream or the two halves); forms that do not exist for them fall back. */
int rtm_ctx_set_snapshots(rtm_ctx *ctx, int every, int precision);
/* Current snapshot setting and the device bytes of the stored snapshots. */
int rtm_ctx_get_snapshots(const rtm_ctx *ctx, int *every, int *precision, size_t *bytes);
/* Autotuner: times nsteps forward and nsteps backward time steps of the
 * first shots of a survey (optional windows as rtm_migrate_stack_windows)
 * for each kernel form (twice, interleaved, keeping each form's faster run)
 * and for shots per launch max_batch, /2, /4, ..., keeps the fastest
 * setting in the context and returns its rate in
 * grid-cell updates per second (/1e9).  Wavefield contents are scratch
 * afterwards. */
int rtm_ctx_autotune(rtm_ctx *ctx, int nshot, const int *src_cells, const int *win_x0,
                     const int *win_nx, int nsteps, double *gcells_per_s);

/* Self-test of the device-side bounded waits (no reference counterpart):
 * a kernel waits `polls` (1..2^20) times on an mbarrier that nothing
 * completes, gives up, and the device error word is read back into *code
 * (RTM_DEVERR_TMA_TIMEOUT = 1 expected); the context stays usable. */
int rtm_selftest_wait_timeout(unsigned polls, unsigned int *code);

/* ======================================================================
 * 5. The reference's file flow.
 * ====================================================================== */

/* Resample.cpp:193-225 (resample, called per trace at kernel.cu:839-845):
 * ntrace traces yin[ntrace][nxin] at interval dxin to yout[ntrace][nxout] at
 * dxout by the 8-point least-squares sinc interpolator; bit-identical to the
 * reference.  flags: RTM_DEVICE_PTRS for device buffers. */
int rtm_resample(const float *yin, int ntrace, int nxin, float dxin, float *yout, int nxout,
                 float dxout, int flags);

/* kernel.cu:542-1098 up to the stacked image: reads the reference's run file
 * (the 2D_Real_RVSP_RTM.txt layout: 28 label/value pairs), the parameter,
 * source-depth, velocity and per-shot gather files it names (paths relative
 * to the working directory, as the reference opens them), resamples the
 * gathers when their interval differs from the modelling step, migrates all
 * shots on the batched engine (max_batch shots per launch, 0: 16) and writes
 * RVSP_RTM_up_<m>.dat / RVSP_RTM_down_<m>.dat per shot,
 * RVSP_Migration_Real_new2.dat and vnew.dat with the reference's names and
 * layouts; for a full-depth output window also the reference's post-stack
 * chain: RVSP_Migration_Real_T.dat (depth to time), _T_phase.dat (phase
 * rotation by `angle`), _D.dat (back to depth) and RVSP_migration_Real.sgy
 * (headers from SGY_Model.sgy in the working directory when present). */
int rtm_run_config(const char *run_file, int max_batch);

/* ======================================================================
 * 6. The reference's post-stack display chain.
 * ====================================================================== */

/* DisToTimeAndTimeToDis1D.cpp:120-180 (D2T): traces img[ntr][nz] at depth
 * step dz with velocities v[ntr][nz] to two-way time at dt: out[ntr][*nt].
 * out may be NULL to query *nt; cap is out's capacity in floats.  flags:
 * RTM_DEVICE_PTRS.  Bit-identical to the reference. */
int rtm_depth_to_time(const float *v, const float *img, int ntr, int nz, float dz, float dt, float *out,
                      long cap, int *nt, int flags);
/* DisToTimeAndTimeToDis1D.cpp:30-118 (T2D): traces img[ntr][nt] at dt back
 * to depth at dz with velocities v[ntr][nzv]: out[ntr][*nz]. */
int rtm_time_to_depth(const float *v, int nzv, const float *img, int ntr, int nt, float dt, float dz,
                      float *out, long cap, int *nz, int flags);
/* phase_correction_ricker_decon.cpp:160-224 (phase_correction): every
 * trace's spectrum rotated by angle degrees (FP64 FFT as the reference;
 * traces up to 8192 samples). */
int rtm_phase_rotate(const float *din, float *dout, int ntr, int nt, float angle, int flags);
/* SGYWrite.cpp:3-55 (WriteSGY): ntr traces of ns samples to a SEG-Y file.
 * With template_path the textual, binary and trace headers come from that
 * file (the reference reads SGY_Model.sgy) and its sample format (IBM or
 * IEEE) is kept; without it, blank headers and IEEE samples.  The binary
 * header gets ns and the interval dt (seconds when < 1, else milliseconds;
 * stored in microseconds); each trace header gets offset, sx, sy (per
 * trace, may be NULL) and gx, gy. */
int rtm_write_segy(const char *path, const char *template_path, const float *data, int ntr, int ns,
                   float dt, const float *sx, const float *sy, float gx, float gy, const float *offset);

#ifdef __cplusplus
}
#endif
#endif /* RTM_GB300_H */
