// Device kernels of the shot-level engine.
//
// Data layout (per context, in HBM):
//   * every wavefield / image array is [shot][NZ][P] fp32 with a row pitch
//     P = NX rounded up to the tile width (128 floats), so tiles never leave
//     a row and every row starts on a 512-byte boundary; shots of a batch are
//     contiguous, so a batch is one 3-D tensor {NX, NZ, B} (row stride P)
//     that one TMA descriptor covers;
//   * the model (v, r_1) is one [NZ][P] grid shared by the batch;
//   * coefficients: one coefficient-major table of float4 groups
//     ctab4[q*nbins + bin] = (c_4q .. c_4q+3) of velocity bin `bin`,
//     zero-padded to the compile-time operator length MMAX, so every cell runs
//     the same unrolled loop (adding 0*x leaves a sum unchanged) and gathers
//     its M+1 coefficients with ceil((MMAX+1)/4) 16-byte loads;
//   * boundary rings: [shot][NT][ring] with ring = 2M(nx+nz) cells
//     (top band M*nx, bottom band M*nx, left band M*nz, right band M*nz).
//
// One time step of a batch is two launches:
//   k_step  : the 2M-order update of every cell of a 128 x 16 tile.  Every
//             input is staged in shared memory by TMA (a halo box for the
//             field being advanced, flat tiles for u_{k-2}, v and the imaging
//             accumulators); each lane owns one column, streams z-neighbours
//             through a register queue and reads x-neighbours as
//             conflict-free 32-bit shared loads.  Pad cells write their
//             pre-blend value to `pre`, interior cells write the result.  The
//             forward variant computes two rows per loop step; the backward
//             variant advances the reconstructed source field and the
//             receiver field in lockstep (one coefficient gather per cell
//             serves both) and updates the imaging accumulators of every
//             interior cell in the same pass.
//   k_pad   : one-way update + blend of every pad cell (reading pre-blend
//             values from `pre`), ring save (forward) or ring restore of the
//             source field (backward), receiver recording (forward).
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "rtm_common.cuh"

// Device-side error word of the engine (zero = fine); read and cleared by
// rtm_device_error().  This header is included by one translation unit only.
__device__ unsigned int g_rtm_dev_error = 0;

namespace eng {

constexpr int WX = 4;               // warps across a tile (one column per lane)
constexpr int WZ = 2;               // warps down a tile
constexpr int RW = 8;               // rows streamed by one warp
constexpr int TX = WX * 32;         // tile width (128 columns)
constexpr int TZ = WZ * RW;         // tile height (16 rows)
constexpr int NTHREADS = WX * WZ * 32;
constexpr int FLAT = TX * TZ;       // floats of one flat (halo-free) tile
constexpr unsigned FLAT_BYTES = FLAT * 4u;

template <int MMAX>
struct Shape {
    static constexpr int XH = (MMAX + 3) / 4 * 4;  // x halo (16-byte aligned)
    static constexpr int ZH = MMAX;                // z halo
    static constexpr int BW = TX + 2 * XH;         // box width (floats)
    static constexpr int BH = TZ + 2 * ZH;         // box height (rows)
    static constexpr int ELEMS = BW * BH;
    static constexpr unsigned BYTES = ELEMS * 4u;
};

// Step kinds of k_step: the forward and backward steps of the ring scheme,
// and the two steps of a migration with source snapshots: a forward step that
// also accumulates the source field's running sum, and a backward step that
// advances the receiver field alone (with its running sum; the imaging at the
// snapshot steps is a separate streaming kernel, k_snap_image).
enum { MODE_FWD = 0, MODE_BWD = 1, MODE_FWDS = 2, MODE_BWDS = 3 };
__host__ __device__ constexpr bool fwd_mode(int m) { return m == MODE_FWD || m == MODE_FWDS; }

// Shared-memory plan of k_step: halo boxes of the field(s) being advanced,
// then flat tiles (u_{k-2} of each field, the per-cell factor v^2 tao^2/h^2,
// the four imaging accumulators in the backward step, the per-cell velocity
// bin), then the mbarrier.
template <int MMAX, int MODE>
struct Smem {
    static constexpr int NBOX = MODE == MODE_BWD ? 2 : 1;
    // fwd: a0, vv, bin; bwd: a0, s0, vv, rel1, rel2, sacc, racc, bin (the bin
    // tile is staged only with adaptive coefficients); the snapshot steps:
    // a0, vv, the running sum (source field forward, receiver field
    // backward), bin
    static constexpr int NFLAT = MODE == MODE_BWD ? 8 : (MODE == MODE_FWDS || MODE == MODE_BWDS) ? 4 : 3;
    static constexpr unsigned BYTES = NBOX * Shape<MMAX>::BYTES + NFLAT * FLAT_BYTES + 16u;
};

struct ImgMaps {
    CUtensorMap rel1, rel2, sacc, racc;
};

// Per-cell model factors staged by the stencil kernels: vv = v^2 tao^2 / h^2
// (float, kernel.cu's v*v*tao2*h2) and the bin word (int); one grid shared by
// the batch or one per shot (vv, bin), and, for shots with their own
// windows, the survey's grid as well (svv, sbin).
struct ModelMaps {
    CUtensorMap vv, bin, svv, sbin;
};

// Flat tiles of the running sum of a migration with source snapshots (the
// source field's in the forward run, the receiver field's in the backward
// run; the [shot][NZ][P] layout of a field).
struct SnapMaps {
    CUtensorMap sum;
};

struct StepArgs {
    int NZ, NX, P, N2, nbins;
    long long ss;              // floats between consecutive shots
    float vmin, dv, tao2, h2, k0, hzx2_1;
    const float *v;            // [NZ][P]
    const float *ctab;         // fixed coefficients c[0..MMAX] (nbins == 1)
    const float4 *ctab4;       // [ceil((MMAX+1)/4)][nbins] coefficient groups (adaptive)
    const float *a0;           // field A (u forward / R backward), level k-2
    float *a2;                 // field A output (interior cells)
    float *pre;                // pre-blend values of pad cells
    const float *s0;           // backward source field, level k+2
    float *s2;                 // backward source field output (interior)
    float *rel1, *rel2, *sacc, *racc;
    int compen;
    const int *src;            // [B] flat z*NX + x
    float wavelet;
    int src_on_a;              // forward: source goes into field A
    // receiver line (Dirichlet injection into field A, backward)
    int rz0, rx0, rdz, rdx, nrec;
    const float *dinj;         // data row for this step, shot 0; shot s at + s*dstride
    long long dstride;
    // per-shot geometry: padded width and receiver start column of each
    // shot's grid; vshot = 1 when every shot has its own model copy
    const int *nxs, *rx0s;
    int vshot;
    int shot0;                 // first shot of this launch (blockIdx.z + shot0)
    // the per-cell bins in global memory (the array the bin tiles are staged
    // from; shot stride gbin_ss, 0 for the shared model): the first rows'
    // coefficients are gathered from it before the tile's copies land
    const int *gbin;
    long long gbin_ss;
    // shots with their own windows: window origin (interior column of the
    // survey) of each shot, and the survey's bins (same pitch P)
    const int *xas;
    const int *gsbin;
    // narrowest padded width among the launch's shots: tiles starting left
    // of it exist in every shot, so they issue their wavefield copies before
    // reading the shot's own width and origin
    int min_nx;
    // snapshot steps (MODE_FWDS / MODE_BWDS): the running sum the step adds
    // its field's interior to (the source field's forward, the receiver
    // field's backward with compensated imaging)
    float *pacc;
};

// Whether a tile of a windowed shot reads its model tiles from the survey's
// grid: its columns lie inside the window's interior, where the window's
// model equals the survey's shifted by the window origin xa (only the
// window's own pad band is an edge extension of its own), and xa keeps the
// survey coordinate x0 + xa a multiple of 4 floats (16 bytes, as TMA needs).
// The survey grid is shared by every shot of the batch, so L2 serves it.
__device__ __forceinline__ bool tile_on_survey(const StepArgs &a, int x0, int NX, int xa)
{
    return a.vshot && (xa & 3) == 0 && x0 >= a.N2 && x0 + TX <= NX - a.N2;
}

__device__ __forceinline__ int mirror_i(int i, int n)
{
    return i < 0 ? -i : (i >= n ? 2 * n - 2 - i : i);
}

// Mirror the out-of-grid halo of a staged box (the reference reflects
// neighbour indices at the array edges, kernel.cu:65-68).  Only the tile's
// own rows need x-halo values and only its own columns need z-halo values.
template <int MMAX, int NT = NTHREADS>
__device__ __forceinline__ void patch_halo(float *t, int x0, int z0, int NX, int NZ)
{
    using S = Shape<MMAX>;
    const int gx0 = x0 - S::XH, gz0 = z0 - S::ZH;
    // x reflection on the tile's in-grid rows, z reflection on its in-grid
    // columns: the written and the read cells of the two passes never overlap.
    if (x0 == 0 || x0 + TX + S::XH > NX) {  // the conditions of tile_at_edge
        for (int idx = threadIdx.x; idx < TZ * S::BW; idx += NT) {
            const int r = S::ZH + idx / S::BW, c = idx % S::BW;
            const int gx = gx0 + c, gz = gz0 + r;
            if ((gx >= 0 && gx < NX) || gz >= NZ) continue;
            const int sc = mirror_i(gx, NX) - gx0;
            t[r * S::BW + c] = (sc >= 0 && sc < S::BW) ? t[r * S::BW + sc] : 0.0f;
        }
    }
    if (z0 == 0 || z0 + TZ + S::ZH > NZ) {
        for (int idx = threadIdx.x; idx < S::BH * TX; idx += NT) {
            const int r = idx / TX, c = S::XH + idx % TX;
            const int gz = gz0 + r, gx = gx0 + c;
            if ((gz >= 0 && gz < NZ) || gx >= NX) continue;
            const int sr = mirror_i(gz, NZ) - gz0;
            t[r * S::BW + c] = (sr >= 0 && sr < S::BH) ? t[sr * S::BW + c] : 0.0f;
        }
    }
}

// Whether a tile's halo box reaches past the grid (patch_halo has work).
template <int MMAX>
__device__ __forceinline__ bool tile_at_edge(int x0, int z0, int NX, int NZ)
{
    using S = Shape<MMAX>;
    return x0 == 0 || x0 + TX + S::XH > NX || z0 == 0 || z0 + TZ + S::ZH > NZ;
}

// Layout of the adaptive table: coefficient-major (float4 group q of bin b
// at q*nbins + b) or bin-major (at b*QP + q, QP = groups rounded up to a
// power of two, so one bin's coefficients fill one aligned 32/64-byte block).
#ifndef RTM_TAB_BINMAJOR
#define RTM_TAB_BINMAJOR 0
#endif
__host__ __device__ constexpr int tab_groups(int mmax) { return (mmax + 4) / 4; }
__host__ __device__ constexpr int tab_pitch(int mmax) { return tab_groups(mmax) == 3 ? 4 : tab_groups(mmax); }
__host__ __device__ __forceinline__ int tab_index(int q, int bin, int nbins, int mmax)
{
    return RTM_TAB_BINMAJOR ? bin * tab_pitch(mmax) + q : q * nbins + bin;
}

// Per-cell bin words: the velocity bin in the low 24 bits and the bin's
// operator length above them (k_model_prep packs them), so a cell learns both
// from one staged int.
constexpr int BIN_BITS = 24;
__device__ __forceinline__ int word_bin(int bw) { return bw & ((1 << BIN_BITS) - 1); }
__device__ __forceinline__ int word_len(int bw) { return (int)((unsigned)bw >> BIN_BITS); }

// Coefficients of one cell: the velocity bin (adaptive; precomputed per cell
// as kernel.cu:55-57 forms it) picks a column of the coefficient-major table;
// only the groups holding c_0..c_len of the cell's own operator length are
// gathered and the others are zero (as the table holds them); with fixed
// coefficients the values are loaded once into registers (cc).  Returns the
// cell's operator length (MMAX with fixed coefficients).
template <int MMAX, bool ADAPT>
__device__ __forceinline__ int load_coefs(const StepArgs &a, int bw, const float *cc, float *cf)
{
    if (!ADAPT) {
#pragma unroll
        for (int l = 0; l <= MMAX; ++l) cf[l] = cc[l];
        return MMAX;
    }
    constexpr int Q = (MMAX + 4) / 4;
    const int bin = word_bin(bw), len = word_len(bw);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const float4 g = (4 * q <= len) ? __ldg(a.ctab4 + tab_index(q, bin, a.nbins, MMAX))
                                        : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (4 * q + 0 <= MMAX) cf[4 * q + 0] = g.x;
        if (4 * q + 1 <= MMAX) cf[4 * q + 1] = g.y;
        if (4 * q + 2 <= MMAX) cf[4 * q + 2] = g.z;
        if (4 * q + 3 <= MMAX) cf[4 * q + 3] = g.w;
    }
    return len;
}

// Longest operator among the warp's cells of one row: terms beyond it have
// zero coefficients for every lane, and adding 0*x leaves a sum unchanged,
// so the stencil loops stop there (the bits of the result do not change).
template <int MMAX, bool ADAPT>
__device__ __forceinline__ int warp_len(int len)
{
    return ADAPT ? min(__reduce_max_sync(0xffffffffu, (unsigned)len), (unsigned)MMAX) : MMAX;
}

// Spatial operator of one cell: w = k0*c0*u + sum_l c_l*((u[z-l]+u[z+l])*hzx2_1
// + u[x-l] + u[x+l]) (kernel.cu:59-72), with q the column's register queue
// (centre at index C) and row the cell's row in the staged halo box.
template <int MMAX, bool ADAPT>
__device__ __forceinline__ float lap_cell(const float *q, int C, const float *row, const float *cf,
                                          float k0, float hzx2_1, int L)
{
    float w1 = k0 * cf[0] * q[C];
#pragma unroll
    for (int l = 1; l <= MMAX; ++l) {
        if (l > L) break;
        const float xs = (q[C - l] + q[C + l]) * hzx2_1 + row[-l];
        w1 = fmaf(cf[l], xs + row[l], w1);
    }
    return w1;
}

__host__ __device__ __forceinline__ float ring16_target(int prec) { return prec == 3 ? 32767.0f : 16384.0f; }

// 16-bit ring codes: 1 BF16, 2 FP16 (floating point: relative rounding
// 2^-9 / 2^-12 of each value), 3 int16 (a fixed-point fraction of the step's
// largest value: absolute rounding of half of max/32767 for every value,
// 16 times finer than FP16 at the largest values that dominate the field).
__device__ __forceinline__ uint16_t ring_quant(float v, float inv, int prec)
{
    if (prec == 1) return __bfloat16_as_ushort(__float2bfloat16_rn(v * inv));
    if (prec == 3) {
        const int q = __float2int_rn(v * inv);  // |v| <= the step's max, so |q| <= 32767
        return (uint16_t)(short)max(-32767, min(32767, q));
    }
    return __half_as_ushort(__float2half_rn(v * inv));
}

__device__ __forceinline__ float ring_dequant(uint16_t q, float sc, int prec)
{
    float f;
    if (prec == 1) f = __bfloat162float(__ushort_as_bfloat16(q));
    else if (prec == 3) f = (float)(short)q;
    else f = __half2float(__ushort_as_half(q));
    return f * sc;
}

// Shared-memory pointers of one pipeline stage (one tile's staged inputs).
template <int MMAX, int MODE>
struct Stage {
    float *tA, *tS, *fA0, *fV, *fS0, *fR1, *fR2, *fSa, *fRa;
    int *fB;
    // snapshot steps: the running sum (in the slot of fS0)
    float *fP;
    __device__ __forceinline__ explicit Stage(float *base)
    {
        using S = Shape<MMAX>;
        tA = base;
        tS = base + S::ELEMS;  // backward only
        float *fl = base + Smem<MMAX, MODE>::NBOX * S::ELEMS;
        fA0 = fl; fV = fl + FLAT;
        fS0 = fl + 2 * FLAT; fR1 = fl + 3 * FLAT; fR2 = fl + 4 * FLAT;
        fSa = fl + 5 * FLAT; fRa = fl + 6 * FLAT;
        fP = fl + 2 * FLAT;
        fB = reinterpret_cast<int *>(fl + (Smem<MMAX, MODE>::NFLAT - 1) * FLAT);
    }
};

// Stage bytes without the barrier word(s), and the bytes its copies bring
// (no bin tile with fixed coefficients).
template <int MMAX, int MODE>
__host__ __device__ constexpr unsigned stage_bytes() { return Smem<MMAX, MODE>::BYTES - 16u; }
template <int MMAX, int MODE, bool ADAPT>
__host__ __device__ constexpr unsigned stage_tx_bytes()
{
    return stage_bytes<MMAX, MODE>() - (ADAPT ? 0u : FLAT_BYTES);
}

// TMA loads of one tile's inputs into a stage, completing on `bar`
// (issued by one thread).
// Backward tiles without interior rows (the top and bottom pad bands) never
// touch the source field or the imaging accumulators: those copies are
// skipped.
__device__ __forceinline__ bool tile_has_interior_rows(int z0, int NZ, int N2)
{
    return z0 + TZ > N2 && z0 < NZ - N2;
}

// The copies of a tile except its model tiles (one arrive on `bar` with the
// byte count of all of them, model tiles included).
template <int MMAX, int MODE, bool ADAPT>
__device__ __forceinline__ void issue_fields(const Stage<MMAX, MODE> &st, uint64_t *bar,
                                             const CUtensorMap &mapA, const CUtensorMap &mapS,
                                             const CUtensorMap &flatA0, const CUtensorMap &flatS0,
                                             const ImgMaps &img, int x0, int z0, int shot, bool with_s,
                                             const SnapMaps *snap = nullptr, const StepArgs *sa = nullptr)
{
    using S = Shape<MMAX>;
    if (MODE == MODE_FWDS || MODE == MODE_BWDS) {
        // snapshot steps: the running sum's tile where the step adds to it
        // (every forward tile; backward, tiles with interior rows when the
        // imaging is compensated)
        const bool sum = MODE == MODE_FWDS || (with_s && sa->compen);
        mbar_arrive_expect_tx(bar, S::BYTES + (sum ? 3u : 2u) * FLAT_BYTES + (ADAPT ? FLAT_BYTES : 0u));
        tma_load_3d(st.tA, &mapA, x0 - S::XH, z0 - S::ZH, shot, bar);
        tma_load_3d(st.fA0, &flatA0, x0, z0, shot, bar);
        if (sum) tma_load_3d(st.fP, &snap->sum, x0, z0, shot, bar);
        return;
    }
    const unsigned skip = (MODE == MODE_BWD && !with_s) ? S::BYTES + 5u * FLAT_BYTES : 0u;
    mbar_arrive_expect_tx(bar, stage_tx_bytes<MMAX, MODE, ADAPT>() - skip);
    tma_load_3d(st.tA, &mapA, x0 - S::XH, z0 - S::ZH, shot, bar);
    tma_load_3d(st.fA0, &flatA0, x0, z0, shot, bar);
    if (MODE == MODE_BWD && with_s) {
        tma_load_3d(st.tS, &mapS, x0 - S::XH, z0 - S::ZH, shot, bar);
        tma_load_3d(st.fS0, &flatS0, x0, z0, shot, bar);
        tma_load_3d(st.fR1, &img.rel1, x0, z0, shot, bar);
        tma_load_3d(st.fR2, &img.rel2, x0, z0, shot, bar);
        tma_load_3d(st.fSa, &img.sacc, x0, z0, shot, bar);
        tma_load_3d(st.fRa, &img.racc, x0, z0, shot, bar);
    }
}

// The model tiles of a tile (vv and, adaptive, the bin words): from the
// survey grid (surv), the shot's own window copy, or the shared grid.
template <int MMAX, int MODE, bool ADAPT>
__device__ __forceinline__ void issue_model(const Stage<MMAX, MODE> &st, uint64_t *bar, const ModelMaps &mod,
                                            int x0, int z0, int shot, int vshot, bool surv, int xa)
{
    if (surv) {
        tma_load_3d(st.fV, &mod.svv, x0 + xa, z0, 0, bar);
        if (ADAPT) tma_load_3d(st.fB, &mod.sbin, x0 + xa, z0, 0, bar);
    } else {
        tma_load_3d(st.fV, &mod.vv, x0, z0, vshot ? shot : 0, bar);
        if (ADAPT) tma_load_3d(st.fB, &mod.bin, x0, z0, vshot ? shot : 0, bar);
    }
}

template <int MMAX, int MODE, bool ADAPT>
__device__ __forceinline__ void issue_tile(const Stage<MMAX, MODE> &st, uint64_t *bar,
                                           const CUtensorMap &mapA, const CUtensorMap &mapS,
                                           const CUtensorMap &flatA0, const CUtensorMap &flatS0,
                                           const ModelMaps &mod, const ImgMaps &img, int x0,
                                           int z0, int shot, int vshot, bool with_s, bool surv = false,
                                           int xa = 0)
{
    issue_fields<MMAX, MODE, ADAPT>(st, bar, mapA, mapS, flatA0, flatS0, img, x0, z0, shot, with_s);
    issue_model<MMAX, MODE, ADAPT>(st, bar, mod, x0, z0, shot, vshot, surv, xa);
}

// The update of one staged 128 x 16 tile (after its copies landed and the
// out-of-grid halo was mirrored): the warp's lanes each own one column and
// stream its rows through register queues; outputs are stored directly.
// Coefficients are gathered PF rows ahead of their use (adaptive mode): a
// gather depends on the staged velocity and usually misses L1, so issuing it
// early hides its latency behind the rows in between.
// Coefficients of the warp's first PRE rows, gathered by each lane from the
// global bins before the tile's copies have landed (their latency then
// overlaps the copies instead of stalling the first rows).
template <int MMAX, bool ADAPT, int PRE>
__device__ __forceinline__ void pre_gather(const StepArgs &a, const float *cc, int x0, int z0, int shot,
                                           int NX, float (&cf)[PRE > 0 ? PRE : 1][MMAX + 1],
                                           int (&len)[PRE > 0 ? PRE : 1], bool surv, int xa)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int zw = z0 + (warp / WX) * RW, gx = x0 + (warp % WX) * 32 + lane;
    const int *gb = surv ? a.gsbin + xa : (a.gbin ? a.gbin + shot * a.gbin_ss : nullptr);
#pragma unroll
    for (int r = 0; r < PRE; ++r) {
        int b = 0;
        if (ADAPT && gb && zw + r < a.NZ && gx < NX) b = __ldg(gb + (long)(zw + r) * a.P + gx);
        len[r] = load_coefs<MMAX, ADAPT>(a, b, cc, cf[r]);
    }
}

// Receiver injection of the backward steps: a receiver cell of the line
// takes the step's recorded value where that is non-zero (kernel.cu's
// Dirichlet injection of the observed data).
__device__ __forceinline__ float inject_line(const StepArgs &a, float rv, int z, int gx, int rx0, int shot)
{
    int j = -1;
    if (a.rdz == 0) {
        if (z == a.rz0 && (gx - rx0) % a.rdx == 0) j = (gx - rx0) / a.rdx;
    } else if (a.rdx == 0) {
        if (gx == rx0 && (z - a.rz0) % a.rdz == 0) j = (z - a.rz0) / a.rdz;
    } else if ((gx - rx0) % a.rdx == 0) {
        const int jj = (gx - rx0) / a.rdx;
        if (z == a.rz0 + jj * a.rdz) j = jj;
    }
    if (j >= 0 && j < a.nrec) {
        const float d = a.dinj[(long long)shot * a.dstride + j];
        if (d != 0.0f) rv = d;
    }
    return rv;
}

template <int MMAX, bool ADAPT, int MODE, int PF, int PRE>
__device__ __forceinline__ void compute_tile(const StepArgs &a, const Stage<MMAX, MODE> &st,
                                             const float *cc, int x0, int z0, int shot, int NX,
                                             const float (&cpre)[PRE > 0 ? PRE : 1][MMAX + 1],
                                             const int (&lpre)[PRE > 0 ? PRE : 1], int src, int rx0)
{
    using S = Shape<MMAX>;
    constexpr int QN = 2 * MMAX + 1;
    const float *tA = st.tA, *tS = st.tS, *fA0 = st.fA0, *fV = st.fV, *fS0 = st.fS0;
    const int *fB = st.fB;
    const float *fR1 = st.fR1, *fR2 = st.fR2, *fSa = st.fSa, *fRa = st.fRa;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int wx = warp % WX, wz = warp / WX;
    const long long so = (long long)shot * a.ss;
    const int zw = z0 + wz * RW;             // first row of this warp
    const int gx = x0 + wx * 32 + lane;      // this lane's column
    const int cx = S::XH + wx * 32 + lane;   // its column in the halo box
    const int rbase = wz * RW;               // box row of zw - MMAX
    const int fr = wz * RW * TX + wx * 32 + lane;  // flat-tile index of row zw
    // source row of this lane's column relative to the warp's first row (-1:
    // the source is not in this column)
    const int src_row = (src % NX == x0 + wx * 32 + lane) ? src / NX - (z0 + wz * RW) : -1;
    const int N2 = a.N2, NZ = a.NZ;
    const bool col_in = gx >= N2 && gx < NX - N2;
    const bool col_ok = gx < NX;
    const long long g0 = so + (long)zw * a.P + gx;  // global index of row zw
    // every cell of the warp's rows and columns is interior and off the
    // first interior ring: no pad stores, no per-cell predicates
    const int xw = x0 + (warp % WX) * 32;
    const bool inner = zw > N2 && zw + RW < NZ - N2 - 1 && xw > N2 && xw + 32 < NX - N2 - 1;

    // Coefficients are gathered PF rows ahead of their use (adaptive mode):
    // a gather depends on the staged velocity and usually misses L1, so
    // issuing it early hides its latency behind the rows in between.
    float cfr[RW][MMAX + 1];
    int lr[RW];  // operator length of the lane's cell in each row
#pragma unroll
    for (int i = 0; i < PRE; ++i) {
        lr[i] = lpre[i];
#pragma unroll
        for (int l = 0; l <= MMAX; ++l) cfr[i][l] = cpre[i][l];
    }
#pragma unroll
    for (int i = PRE; i < PF; ++i) lr[i] = load_coefs<MMAX, ADAPT>(a, ADAPT ? fB[fr + i * TX] : 0, cc, cfr[i]);

    bool line_hit = false;
    if (!fwd_mode(MODE) && a.nrec > 0) {
        const int zb = a.rz0 + (a.nrec - 1) * a.rdz, xb = rx0 + (a.nrec - 1) * a.rdx;
        const int zlo = min(a.rz0, zb), zhi = max(a.rz0, zb), xlo = min(rx0, xb), xhi = max(rx0, xb);
        line_hit = !(zhi < zw || zlo >= zw + RW || xhi < x0 + wx * 32 || xlo >= x0 + wx * 32 + 32);
    }
    if (fwd_mode(MODE) || MODE == MODE_BWDS) {
        // One field (forward: the source field; backward with snapshots: the
        // receiver field, injected at the receivers), two rows per iteration:
        // two independent accumulation chains.  The snapshot steps also add
        // the field's interior to its running sum.
        const bool sum = MODE == MODE_FWDS || (MODE == MODE_BWDS && a.compen);
        float q[QN + 1];
#pragma unroll
        for (int j = 0; j < QN - 1; ++j) q[j] = tA[(rbase + j) * S::BW + cx];
#pragma unroll
        for (int i = 0; i < RW; i += 2) {
#pragma unroll
            for (int h = 0; h < 2; ++h)
                if (i + h + PF < RW && i + h + PF >= PRE)
                    lr[i + h + PF] =
                        load_coefs<MMAX, ADAPT>(a, ADAPT ? fB[fr + (i + h + PF) * TX] : 0, cc, cfr[i + h + PF]);
            q[QN - 1] = tA[(rbase + i + QN - 1) * S::BW + cx];
            q[QN] = tA[(rbase + i + QN) * S::BW + cx];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int z = zw + i + h;
                if (z >= NZ) continue;
                const int t = fr + (i + h) * TX;
                const float *cf = cfr[i + h];
                const float *row = tA + (rbase + i + h + MMAX) * S::BW + cx;
                const int L = warp_len<MMAX, ADAPT>(lr[i + h]);
                const float w1 = lap_cell<MMAX, ADAPT>(q, MMAX + h, row, cf, a.k0, a.hzx2_1, L);
                float val = fmaf(fV[t], w1, 2.0f * q[MMAX + h] - fA0[t]);
                if (fwd_mode(MODE)) {
                    if (i + h == src_row) val += a.wavelet;
                } else if (line_hit) {
                    val = inject_line(a, val, z, gx, rx0, shot);
                }
                const long long g = g0 + (long)(i + h) * a.P;
                if (inner) {
                    a.a2[g] = val;
                    if (sum) a.pacc[g] = st.fP[t] + val;
                } else if (col_ok) {
                    const bool interior = col_in && z >= N2 && z < NZ - N2;
                    if (interior) a.a2[g] = val;
                    if (sum && interior) a.pacc[g] = st.fP[t] + val;
                    if (!interior || gx == N2 || gx == NX - 1 - N2 || z == N2 || z == NZ - 1 - N2)
                        a.pre[g] = val;
                }
            }
#pragma unroll
            for (int j = 0; j < QN - 1; ++j) q[j] = q[j + 2];
        }
        return;
    }

    // Backward: receiver field R on every cell, reconstructed source field S
    // on the interior, advanced in lockstep so both share the coefficients and
    // the imaging condition sees both at once.
    const bool rows_s = (zw + RW > N2) && (zw < NZ - N2);
    float qr[QN], qs[QN];
#pragma unroll
    for (int j = 0; j < QN - 1; ++j) {
        qr[j] = tA[(rbase + j) * S::BW + cx];
        qs[j] = rows_s ? tS[(rbase + j) * S::BW + cx] : 0.0f;
    }
#pragma unroll
    for (int i = 0; i < RW; ++i) {
        if (i + PF < RW && i + PF >= PRE)
            lr[i + PF] = load_coefs<MMAX, ADAPT>(a, ADAPT ? fB[fr + (i + PF) * TX] : 0, cc, cfr[i + PF]);
        qr[QN - 1] = tA[(rbase + i + QN - 1) * S::BW + cx];
        if (rows_s) qs[QN - 1] = tS[(rbase + i + QN - 1) * S::BW + cx];
        const int z = zw + i;
        if (z < NZ) {
            const int t = fr + i * TX;
            const float vv = fV[t];
            const float *cf = cfr[i];
            const float *rowR = tA + (rbase + i + MMAX) * S::BW + cx;
            const float *rowS = tS + (rbase + i + MMAX) * S::BW + cx;
            const float c0 = cf[0];
            float wr = a.k0 * c0 * qr[MMAX];
            float ws = a.k0 * c0 * qs[MMAX];
            const int L = warp_len<MMAX, ADAPT>(lr[i]);
#pragma unroll
            for (int l = 1; l <= MMAX; ++l) {
                if (l > L) break;
                const float cl = cf[l];
                wr = fmaf(cl, (qr[MMAX - l] + qr[MMAX + l]) * a.hzx2_1 + rowR[-l] + rowR[l], wr);
                if (rows_s)
                    ws = fmaf(cl, (qs[MMAX - l] + qs[MMAX + l]) * a.hzx2_1 + rowS[-l] + rowS[l], ws);
            }
            float rv = fmaf(vv, wr, 2.0f * qr[MMAX] - fA0[t]);
            if (line_hit) rv = inject_line(a, rv, z, gx, rx0, shot);
            const bool interior = inner || (col_in && z >= N2 && z < NZ - N2);
            const long long g = g0 + (long)i * a.P;
            if (inner) {
                a.a2[g] = rv;
            } else if (col_ok) {
                if (interior) a.a2[g] = rv;
                if (!interior || gx == N2 || gx == NX - 1 - N2 || z == N2 || z == NZ - 1 - N2)
                    a.pre[g] = rv;
            }
            if (interior) {
                float sv = fmaf(vv, ws, 2.0f * qs[MMAX] - fS0[t]);
                if (i == src_row) sv += a.wavelet;
                a.s2[g] = sv;
                // imaging (kernel.cu:489-517)
                if (a.compen) {
                    const float sa = fSa[t] + sv;
                    const float ra = fRa[t] + rv;
                    a.sacc[g] = sa;
                    a.racc[g] = ra;
                    a.rel1[g] = fR1[t] + ra * sa;
                } else {
                    a.rel1[g] = fR1[t] + rv * sv;
                }
                a.rel2[g] = fR2[t] + sv * sv;
            }
        }
#pragma unroll
        for (int j = 0; j < QN - 1; ++j) {
            qr[j] = qr[j + 1];
            qs[j] = qs[j + 1];
        }
    }
}

#ifndef RTM_FWD_MINB
#define RTM_FWD_MINB 4
#endif
#ifndef RTM_FWD_PF
#define RTM_FWD_PF 0
#endif
#ifndef RTM_BWD_PF
#define RTM_BWD_PF 2
#endif
#ifndef RTM_BWD_PRE
#define RTM_BWD_PRE 6   // rows whose coefficients are gathered before the tile lands
#endif
#ifndef RTM_FWD_PRE
#define RTM_FWD_PRE 2
#endif
#ifndef RTM_PIPE_FWD_PF
#define RTM_PIPE_FWD_PF 2
#endif

// One time step of a batch of shots, one CTA per 128 x 16 tile (grid: tiles
// x tiles x shots).  All inputs arrive by TMA into shared memory under one
// mbarrier.
template <int MMAX, bool ADAPT, int MODE>
__global__ void __launch_bounds__(NTHREADS, MODE == MODE_BWD || MMAX > 8 ? 2 : RTM_FWD_MINB)
    k_step(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapS,
           const __grid_constant__ CUtensorMap flatA0, const __grid_constant__ CUtensorMap flatS0,
           const __grid_constant__ ModelMaps mod, const __grid_constant__ ImgMaps img,
           const __grid_constant__ SnapMaps snap, const StepArgs a)
{
    using SM = Smem<MMAX, MODE>;
    constexpr int PF = MODE != MODE_BWD ? RTM_FWD_PF : (MMAX <= 8 ? RTM_BWD_PF : 2);  // register budget
    extern __shared__ __align__(128) float smem[];
    const Stage<MMAX, MODE> st(smem);
    uint64_t &bar = *reinterpret_cast<uint64_t *>(reinterpret_cast<char *>(smem) + stage_bytes<MMAX, MODE>());
    const int x0 = blockIdx.x * TX, z0 = blockIdx.y * TZ, shot = blockIdx.z + a.shot0;
    const bool with_s = tile_has_interior_rows(z0, a.NZ, a.N2);
    // a tile every shot of the launch has issues its wavefield copies before
    // anything else; the shot's width and window origin (loads only when
    // shots have their own windows) arrive while those copies fly
    const bool early = x0 < a.min_nx;
    if (early && threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_barrier_init();
        issue_fields<MMAX, MODE, ADAPT>(st, &bar, mapA, mapS, flatA0, flatS0, img, x0, z0, shot, with_s, &snap, &a);
    }
    const int NX = a.vshot ? a.nxs[shot] : a.NX;
    const int xa = a.vshot ? a.xas[shot] : 0;
    if (x0 >= NX) return;  // tile beyond this shot's (narrower) grid (never an early tile)
    const bool surv = tile_on_survey(a, x0, NX, xa);
    if (threadIdx.x == 0) {
        if (!early) {
            mbar_init(&bar, 1);
            fence_barrier_init();
            issue_fields<MMAX, MODE, ADAPT>(st, &bar, mapA, mapS, flatA0, flatS0, img, x0, z0, shot, with_s, &snap, &a);
        }
        issue_model<MMAX, MODE, ADAPT>(st, &bar, mod, x0, z0, shot, a.vshot, surv, xa);
    }
    // fixed coefficients: once per thread, while the copies are in flight;
    // the first rows' adaptive coefficients likewise (issued by every thread
    // while thread 0 is still issuing the copies)
    float cc[MMAX + 1];
#pragma unroll
    for (int l = 0; l <= MMAX; ++l) cc[l] = ADAPT ? 0.0f : __ldg(a.ctab + l);
    // (the 12-wide backward gathers two rows early: six rows of 13
    // coefficients would not fit its registers)
    constexpr int PRE = !ADAPT ? 0 : (MODE == MODE_BWD ? (MMAX <= 8 ? RTM_BWD_PRE : 2) : RTM_FWD_PRE);
    float cpre[PRE > 0 ? PRE : 1][MMAX + 1];
    int lpre[PRE > 0 ? PRE : 1];
    pre_gather<MMAX, ADAPT, PRE>(a, cc, x0, z0, shot, NX, cpre, lpre, surv, xa);
    const int src = __ldg(a.src + shot), rx0 = !fwd_mode(MODE) ? __ldg(a.rx0s + shot) : 0;
    __syncthreads();  // the barrier is initialised before any thread waits on it
    const bool ok = mbar_wait_bounded(&bar, 0, &g_rtm_dev_error);
    if (tile_at_edge<MMAX>(x0, z0, NX, a.NZ)) {
        // out-of-grid halo mirrored by all threads before any reads it
        if (ok) {
            patch_halo<MMAX>(st.tA, x0, z0, NX, a.NZ);
            if (MODE == MODE_BWD && with_s) patch_halo<MMAX>(st.tS, x0, z0, NX, a.NZ);
        }
        if (!__syncthreads_and(ok)) {
            mbar_wait_bounded(&bar, 0, &g_rtm_dev_error);  // let an in-flight copy land before exit
            return;
        }
    } else if (!ok) {
        // no halo to mirror: every warp starts as soon as its own wait is over
        mbar_wait_bounded(&bar, 0, &g_rtm_dev_error);
        return;
    }
    compute_tile<MMAX, ADAPT, MODE, PF, PRE>(a, st, cc, x0, z0, shot, NX, cpre, lpre, src, rx0);
}

// Forward step with two columns per lane (kernel form RTM_KERNEL_X2): the
// same 128 x 16 tile and staging as k_step with 4 warps (2 across, 2 down);
// each lane owns two adjacent columns, reads their z-queue entries and their
// 2M+2 x-neighbours as 8-byte shared loads, and computes both cells with
// k_step's operation order (bit-identical results).
constexpr int X2_THREADS = 128;

template <int MMAX, bool ADAPT>
__device__ __forceinline__ float lap_regs(const float *q, int C, const float *xv, int o, const float *cf,
                                          float k0, float hzx2_1, int L)
{
    // xv[o + j] is the row's value at column (cell - MMAX + j)
    float w1 = k0 * cf[0] * q[C];
#pragma unroll
    for (int l = 1; l <= MMAX; ++l) {
        if (l > L) break;
        const float xs = (q[C - l] + q[C + l]) * hzx2_1 + xv[o + MMAX - l];
        w1 = fmaf(cf[l], xs + xv[o + MMAX + l], w1);
    }
    return w1;
}

#ifndef RTM_X2_MINB
#define RTM_X2_MINB 4
#endif

template <int MMAX, bool ADAPT>
__global__ void __launch_bounds__(X2_THREADS, RTM_X2_MINB)
    k_step_x2(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapS,
              const __grid_constant__ CUtensorMap flatA0, const __grid_constant__ CUtensorMap flatS0,
              const __grid_constant__ ModelMaps mod, const __grid_constant__ ImgMaps img, const StepArgs a)
{
    using S = Shape<MMAX>;
    constexpr int QN = 2 * MMAX + 1;
    constexpr int NXV = 2 * MMAX + 2;  // x values covering both columns' stencils
    extern __shared__ __align__(128) float smem[];
    const Stage<MMAX, MODE_FWD> st(smem);
    uint64_t &bar = *reinterpret_cast<uint64_t *>(reinterpret_cast<char *>(smem) + stage_bytes<MMAX, MODE_FWD>());
    const int x0 = blockIdx.x * TX, z0 = blockIdx.y * TZ, shot = blockIdx.z + a.shot0;
    const bool early = x0 < a.min_nx;  // as in k_step
    if (early && threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_barrier_init();
        issue_fields<MMAX, MODE_FWD, ADAPT>(st, &bar, mapA, mapS, flatA0, flatS0, img, x0, z0, shot, false);
    }
    const int NX = a.vshot ? a.nxs[shot] : a.NX;
    const int xa = a.vshot ? a.xas[shot] : 0;
    if (x0 >= NX) return;
    const bool surv = tile_on_survey(a, x0, NX, xa);
    if (threadIdx.x == 0) {
        if (!early) {
            mbar_init(&bar, 1);
            fence_barrier_init();
            issue_fields<MMAX, MODE_FWD, ADAPT>(st, &bar, mapA, mapS, flatA0, flatS0, img, x0, z0, shot, false);
        }
        issue_model<MMAX, MODE_FWD, ADAPT>(st, &bar, mod, x0, z0, shot, a.vshot, surv, xa);
    }
    float cc[MMAX + 1];
#pragma unroll
    for (int l = 0; l <= MMAX; ++l) cc[l] = ADAPT ? 0.0f : __ldg(a.ctab + l);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int wx = warp & 1, wz = warp >> 1;
    const int c0 = wx * 64 + 2 * lane;        // first of the lane's two columns in the tile
    const int gx = x0 + c0;
    const int zw = z0 + wz * RW;
    // coefficients of the first row pair, gathered from the global bins
    // while the tile's copies are in flight
    float cpa[2][MMAX + 1], cpb[2][MMAX + 1];
    int lpa[2], lpb[2];
    {
        const int *gb = !ADAPT ? nullptr : (surv ? a.gsbin + xa : (a.gbin ? a.gbin + shot * a.gbin_ss : nullptr));
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            int ba = 0, bb = 0;
            if (gb && zw + r < a.NZ) {
                const int *rowb = gb + (long)(zw + r) * a.P + gx;
                if (gx < NX) ba = __ldg(rowb);
                if (gx + 1 < NX) bb = __ldg(rowb + 1);
            }
            lpa[r] = load_coefs<MMAX, ADAPT>(a, ba, cc, cpa[r]);
            lpb[r] = load_coefs<MMAX, ADAPT>(a, bb, cc, cpb[r]);
        }
    }
    const int src = __ldg(a.src + shot);
    __syncthreads();  // the barrier is initialised before any thread waits on it
    const bool ok = mbar_wait_bounded(&bar, 0, &g_rtm_dev_error);
    if (tile_at_edge<MMAX>(x0, z0, NX, a.NZ)) {
        if (ok) patch_halo<MMAX, X2_THREADS>(st.tA, x0, z0, NX, a.NZ);
        if (!__syncthreads_and(ok)) {
            mbar_wait_bounded(&bar, 0, &g_rtm_dev_error);
            return;
        }
    } else if (!ok) {
        mbar_wait_bounded(&bar, 0, &g_rtm_dev_error);
        return;
    }
    const float *tA = st.tA, *fA0 = st.fA0, *fV = st.fV;
    const int *fB = st.fB;
    const int cx = S::XH + c0;                // its column in the halo box (even)
    const int rbase = wz * RW;
    const int fr = wz * RW * TX + c0;
    const int sx = src % NX;
    const int src_row0 = (sx == gx) ? src / NX - zw : -1;
    const int src_row1 = (sx == gx + 1) ? src / NX - zw : -1;
    const int N2 = a.N2, NZ = a.NZ;
    const long long g0 = (long long)shot * a.ss + (long)zw * a.P + gx;
    // every cell of the warp's rows and columns is interior and off the
    // first interior ring: paired 8-byte stores without per-cell predicates
    const int xw = x0 + wx * 64;
    const bool inner = zw > N2 && zw + RW < NZ - N2 - 1 && xw > N2 && xw + 64 < NX - N2 - 1;
    float qa[QN + 1], qb[QN + 1];  // z-queues of the two columns
#pragma unroll
    for (int j = 0; j < QN - 1; ++j) {
        const float2 v = *reinterpret_cast<const float2 *>(tA + (rbase + j) * S::BW + cx);
        qa[j] = v.x;
        qb[j] = v.y;
    }
#pragma unroll
    for (int i = 0; i < RW; i += 2) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const float2 v = *reinterpret_cast<const float2 *>(tA + (rbase + i + QN - 1 + h) * S::BW + cx);
            qa[QN - 1 + h] = v.x;
            qb[QN - 1 + h] = v.y;
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int z = zw + i + h;
            if (z >= NZ) continue;
            const int t = fr + (i + h) * TX;
            const float *row = tA + (rbase + i + h + MMAX) * S::BW + cx - MMAX;  // even offset
            float cfa[MMAX + 1], cfb[MMAX + 1];
            int la, lb;
            if (i == 0) {
                la = lpa[h];
                lb = lpb[h];
#pragma unroll
                for (int l = 0; l <= MMAX; ++l) {
                    cfa[l] = cpa[h][l];
                    cfb[l] = cpb[h][l];
                }
            } else {
                const int2 bins = ADAPT ? *reinterpret_cast<const int2 *>(fB + t) : make_int2(0, 0);
                la = load_coefs<MMAX, ADAPT>(a, bins.x, cc, cfa);
                lb = load_coefs<MMAX, ADAPT>(a, bins.y, cc, cfb);
            }
            const int L = warp_len<MMAX, ADAPT>(max(la, lb));
            // x values the warp's operators reach: columns MMAX-L .. MMAX+1+L of xv
            float xv[NXV];
#pragma unroll
            for (int j = 0; j < NXV; j += 2) {
                if (j + 1 < MMAX - L || j > MMAX + 1 + L) {
                    xv[j] = xv[j + 1] = 0.0f;
                    continue;
                }
                const float2 v = *reinterpret_cast<const float2 *>(row + j);
                xv[j] = v.x;
                xv[j + 1] = v.y;
            }
            const float2 vv = *reinterpret_cast<const float2 *>(fV + t);
            const float2 u0 = *reinterpret_cast<const float2 *>(fA0 + t);
            const float wa = lap_regs<MMAX, ADAPT>(qa, MMAX + h, xv, 0, cfa, a.k0, a.hzx2_1, L);
            const float wb = lap_regs<MMAX, ADAPT>(qb, MMAX + h, xv, 1, cfb, a.k0, a.hzx2_1, L);
            float va = fmaf(vv.x, wa, 2.0f * qa[MMAX + h] - u0.x);
            float vb = fmaf(vv.y, wb, 2.0f * qb[MMAX + h] - u0.y);
            if (i + h == src_row0) va += a.wavelet;
            if (i + h == src_row1) vb += a.wavelet;
            const long long g = g0 + (long)(i + h) * a.P;
            if (inner) {
                *reinterpret_cast<float2 *>(a.a2 + g) = make_float2(va, vb);
                continue;
            }
            const bool zin = z >= N2 && z < NZ - N2, zring = z == N2 || z == NZ - 1 - N2;
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                const int x = gx + c;
                if (x >= NX) continue;
                const float val = c ? vb : va;
                const bool interior = zin && x >= N2 && x < NX - N2;
                if (interior) a.a2[g + c] = val;
                if (!interior || x == N2 || x == NX - 1 - N2 || zring) a.pre[g + c] = val;
            }
        }
#pragma unroll
        for (int j = 0; j < QN - 1; ++j) {
            qa[j] = qa[j + 2];
            qb[j] = qb[j + 2];
        }
    }
}

// Persistent form of k_step: a fixed grid of CTAs walks the batch's tiles
// (item i -> shot, tile row, tile column; shots may differ in width) with a
// two-stage TMA pipeline, loading tile k+1 while tile k is computed.
// items[s] = first item of shot s (items[nb] = total).
template <int MMAX, int MODE>
struct PipeSmem {
    static constexpr unsigned BYTES = 2 * stage_bytes<MMAX, MODE>() + 16u;
};

__device__ __forceinline__ void decode_item(const int *items, int nb, const int *nxs, int NZ, int it,
                                            int &shot, int &x0, int &z0)
{
    int lo = 0, hi = nb - 1;  // last shot whose first item is <= it
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(items + mid) <= it) lo = mid; else hi = mid - 1;
    }
    shot = lo;
    const int ntx = (__ldg(nxs + shot) + TX - 1) / TX;
    const int r = it - __ldg(items + shot);
    z0 = (r / ntx) * TZ;
    x0 = (r % ntx) * TX;
}

template <int MMAX, bool ADAPT, int MODE>
__global__ void __launch_bounds__(NTHREADS, MODE == MODE_BWD ? 1 : 2)
    k_step_pipe(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapS,
                const __grid_constant__ CUtensorMap flatA0, const __grid_constant__ CUtensorMap flatS0,
                const __grid_constant__ ModelMaps mod, const __grid_constant__ ImgMaps img,
                const StepArgs a, const int *__restrict__ items, int nb)
{
    constexpr int PF = MODE == MODE_BWD ? RW : RTM_PIPE_FWD_PF;
    constexpr unsigned SB = stage_bytes<MMAX, MODE>();
    extern __shared__ __align__(128) float smem[];
    const Stage<MMAX, MODE> st0(smem), st1(reinterpret_cast<float *>(reinterpret_cast<char *>(smem) + SB));
    uint64_t *bar = reinterpret_cast<uint64_t *>(reinterpret_cast<char *>(smem) + 2 * SB);
    const int total = __ldg(items + nb);
    int it = blockIdx.x;
    if (it >= total) return;
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        mbar_init(bar + 1, 1);
        fence_barrier_init();
    }
    __syncthreads();
    int shot, x0, z0;
    decode_item(items, nb, a.nxs, a.NZ, it, shot, x0, z0);
    if (threadIdx.x == 0)
        issue_tile<MMAX, MODE, ADAPT>(st0, bar, mapA, mapS, flatA0, flatS0, mod, img, x0, z0, shot, a.vshot,
                                      tile_has_interior_rows(z0, a.NZ, a.N2));
    float cc[MMAX + 1];
#pragma unroll
    for (int l = 0; l <= MMAX; ++l) cc[l] = ADAPT ? 0.0f : __ldg(a.ctab + l);
    unsigned phase = 0;  // bit s: parity of stage s's next completion
    for (int k = 0; it < total; ++k, it += gridDim.x) {
        const int s = k & 1;
        const Stage<MMAX, MODE> &cur = s ? st1 : st0;
        const int nit = it + gridDim.x;
        int nshot = 0, nx0 = 0, nz0 = 0;
        if (nit < total) {
            decode_item(items, nb, a.nxs, a.NZ, nit, nshot, nx0, nz0);
            if (threadIdx.x == 0) {
                // the other stage was last read (and patched) in the previous
                // iteration, which ended with a block barrier
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue_tile<MMAX, MODE, ADAPT>(s ? st0 : st1, bar + (s ^ 1), mapA, mapS, flatA0, flatS0,
                                              mod, img, nx0, nz0, nshot, a.vshot,
                                              tile_has_interior_rows(nz0, a.NZ, a.N2));
            }
        }
        const int NX = __ldg(a.nxs + shot);
        const bool ok = mbar_wait_bounded(bar + s, (phase >> s) & 1u, &g_rtm_dev_error);
        if (ok) {
            patch_halo<MMAX>(cur.tA, x0, z0, NX, a.NZ);
            if (MODE == MODE_BWD && tile_has_interior_rows(z0, a.NZ, a.N2))
                patch_halo<MMAX>(cur.tS, x0, z0, NX, a.NZ);
        }
        if (!__syncthreads_and(ok)) {
            // let the copies in flight land before the CTA exits
            mbar_wait_bounded(bar + s, (phase >> s) & 1u, &g_rtm_dev_error);
            if (nit < total) mbar_wait_bounded(bar + (s ^ 1), (phase >> (s ^ 1)) & 1u, &g_rtm_dev_error);
            return;
        }
        phase ^= 1u << s;
        const float nopre[1][MMAX + 1] = {};
        const int nolen[1] = {0};
        compute_tile<MMAX, ADAPT, MODE, PF, 0>(a, cur, cc, x0, z0, shot, NX, nopre, nolen,
                                               __ldg(a.src + shot), __ldg(a.rx0s + shot));
        __syncthreads();  // every thread is done with this stage before it is reloaded
        shot = nshot; x0 = nx0; z0 = nz0;
    }
}

// ---------------------------------------------------------------------------
// Pad kernel: one-way update + blend of the absorbing pad (kernel.cu:116-183),
// ring save / restore, receiver recording.

// The band of cells around a shot's receiver line that a migration with
// snapshots images at every step (rows z0 .. z0+zn-1 of the padded grid,
// inside the interior; xn columns from the shot's first receiver column plus
// xoff, clipped to its interior).  There the receiver field is held to the
// recorded data, whose content reaches far above the sampled steps' rate.
struct SnapBand {
    int z0, zn, xoff, xn;
};

__device__ __forceinline__ bool in_band(const SnapBand &b, int z, int x, int rx0)
{
    const int xb = x - (rx0 + b.xoff);
    return z >= b.z0 && z < b.z0 + b.zn && xb >= 0 && xb < b.xn;
}

// Band cell i of a shot: its padded-grid row and column (false: outside the
// shot's interior).
__device__ __forceinline__ bool band_cell(const SnapBand &b, long long i, int rx0, int NX, int N2, int &z,
                                          int &x)
{
    z = b.z0 + (int)(i / b.xn);
    x = rx0 + b.xoff + (int)(i % b.xn);
    return x >= N2 && x < NX - N2;
}

// The receiver band's cells of the two start levels (forward run, before
// its first step): level 0 (zero) in slot 0 and level 1 (the start-up spike)
// in slot 1, their running sums before them being zero.
__global__ void k_band_start(const float *S1, long long ss, int P, int N2, const int *nxs, const int *rx0s,
                             SnapBand b, int nsteps, float *bS, float *bP)
{
    const int shot = blockIdx.y;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)b.zn * b.xn) return;
    int z, x;
    if (!band_cell(b, i, rx0s[shot], nxs[shot], N2, z, x)) return;
    const long long o0 = (long long)shot * nsteps * b.zn * b.xn + i, o1 = o0 + (long long)b.zn * b.xn;
    bS[o0] = 0.0f;
    bS[o1] = S1[(long long)shot * ss + (long long)z * P + x];
    if (bP) bP[o0] = bP[o1] = 0.0f;
}

struct PadArgs {
    int NZ, P, N2, M;
    int shot0;                // first shot of this launch (blockIdx.y + shot0)
    long long ss;
    long nabc;                // pad cells of the widest grid (threads per shot)
    const int *nxs, *rx0s;    // per-shot padded width and receiver start column
    long long tab_ss;         // pad-table entries between shots (0: shared table)
    const int4 *meta;         // [nabc] pad_meta(): {cell, d1, d2, (ring slot + 1) << 1 | corner}
    const float4 *fac;        // [nabc] side: {taoh*v, 1/(taoh*v+1), taoh2*vq*vq, w}
                              //        corner: {r_1, 1/(2 r_1+1), 0, w}
    const float *a0, *a1;     // field A levels k-2, k-1
    float *a2;                // field A level k (interior final, pad written here)
    const float *pre;         // pre-blend pad values of level k
    // ring
    float *ring;              // shot 0, slot k (forward save) or slot k (backward restore)
    long long ring_ss;        // floats between shots in the ring store
    int ring_mode;            // 0 none, 1 save a2, 2 restore into s2
    float *s2;                // backward source field receiving the restore
    // recording (forward): rec[shot*rec_ss + j] = a1[cell_j]
    float *rec;
    long long rec_ss;
    int rz0, rx0, rdz, rdx, nrec;
    // 16-bit ring store (ring_prec 1: bf16, 2: fp16, 3: int16) with per-step max-abs
    // scaling.  Forward: the blended ring values of step k go to the FP32
    // stage (stage + shot*ringsz) and their max |value| to amax[shot][k];
    // the quantisation of slot qslot (= k-1, whose max is final by now) from
    // qstage runs on extra threads of the same launch.  Backward: slot k is
    // read back as q * scale[shot][k].
    int ring_prec;
    long ringsz;
    long long slots;         // NT: slots per shot in ring16 / amax / scale
    uint16_t *ring16;        // [shot][NT][ringsz]
    float *stage;            // FP32 values of this step   [shot][ringsz]
    const float *qstage;     // FP32 values of slot qslot  [shot][ringsz]
    unsigned *amax;          // [shot][NT] float bits of max |value|
    float *scale;            // [shot][NT] dequantisation factor
    int slot, qslot;         // slot written (fwd) / restored (bwd); slot to quantise (<0: none)
    // the receiver band of a migration with source snapshots, on extra
    // threads after the others: band_mode 1 (forward) stores the band cells
    // of the source field of step band_k and its running sum before the step
    // (sum: the running sum after it; band_qzero: level 0), fp32, at
    // [shot][band_k][cell]; band_mode 2 (backward) applies the imaging
    // condition of step band_k to them with weight 1 (sum: the forward
    // total; racc: the receiver field's running sum; R(k): a2)
    SnapBand band;
    int band_mode, band_k, band_steps, band_qzero, compen;
    float *bandS, *bandP;
    const float *sum, *racc;
    float *rel1, *rel2;
};

// Value a step's max |ring value| maps to: 16384 for FP16 / BF16 (FP16 keeps
// headroom below 65504; BF16 uses the same scale), 32767 for the scaled
// integers of RTM_RING_I16, whose values then fill the int16 range.
// Source snapshots.  At a snapshot step of the forward run, S is the step's
// source field and P its running sum after the step, so P - S is the sum of
// the levels before the step.  A slot holds both over the shot's interior
// (qzero: the slot of level 0, whose sum is zero) at plane shot*nslots+slot,
// row z - N2, column x - N2 + off: S as fp32 or as 16-bit codes, fractions
// of the slot's largest |S| (as the rings' codes); the running sum always as
// fp32 -- it changes slowly from slot to slot, so 16-bit rounding of it would
// repeat over many slots instead of averaging out, and the image's Laplacian
// filter would bring that cell-to-cell noise out (FP16: 3e-3 of the image).
__global__ void k_snap_max(const float *S, long long ss, int NZ, int P, int N2, const int *nxs,
                           unsigned *amax, int nslots, int slot, int shot0)
{
    const int shot = blockIdx.y + shot0;
    const int nx = nxs[shot] - 2 * N2, nz = NZ - 2 * N2;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned bs = 0;
    if (i < (long long)nz * nx) {
        const int z = N2 + (int)(i / nx), x = N2 + (int)(i % nx);
        bs = __float_as_uint(fabsf(S[(long long)shot * ss + (long long)z * P + x]));
    }
    bs = __reduce_max_sync(0xffffffffu, bs);
    if ((threadIdx.x & 31) == 0 && bs) atomicMax(amax + (long long)shot * nslots + slot, bs);
}

__global__ void k_snap_store(const float *S, const float *pacc, long long ss, int NZ, int P, int N2,
                             const int *nxs, const unsigned *amax, float *scale, int nslots, int slot,
                             int qzero, int prec, int pitch, int off, void *outS, float *outQ, int shot0)
{
    const int shot = blockIdx.y + shot0;
    const int nx = nxs[shot] - 2 * N2, nz = NZ - 2 * N2;
    const long long sl = (long long)shot * nslots + slot;
    float inv = 1.0f;
    if (prec) {
        const float tgt = ring16_target(prec);
        const float ms = __uint_as_float(amax[sl]);
        inv = ms > 0.0f ? tgt / ms : 0.0f;
        if (blockIdx.x == 0 && threadIdx.x == 0) scale[sl] = ms / tgt;
    }
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)nz * nx) return;
    const int z = N2 + (int)(i / nx), x = N2 + (int)(i % nx);
    const long long g = (long long)shot * ss + (long long)z * P + x;
    const float sv = S[g];
    const long long o = (sl * nz + (z - N2)) * pitch + (x - N2 + off);
    if (prec == 0) static_cast<float *>(outS)[o] = sv;
    else static_cast<uint16_t *>(outS)[o] = ring_quant(sv, inv, prec);
    if (outQ) outQ[o] = qzero ? 0.0f : pacc[g] - sv;
}

// Imaging at snapshot step k of the backward run, over the interior of the
// launch's shots outside the receiver band (a streaming pass after the
// step's stencil): with the stored source field S(k) and, compensated, the
// source's running sum Tot - P_k (Tot: the forward run's total, P_k: the
// stored prefix) times the receiver field's running sum, or, plain, the
// receiver field R(k) itself; w is the step's share of the time sum
// (kernel.cu:489-517's accumulations).
__global__ void k_snap_image(const float *R, const float *racc, const float *tot, const void *snapS,
                             const float *snapQ, const float *scale, float *rel1, float *rel2, long long ss,
                             int NZ, int P, int N2, const int *nxs, const int *rx0s, SnapBand b, int nslots,
                             int slot, int prec, int pitch, int off, float w, int compen, int shot0)
{
    const int shot = blockIdx.y + shot0;
    const int nx = nxs[shot] - 2 * N2, nz = NZ - 2 * N2;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)nz * nx) return;
    const int z = N2 + (int)(i / nx), x = N2 + (int)(i % nx);
    if (in_band(b, z, x, rx0s[shot])) return;  // imaged at every step
    const long long g = (long long)shot * ss + (long long)z * P + x;
    const long long sl = (long long)shot * nslots + slot;
    const long long o = (sl * nz + (z - N2)) * pitch + (x - N2 + off);
    const float sv = prec == 0 ? static_cast<const float *>(snapS)[o]
                               : ring_dequant(static_cast<const uint16_t *>(snapS)[o], __ldg(scale + sl), prec);
    if (compen) rel1[g] = fmaf(w, racc[g] * (tot[g] - snapQ[o]), rel1[g]);
    else rel1[g] = fmaf(w, R[g] * sv, rel1[g]);
    rel2[g] = fmaf(w, sv * sv, rel2[g]);
}

enum { PAD_ROWEDGE = 0, PAD_COLEDGE = 1, PAD_CORNER = 2 };

__host__ __device__ __forceinline__ long ring_index(int z, int x, int NZ, int NX, int N2, int M,
                                                    int nz, int nx)
{
    if (x >= N2 && x < NX - N2) {
        if (z < N2 && z >= N2 - M) return (long)(N2 - 1 - z) * nx + (x - N2);
        if (z >= NZ - N2 && z < NZ - N2 + M) return (long)M * nx + (long)(z - (NZ - N2)) * nx + (x - N2);
    }
    if (z >= N2 && z < NZ - N2) {
        if (x < N2 && x >= N2 - M) return 2L * M * nx + (long)(N2 - 1 - x) * nz + (z - N2);
        if (x >= NX - N2 && x < NX - N2 + M)
            return 2L * M * nx + (long)M * nz + (long)(x - (NX - N2)) * nz + (z - N2);
    }
    return -1;
}

// Geometry of pad cell t as flat offsets in a grid of pitch P:
// {cell, d1, d2, (ring slot + 1) << 1 | corner}.  Row-edge cell: inward
// neighbour cell+d1 (d1 = dz*P), lateral step d2 = 1; column-edge cell:
// d1 = dx, d2 = P; corner: its two inward neighbours cell+d1 (d1 = dx) and
// cell+d2 (d2 = dz*P).  dz / dx point into the grid.  Ring slot -1 (stored as
// 0) when the cell is not on the saved ring.
__host__ __device__ __forceinline__ int4 pad_meta(long t, int NZ, int NX, int P, int N2, int M)
{
    const AbcCell cc = abc_cell(t, NZ, NX, N2);
    const int z = cc.z, x = cc.x;
    const int ea = min(z, NZ - 1 - z), ee = min(x, NX - 1 - x);
    const int dz = (z < NZ - 1 - z) ? 1 : -1, dx = (x < NX - 1 - x) ? 1 : -1;
    const long ri = M > 0 ? ring_index(z, x, NZ, NX, N2, M, NZ - 2 * N2, NX - 2 * N2) : -1;
    int d1, d2, corner = 0;
    if (ee >= ea + 2) {
        d1 = dz * P; d2 = 1;
    } else if (ea >= ee + 2) {
        d1 = dx; d2 = P;
    } else {
        d1 = dx; d2 = dz * P; corner = 1;
    }
    return make_int4(z * P + x, d1, d2, (int)((ri + 1) << 1) | corner);
}

// One-way update + blend of one pad cell (kernel.cu:116-183).  Side cell c
// with inward neighbour n and lateral step s:
//   b = inv*(A*(u2[n]-u0[n]+u0[c]) - (-2u1[c]+u0[c]+u2[n]-2u1[n]+u0[n])
//           + Q*(u2[n+s]-2u2[n]+u2[n-s]+u0[c+s]-2u0[c]+u0[c-s]))
// corner: b = inv*(u1[c] + r_1*(u2[c+dx]+u2[c+dz])); u2 is read before
// blending (pre-blend pad values from `pre`, interior values from a2);
// out = (1-w)*u2[c] + w*b.
#ifndef RTM_PAD_CPT
#define RTM_PAD_CPT 2
#endif
constexpr int PAD_CPT = RTM_PAD_CPT;  // pad cells per thread

// The update of pad cell t of one shot, without branches on its kind: a
// corner cell reads its side-cell operands at zero lateral offset (valid
// addresses) and the corner formula is selected at the end, so the loads of
// several cells of a thread can all be in flight together.
struct PadOut {
    float out;
    long c, ri;
};

__device__ __forceinline__ PadOut pad_cell(const PadArgs &a, int shot, long long so, long t)
{
    const int4 m = __ldg(a.meta + shot * a.tab_ss + t);
    const float4 f = __ldg(a.fac + shot * a.tab_ss + t);
    const bool corner = m.w & 1;
    const long c = m.x, n = c + m.y, sd = corner ? 0 : m.z, zc = corner ? m.z : 0;
    const float *u0 = a.a0 + so, *u1 = a.a1 + so, *pr = a.pre + so;
    const float u2n = pr[n], pnp = pr[n + sd], pnm = pr[n - sd], pcz = pr[c + zc], pc = pr[c];
    const float u0c = u0[c], u0n = u0[n], u0p = u0[c + sd], u0m = u0[c - sd];
    const float u1c = u1[c], u1n = u1[n];
    const float lat = pnp - 2.0f * u2n + pnm + u0p - 2.0f * u0c + u0m;
    const float bs = f.y * (f.x * (u2n - u0n + u0c) - (-2.0f * u1c + u0c + u2n - 2.0f * u1n + u0n) +
                            f.z * lat);
    const float bc = f.y * (u1c + f.x * (u2n + pcz));
    PadOut r;
    r.out = (1.0f - f.w) * pc + f.w * (corner ? bc : bs);
    r.c = c;
    r.ri = a.ring_mode ? (long)(m.w >> 1) - 1 : -1;
    return r;
}

__global__ void __launch_bounds__(256) k_pad(const PadArgs a)
{
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int shot = blockIdx.y + a.shot0;
    const long long so = (long long)shot * a.ss;
    const long npadt = (a.nabc + PAD_CPT - 1) / PAD_CPT;  // threads of the pad cells
    if (t >= npadt) {
        long j = t - npadt;
        if (a.rec && j < a.nrec) {
            const int z = a.rz0 + (int)j * a.rdz, x = a.rx0s[shot] + (int)j * a.rdx;
            a.rec[(long long)shot * a.rec_ss + j] = a.a1[so + (long)z * a.P + x];
            return;
        }
        if (a.rec) j -= a.nrec;
        if (a.ring_prec && a.ring_mode == 1 && a.qslot >= 0 && j < a.ringsz) {
            const long long sl = (long long)shot * a.slots + a.qslot;
            const float mx = __uint_as_float(a.amax[sl]);
            const float tgt = ring16_target(a.ring_prec);
            const float inv = mx > 0.0f ? tgt / mx : 0.0f;
            a.ring16[sl * a.ringsz + j] = ring_quant(a.qstage[(long long)shot * a.ringsz + j], inv, a.ring_prec);
            if (j == 0) a.scale[sl] = mx / tgt;
            return;
        }
        if (a.ring_prec && a.ring_mode == 1) j -= a.ringsz;
        if (a.band_mode) {
            const long nb = (long)a.band.zn * a.band.xn;
            int z, x;
            if (j < nb) {
                if (!band_cell(a.band, j, a.rx0s[shot], a.nxs[shot], a.N2, z, x)) return;
                const long long g = so + (long long)z * a.P + x;
                const long long o = ((long long)shot * a.band_steps + a.band_k) * nb + j;
                if (a.band_mode == 1) {
                    const float sv = a.a2[g];
                    a.bandS[o] = sv;
                    if (a.bandP) a.bandP[o] = a.band_qzero ? 0.0f : a.sum[g] - sv;
                } else {
                    const float sv = a.bandS[o];
                    if (a.compen) a.rel1[g] = fmaf(a.racc[g], a.sum[g] - a.bandP[o], a.rel1[g]);
                    else a.rel1[g] = fmaf(a.a2[g], sv, a.rel1[g]);
                    a.rel2[g] = fmaf(sv, sv, a.rel2[g]);
                }
                return;
            }
            j -= nb;
        }
        return;
    }
    // this shot's pad may be smaller (own window); with one shared table
    // every shot has the full pad, and no width load delays the cells
    const long nmine = a.tab_ss ? abc_count(a.NZ, a.nxs[shot], a.N2) : a.nabc;
    PadOut r[PAD_CPT];
    bool on[PAD_CPT];
#pragma unroll
    for (int k = 0; k < PAD_CPT; ++k) {
        const long tk = t * PAD_CPT + k;
        on[k] = tk < nmine;
        if (on[k]) r[k] = pad_cell(a, shot, so, tk);
    }
    unsigned bits = 0u;
#pragma unroll
    for (int k = 0; k < PAD_CPT; ++k) {
        if (!on[k]) continue;
        const long c = r[k].c, ri = r[k].ri;
        const float out = r[k].out;
        a.a2[so + c] = out;
        if (ri >= 0) {
            if (a.ring_prec == 0) {
                if (a.ring_mode == 1)
                    a.ring[(long long)shot * a.ring_ss + ri] = out;
                else
                    a.s2[so + c] = a.ring[(long long)shot * a.ring_ss + ri];
            } else if (a.ring_mode == 1) {
                a.stage[(long long)shot * a.ringsz + ri] = out;
                bits = max(bits, __float_as_uint(fabsf(out)));
            } else {
                const long long sl = (long long)shot * a.slots + a.slot;
                a.s2[so + c] = ring_dequant(a.ring16[sl * a.ringsz + ri], a.scale[sl], a.ring_prec);
            }
        }
    }
    if (a.ring_prec && a.ring_mode == 1) {
        // max |value| of the step's ring: reduced over the warp first (all
        // lanes of a block belong to one shot), one atomic per warp.  Float
        // bits of non-negative values order like unsigned integers.
        const unsigned mask = __activemask();
        bits = __reduce_max_sync(mask, bits);
        if ((threadIdx.x & 31) == __ffs(mask) - 1 && bits)
            atomicMax(a.amax + (long long)shot * a.slots + a.slot, bits);
    }
}

// Ring of one level (slot 1 at start-up): ring[ri] = u[cell].  With a 16-bit
// store the values go to the FP32 stage and the slot's max-abs, and the next
// pad launch quantises them.
__global__ void k_ring_fill(const float *__restrict__ u, float *__restrict__ ring, long long ss,
                            long long ring_ss, int NZ, const int *nxs, int P, int N2, int M,
                            unsigned *amax, long long amax_ss)
{
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int shot = blockIdx.y;
    const int NX = nxs[shot];
    if (t >= abc_count(NZ, NX, N2)) return;
    const AbcCell cc = abc_cell(t, NZ, NX, N2);
    const long ri = ring_index(cc.z, cc.x, NZ, NX, N2, M, NZ - 2 * N2, NX - 2 * N2);
    if (ri < 0) return;
    const float val = u[(long long)shot * ss + (long)cc.z * P + cc.x];
    ring[(long long)shot * ring_ss + ri] = val;
    if (amax) atomicMax(amax + (long long)shot * amax_ss, __float_as_uint(fabsf(val)));
}

// Start of a shot: u0 = 0, u1 = spike at the source (kernel.cu:798-803).
__global__ void k_shot_init(float *u0, float *u1, float *u2, float *pre, const int *src,
                            const int *nxs, float spike, long long ss, int P)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int shot = blockIdx.y;
    if (i >= ss) return;
    const long long o = (long long)shot * ss + i;
    u0[o] = 0.0f;
    u2[o] = 0.0f;
    pre[o] = 0.0f;
    const int s = src[shot], NX = nxs[shot];
    const long si = (long)(s / NX) * P + s % NX;
    u1[o] = (i == si) ? spike : 0.0f;
}

// Hand-off to the backward pass and image initialisation (kernel.cu:822-885).
// F1 = u_{NT-1}, F0 = u_{NT-2} of the forward run; the host-side forward
// arrays the reference reads here still hold the initial state (zeros plus
// the start spike at the source).
__global__ void k_img_init(const float *F1, const float *F0, float *R0, float *R1, float *R2,
                           float *rel1, float *rel2, float *sacc, float *racc, const int *src,
                           const int *nxs, float spike, int compen, long long ss, int P)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int shot = blockIdx.y;
    if (i >= ss) return;
    const long long o = (long long)shot * ss + i;
    const int s = src[shot], NX = nxs[shot];
    const long si = (long)(s / NX) * P + s % NX;
    const float h1 = (i == si) ? spike : 0.0f, h0 = 0.0f;
    const float b0 = F1[o], b1 = F0[o];  // BW0 = u_{NT-1}, BW1 = u_{NT-2}
    if (compen) {
        const float bw2 = b0 + b1, fw2 = h0 + h1;
        rel1[o] = fw2 * bw2 + h0 * b0;
        rel2[o] = b1 * b1 + b0 * b0;
        sacc[o] = bw2;
        racc[o] = fw2;
    } else {
        rel1[o] = h1 * b1 + h0 * b0;
        rel2[o] = b1 * b1 + b0 * b0;
    }
    R0[o] = 0.0f;
    R1[o] = 0.0f;
    R2[o] = 0.0f;
}

// Receiver samples of a level (used for the first and last recorded steps).
__global__ void k_record(const float *u, float *rec, long long ss, long long rec_ss, int P, int rz0,
                         const int *rx0s, int rdz, int rdx, int nrec)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int shot = blockIdx.y;
    if (j >= nrec) return;
    const int z = rz0 + j * rdz, x = rx0s[shot] + j * rdx;
    rec[(long long)shot * rec_ss + j] = u[(long long)shot * ss + (long)z * P + x];
}

// Model of each shot's aperture window: interior columns [xa, xa+nx) of the
// survey model, padded by edge extension as the reference pads a model it
// reads (GPU_velocity_real.cpp:20-80); v and r_1 copied from the survey's
// padded grid (survey pitch Pg) so the values are bit-identical.
__global__ void k_window_model(const float *vg, const float *r1g, int Pg, const int *xas,
                               const int *nxs, float *vs, float *r1s, long long ss, int NZ, int P,
                               int N2)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int shot = blockIdx.y;
    if (i >= ss) return;
    const int z = (int)(i / P), x = (int)(i % P);
    const int NX = nxs[shot], nx = NX - 2 * N2;
    const int xi = min(max(x - N2, 0), nx - 1);   // pitch columns repeat the last column
    const long gi = (long)z * Pg + N2 + xas[shot] + xi;
    const long long o = (long long)shot * ss + i;
    const int zc = min(max(z, N2), NZ - N2 - 1);
    const long gz = (long)zc * Pg + N2 + xas[shot] + xi;
    vs[o] = vg[(z >= N2 && z < NZ - N2) ? gi : gz];
    r1s[o] = r1g[(z >= N2 && z < NZ - N2) ? gi : gz];
}

// Per-cell model factors of nshot grids [shot][NZ][P]: vv = v*v*tao2*h2 in
// the reference's float order, and the bin word: the velocity bin
// int((v-vmin)/dv + 0.5), with the 0.5 added in double as the reference's
// kernels do (kernel.cu:56) and clamped to the table, packed with that bin's
// operator length blen[bin] (word_bin / word_len).
__global__ void k_model_prep(const float *__restrict__ v, long long ncell, float tao2, float h2,
                             float vmin, float dv, int nbins, const int *__restrict__ blen,
                             float *__restrict__ vv, int *__restrict__ bin)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ncell) return;
    const float x = v[i];
    vv[i] = __fmul_rn(__fmul_rn(__fmul_rn(x, x), tao2), h2);
    if (bin) {
        const float q = __fdiv_rn(__fsub_rn(x, vmin), dv);
        const int b = min(max((int)((double)q + 0.5), 0), nbins - 1);
        bin[i] = b | (blen[b] << BIN_BITS);
    }
}

// Pad tables of each shot's grid (the device form of the table rtm_ctx_create
// builds for a single grid): classification, inward directions, ring slot and
// the model factors, from the shot's own padded model.

__global__ void k_pad_tables(const float *vs, const float *r1s, const float *w, const int *nxs,
                             long long ss, long long tab_ss, int NZ, int P, int N2, int M,
                             float taoh, float taoh2, int quirk, int4 *meta, float4 *fac)
{
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int shot = blockIdx.y;
    const int NX = nxs[shot];
    if (t >= abc_count(NZ, NX, N2)) return;
    const AbcCell cc = abc_cell(t, NZ, NX, N2);
    const int z = cc.z, x = cc.x;
    const int ea = min(z, NZ - 1 - z), ee = min(x, NX - 1 - x);
    const int dz = (z < NZ - 1 - z) ? 1 : -1, dx = (x < NX - 1 - x) ? 1 : -1;
    int kind;
    long q = (long)z * NX + x;  // flat index (reference pitch NX) of the lateral-term velocity
    if (ee >= ea + 2) {
        kind = PAD_ROWEDGE;
        if (quirk && dz < 0) q = (long)(NZ - 1 - z) * NX + x;
    } else if (ea >= ee + 2) {
        kind = PAD_COLEDGE;
        if (quirk) q = (dx > 0) ? (long)x * NX + z : (long)(NX - 1 - x) * NX + z;
    } else {
        kind = PAD_CORNER;
    }
    const float *v = vs + shot * ss, *r1 = r1s + shot * ss;
    const float wj = w[blend_index(z, x, NZ, NX, N2)];
    float4 f;
    if (kind == PAD_CORNER) {
        const float rr = r1[(long)z * P + x];
        f = make_float4(rr, __fdiv_rn(1.0f, __fadd_rn(__fmul_rn(2.0f, rr), 1.0f)), 0.0f, wj);
    } else {
        const float vc = v[(long)z * P + x];
        const float vq = v[(q / NX) * P + q % NX];
        const float tv = __fmul_rn(taoh, vc);
        f = make_float4(tv, __fdiv_rn(1.0f, __fadd_rn(tv, 1.0f)), __fmul_rn(__fmul_rn(taoh2, vq), vq), wj);
    }
    meta[shot * tab_ss + t] = pad_meta(t, NZ, NX, P, N2, M);
    fac[shot * tab_ss + t] = f;
}

// ---------------------------------------------------------------------------
// Per-shot finishing (kernel.cu:935-990) and the compensated stack.

__global__ void k_illum_max(const float *rel2, unsigned *mx, long long ss, int NZ, const int *nxs,
                            int P, int N2)
{
    const int shot = blockIdx.y;
    const int nz = NZ - 2 * N2, nx = nxs[shot] - 2 * N2;
    float m = 0.0f;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < (long)nz * nx;
         t += (long)gridDim.x * blockDim.x) {
        const int zi = (int)(t / nx), xi = (int)(t % nx);
        m = fmaxf(m, fabsf(rel2[(long long)shot * ss + (long)(zi + N2) * P + xi + N2]));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(mx + shot, __float_as_uint(m));
}

// up = -(Laplacian of rel1) * v^2 / vmax^2 with even reflection at the
// interior edges, down = rel2 + whitecoe*max|rel2|; outputs
// [shot][nz][ostride] (ostride >= the shot's interior width).
__global__ void k_finish(const float *rel1, const float *rel2, const float *v, long long vss,
                         const unsigned *mx, float *up, float *down, long long ss, int NZ,
                         const int *nxs, int P, int N2, int ostride, float vmax, float whitecoe)
{
    const int shot = blockIdx.y;
    const int NX = nxs[shot];
    const int nz = NZ - 2 * N2, nx = NX - 2 * N2;
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long)nz * nx) return;
    const int zi = (int)(t / nx), xi = (int)(t % nx);
    const int i = zi + N2, j = xi + N2;
    int i1 = i - 1, i2 = i + 1, j1 = j - 1, j2 = j + 1;
    if (i1 < N2) i1 = 2 * N2 - i1;
    if (j1 < N2) j1 = 2 * N2 - j1;
    if (i2 >= NZ - N2) i2 = 2 * (NZ - N2 - 1) - i2;
    if (j2 >= NX - N2) j2 = 2 * (NX - N2 - 1) - j2;
    const float *g = rel1 + (long long)shot * ss;
    const float s = g[(long)i * P + j2] + g[(long)i * P + j1] + g[(long)i2 * P + j] +
                    g[(long)i1 * P + j] - 4.0f * g[(long)i * P + j];
    const float vv = v[shot * vss + (long)i * P + j];
    const long long o = ((long long)shot * nz + zi) * ostride + xi;
    up[o] = -1.0f * s * vv * vv / (vmax * vmax);
    const float stable = __uint_as_float(mx[shot]) * whitecoe;
    down[o] = rel2[(long long)shot * ss + (long)i * P + j] + stable;
}

// Compensated (Kahan) accumulation of per-shot images into the survey frame,
// in shot order; shot m covers survey columns [xa[m], xa[m]+nx_m).
// sum/comp persist across batches.
__global__ void k_stack_kahan(const float *up, const float *down, int nshot, int nz, int nxg,
                              int ostride, const int *xas, const int *nxs, int N2, float *s1,
                              float *c1, float *s2, float *c2)
{
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long)nz * nxg) return;
    const int zi = (int)(t / nxg), xg = (int)(t % nxg);
    float a1 = s1[t], e1 = c1[t], a2 = s2[t], e2 = c2[t];
    for (int m = 0; m < nshot; ++m) {
        const int xi = xg - xas[m];
        if (xi < 0 || xi >= nxs[m] - 2 * N2) continue;
        const long long o = ((long long)m * nz + zi) * ostride + xi;
        const float y1 = __fsub_rn(up[o], e1);
        const float t1 = __fadd_rn(a1, y1);
        e1 = __fsub_rn(__fsub_rn(t1, a1), y1);
        a1 = t1;
        const float y2 = __fsub_rn(down[o], e2);
        const float t2 = __fadd_rn(a2, y2);
        e2 = __fsub_rn(__fsub_rn(t2, a2), y2);
        a2 = t2;
    }
    s1[t] = a1; c1[t] = e1; s2[t] = a2; c2[t] = e2;
}

__global__ void k_stack_final(const float *s1, const float *s2, float *img, float *ill, long ncell,
                              int nrec, int inorm)
{
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ncell) return;
    float g1 = s1[t] / (float)nrec, g2 = s2[t] / (float)nrec;
    if (inorm) g1 = g1 / g2;
    img[t] = g1;
    ill[t] = g2;
}

}  // namespace eng
