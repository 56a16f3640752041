// Kernel-level drop-in entry points: one per __global__ kernel of the
// reference's kernel.cu, same arguments and [iz*NX + ix] layout.
//
// Design: lanes run along x (the contiguous axis) so every warp touches
// 128 contiguous bytes per row (the reference maps threadIdx.x to z, which
// makes each warp straddle 16 rows); boundary kernels launch over the pad or
// ring cells only instead of the full grid; the rotation kernels are plain
// vectorisable copies.  No allocation happens here.
#include <cstdio>
#include <vector>

#include "rtm_common.cuh"

namespace {

constexpr int BX = 32, BY = 8;

inline dim3 grid_cells(int NZ, int NX) { return dim3((NX + BX - 1) / BX, (NZ + BY - 1) / BY); }

__device__ __forceinline__ int mirror_idx(int i, int n)
{
    return i < 0 ? -i : (i >= n ? 2 * n - 2 - i : i);
}

// Spatial operator of kernel.cu:59-72 at (z,x) with coefficients c[0..cnt]:
// (1+hzx2_1)*c0*u + sum_l c_l*((u[z-l]+u[z+l])*hzx2_1 + u[x-l] + u[x+l]).
__device__ __forceinline__ float lap_at(const float *__restrict__ u, const float *__restrict__ c,
                                        int cnt, int z, int x, int NZ, int NX, float hzx2_1)
{
    float w1 = (1.0f + hzx2_1) * __ldg(c) * u[(long)z * NX + x];
    for (int l = 1; l <= cnt; ++l) {
        int z1 = mirror_idx(z - l, NZ), z2 = mirror_idx(z + l, NZ);
        int x1 = mirror_idx(x - l, NX), x2 = mirror_idx(x + l, NX);
        w1 += __ldg(c + l) * ((u[(long)z1 * NX + x] + u[(long)z2 * NX + x]) * hzx2_1 +
                              u[(long)z * NX + x1] + u[(long)z * NX + x2]);
    }
    return w1;
}

// Coefficient window of a cell from its velocity bin (kernel.cu:55-57).
__device__ __forceinline__ void bin_window(float v, float vmin, float dv, const int *idx, int *top,
                                           int *cnt)
{
    float q = (v - vmin) / dv;
    int t = __ldg(idx + (int)(q + 0.5f));
    int e = __ldg(idx + (int)(q + 1.5f));
    *top = t;
    *cnt = e - t - 1;
}

enum { ST_FULL = 0, ST_INTERIOR = 1 };

template <bool ADAPT, int REGION>
__global__ void k_add(const float *__restrict__ v, float *__restrict__ u2,
                      const float *__restrict__ u0, const float *__restrict__ u1,
                      const float *__restrict__ c, const int *__restrict__ idx, float tao2,
                      float h2, float vmin, float dv, int M, int N2, int NZ, int NX, int r_u,
                      int r_x, float wavelet, float hzx2_1)
{
    int x = blockIdx.x * BX + threadIdx.x, z = blockIdx.y * BY + threadIdx.y;
    if (z >= NZ || x >= NX) return;
    if (REGION == ST_INTERIOR && (z < N2 || z >= NZ - N2 || x < N2 || x >= NX - N2)) return;
    long i = (long)z * NX + x;
    float vc = v[i];
    float w1;
    if (ADAPT) {
        int top, cnt;
        bin_window(vc, vmin, dv, idx, &top, &cnt);
        w1 = lap_at(u1, c + top, cnt, z, x, NZ, NX, hzx2_1);
    } else {
        w1 = lap_at(u1, c, M, z, x, NZ, NX, hzx2_1);
    }
    float out = 2.0f * u1[i] - u0[i] + vc * vc * tao2 * h2 * w1;
    if (z == r_u && x == r_x) out += wavelet;
    u2[i] = out;
}

// kernel.cu:339-418: receiver-side update with Dirichlet replacement on the
// line z=s_z, x = s_l + s*ds <= s_r when seis[s] != 0.
template <bool ADAPT>
__global__ void k_bkadd(const float *__restrict__ v, float *__restrict__ u2,
                        const float *__restrict__ u1, const float *__restrict__ u0,
                        const float *__restrict__ c, const int *__restrict__ idx,
                        const float *__restrict__ seis, float tao2, float h2, float vmin, float dv,
                        int M, int NZ, int NX, int s_l, int s_r, int s_z, int ds, float hzx2_1)
{
    int x = blockIdx.x * BX + threadIdx.x, z = blockIdx.y * BY + threadIdx.y;
    if (z >= NZ || x >= NX) return;
    long i = (long)z * NX + x;
    if (z == s_z && x >= s_l && x <= s_r && (x - s_l) % ds == 0) {
        float d = seis[(x - s_l) / ds];
        if (d != 0.0f) {
            u2[i] = d;
            return;
        }
    }
    float vc = v[i];
    float w1;
    if (ADAPT) {
        int top, cnt;
        bin_window(vc, vmin, dv, idx, &top, &cnt);
        w1 = lap_at(u1, c + top, cnt, z, x, NZ, NX, hzx2_1);
    } else {
        w1 = lap_at(u1, c, M, z, x, NZ, NX, hzx2_1);
    }
    u2[i] = 2.0f * u1[i] - u0[i] + vc * vc * tao2 * h2 * w1;
}

// One-way value of every pad cell (kernel.cu:116-158); see rtm_common.cuh for
// the cell classification.  Launched over the pad only.
__global__ void k_hybrid1(const float *__restrict__ u1, const float *__restrict__ u0,
                          const float *__restrict__ u2, float *__restrict__ b,
                          const float *__restrict__ v, const float *__restrict__ r1, int NZ,
                          int NX, int N2, float taoh, float taoh2)
{
    long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= abc_count(NZ, NX, N2)) return;
    AbcCell cc = abc_cell(t, NZ, NX, N2);
    int z = cc.z, x = cc.x;
    long c = (long)z * NX + x;
    int a = min(z, NZ - 1 - z), e = min(x, NX - 1 - x);
    int dz = (z < NZ - 1 - z) ? 1 : -1, dx = (x < NX - 1 - x) ? 1 : -1;
    if (e >= a + 2 || a >= e + 2) {
        long n, s, q;
        if (e >= a + 2) {
            n = c + (long)dz * NX;
            s = 1;
            q = (dz > 0) ? c : (long)(NZ - 1 - z) * NX + x;
        } else {
            n = c + dx;
            s = NX;
            q = (dx > 0) ? (long)x * NX + z : (long)(NX - 1 - x) * NX + z;
        }
        float vc = v[c], vq = v[q];
        b[c] = 1.0f / (taoh * vc + 1.0f) *
               (taoh * vc * (u2[n] - u0[n] + u0[c]) -
                (-2.0f * u1[c] + u0[c] + u2[n] - 2.0f * u1[n] + u0[n]) +
                taoh2 * vq * vq * (u2[n + s] - 2.0f * u2[n] + u2[n - s] + u0[c + s] - 2.0f * u0[c] +
                                   u0[c - s]));
    } else {
        float rr = r1[c];
        b[c] = 1.0f / (2.0f * rr + 1.0f) * (u1[c] + rr * (u2[c + dx] + u2[c + (long)dz * NX]));
    }
}

// Blend of kernel.cu:160-183: u2 = (1-w[j])*u2 + w[j]*b on the pad.
__global__ void k_hybrid2(float *__restrict__ u2, const float *__restrict__ b,
                          const float *__restrict__ w, int NZ, int NX, int N2)
{
    long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= abc_count(NZ, NX, N2)) return;
    AbcCell cc = abc_cell(t, NZ, NX, N2);
    long c = (long)cc.z * NX + cc.x;
    float wj = w[blend_index(cc.z, cc.x, NZ, NX, N2)];
    u2[c] = (1.0f - wj) * u2[c] + wj * b[c];
}

// Ring store in the reference layout (kernel.cu:18-45, 184-208, 222-245):
// slot s: lf/rt [s][nz][M], up/dw [s][M][nx].  dir=0 saves u into slot
// `slot`, dir=1 restores slot `slot` into u.
__global__ void k_ring(float *__restrict__ lf, float *__restrict__ rt, float *__restrict__ up,
                       float *__restrict__ dw, float *__restrict__ u, int NZ, int NX, int N2,
                       int M, long slot, int dir)
{
    int nz = NZ - 2 * N2, nx = NX - 2 * N2;
    long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    long nside = (long)nz * M, ntop = (long)M * nx;
    if (t < nside) {
        int zi = (int)(t / M), m = (int)(t % M);
        long ri = slot * nside + t;
        long cl = (long)(N2 + zi) * NX + (N2 - 1 - m), cr = (long)(N2 + zi) * NX + (NX - N2 + m);
        if (dir) { u[cl] = lf[ri]; u[cr] = rt[ri]; }
        else     { lf[ri] = u[cl]; rt[ri] = u[cr]; }
        return;
    }
    t -= nside;
    if (t < ntop) {
        int m = (int)(t / nx), xi = (int)(t % nx);
        long ri = slot * ntop + t;
        long cu = (long)(N2 - 1 - m) * NX + (N2 + xi), cd = (long)(NZ - N2 + m) * NX + (N2 + xi);
        if (dir) { u[cu] = up[ri]; u[cd] = dw[ri]; }
        else     { up[ri] = u[cu]; dw[ri] = u[cd]; }
    }
}

__global__ void k_deliver(float *__restrict__ u1, float *__restrict__ u0,
                          const float *__restrict__ u2, int NZ, int NX, int lo)
{
    int x = blockIdx.x * BX + threadIdx.x, z = blockIdx.y * BY + threadIdx.y;
    if (z < lo || z >= NZ - lo || x < lo || x >= NX - lo) return;
    long i = (long)z * NX + x;
    u0[i] = u1[i];
    u1[i] = u2[i];
}

// kernel.cu:489-517: S is the source wavefield, R the receiver wavefield.
template <bool COMPEN>
__global__ void k_rel(const float *__restrict__ S, const float *__restrict__ R,
                      float *__restrict__ Sacc, float *__restrict__ Racc, float *__restrict__ rel1,
                      float *__restrict__ rel2, long n)
{
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float s = S[i], r = R[i];
    if (COMPEN) {
        float sa = Sacc[i] + s, ra = Racc[i] + r;
        Sacc[i] = sa;
        Racc[i] = ra;
        rel1[i] += ra * sa;
    } else {
        rel1[i] += r * s;
    }
    rel2[i] += s * s;
}

int check_grid(int NZ, int NX, int N2, int M)
{
    if (NZ <= 2 * N2 || NX <= 2 * N2 || N2 < 2 || M < 0 || M > N2 || NZ < 3 || NX < 3) {
        rtm_set_last_error("invalid grid: need NZ,NX > 2*N2, N2 >= 2, 0 <= nfdmax <= N2");
        return RTM_ERR_ARG;
    }
    return RTM_OK;
}

inline unsigned blocks_for(long n, int t) { return (unsigned)((n + t - 1) / t); }

} // namespace

extern "C" {

int rtm_k_Equal(float *Dlf, float *Drt, float *Dup, float *Ddw, float *DFW0, float *DFW1, int NZ,
                int NX, int N2, int nfdmax, rtm_stream_t s)
{
    if (int rc = check_grid(NZ, NX, N2, nfdmax)) return rc;
    long n = (long)nfdmax * ((NZ - 2 * N2) + (NX - 2 * N2));
    if (n == 0) return RTM_OK;
    k_ring<<<blocks_for(n, 256), 256, 0, s>>>(Dlf, Drt, Dup, Ddw, DFW0, NZ, NX, N2, nfdmax, 0, 0);
    k_ring<<<blocks_for(n, 256), 256, 0, s>>>(Dlf, Drt, Dup, Ddw, DFW1, NZ, NX, N2, nfdmax, 1, 0);
    RTM_LAUNCH_CHECK();
    return RTM_OK;
}

int rtm_k_Add(float *Dv, float *DFW2, float *DFW0, float *DFW1, float *Dc, int *DIndex, float tao2,
              float h2, float vmin, float dv, int nfdmax, int NZ, int NX, int NXZ, int r_u, int r_x,
              float wavelet, float hzx2_1, rtm_stream_t s)
{
    (void)NXZ;
    if (NZ < 3 || NX < 3) return RTM_ERR_ARG;
    k_add<true, ST_FULL><<<grid_cells(NZ, NX), dim3(BX, BY), 0, s>>>(
        Dv, DFW2, DFW0, DFW1, Dc, DIndex, tao2, h2, vmin, dv, nfdmax, 0, NZ, NX, r_u, r_x, wavelet,
        hzx2_1);
    RTM_LAUNCH_CHECK();
    return RTM_OK;
}

int rtm_k_Add_Con(float *Dv, float *DFW2, float *DFW0, float *DFW1, float *Dc, float tao2, float h2,
                  int nfdmax, int NZ, int NX, int NXZ, int r_u, int r_x, float wavelet,
                  float hzx2_1, rtm_stream_t s)
{
    (void)NXZ;
    if (NZ < 3 || NX < 3) return RTM_ERR_ARG;
    k_add<false, ST_FULL><<<grid_cells(NZ, NX), dim3(BX, BY), 0, s>>>(
        Dv, DFW2, DFW0, DFW1, Dc, nullptr, tao2, h2, 0.f, 1.f, nfdmax, 0, NZ, NX, r_u, r_x, wavelet,
        hzx2_1);
    RTM_LAUNCH_CHECK();
    return RTM_OK;
}

int rtm_k_Hybrid1(float *DFW1, float *DFW0, float *DFW2, float *DFWb, float *Dlf, float *Drt,
                  float *Dup, float *Ddw, float *Dv, float *Dr_1, float *Dw, int NZ, int NX, int N2,
                  int nfdmax, int k, float taoh, float taoh2, rtm_stream_t s)
{
    (void)Dlf; (void)Drt; (void)Dup; (void)Ddw; (void)Dw; (void)k;
    if (int rc = check_grid(NZ, NX, N2, nfdmax)) return rc;
    long n = abc_count(NZ, NX, N2);
    k_hybrid1<<<blocks_for(n, 256), 256, 0, s>>>(DFW1, DFW0, DFW2, DFWb, Dv, Dr_1, NZ, NX, N2, taoh,
                                                 taoh2);
    RTM_LAUNCH_CHECK();
    return RTM_OK;
}

int rtm_k_Hybrid2(float *DFW1, float *DFW0, float *DFW2, float *DFWb, float *Dlf, float *Drt,
                  float *Dup, float *Ddw, float *Dv, float *Dr_1, float *Dw, int NZ, int NX, int N2,
                  int nfdmax, int k, float taoh, float taoh2, rtm_stream_t s)
{
    (void)DFW1; (void)DFW0; (void)Dlf; (void)Drt; (void)Dup; (void)Ddw; (void)Dv; (void)Dr_1;
    (void)k; (void)taoh; (void)taoh2;
    if (int rc = check_grid(NZ, NX, N2, nfdmax)) return rc;
    long n = abc_count(NZ, NX, N2);
    k_hybrid2<<<blocks_for(n, 256), 256, 0, s>>>(DFW2, DFWb, Dw, NZ, NX, N2);
    RTM_LAUNCH_CHECK();
    return RTM_OK;
}

int rtm_k_Hybrid3(float *DFW1, float *DFW0, float *DFW2, float *DFWb, float *Dlf, float *Drt,
                  float *Dup, float *Ddw, float *Dv, float *Dr_1, float *Dw, int NZ, int NX, int N2,
                  int nfdmax, int k, float taoh, float taoh2, rtm_stream_t s)
{
    (void)DFW1; (void)DFW0; (void)DFWb; (void)Dv; (void)Dr_1; (void)Dw; (void)taoh; (void)taoh2;
    if (int rc = check_grid(NZ, NX, N2, nfdmax)) return rc;
    long n = (long)nfdmax * ((NZ - 2 * N2) + (NX - 2 * N2));
    if (n == 0) return RTM_OK;
    k_ring<<<blocks_for(n, 256), 256, 0, s>>>(Dlf, Drt, Dup, Ddw, DFW2, NZ, NX, N2, nfdmax, k, 0);
    RTM_LAUNCH_CHECK();
    return RTM_OK;
}

int rtm_k_Deliver(float *DFW1, float *DFW0, float *DFW2, int NZ, int NX, rtm_stream_t s)
{
    if (NZ < 1 || NX < 1) return RTM_ERR_ARG;
    k_deliver<<<grid_cells(NZ, NX), dim3(BX, BY), 0, s>>>(DFW1, DFW0, DFW2, NZ, NX, 0);
    RTM_LAUNCH_CHECK();
    return RTM_OK;
}

int rtm_k_BKEqual(float *Dlf, float *Drt, float *Dup, float *Ddw, float *DFW1, int NZ, int NX,
                  int N2, int nfdmax, int k, rtm_stream_t s)
{
    if (int rc = check_grid(NZ, NX, N2, nfdmax)) return rc;
    long n = (long)nfdmax * ((NZ - 2 * N2) + (NX - 2 * N2));
    if (n == 0) return RTM_OK;
    k_ring<<<blocks_for(n, 256), 256, 0, s>>>(Dlf, Drt, Dup, Ddw, DFW1, NZ, NX, N2, nfdmax,
                                              (long)k + 1, 1);
    RTM_LAUNCH_CHECK();
    return RTM_OK;
}

int rtm_k_BKAdd_EFF(float *Dv, float *DFW2, float *DFW0, float *DFW1, float *Dc, int *DIndex,
                    float tao2, float h2, float vmin, float dv, int N2, int NZ, int NX, int NXZ,
                    int r_u, int r_x, float wavelet, float hzx2_1, rtm_stream_t s)
{
    (void)NXZ;
    if (NZ <= 2 * N2 || NX <= 2 * N2) return RTM_ERR_ARG;
    k_add<true, ST_INTERIOR><<<grid_cells(NZ, NX), dim3(BX, BY), 0, s>>>(
        Dv, DFW2, DFW0, DFW1, Dc, DIndex, tao2, h2, vmin, dv, 0, N2, NZ, NX, r_u, r_x, wavelet,
        hzx2_1);
    RTM_LAUNCH_CHECK();
    return RTM_OK;
}

int rtm_k_BKAdd_EFF_Con(float *Dv, float *DFW2, float *DFW0, float *DFW1, float *Dc, float tao2,
                        float h2, int N2, int NZ, int NX, int NXZ, int r_u, int r_x, int nfdmax,
                        float wavelet, float hzx2_1, rtm_stream_t s)
{
    (void)NXZ;
    if (NZ <= 2 * N2 || NX <= 2 * N2) return RTM_ERR_ARG;
    k_add<false, ST_INTERIOR><<<grid_cells(NZ, NX), dim3(BX, BY), 0, s>>>(
        Dv, DFW2, DFW0, DFW1, Dc, nullptr, tao2, h2, 0.f, 1.f, nfdmax, N2, NZ, NX, r_u, r_x,
        wavelet, hzx2_1);
    RTM_LAUNCH_CHECK();
    return RTM_OK;
}

int rtm_k_Deliver_EFF(float *DFW1, float *DFW0, float *DFW2, int N2, int NZ, int NX,
                      rtm_stream_t s)
{
    if (NZ <= 2 * N2 || NX <= 2 * N2) return RTM_ERR_ARG;
    k_deliver<<<grid_cells(NZ, NX), dim3(BX, BY), 0, s>>>(DFW1, DFW0, DFW2, NZ, NX, N2);
    RTM_LAUNCH_CHECK();
    return RTM_OK;
}

int rtm_k_BKAdd(float *Dv, float *DBW2, float *DBW1, float *DBW0, float *Dc, int *DIndex,
                float *Dseis, float tao2, float h2, float vmin, float dv, int nfdmax, int NZ,
                int NX, int NXZ, int s_l, int s_r, int s_z, int ds, float hzx2_1, rtm_stream_t s)
{
    (void)NXZ;
    if (NZ < 3 || NX < 3 || ds < 1) return RTM_ERR_ARG;
    k_bkadd<true><<<grid_cells(NZ, NX), dim3(BX, BY), 0, s>>>(Dv, DBW2, DBW1, DBW0, Dc, DIndex,
                                                               Dseis, tao2, h2, vmin, dv, nfdmax, NZ,
                                                               NX, s_l, s_r, s_z, ds, hzx2_1);
    RTM_LAUNCH_CHECK();
    return RTM_OK;
}

int rtm_k_BKAdd_Con(float *Dv, float *DBW2, float *DBW1, float *DBW0, float *Dc, float *Dseis,
                    float tao2, float h2, int nfdmax, int NZ, int NX, int NXZ, int s_l, int s_r,
                    int s_z, int ds, float hzx2_1, rtm_stream_t s)
{
    (void)NXZ;
    if (NZ < 3 || NX < 3 || ds < 1) return RTM_ERR_ARG;
    k_bkadd<false><<<grid_cells(NZ, NX), dim3(BX, BY), 0, s>>>(Dv, DBW2, DBW1, DBW0, Dc, nullptr,
                                                                Dseis, tao2, h2, 0.f, 1.f, nfdmax,
                                                                NZ, NX, s_l, s_r, s_z, ds, hzx2_1);
    RTM_LAUNCH_CHECK();
    return RTM_OK;
}

int rtm_k_BKHybrid1(float *DFW1, float *DFW0, float *DFW2, float *DFWb, float *Dv, float *Dr_1,
                    float *Dw, int NZ, int NX, int N2, float taoh, float taoh2, rtm_stream_t s)
{
    (void)Dw;
    if (int rc = check_grid(NZ, NX, N2, 0)) return rc;
    long n = abc_count(NZ, NX, N2);
    k_hybrid1<<<blocks_for(n, 256), 256, 0, s>>>(DFW1, DFW0, DFW2, DFWb, Dv, Dr_1, NZ, NX, N2, taoh,
                                                 taoh2);
    RTM_LAUNCH_CHECK();
    return RTM_OK;
}

int rtm_k_BKHybrid2(float *DFW1, float *DFW0, float *DFW2, float *DFWb, float *Dv, float *Dr_1,
                    float *Dw, int NZ, int NX, int N2, float taoh, float taoh2, rtm_stream_t s)
{
    (void)DFW1; (void)DFW0; (void)Dv; (void)Dr_1; (void)taoh; (void)taoh2;
    if (int rc = check_grid(NZ, NX, N2, 0)) return rc;
    long n = abc_count(NZ, NX, N2);
    k_hybrid2<<<blocks_for(n, 256), 256, 0, s>>>(DFW2, DFWb, Dw, NZ, NX, N2);
    RTM_LAUNCH_CHECK();
    return RTM_OK;
}

int rtm_k_Rel_NonCompen(float *DBW2, float *DFW2, float *Drel1, float *Drel2, int NZ, int NX,
                        rtm_stream_t s)
{
    // The reference's parameter named DFW2 carries the source wavefield and
    // DBW2 the receiver wavefield (kernel.cu:925-929 passes them that way).
    long n = (long)NZ * NX;
    if (n <= 0) return RTM_ERR_ARG;
    k_rel<false><<<blocks_for(n, 256), 256, 0, s>>>(DFW2, DBW2, nullptr, nullptr, Drel1, Drel2, n);
    RTM_LAUNCH_CHECK();
    return RTM_OK;
}

int rtm_k_Rel_Compen(float *DBW2, float *DFW2, float *DBWADD, float *DFWADD, float *Drel1,
                     float *Drel2, int NZ, int NX, rtm_stream_t s)
{
    long n = (long)NZ * NX;
    if (n <= 0) return RTM_ERR_ARG;
    // Parameter DFWADD accumulates DFW2 (source), DBWADD accumulates DBW2.
    k_rel<true><<<blocks_for(n, 256), 256, 0, s>>>(DFW2, DBW2, DFWADD, DBWADD, Drel1, Drel2, n);
    RTM_LAUNCH_CHECK();
    return RTM_OK;
}

} // extern "C"

// ---------------------------------------------------------------------------
// The reference's per-shot loop (kernel.cu:798-933) on the drop-in kernels:
// 5 launches per forward step, 8 launches and one synchronous host-to-device
// copy of the step's trace samples per backward step, on the legacy default
// stream -- the "plain single-shot GPU drop-in" the batched engine is
// measured against.  Host inputs/outputs; device buffers are allocated and
// freed here.  The receivers are the problem's line (rdz == 0).
namespace {

template <class T>
struct DevArr {
    T *p = nullptr;
    ~DevArr()
    {
        if (p) cudaFree(p);
    }
    int alloc(size_t n)
    {
        if (cudaMalloc(&p, sizeof(T) * (n ? n : 1)) != cudaSuccess) {
            cudaGetLastError();
            rtm_set_last_error("cudaMalloc failed");
            return RTM_ERR_NOMEM;
        }
        if (cudaMemset(p, 0, sizeof(T) * (n ? n : 1)) != cudaSuccess) {
            rtm_set_last_error("cudaMemset failed");
            return RTM_ERR_CUDA;
        }
        return RTM_OK;
    }
};

}  // namespace

extern "C" int rtm_plain_migrate_shot(const rtm_problem *p, int src_cell, const float *seis,
                                      float *rel1, float *rel2)
{
    if (!p || !seis || !rel1 || !rel2 || p->rdz != 0 || p->rdx < 1 || p->nrec < 1) return RTM_ERR_ARG;
    const int N2 = p->N2, M = p->M, NT = p->NT;
    const int NZ = p->nz + 2 * N2, NX = p->nx + 2 * N2, nz = p->nz, nx = p->nx;
    if (int rc = check_grid(NZ, NX, N2, M)) return rc;
    const long nxz = (long)NZ * NX;
    const size_t gb = sizeof(float) * nxz;
    const int r_u = src_cell / NX, r_x = src_cell % NX;
    const int s_l = p->rx0, s_z = p->rz0, ds = p->rdx, n = p->nrec, s_r = (n - 1) * ds + s_l;
    DevArr<float> FW0, FW1, FW2, FWb, BW0, BW1, BW2, FA, BA, R1, R2, v, r1, w, c, lf, rt, up, dw, sd;
    DevArr<int> idx;
    int rc;
    DevArr<float> *g[] = {&FW0, &FW1, &FW2, &FWb, &BW0, &BW1, &BW2, &FA, &BA, &R1, &R2, &v, &r1};
    for (auto *a : g)
        if ((rc = a->alloc(nxz))) return rc;
    const int nc = p->adaptive ? p->index[p->nbins] : M + 1;
    if ((rc = w.alloc(N2 + 1)) || (rc = c.alloc(nc)) || (rc = idx.alloc(p->adaptive ? p->nbins + 1 : 1)) ||
        (rc = lf.alloc((size_t)M * nz * NT)) || (rc = rt.alloc((size_t)M * nz * NT)) ||
        (rc = up.alloc((size_t)M * nx * NT)) || (rc = dw.alloc((size_t)M * nx * NT)) ||
        (rc = sd.alloc(n)))
        return rc;
    RTM_CUDA_TRY(cudaMemcpy(v.p, p->v, gb, cudaMemcpyHostToDevice));
    RTM_CUDA_TRY(cudaMemcpy(r1.p, p->r1, gb, cudaMemcpyHostToDevice));
    RTM_CUDA_TRY(cudaMemcpy(w.p, p->w, sizeof(float) * (N2 + 1), cudaMemcpyHostToDevice));
    RTM_CUDA_TRY(cudaMemcpy(c.p, p->coef, sizeof(float) * nc, cudaMemcpyHostToDevice));
    if (p->adaptive)
        RTM_CUDA_TRY(cudaMemcpy(idx.p, p->index, sizeof(int) * (p->nbins + 1), cudaMemcpyHostToDevice));
    const float spike = p->spike;
    RTM_CUDA_TRY(cudaMemcpy(FW1.p + (long)r_u * NX + r_x, &spike, sizeof(float), cudaMemcpyHostToDevice));
    const float tao2 = p->tao2, h2 = p->h2, vmin = p->vmin, dv = p->dv, hzx2_1 = p->hzx2_1;
    const float taoh = p->taoh, taoh2 = p->taoh2;
#define TRYK(x)                      \
    do {                             \
        if ((rc = (x)) != RTM_OK) return rc; \
    } while (0)
    TRYK(rtm_k_Equal(lf.p, rt.p, up.p, dw.p, FW0.p, FW1.p, NZ, NX, N2, M, nullptr));
    for (int k = 2; k < NT; ++k) {
        const float wav = (k < p->NT2) ? p->wav[k - 1] : 0.0f;
        if (p->adaptive)
            TRYK(rtm_k_Add(v.p, FW2.p, FW0.p, FW1.p, c.p, idx.p, tao2, h2, vmin, dv, M, NZ, NX, (int)nxz,
                           r_u, r_x, wav, hzx2_1, nullptr));
        else
            TRYK(rtm_k_Add_Con(v.p, FW2.p, FW0.p, FW1.p, c.p, tao2, h2, M, NZ, NX, (int)nxz, r_u, r_x, wav,
                               hzx2_1, nullptr));
        TRYK(rtm_k_Hybrid1(FW1.p, FW0.p, FW2.p, FWb.p, lf.p, rt.p, up.p, dw.p, v.p, r1.p, w.p, NZ, NX, N2,
                           M, k, taoh, taoh2, nullptr));
        TRYK(rtm_k_Hybrid2(FW1.p, FW0.p, FW2.p, FWb.p, lf.p, rt.p, up.p, dw.p, v.p, r1.p, w.p, NZ, NX, N2,
                           M, k, taoh, taoh2, nullptr));
        TRYK(rtm_k_Hybrid3(FW1.p, FW0.p, FW2.p, FWb.p, lf.p, rt.p, up.p, dw.p, v.p, r1.p, w.p, NZ, NX, N2,
                           M, k, taoh, taoh2, nullptr));
        TRYK(rtm_k_Deliver(FW1.p, FW0.p, FW2.p, NZ, NX, nullptr));
    }
    // hand-off (kernel.cu:822-825) and image initialisation (:859-885)
    RTM_CUDA_TRY(cudaMemcpy(BW0.p, FW1.p, gb, cudaMemcpyDeviceToDevice));
    RTM_CUDA_TRY(cudaMemcpy(BW1.p, FW0.p, gb, cudaMemcpyDeviceToDevice));
    {
        std::vector<float> b0(nxz), b1(nxz), m1(nxz), m2(nxz), ba(nxz, 0.0f), fa(nxz, 0.0f);
        RTM_CUDA_TRY(cudaMemcpy(b0.data(), BW0.p, gb, cudaMemcpyDeviceToHost));
        RTM_CUDA_TRY(cudaMemcpy(b1.data(), BW1.p, gb, cudaMemcpyDeviceToHost));
        const long src = (long)r_u * NX + r_x;
        for (long i = 0; i < nxz; ++i) {
            const float h0 = 0.0f, h1 = (i == src) ? spike : 0.0f;
            if (p->compen) {
                ba[i] = b0[i] + b1[i];
                fa[i] = h0 + h1;
                m1[i] = fa[i] * ba[i] + h0 * b0[i];
            } else {
                m1[i] = h1 * b1[i] + h0 * b0[i];
            }
            m2[i] = b1[i] * b1[i] + b0[i] * b0[i];
        }
        RTM_CUDA_TRY(cudaMemcpy(R1.p, m1.data(), gb, cudaMemcpyHostToDevice));
        RTM_CUDA_TRY(cudaMemcpy(R2.p, m2.data(), gb, cudaMemcpyHostToDevice));
        RTM_CUDA_TRY(cudaMemcpy(BA.p, ba.data(), gb, cudaMemcpyHostToDevice));
        RTM_CUDA_TRY(cudaMemcpy(FA.p, fa.data(), gb, cudaMemcpyHostToDevice));
        RTM_CUDA_TRY(cudaMemcpy(FW2.p, fa.data(), gb, cudaMemcpyHostToDevice));
        RTM_CUDA_TRY(cudaMemset(FW0.p, 0, gb));
        RTM_CUDA_TRY(cudaMemset(FW1.p, 0, gb));
        RTM_CUDA_TRY(cudaMemset(FWb.p, 0, gb));
    }
    std::vector<float> cs(n);
    for (int k = NT - 3; k >= 0; --k) {
        const float wav = (k < p->NT2) ? p->wav[k + 1] : 0.0f;
        TRYK(rtm_k_BKEqual(lf.p, rt.p, up.p, dw.p, BW1.p, NZ, NX, N2, M, k, nullptr));
        if (p->adaptive)
            TRYK(rtm_k_BKAdd_EFF(v.p, BW2.p, BW0.p, BW1.p, c.p, idx.p, tao2, h2, vmin, dv, N2, NZ, NX,
                                 (int)nxz, r_u, r_x, wav, hzx2_1, nullptr));
        else
            TRYK(rtm_k_BKAdd_EFF_Con(v.p, BW2.p, BW0.p, BW1.p, c.p, tao2, h2, N2, NZ, NX, (int)nxz, r_u,
                                     r_x, M, wav, hzx2_1, nullptr));
        TRYK(rtm_k_Deliver_EFF(BW1.p, BW0.p, BW2.p, N2, NZ, NX, nullptr));
        for (int j = 0; j < n; ++j) cs[j] = seis[(long)j * NT + k + 1];
        RTM_CUDA_TRY(cudaMemcpy(sd.p, cs.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
        if (p->adaptive)
            TRYK(rtm_k_BKAdd(v.p, FW2.p, FW1.p, FW0.p, c.p, idx.p, sd.p, tao2, h2, vmin, dv, M, NZ, NX,
                             (int)nxz, s_l, s_r, s_z, ds, hzx2_1, nullptr));
        else
            TRYK(rtm_k_BKAdd_Con(v.p, FW2.p, FW1.p, FW0.p, c.p, sd.p, tao2, h2, M, NZ, NX, (int)nxz, s_l,
                                 s_r, s_z, ds, hzx2_1, nullptr));
        TRYK(rtm_k_BKHybrid1(FW1.p, FW0.p, FW2.p, FWb.p, v.p, r1.p, w.p, NZ, NX, N2, taoh, taoh2, nullptr));
        TRYK(rtm_k_BKHybrid2(FW1.p, FW0.p, FW2.p, FWb.p, v.p, r1.p, w.p, NZ, NX, N2, taoh, taoh2, nullptr));
        TRYK(rtm_k_Deliver(FW1.p, FW0.p, FW2.p, NZ, NX, nullptr));
        if (p->compen)
            TRYK(rtm_k_Rel_Compen(FW2.p, BW2.p, FA.p, BA.p, R1.p, R2.p, NZ, NX, nullptr));
        else
            TRYK(rtm_k_Rel_NonCompen(FW2.p, BW2.p, R1.p, R2.p, NZ, NX, nullptr));
    }
#undef TRYK
    RTM_CUDA_TRY(cudaMemcpy(rel1, R1.p, gb, cudaMemcpyDeviceToHost));
    RTM_CUDA_TRY(cudaMemcpy(rel2, R2.p, gb, cudaMemcpyDeviceToHost));
    return RTM_OK;
}
