/*
 * Runs the reference's own GPU kernels on the GPU, as a yardstick and a
 * parity target.  TEST INFRASTRUCTURE ONLY (tests/ and bench.py's reference
 * arm load it; the product never does).
 *
 * build_ref.py compiles this file with nvcc into oracle/_ref/libref_gpu.so
 * together with the unchanged __global__ kernels of kernel.cu (the block from
 * "#define BLOCKSIZE 16" up to the Ricker prototype, kernel.cu:15-517, copied
 * verbatim into the git-ignored oracle/_ref/ref_kernels.inc).  The host code
 * below restates the per-shot sequence of the reference's main()
 * (kernel.cu:788-933) on those kernels: the stock launch shape
 * dim3(16,16) over ceil(NZ/16) x ceil(NX/16) blocks on the default stream,
 * the host-side hand-off and image initialisation with their synchronous
 * copies, and one synchronous host-to-device copy of the receiver samples
 * per backward step.  Device buffers are allocated and freed per call, as
 * the reference allocates them once per run; they are zero-filled after
 * allocation (the reference never writes the pad of DBW2 and reads it in
 * Rel_Compen, which a fresh allocation holds as zero).
 */
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "ref_kernels.inc" /* generated from kernel.cu */

extern "C" {
#include "rtm_oracle.h"
}

namespace {

struct Dev {
    std::vector<void *> ptrs;
    bool ok = true;
    template <class T>
    T *alloc(size_t n)
    {
        void *p = nullptr;
        if (cudaMalloc(&p, (n ? n : 1) * sizeof(T)) != cudaSuccess) {
            ok = false;
            return nullptr;
        }
        cudaMemset(p, 0, (n ? n : 1) * sizeof(T));
        ptrs.push_back(p);
        return static_cast<T *>(p);
    }
    ~Dev()
    {
        for (void *p : ptrs) cudaFree(p);
    }
};

// Receivers given as a cell list (the generalisation the oracle's driver
// makes for geometries the reference's line cannot express, e.g. a vertical
// well, rtm_driver_body.h): after BKAdd, each listed cell takes its sample
// when the sample is non-zero, as the line rule does (kernel.cu:351-353).
__global__ void refgpu_inject_list(float *u, const int *cells, const float *seis, int n)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n && seis[j] != 0.0f) u[cells[j]] = seis[j];
}

}  // namespace

extern "C" {

/* One migration (kernel.cu:798-933) on the reference's kernels.  Inputs as
 * or_migrate_f32 (oracle/rtm_oracle.h) plus the bin count nvel (DIndex holds
 * nvel+1 offsets) and the length of the coefficient table c.  Receivers are
 * the reference's line (s_l, s_r, s_z, ds, n) or, when P->rec_cells is set,
 * a cell list injected after BKAdd by the line's rule.  rel1 / rel2: full padded grids.
 * seconds: wall-clock time of the shot (first launch to last copy back).
 * Returns 0, or -1 on a CUDA error / unsupported geometry. */
int refgpu_migrate(const or_params *P, const float *v, const float *r1, const float *w,
                   const float *c, const int *idx, int nvel, int ncoef, const float *wav,
                   const float *seis, float *rel1, float *rel2, double *seconds)
{
    const bool list = P->rec_cells != nullptr;
    const int n = list ? P->nrec_list : P->n;
    if (n < 1) return -1;
    const int NZ = P->NZ, NX = P->NX, N2 = P->N2, nfdmax = P->M, NT = P->NT;
    const long NXZ = (long)NZ * NX;
    const int nz = NZ - 2 * N2, nx = NX - 2 * N2;
    const size_t sizeLF = (size_t)nfdmax * nz * NT, sizeUP = (size_t)nfdmax * nx * NT;
    const int nvel1 = P->adaptive ? nvel + 1 : 1;
    const int nc = ncoef;

    Dev d;
    float *DFWADD = d.alloc<float>(NXZ), *DFW2 = d.alloc<float>(NXZ), *DFW1 = d.alloc<float>(NXZ);
    float *DFW0 = d.alloc<float>(NXZ), *DFWb = d.alloc<float>(NXZ), *DBWADD = d.alloc<float>(NXZ);
    float *DBW2 = d.alloc<float>(NXZ), *DBW1 = d.alloc<float>(NXZ), *DBW0 = d.alloc<float>(NXZ);
    float *Dv = d.alloc<float>(NXZ), *Dr_1 = d.alloc<float>(NXZ), *Dw = d.alloc<float>(N2 + 1);
    float *Dc = d.alloc<float>(nc), *Drel1 = d.alloc<float>(NXZ), *Drel2 = d.alloc<float>(NXZ);
    float *Dseis = d.alloc<float>(n);
    int *Dcells = d.alloc<int>(list ? n : 1);
    int *DIndex = d.alloc<int>(nvel1);
    float *Dlf = d.alloc<float>(sizeLF), *Drt = d.alloc<float>(sizeLF);
    float *Dup = d.alloc<float>(sizeUP), *Ddw = d.alloc<float>(sizeUP);
    if (!d.ok) return -1;
    const size_t size = sizeof(float) * NXZ;
    cudaMemcpy(Dv, v, size, cudaMemcpyHostToDevice);
    cudaMemcpy(Dr_1, r1, size, cudaMemcpyHostToDevice);
    cudaMemcpy(Dw, w, sizeof(float) * (N2 + 1), cudaMemcpyHostToDevice);
    cudaMemcpy(Dc, c, sizeof(float) * nc, cudaMemcpyHostToDevice);
    if (P->adaptive) cudaMemcpy(DIndex, idx, sizeof(int) * nvel1, cudaMemcpyHostToDevice);
    if (list) cudaMemcpy(Dcells, P->rec_cells, sizeof(int) * n, cudaMemcpyHostToDevice);
    if (cudaDeviceSynchronize() != cudaSuccess) return -1;

    std::vector<float> FW0(NXZ, 0.f), FW1(NXZ, 0.f), FW2(NXZ), FWb(NXZ, 0.f), BW0(NXZ), BW1(NXZ),
        BW2(NXZ), MIG1(NXZ), MIG2(NXZ), Cseis(n);
    dim3 blockDim(BLOCKSIZE, BLOCKSIZE);
    dim3 gridDim((NZ + blockDim.x - 1) / blockDim.x, (NX + blockDim.y - 1) / blockDim.y);
    const float tao2 = P->tao2, h2 = P->h2, vmin = P->vmin, dv = P->dv, hzx2_1 = P->hzx2_1;
    const float taoh = P->taoh, taoh2 = P->taoh2;
    const int r_u = P->r_u, r_x = P->r_x, s_l = P->s_l, s_r = P->s_r, s_z = P->s_z, ds = P->ds;

    auto t0 = std::chrono::steady_clock::now();
    FW1[(long)r_u * NX + r_x] = P->spike;
    cudaMemcpy(DFW0, FW0.data(), size, cudaMemcpyHostToDevice);
    cudaMemcpy(DFW1, FW1.data(), size, cudaMemcpyHostToDevice);
    Equal<<<gridDim, blockDim>>>(Dlf, Drt, Dup, Ddw, DFW0, DFW1, NZ, NX, N2, nfdmax);
    for (int k = 2; k < NT; ++k) {
        const float wavelet = (k < P->NT2) ? wav[k - 1] : 0.0f;
        if (P->adaptive)
            Add<<<gridDim, blockDim>>>(Dv, DFW2, DFW0, DFW1, Dc, DIndex, tao2, h2, vmin, dv, nfdmax, NZ,
                                       NX, (int)NXZ, r_u, r_x, wavelet, hzx2_1);
        else
            Add_Con<<<gridDim, blockDim>>>(Dv, DFW2, DFW0, DFW1, Dc, tao2, h2, nfdmax, NZ, NX, (int)NXZ,
                                           r_u, r_x, wavelet, hzx2_1);
        Hybrid1<<<gridDim, blockDim>>>(DFW1, DFW0, DFW2, DFWb, Dlf, Drt, Dup, Ddw, Dv, Dr_1, Dw, NZ, NX,
                                       N2, nfdmax, k, taoh, taoh2);
        Hybrid2<<<gridDim, blockDim>>>(DFW1, DFW0, DFW2, DFWb, Dlf, Drt, Dup, Ddw, Dv, Dr_1, Dw, NZ, NX,
                                       N2, nfdmax, k, taoh, taoh2);
        Hybrid3<<<gridDim, blockDim>>>(DFW1, DFW0, DFW2, DFWb, Dlf, Drt, Dup, Ddw, Dv, Dr_1, Dw, NZ, NX,
                                       N2, nfdmax, k, taoh, taoh2);
        Deliver<<<gridDim, blockDim>>>(DFW1, DFW0, DFW2, NZ, NX);
    }
    cudaMemcpy(BW0.data(), DFW1, size, cudaMemcpyDeviceToHost);
    cudaMemcpy(BW1.data(), DFW0, size, cudaMemcpyDeviceToHost);
    cudaMemcpy(DBW1, BW1.data(), size, cudaMemcpyHostToDevice);
    cudaMemcpy(DBW0, BW0.data(), size, cudaMemcpyHostToDevice);
    /* kernel.cu:859-885: the host forward arrays still hold the start state */
    for (long i = 0; i < NXZ; ++i) {
        FWb[i] = 0.0f;
        if (P->compen) {
            BW2[i] = BW0[i] + BW1[i];
            FW2[i] = FW0[i] + FW1[i];
            MIG1[i] = FW2[i] * BW2[i] + FW0[i] * BW0[i];
            MIG2[i] = BW1[i] * BW1[i] + BW0[i] * BW0[i];
        } else {
            BW2[i] = 0.0f;
            FW2[i] = 0.0f;
            MIG1[i] = FW1[i] * BW1[i] + FW0[i] * BW0[i];
            MIG2[i] = BW1[i] * BW1[i] + BW0[i] * BW0[i];
        }
    }
    cudaMemcpy(DFW2, FW2.data(), size, cudaMemcpyHostToDevice);
    cudaMemcpy(DFWb, FWb.data(), size, cudaMemcpyHostToDevice);
    cudaMemcpy(DFW0, FWb.data(), size, cudaMemcpyHostToDevice);
    cudaMemcpy(DFW1, FWb.data(), size, cudaMemcpyHostToDevice);
    cudaMemcpy(DFWADD, FW2.data(), size, cudaMemcpyHostToDevice);
    cudaMemcpy(DBWADD, BW2.data(), size, cudaMemcpyHostToDevice);
    cudaMemcpy(Drel1, MIG1.data(), size, cudaMemcpyHostToDevice);
    cudaMemcpy(Drel2, MIG2.data(), size, cudaMemcpyHostToDevice);
    for (int k = NT - 3; k >= 0; --k) {
        const float wavelet = (k < P->NT2) ? wav[k + 1] : 0.0f;
        BKEqual<<<gridDim, blockDim>>>(Dlf, Drt, Dup, Ddw, DBW1, NZ, NX, N2, nfdmax, k);
        if (P->adaptive)
            BKAdd_EFF<<<gridDim, blockDim>>>(Dv, DBW2, DBW0, DBW1, Dc, DIndex, tao2, h2, vmin, dv, N2, NZ,
                                             NX, (int)NXZ, r_u, r_x, wavelet, hzx2_1);
        else
            BKAdd_EFF_Con<<<gridDim, blockDim>>>(Dv, DBW2, DBW0, DBW1, Dc, tao2, h2, N2, NZ, NX, (int)NXZ,
                                                 r_u, r_x, nfdmax, wavelet, hzx2_1);
        Deliver_EFF<<<gridDim, blockDim>>>(DBW1, DBW0, DBW2, N2, NZ, NX);
        for (int j = 0; j < n; ++j) Cseis[j] = seis[(long)j * NT + k + 1];
        cudaMemcpy(Dseis, Cseis.data(), sizeof(float) * n, cudaMemcpyHostToDevice);
        if (P->adaptive)
            BKAdd<<<gridDim, blockDim>>>(Dv, DFW2, DFW1, DFW0, Dc, DIndex, Dseis, tao2, h2, vmin, dv,
                                         nfdmax, NZ, NX, (int)NXZ, s_l, s_r, s_z, ds, hzx2_1);
        else
            BKAdd_Con<<<gridDim, blockDim>>>(Dv, DFW2, DFW1, DFW0, Dc, Dseis, tao2, h2, nfdmax, NZ, NX,
                                             (int)NXZ, s_l, s_r, s_z, ds, hzx2_1);
        if (list) refgpu_inject_list<<<(n + 127) / 128, 128>>>(DFW2, Dcells, Dseis, n);
        BKHybrid1<<<gridDim, blockDim>>>(DFW1, DFW0, DFW2, DFWb, Dv, Dr_1, Dw, NZ, NX, N2, taoh, taoh2);
        BKHybrid2<<<gridDim, blockDim>>>(DFW1, DFW0, DFW2, DFWb, Dv, Dr_1, Dw, NZ, NX, N2, taoh, taoh2);
        Deliver<<<gridDim, blockDim>>>(DFW1, DFW0, DFW2, NZ, NX);
        if (P->compen)
            Rel_Compen<<<gridDim, blockDim>>>(DFW2, DBW2, DFWADD, DBWADD, Drel1, Drel2, NZ, NX);
        else
            Rel_NonCompen<<<gridDim, blockDim>>>(DFW2, DBW2, Drel1, Drel2, NZ, NX);
    }
    cudaMemcpy(rel1, Drel1, size, cudaMemcpyDeviceToHost);
    cudaMemcpy(rel2, Drel2, size, cudaMemcpyDeviceToHost);
    const cudaError_t e = cudaDeviceSynchronize();
    auto t1 = std::chrono::steady_clock::now();
    if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
    if (e != cudaSuccess || cudaGetLastError() != cudaSuccess) {
        fprintf(stderr, "refgpu_migrate: %s\n", cudaGetErrorString(e));
        return -1;
    }
    return 0;
}

} /* extern "C" */
