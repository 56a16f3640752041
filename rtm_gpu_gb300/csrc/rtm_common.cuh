// Shared device/host helpers for the GB300 RTM kernels: status codes, the
// bounded-wait mbarrier and TMA (cp.async.bulk.tensor) wrappers, and the
// absorbing-boundary cell classification.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/rtm_gb300.h"

#define RTM_CUDA_TRY(expr)                                   \
    do {                                                     \
        cudaError_t e_ = (expr);                             \
        if (e_ != cudaSuccess) {                             \
            rtm_set_last_error(cudaGetErrorString(e_));      \
            return RTM_ERR_CUDA;                             \
        }                                                    \
    } while (0)

#define RTM_LAUNCH_CHECK()                                   \
    do {                                                     \
        cudaError_t e_ = cudaGetLastError();                 \
        if (e_ != cudaSuccess) {                             \
            rtm_set_last_error(cudaGetErrorString(e_));      \
            return RTM_ERR_CUDA;                             \
        }                                                    \
    } while (0)

void rtm_set_last_error(const char *msg);

#define RTM_DEVERR_TMA_TIMEOUT 1u

// Bounds of every spin on an mbarrier: at most RTM_SPIN_LIMIT polls and at
// most RTM_WAIT_NS nanoseconds of the GPU's global timer, whichever ends the
// wait first (try_wait suspends for a hardware-chosen interval per call, so
// the poll count alone gives no time bound).
#define RTM_SPIN_LIMIT (1u << 26)
#define RTM_WAIT_NS 2000000000ull

__device__ __forceinline__ unsigned smem_u32(const void *p)
{
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}

__device__ __forceinline__ void fence_barrier_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Waits for phase `parity` of the barrier, at most `limit` polls and
// RTM_WAIT_NS nanoseconds (the clock is read only once the first poll has
// failed, and then every 64 polls).  Returns false (and ORs
// RTM_DEVERR_TMA_TIMEOUT into *err) when a bound is hit, so a lost copy
// ends the kernel with an error instead of a hang.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, unsigned parity, unsigned *err,
                                                  unsigned limit = RTM_SPIN_LIMIT)
{
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    for (unsigned it = 1; it < limit; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 63u) == 0 && global_ns() - t0 > RTM_WAIT_NS) break;
    }
    atomicOr(err, RTM_DEVERR_TMA_TIMEOUT);
    return false;
}

// 3-D tiled TMA load of one box into shared memory, completing on `bar`.
// The innermost coordinate x must be a multiple of 4 (16 bytes of fp32).
__device__ __forceinline__ void tma_load_3d(void *smem_dst, const CUtensorMap *map, int x, int y,
                                            int z, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(smem_dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

// ---------------------------------------------------------------------------
// Absorbing-boundary (ABC) pad geometry.  With a = distance to the nearer of
// the top/bottom edges and e = distance to the nearer of the left/right edges,
// a pad cell takes the row-edge one-way update when e >= a+2, the column-edge
// update when a >= e+2 and the 45-degree corner update otherwise; its blend
// weight index is j = max(N2-z, N2-x, z-(NZ-N2)+1, x-(NX-N2)+1).  These are
// exactly the index sets of the reference's Hybrid1/Hybrid2 thread conditions
// (kernel.cu:116-183), verified by enumeration in the tests.

struct AbcCell {
    int z, x;
};

// Compact enumeration of the pad: top strip, bottom strip, then the left and
// right strips row by row (N2 left cells followed by N2 right cells).
__host__ __device__ __forceinline__ AbcCell abc_cell(long t, int NZ, int NX, int N2)
{
    AbcCell c;
    long top = (long)N2 * NX;
    if (t < top) {
        c.z = (int)(t / NX);
        c.x = (int)(t % NX);
    } else if (t < 2 * top) {
        t -= top;
        c.z = NZ - N2 + (int)(t / NX);
        c.x = (int)(t % NX);
    } else {
        t -= 2 * top;
        int r = (int)(t / (2 * N2)), q = (int)(t % (2 * N2));
        c.z = N2 + r;
        c.x = q < N2 ? q : NX - 2 * N2 + q;
    }
    return c;
}

__host__ __device__ __forceinline__ long abc_count(int NZ, int NX, int N2)
{
    return (long)NZ * NX - (long)(NZ - 2 * N2) * (NX - 2 * N2);
}

__host__ __device__ __forceinline__ bool is_pad(int z, int x, int NZ, int NX, int N2)
{
    return z < N2 || z >= NZ - N2 || x < N2 || x >= NX - N2;
}

__host__ __device__ __forceinline__ int blend_index(int z, int x, int NZ, int NX, int N2)
{
    int j = N2 - z;
    j = max(j, N2 - x);
    j = max(j, z - (NZ - N2) + 1);
    j = max(j, x - (NX - N2) + 1);
    return j;
}
