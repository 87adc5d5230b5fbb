// Persistent cooperative grid of one solve: the bounded grid-wide barrier, the grid's
// row-unit / column-group shape and the column pass with the propagator values held in
// registers. Shared by the plain march (k_march_coop, shg_march.cu) and the THERMAL march
// (k_march_coop_th, shg_thermal.cu); the row passes are those of the streaming kernels
// with one thread per point, so a run gives their results bit for bit.
#pragma once

#include <cuda_runtime.h>

#include "shg_march.cuh"

namespace shg {

// Poll limit of a grid-barrier wait (about a second).
constexpr long long kGridWaitLimit = 1ll << 22;

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void red_release_gpu(unsigned *p, unsigned v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Grid-wide barrier of a cooperative launch on a monotonic arrival counter (zeroed before
// the launch): barrier number e of the run completes once e * gridDim.x arrivals are in.
// Thread 0 of each block arrives with a release add (ordering the block's writes, which the
// block barrier made its own, before the arrival) and polls with acquire loads (ordering
// the other blocks' writes before this block's later loads). No reset step: a waiter reads
// one word. Every wait is bounded: on timeout `code` is or-ed into *err and false is
// returned (the caller leaves the kernel), and a wait also ends once *err is non-zero.
__device__ __forceinline__ bool grid_barrier(unsigned *count, unsigned target, int *err, int code = 1) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        red_release_gpu(count, 1u);
        int good = 1;
        for (long long it = 0; ld_acquire_gpu(count) < target; ++it) {
            if (it >= kGridWaitLimit || *(volatile int *)err) {
                atomicOr(err, code);
                good = 0;
                break;
            }
            if (it >= 64) __nanosleep(32);
        }
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

template <int N>
struct CoopShape {
    static constexpr int G = LineShape<N>::G, E = N / G;
    static constexpr int LPB = (512 / N < N) ? 512 / N : N;  // lines per row unit
    static constexpr int TPB = LPB * N;                     // one thread per point of a unit
    static constexpr int TC = 32 / G;                    // columns per column group (one warp)
    static constexpr int ROW_UNITS = N / LPB;            // groups of LPB lines
    static constexpr int COL_UNITS = 2 * (N / TC);       // column groups of both fields
    static_assert(TC * G == 32, "a column group is one warp");
};

// cols_body with the column's propagator values already in registers.
template <int N, int TC>
__device__ __forceinline__ void cols_body_h(const InstDesc &d, int x, int f, int t, float2 *sc,
                                            const float2 (&h)[N / LineShape<N>::G], const float2 *tab) {
    constexpr int G = LineShape<N>::G, E = N / G;  // tab: the split's pair table in shared memory
    float2 *F = f == 0 ? d.P : d.S;
    constexpr size_t NN = (size_t)N * N;
    float2 v[E];
#pragma unroll
    for (int j = 0; j < E; ++j) v[j] = SHG_AT(F, (size_t)(t + G * j) * N + x, NN, kChkCoop);
    fft_nat_to_spec<N, G, +1, false, TC, G, true>(v, t, sc, tab);
#pragma unroll
    for (int r = 0; r < E; ++r) v[r] = c_mul(v[r], h[r]);
    fft_spec_to_nat<N, G, -1, false, TC, G, true>(v, t, sc, tab);
#pragma unroll
    for (int j = 0; j < E; ++j) SHG_AT(F, (size_t)(t + G * j) * N + x, NN, kChkCoop) = v[j];
}

}  // namespace shg
