// Resident z-march kernel template (design notes in shg_resident_variants.cu); instantiated per grid size in
// shg_resident_<n>.cu.
#pragma once

#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "shg_internal.h"
#include "shg_march.cuh"

namespace cg = cooperative_groups;

namespace shg {

// Shape of one resident variant: CS CTAs per cluster, MINB CTAs per SM requested from the
// register allocator.
template <int N, int CS_, int MINB_, int G_ = LineShape<N>::G>
struct ResShape {
    static constexpr int CS = CS_, MINB = MINB_;
    static constexpr int G = G_, E = N / G;   // line FFT split: E-point register DFTs, then G-point
    static constexpr int R = N / CS;             // rows (and columns) per CTA
    static constexpr int THREADS = R * G;
    static constexpr int SC_ROW = LineScratch<N, G>::SIZE;
    static constexpr int FIELD = R * N;          // complex values per field per CTA
    static constexpr int SCR = (R * SC_ROW > R * N) ? R * SC_ROW : R * N;
    static constexpr size_t SMEM = (size_t)(2 * FIELD + SCR) * sizeof(float2);
};

template <int CS>
__device__ __forceinline__ void cluster_barrier() {
    if constexpr (CS > 1)
        cg::this_cluster().sync();
    else
        __syncthreads();
}

__device__ __forceinline__ void block_add_double_res(double v, double *dst) {
    __shared__ double red[32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    if (w == 0) {
        v = (l < (int)(blockDim.x >> 5)) ? red[l] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (l == 0 && v != 0.0) atomicAdd(dst, v);
    }
}

template <int N, int CS_, int MINB_, int G_>
__global__ void __launch_bounds__(ResShape<N, CS_, MINB_, G_>::THREADS, MINB_)
    k_march_resident(const InstDesc *__restrict__ inst, const int *__restrict__ list, int njobs, int *counter) {
    using Sh = ResShape<N, CS_, MINB_, G_>;
    constexpr int CS = Sh::CS, G = Sh::G, E = Sh::E, R = Sh::R, FIELD = Sh::FIELD, SC_ROW = Sh::SC_ROW;
    extern __shared__ float2 smem[];
    float2 *sP = smem, *sS = smem + FIELD, *scr = smem + 2 * FIELD;
    __shared__ int job_s;
    // this split's inter-stage twiddle pairs, staged in shared memory once per launch (the
    // transforms then read them with shared loads instead of global ones)
    __shared__ __align__(16) float2 tab[N];
    {
        const float2 *src = twiddle_split<N, G>(g_twiddle + N);
        for (int i = threadIdx.x; i < N; i += blockDim.x) tab[i] = src[i];
    }
    __syncthreads();
    int rank = 0;
    if constexpr (CS > 1) rank = (int)cg::this_cluster().block_rank();
    const int tid = threadIdx.x;
    // row-phase roles
    const int line = tid / G, t = tid % G;
    float2 *rsc = scr + line * SC_ROW;
    // column-phase roles
    const int cc = tid % R, ct = tid / R;

    for (;;) {
        if (rank == 0 && tid == 0) job_s = atomicAdd(counter, 1);
        cluster_barrier<CS>();
        int job;
        if constexpr (CS > 1)
            job = *cg::this_cluster().map_shared_rank(&job_s, 0);
        else
            job = job_s;
        // every CTA has read the job index before rank 0 may exit or overwrite it
        cluster_barrier<CS>();
        if (job >= njobs) break;
        const InstDesc &d = inst[list[job]];
        // a bad descriptor skips the job in every CTA of the cluster alike (no barrier inside)
        if (!SHG_REQUIRE(d.n == N && d.nsteps < d.nz && d.nsteps >= 1, kChkDescriptor, job)) continue;
        // load this CTA's rows of both fields
        {
            const float4 *gP = reinterpret_cast<const float4 *>(d.P + (size_t)rank * FIELD);
            const float4 *gS = reinterpret_cast<const float4 *>(d.S + (size_t)rank * FIELD);
            float4 *lP = reinterpret_cast<float4 *>(sP), *lS = reinterpret_cast<float4 *>(sS);
            for (int i = tid; i < FIELD / 2; i += Sh::THREADS) {
                lP[i] = gP[i];
                lS[i] = gS[i];
            }
        }
        __syncthreads();
        const int K = d.nsteps;
        for (int s = 0; s <= K; ++s) {
            // ---- row phase (local rows)
            {
                float2 *rowP = sP + line * N, *rowS = sS + line * N;
                // step constants of slices s-1 and s (s <= K < nz), loaded before the transform
                const float4 cprev = d.stepc[s > 0 ? s - 1 : 0], ccur = d.stepc[s];
                float2 vp[E], vs[E];
#pragma unroll
                for (int j = 0; j < E; ++j) {
                    vp[j] = rowP[t + G * j];
                    vs[j] = rowS[t + G * j];
                }
                if (s == 0) {
                    const float4 c = ccur;
#pragma unroll
                    for (int j = 0; j < E; ++j) rk4_point(vp[j], vs[j], c, d);
                    fft_nat_to_spec<N, G, +1, false, 1, G + 1, true>(vp, t, rsc, tab);
                    fft_nat_to_spec<N, G, +1, false, 1, G + 1, true>(vs, t, rsc, tab);
                    __syncwarp();
#pragma unroll
                    for (int r = 0; r < E; ++r) {
                        const int k = spec_index<N, G>(t, r);
                        rowP[k] = vp[r];
                        rowS[k] = vs[r];
                    }
                } else {
                    fft_nat_to_spec<N, G, -1, false, 1, G + 1, true>(vp, t, rsc, tab);
                    fft_nat_to_spec<N, G, -1, false, 1, G + 1, true>(vs, t, rsc, tab);
                    const float4 c1 = cprev;
#pragma unroll
                    for (int r = 0; r < E; ++r) rk4_point(vp[r], vs[r], c1, d);
                    if (d.slices && s < d.nz) {
                        float2 *sl = d.slices + (size_t)s * 2 * N * N;
                        const size_t base = (size_t)(rank * R + line) * N;
#pragma unroll
                        for (int r = 0; r < E; ++r) {
                            const int k = spec_index<N, G>(t, r);
                            SHG_AT(sl, base + k, (size_t)2 * N * N, kChkSlices) = vp[r];
                            SHG_AT(sl, (size_t)N * N + base + k, (size_t)2 * N * N, kChkSlices) = vs[r];
                        }
                    }
                    if (s == K) {
                        const size_t base = (size_t)(rank * R + line) * N;
                        double aS = 0.0, aP = 0.0;
#pragma unroll
                        for (int r = 0; r < E; ++r) {
                            const int k = spec_index<N, G>(t, r);
                            SHG_AT(d.Pout, base + k, (size_t)N * N, kChkResidentLoad) = vp[r];
                            SHG_AT(d.Sout, base + k, (size_t)N * N, kChkResidentLoad) = vs[r];
                            aS += (double)vs[r].x * vs[r].x + (double)vs[r].y * vs[r].y;
                            aP += (double)vp[r].x * vp[r].x + (double)vp[r].y * vp[r].y;
                        }
                        block_add_double_res(aS, d.acc + 1);
                        block_add_double_res(aP, d.acc + 2);
                    } else {
                        const float4 c2 = ccur;
#pragma unroll
                        for (int r = 0; r < E; ++r) rk4_point(vp[r], vs[r], c2, d);
                        fft_spec_to_nat<N, G, +1, false, 1, G + 1, true>(vp, t, rsc, tab);
                        fft_spec_to_nat<N, G, +1, false, 1, G + 1, true>(vs, t, rsc, tab);
#pragma unroll
                        for (int j = 0; j < E; ++j) {
                            rowP[t + G * j] = vp[j];
                            rowS[t + G * j] = vs[j];
                        }
                    }
                }
            }
            if (s == K) break;
            cluster_barrier<CS>();
            // ---- column phase: columns [rank*R, rank*R + R)
            {
                const int x = rank * R + cc;
#pragma unroll 1
                for (int f = 0; f < 2; ++f) {
                    float2 *F = f == 0 ? sP : sS;
                    const float2 *__restrict__ H = f == 0 ? d.Hp : d.Hs;
                    auto at = [&](int j) -> float2 * {
                        const int y = ct + G * j;
                        int rk = y / R, li = (y % R) * N + x;
                        if (!SHG_REQUIRE(rk < CS && li < FIELD, kChkResidentCol, y)) rk = rank, li = 0;
                        float2 *p = F + li;
                        if constexpr (CS > 1) p = cg::this_cluster().map_shared_rank(p, rk);
                        return p;
                    };
                    // propagator values first: their L2 latency overlaps the column transform
                    float2 h[E];
                    if constexpr (G == LineShape<N>::G) {
                        hprop_load<N>(H, x, ct, h);
                    } else {
#pragma unroll
                        for (int r = 0; r < E; ++r) h[r] = __ldg(H + hprop_index<N>(spec_index<N, G>(ct, r), x));
                    }
                    float2 v[E];
#pragma unroll
                    for (int j = 0; j < E; ++j) v[j] = *at(j);
                    fft_nat_to_spec<N, G, +1, true, R, G, true>(v, ct, scr + cc, tab);
#pragma unroll
                    for (int r = 0; r < E; ++r) v[r] = c_mul(v[r], h[r]);
                    fft_spec_to_nat<N, G, -1, true, R, G, true>(v, ct, scr + cc, tab);
#pragma unroll
                    for (int j = 0; j < E; ++j) *at(j) = v[j];
                    __syncthreads();  // scratch reuse by the second field
                }
            }
            cluster_barrier<CS>();
        }
        // The next job's loads touch only this CTA's shared memory; all remote accesses of
        // this job ended before the last cluster barrier.
    }
}

template <int N, int CS, int MINB, int G>
static cudaLaunchConfig_t resident_config(cudaLaunchAttribute *attr, cudaStream_t st) {
    using Sh = ResShape<N, CS, MINB, G>;
    cudaLaunchConfig_t cfg = {};
    cfg.blockDim = dim3(Sh::THREADS, 1, 1);
    cfg.dynamicSmemBytes = Sh::SMEM;
    cfg.stream = st;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = Sh::CS;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cfg;
}

// Once per device, outside any stream capture: shared-memory limit, cluster size above the
// portable 8 where asked, and the number of clusters that fit at once (0: does not fit).
template <int N, int CS, int MINB, int G>
cudaError_t prepare_resident_t(int *max_clusters) {
    using Sh = ResShape<N, CS, MINB, G>;
    auto k = k_march_resident<N, CS, MINB, G>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Sh::SMEM);
    if (e != cudaSuccess) return e;
    if (CS > 8) {
        e = cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) return e;
    }
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = resident_config<N, CS, MINB, G>(attr, nullptr);
    cfg.gridDim = dim3(Sh::CS, 1, 1);
    return cudaOccupancyMaxActiveClusters(max_clusters, k, &cfg);
}

template <int N, int CS, int MINB, int G>
cudaError_t launch_resident_t(const InstDesc *inst, const int *list, int njobs, int *counter, int max_clusters,
                              cudaStream_t st) {
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = resident_config<N, CS, MINB, G>(attr, st);
    int clusters = max_clusters;
    if (clusters > njobs) clusters = njobs;
    if (clusters < 1) clusters = 1;
    cfg.gridDim = dim3(clusters * CS, 1, 1);
    return cudaLaunchKernelEx(&cfg, k_march_resident<N, CS, MINB, G>, inst, list, njobs, counter);
}

// Variants compiled for grid n (its translation unit), as (CS, MINB, G) triples.
#define SHG_RESIDENT_INSTANTIATE(N, CS, MINB, G)                                                              \
    template cudaError_t prepare_resident_t<N, CS, MINB, G>(int *);                                         \
    template cudaError_t launch_resident_t<N, CS, MINB, G>(const InstDesc *, const int *, int, int *, int,  \
                                                           cudaStream_t);

}  // namespace shg
