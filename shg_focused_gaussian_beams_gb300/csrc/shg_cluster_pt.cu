// Cluster march with one thread per point: the whole z-march of a solve
// (Solver::CWES -> SSFM, Solver.h:236-276) in one thread-block cluster, both fields held in
// the cluster's shared memory for the whole run.
//
// CTA `rank` of the cluster owns rows [rank R, rank R + R) of both fields (row phase) and
// columns [rank R, rank R + R) (column phase, read and written through distributed shared
// memory); a cluster barrier separates the phases. Against the resident cluster march
// (shg_resident.cuh, R * G threads per CTA, each carrying N / G points through both RK4
// calls) every CTA here has 512 threads: the line transforms run on 2 R G of them and the
// two RK4 calls on all of them, R N / 512 points each, through the shared field rows. The
// arithmetic is that of the streaming row and column passes (k_rows_pt, k_cols in
// shg_march.cu): the same transforms, RK4 and propagator products in the same order, so
// the output fields are bit-identical. Meant for lone solves (the march's latency is set by
// on-chip exchanges instead of two dependent kernel launches per z-step); one cluster per
// solve of a class.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "shg_internal.h"
#include "shg_march.cuh"

namespace cg = cooperative_groups;

namespace shg {

const float2 *twiddle_symbol_address_cluster_pt() {
    void *p = nullptr;
    cudaGetSymbolAddress(&p, g_twiddle);
    return static_cast<const float2 *>(p);
}
SHG_CHECK_TU(cluster_pt)

template <int N>
struct CptCluster;
template <> struct CptCluster<64> { static constexpr int CS = 8; };
template <> struct CptCluster<128> { static constexpr int CS = 16; };
template <> struct CptCluster<256> { static constexpr int CS = 16; };

template <int N>
struct CptShape {
    static constexpr int CS = CptCluster<N>::CS;       // CTAs per cluster (16: non-portable)
    static constexpr int G = LineShape<N>::G, E = N / G;
    static constexpr int R = N / CS;                   // rows (and columns) per CTA
    static constexpr int TPB = 512;
    static constexpr int PTS = R * N / TPB;            // points per thread in the pointwise phase
    static constexpr int XF = 2 * R * G;               // transform threads (both fields' lines)
    static constexpr int TC = 32 / G;                  // columns per warp in the column phase
    static constexpr int SC = LineScratch<N, G>::SIZE;
    static constexpr int FIELD = R * N;                // complex values per field per CTA
    static constexpr int SCR = (2 * R * SC > 2 * FIELD) ? 2 * R * SC : 2 * FIELD;
    static constexpr size_t SMEM = (size_t)(2 * FIELD + SCR) * sizeof(float2);
    static_assert(PTS * TPB == R * N && XF <= TPB && XF % 32 == 0, "thread roles fill whole warps");
    static_assert(TC * G == 32 && R % TC == 0, "a column warp holds TC columns of one field");
};

__device__ __forceinline__ void cpt_block_add(double v, double *dst) {
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

// Grid: count clusters of CS CTAs, cluster c marching solve list[c].
template <int N>
__global__ void __launch_bounds__(CptShape<N>::TPB, 1)
    k_march_cluster_pt(const InstDesc *__restrict__ inst, const int *__restrict__ list) {
    using Sh = CptShape<N>;
    constexpr int G = Sh::G, E = Sh::E, R = Sh::R, N2 = R * G, TC = Sh::TC, FIELD = Sh::FIELD;
    extern __shared__ float2 smem[];
    float2 *const sP = smem, *const sS = smem + FIELD, *const scr = smem + 2 * FIELD;
    // the split's twiddle pairs, staged in shared memory once per launch
    __shared__ __align__(16) float2 tab[N];
    {
        const float2 *src = twiddle_split<N, G>(g_twiddle + N);
        for (int i = threadIdx.x; i < N; i += blockDim.x) tab[i] = src[i];
    }
    __syncthreads();
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    const InstDesc &d = inst[list[blockIdx.x / Sh::CS]];
    // every CTA of the cluster reads the same descriptor: all leave before the first barrier
    if (!SHG_REQUIRE(d.n == N && d.nsteps >= 1 && d.nsteps < d.nz, kChkDescriptor, d.n)) return;
    const int tid = threadIdx.x, K = d.nsteps;
    const size_t row0 = (size_t)rank * R * N;  // this CTA's first point in the N x N field

    // row-phase transform role: field rf, local line rl, thread rt of the line's G
    const bool xf = tid < Sh::XF;
    const int rf = tid / N2, rl = (tid % N2) / G, rt = tid % G;
    float2 *const rline = (rf == 0 ? sP : sS) + rl * N;
    float2 *const rsc = scr + (size_t)(rf * R + rl) * Sh::SC;
    // column-phase role: warp w holds columns of one field, lane = column + TC * thread
    const int w = tid >> 5, lane = tid & 31;
    const int cgi = w * TC + lane % TC;  // column group index in [0, 2R) for transform warps
    const int cf = cgi / R, cx = rank * R + cgi % R, ct = lane / TC;
    float2 *const cfield = cf == 0 ? sP : sS;
    float2 *const csc = scr + (size_t)w * TC * N + lane % TC;
    // the column's propagator values, held in registers for the whole run
    float2 h[E];
    if (xf) hprop_load<N>(cf == 0 ? d.Hp : d.Hs, cx, ct, h);

    // this CTA's rows of both fields (16-byte loads)
    {
        const float4 *gP = reinterpret_cast<const float4 *>(d.P + row0);
        const float4 *gS = reinterpret_cast<const float4 *>(d.S + row0);
        float4 *lP = reinterpret_cast<float4 *>(sP), *lS = reinterpret_cast<float4 *>(sS);
        for (int i = tid; i < FIELD / 2; i += Sh::TPB) {
            lP[i] = gP[i];
            lS[i] = gS[i];
        }
    }
    __syncthreads();

    for (int s = 0; s <= K; ++s) {
        // ---- row phase on the local rows (k_rows_pt's arithmetic)
        if (s == 0) {
            const float4 c = d.stepc[0];
#pragma unroll
            for (int k = 0; k < Sh::PTS; ++k) {
                const int i = tid + Sh::TPB * k;
                float2 p = sP[i], q = sS[i];
                rk4_point(p, q, c, d);
                sP[i] = p;
                sS[i] = q;
            }
            __syncthreads();
            if (xf) {
                float2 v[E];
#pragma unroll
                for (int j = 0; j < E; ++j) v[j] = rline[rt + G * j];
                fft_nat_to_spec<N, G, +1, false, 1, G + 1, true>(v, rt, rsc, tab);
#pragma unroll
                for (int r = 0; r < E; ++r) rline[spec_index<N, G>(rt, r)] = v[r];
            }
        } else {
            const float4 cprev = d.stepc[s - 1], ccur = d.stepc[s];  // s <= K < nz
            if (xf) {
                // in place: every lane of the line has loaded before the transform's first
                // warp synchronisation, and the stores follow it
                float2 v[E];
#pragma unroll
                for (int j = 0; j < E; ++j) v[j] = rline[rt + G * j];
                fft_nat_to_spec<N, G, -1, false, 1, G + 1, true>(v, rt, rsc, tab);
#pragma unroll
                for (int r = 0; r < E; ++r) rline[spec_index<N, G>(rt, r)] = v[r];
            }
            __syncthreads();
            double aS = 0.0, aP = 0.0;
#pragma unroll 2
            for (int k = 0; k < Sh::PTS; ++k) {
                const int i = tid + Sh::TPB * k;
                float2 p = sP[i], q = sS[i];
                rk4_point(p, q, cprev, d);
                if (d.slices && s < d.nz) {
                    float2 *sl = d.slices + (size_t)s * 2 * N * N;
                    SHG_AT(sl, row0 + i, (size_t)2 * N * N, kChkSlices) = p;
                    SHG_AT(sl, (size_t)N * N + row0 + i, (size_t)2 * N * N, kChkSlices) = q;
                }
                if (s == K) {
                    SHG_AT(d.Pout, row0 + i, (size_t)N * N, kChkClusterPtRow) = p;
                    SHG_AT(d.Sout, row0 + i, (size_t)N * N, kChkClusterPtRow) = q;
                    aS += (double)q.x * q.x + (double)q.y * q.y;
                    aP += (double)p.x * p.x + (double)p.y * p.y;
                } else {
                    rk4_point(p, q, ccur, d);
                    sP[i] = p;
                    sS[i] = q;
                }
            }
            if (s == K) {
                cpt_block_add(aS, d.acc + 1);
                cpt_block_add(aP, d.acc + 2);
                break;
            }
            __syncthreads();
            if (xf) {
                float2 v[E];
#pragma unroll
                for (int r = 0; r < E; ++r) v[r] = rline[spec_index<N, G>(rt, r)];
                fft_spec_to_nat<N, G, +1, false, 1, G + 1, true>(v, rt, rsc, tab);
#pragma unroll
                for (int j = 0; j < E; ++j) rline[rt + G * j] = v[j];
            }
        }
        // every CTA's rows are finished before any column is read
        cluster.sync();
        // ---- column phase on columns [rank R, rank R + R) of both fields (k_cols' arithmetic)
        // element y of this thread's column: rank y / R, local row y % R (checked build:
        // a bad element is redirected to this CTA's own first entry)
        auto col_at = [&](int y) -> float2 * {
            int rk = y / R, li = (y % R) * N + cx;
            if (!SHG_REQUIRE(rk < Sh::CS && li < FIELD, kChkClusterPtCol, y)) rk = rank, li = 0;
            return cluster.map_shared_rank(cfield + li, rk);
        };
        if (xf) {
            float2 v[E];
#pragma unroll
            for (int j = 0; j < E; ++j) v[j] = *col_at(ct + G * j);
            fft_nat_to_spec<N, G, +1, false, TC, G, true>(v, ct, csc, tab);
#pragma unroll
            for (int r = 0; r < E; ++r) v[r] = c_mul(v[r], h[r]);
            fft_spec_to_nat<N, G, -1, false, TC, G, true>(v, ct, csc, tab);
#pragma unroll
            for (int j = 0; j < E; ++j) *col_at(ct + G * j) = v[j];
        }
        // every column is written back before any row is read again
        cluster.sync();
    }
    // The last remote access of the run preceded the last cluster barrier: no CTA reads or
    // writes another's shared memory after that, so CTAs may exit independently.
}

template <int N>
static cudaLaunchConfig_t cpt_config(cudaLaunchAttribute *attr, cudaStream_t st) {
    using Sh = CptShape<N>;
    cudaLaunchConfig_t cfg = {};
    cfg.blockDim = dim3(Sh::TPB, 1, 1);
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

template <int N>
static cudaError_t prepare_cpt_t(int *max_clusters) {
    using Sh = CptShape<N>;
    auto k = k_march_cluster_pt<N>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Sh::SMEM);
    if (e != cudaSuccess) return e;
    if (Sh::CS > 8 && (e = cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1)) != cudaSuccess)
        return e;
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = cpt_config<N>(attr, nullptr);
    cfg.gridDim = dim3(Sh::CS, 1, 1);
    return cudaOccupancyMaxActiveClusters(max_clusters, k, &cfg);
}

template <int N>
static cudaError_t launch_cpt_t(const InstDesc *inst, const int *list, int count, cudaStream_t st) {
    using Sh = CptShape<N>;
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = cpt_config<N>(attr, st);
    cfg.gridDim = dim3((unsigned)count * Sh::CS, 1, 1);
    return cudaLaunchKernelEx(&cfg, k_march_cluster_pt<N>, inst, list);
}

int cluster_pt_size(int n) {
    switch (n) {
        case 64: return CptShape<64>::CS;
        case 128: return CptShape<128>::CS;
        case 256: return CptShape<256>::CS;
        default: return 0;
    }
}

cudaError_t prepare_cluster_pt(int n, int *max_clusters) {
    *max_clusters = 0;
    switch (n) {
        case 64: return prepare_cpt_t<64>(max_clusters);
        case 128: return prepare_cpt_t<128>(max_clusters);
        case 256: return prepare_cpt_t<256>(max_clusters);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_cluster_pt(int n, const InstDesc *inst, const int *list, int count, cudaStream_t st) {
    if (count < 1) return cudaErrorInvalidValue;
    switch (n) {
        case 64: return launch_cpt_t<64>(inst, list, count, st);
        case 128: return launch_cpt_t<128>(inst, list, count, st);
        case 256: return launch_cpt_t<256>(inst, list, count, st);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace shg
