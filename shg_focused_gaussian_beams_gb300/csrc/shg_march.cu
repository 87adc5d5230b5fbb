// Plain SSFM z-march kernels (Solver.h:236-276 without THERMAL), batched over solves.
//
// One SSFM step of the reference is RK4(z) -> diffraction -> RK4(z) (Solver.h:236-242),
// where diffraction is FFT_backward -> propagator product -> FFT_forward -> 1/(NX*NY)
// (Solver.h:156-190). The march here regroups the work of consecutive steps into two
// passes per step so that each field crosses memory twice per step:
//
//   row pass (k_rows, lines along x): finish the forward 2D transform of step s-1 along x,
//       second RK4 of step s-1, [capture at the top of slice nz-1], first RK4 of step s,
//       start the backward 2D transform of step s along x;
//   column pass (k_cols, lines along y): backward transform along y, product with the
//       shifted propagator (pre-scaled by 1/(NX*NY), exact for power-of-two grids), forward
//       transform along y.
//
// The row-pass transforms use the spectral register layout between the forward and the
// backward transform, so the RK4 work never reorders data (shg_fft.cuh).
#include <cuda_runtime.h>
#include <math.h>

#include "shg_internal.h"
#include "shg_coop.cuh"
#include "shg_march.cuh"

namespace shg {

const float2 *twiddle_symbol_address_march() {
    void *p = nullptr;
    cudaGetSymbolAddress(&p, g_twiddle);
    return static_cast<const float2 *>(p);
}
SHG_CHECK_TU(march)

// Check build: the descriptor matches the kernel's grid and stage s is a valid SSFM stage.
template <int N>
__device__ __forceinline__ bool check_solve(const InstDesc &d, int s) {
    return SHG_REQUIRE(d.n == N, kChkDescriptor, d.n) &&
           SHG_REQUIRE(s >= 0 && s <= d.nsteps && d.nsteps < d.nz, kChkStage, s);
}

// Check-build self test: records (kChkSelfTest, value) without touching memory.
__global__ void k_check_selftest(long long value) {
    if (threadIdx.x == 0) SHG_REQUIRE(false, kChkSelfTest, value);
}
cudaError_t launch_check_selftest(long long value) {
    k_check_selftest<<<1, 32>>>(value);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------
// Setup: phase table, Gaussian pump, shifted propagators, input power.

// z accumulates in float (Solver.h:271), one thread walks the slices of one solve; the
// phase exp(-+ i z dk) enters dA/dz through cosf/sinf of fl(z*dk) (Operators.h:105-117).
__global__ void k_setup_steps(const InstDesc *__restrict__ inst, int n_inst) {
    extern __shared__ float zs[];
    const InstDesc &d = inst[blockIdx.x];
    if (threadIdx.x == 0) {
        float z = 0.0f;
        for (int s = 0; s < d.nz; ++s) {
            zs[s] = z;
            z = __fadd_rn(z, d.dz);
        }
    }
    __syncthreads();
    for (int s = threadIdx.x; s < d.nz; s += blockDim.x) {
        const float arg = __fmul_rn(zs[s], d.dk);
        float sn, cs;
        sincosf(arg, &sn, &cs);
        d.stepc[s] = make_float4(d.kp * sn, d.kp * cs, -d.ks * sn, d.ks * cs);
    }
}

__device__ __forceinline__ void block_add_double(double v, double *dst) {
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

// Efields.h:74-104 (pump) and Efields.h:107-126 + 32-71 (propagators), with the float
// operations of the reference kept in order (no contraction); only cosf/sinf/expf are the
// device's. Grid: (chunks of 4*blockDim pixels, solves).
__global__ void k_setup_fields(const InstDesc *__restrict__ inst) {
    const InstDesc &d = inst[blockIdx.y];
    const int n = d.n, nn = n * n, half = n / 2;
    double acc = 0.0;
    for (int q = 0; q < 4; ++q) {
        const int i = (blockIdx.x * 4 + q) * blockDim.x + threadIdx.x;
        if (i >= nn) break;
        const int ix = i % n, iy = i / n;
        if (!d.pump_given) {
            const float ax = __fmul_rn(__fsub_rn((float)ix, d.uX), d.dx);
            const float ay = __fmul_rn(__fsub_rn((float)iy, d.uY), d.dy);
            const float num = __fsub_rn(-__fmul_rn(ax, ax), __fmul_rn(ay, ay));
            const float re = __fdiv_rn(__fmul_rn(num, d.wM.x), d.wM_den);
            const float im = __fdiv_rn(__fmul_rn(-num, d.wM.y), d.wM_den);
            const float e = expf(re);
            float sn, cs;
            sincosf(im, &sn, &cs);
            const float er = __fmul_rn(e, cs), ei = __fmul_rn(e, sn);
            const float2 p = make_float2(__fsub_rn(__fmul_rn(d.amp.x, er), __fmul_rn(d.amp.y, ei)),
                                         __fadd_rn(__fmul_rn(d.amp.x, ei), __fmul_rn(d.amp.y, er)));
            d.P[i] = p;
        }
        const float2 p = d.P[i];
        acc += (double)p.x * p.x + (double)p.y * p.y;
        // shifted propagator: H_shift[ix, iy] = H[(ix + n/2) % n, (iy + n/2) % n]
        const int ux = (ix + half) & (n - 1), uy = (iy + half) & (n - 1);
        const float tx = __fsub_rn((float)ux, d.uX), ty = __fsub_rn((float)uy, d.uY);
        const float q2 = __fadd_rn(__fmul_rn(d.dfX2, __fmul_rn(tx, tx)), __fmul_rn(d.dfY2, __fmul_rn(ty, ty)));
        const float php = __fmul_rn(d.mdz, __fadd_rn(__fmul_rn(d.gp, q2), __fmul_rn(d.linp, tx)));
        const float phs = __fmul_rn(d.mdz, __fadd_rn(__fmul_rn(d.gs, q2), __fmul_rn(d.lins, tx)));
        float s1, c1, s2, c2;
        sincosf(php, &s1, &c1);
        sincosf(phs, &s2, &c2);
        // stored in the column transforms' order (hprop_index_rt, shg_fft.cuh)
        const size_t ih = hprop_index_rt(n, iy, ix);
        d.Hp[ih] = make_float2(c1 * d.inv_nn, s1 * d.inv_nn);
        d.Hs[ih] = make_float2(c2 * d.inv_nn, s2 * d.inv_nn);
    }
    block_add_double(acc, d.acc + 0);
}

// ---------------------------------------------------------------------------------------
// Row pass. Block = 256 threads = 256/G lines of one solve; mode from the stage s:
//   s == 0           : RK4(z_0), backward transform along x, store in frequency order;
//   0 < s < nsteps   : forward transform along x, RK4(z_{s-1}), RK4(z_s), backward;
//   s == nsteps      : forward transform along x, RK4(z_{s-1}), capture, power sums.
template <int N>
struct RowShape {
    static constexpr int G = LineShape<N>::G;
    static constexpr int TPB = (N * G < 256) ? N * G : 256;  // threads per block
    static constexpr int LPB = TPB / G;                      // lines per block
    static constexpr int BPI = N / LPB;                      // blocks per solve
};

template <int N>
__global__ void __launch_bounds__(RowShape<N>::TPB) k_rows(const InstDesc *__restrict__ inst, const int *__restrict__ list, int s) {
    constexpr int G = LineShape<N>::G, E = N / G, LPB = RowShape<N>::LPB, BPI = RowShape<N>::BPI;
    constexpr int SC = LineScratch<N, G>::SIZE;
    static_assert(N % LPB == 0, "blocks must not straddle solves");
    __shared__ float2 scratch[LPB * SC];
    const InstDesc &d = inst[list[blockIdx.x / BPI]];
    if (!check_solve<N>(d, s)) return;  // whole block (d and s are block-uniform)
    constexpr size_t NN = (size_t)N * N;
    const float2 *__restrict__ tab = g_twiddle + N;
    const int line = (blockIdx.x % BPI) * LPB + threadIdx.x / G;
    const int t = threadIdx.x % G;
    float2 *sc = scratch + (threadIdx.x / G) * SC;
    const size_t base = (size_t)line * N;
    float2 vp[E], vs[E];
#pragma unroll
    for (int j = 0; j < E; ++j) {
        vp[j] = SHG_AT(d.P, base + t + G * j, NN, kChkRowsGlobal);
        vs[j] = SHG_AT(d.S, base + t + G * j, NN, kChkRowsGlobal);
    }
    if (s == 0) {
        const float4 c = d.stepc[0];
#pragma unroll
        for (int j = 0; j < E; ++j) rk4_point(vp[j], vs[j], c, d);
        fft_nat_to_spec<N, G, +1>(vp, t, sc, tab);
        fft_nat_to_spec<N, G, +1>(vs, t, sc, tab);
#pragma unroll
        for (int r = 0; r < E; ++r) {
            const int k = spec_index<N, G>(t, r);
            SHG_AT(d.P, base + k, NN, kChkRowsGlobal) = vp[r];
            SHG_AT(d.S, base + k, NN, kChkRowsGlobal) = vs[r];
        }
        return;
    }
    fft_nat_to_spec<N, G, -1>(vp, t, sc, tab);
    fft_nat_to_spec<N, G, -1>(vs, t, sc, tab);
    const float4 c1 = d.stepc[s - 1];
#pragma unroll
    for (int r = 0; r < E; ++r) rk4_point(vp[r], vs[r], c1, d);
    if (d.slices && s < d.nz) {
        float2 *sl = d.slices + (size_t)s * 2 * N * N;
#pragma unroll
        for (int r = 0; r < E; ++r) {
            const int k = spec_index<N, G>(t, r);
            SHG_AT(sl, base + k, 2 * NN, kChkSlices) = vp[r];
            SHG_AT(sl, NN + base + k, 2 * NN, kChkSlices) = vs[r];
        }
    }
    if (s == d.nsteps) {
        double aS = 0.0, aP = 0.0;
#pragma unroll
        for (int r = 0; r < E; ++r) {
            const int k = spec_index<N, G>(t, r);
            SHG_AT(d.Pout, base + k, NN, kChkRowsGlobal) = vp[r];
            SHG_AT(d.Sout, base + k, NN, kChkRowsGlobal) = vs[r];
            aS += (double)vs[r].x * vs[r].x + (double)vs[r].y * vs[r].y;
            aP += (double)vp[r].x * vp[r].x + (double)vp[r].y * vp[r].y;
        }
        block_add_double(aS, d.acc + 1);
        block_add_double(aP, d.acc + 2);
        return;
    }
    const float4 c2 = d.stepc[s];
#pragma unroll
    for (int r = 0; r < E; ++r) rk4_point(vp[r], vs[r], c2, d);
    fft_spec_to_nat<N, G, +1>(vp, t, sc, tab);
    fft_spec_to_nat<N, G, +1>(vs, t, sc, tab);
#pragma unroll
    for (int j = 0; j < E; ++j) {
        SHG_AT(d.P, base + t + G * j, NN, kChkRowsGlobal) = vp[j];
        SHG_AT(d.S, base + t + G * j, NN, kChkRowsGlobal) = vs[j];
    }
}

// Row pass for one to three solves: the same work as k_rows with one thread per point.
// Block = LPB lines x N threads; the row transforms run on 2 * LPB * G threads (pump lines
// first, then SH lines), both RK4 calls on every thread for its point through a
// shared-memory line buffer, so a lone solve occupies N * N threads instead of N * G.
template <int N>
struct PtRowShape {
    static constexpr int G = LineShape<N>::G;
    static constexpr int LPB = (512 / N < N) ? 512 / N : N;
    static constexpr int TPB = LPB * N;
    static constexpr int BPI = N / LPB;
    static constexpr int FT = LPB * G;  // transform threads per field
    static_assert(FT % 32 == 0 && 2 * FT <= TPB && N % LPB == 0, "transform threads fill whole warps");
};

// The row pass of k_rows_pt for lines [line0, line0 + LPB) of solve d at stage s, on a block
// of PtRowShape<N>::TPB threads (shared by the streaming launch and the persistent grid).
// twiddles: the line length's global block g_twiddle + N, or with TS the split's own pair
// table staged in shared memory by the caller.
template <int N, bool TS = false>
__device__ __forceinline__ void rows_pt_body(const InstDesc &d, int line0, int s, float2 *scratch, float2 *lines0,
                                             float2 *lines1, const float2 *tab) {
    using Sh = PtRowShape<N>;
    constexpr int G = Sh::G, E = N / G, LPB = Sh::LPB, FT = Sh::FT;
    constexpr int SC = LineScratch<N, G>::SIZE;
    const int tid = threadIdx.x;
    // transform role
    const bool xf = tid < 2 * FT;
    const int f = tid / FT, fl = (tid % FT) / G, t = tid % G;
    float2 *const F = f == 0 ? d.P : d.S;
    float2 *const fline = ((f & 1) ? lines1 : lines0) + fl * N;
    float2 *const fsc = scratch + (size_t)((f & 1) * LPB + fl) * SC;
    const size_t fbase = (size_t)(line0 + fl) * N;
    // point role
    const int l = tid / N, x = tid % N;
    const size_t i2 = (size_t)(line0 + l) * N + x;
    float2 *const pP = lines0 + l * N + x, *const pS = lines1 + l * N + x;
    constexpr size_t NN = (size_t)N * N;
    if (!SHG_REQUIRE(line0 >= 0 && line0 + LPB <= N, kChkRowsGlobal, line0)) return;  // block-uniform

    if (s == 0) {
        float2 vp = d.P[i2], vs = d.S[i2];
        rk4_point(vp, vs, d.stepc[0], d);
        *pP = vp;
        *pS = vs;
        __syncthreads();
        if (xf) {
            float2 v[E];
#pragma unroll
            for (int j = 0; j < E; ++j) v[j] = fline[t + G * j];
            fft_nat_to_spec<N, G, +1, false, 1, G + 1, TS>(v, t, fsc, tab);
#pragma unroll
            for (int r = 0; r < E; ++r) F[fbase + spec_index<N, G>(t, r)] = v[r];
        }
        return;
    }
    if (xf) {
        float2 v[E];
#pragma unroll
        for (int j = 0; j < E; ++j) v[j] = F[fbase + t + G * j];
        fft_nat_to_spec<N, G, -1, false, 1, G + 1, TS>(v, t, fsc, tab);
#pragma unroll
        for (int r = 0; r < E; ++r) fline[spec_index<N, G>(t, r)] = v[r];
    }
    __syncthreads();
    float2 vp = *pP, vs = *pS;
    rk4_point(vp, vs, d.stepc[s - 1], d);
    if (d.slices && s < d.nz) {
        float2 *sl = d.slices + (size_t)s * 2 * N * N;
        sl[i2] = vp;
        sl[(size_t)N * N + i2] = vs;
    }
    if (s == d.nsteps) {
        d.Pout[i2] = vp;
        d.Sout[i2] = vs;
        block_add_double((double)vs.x * vs.x + (double)vs.y * vs.y, d.acc + 1);
        block_add_double((double)vp.x * vp.x + (double)vp.y * vp.y, d.acc + 2);
        return;
    }
    rk4_point(vp, vs, d.stepc[s], d);
    *pP = vp;
    *pS = vs;
    __syncthreads();
    if (xf) {
        float2 v[E];
#pragma unroll
        for (int r = 0; r < E; ++r) v[r] = fline[spec_index<N, G>(t, r)];
        fft_spec_to_nat<N, G, +1, false, 1, G + 1, TS>(v, t, fsc, tab);
#pragma unroll
        for (int j = 0; j < E; ++j) F[fbase + t + G * j] = v[j];
    }
}

template <int N>
__global__ void __launch_bounds__(PtRowShape<N>::TPB) k_rows_pt(const InstDesc *__restrict__ inst, const int *__restrict__ list, int s) {
    using Sh = PtRowShape<N>;
    __shared__ float2 scratch[2 * Sh::LPB * LineScratch<N, Sh::G>::SIZE];
    __shared__ float2 lines[2][Sh::LPB * N];  // [field][line * N + x], natural x order
    const InstDesc &d = inst[list[blockIdx.x / Sh::BPI]];
    if (!check_solve<N>(d, s)) return;  // whole block
    rows_pt_body<N>(d, (blockIdx.x % Sh::BPI) * Sh::LPB, s, scratch, lines[0], lines[1], g_twiddle + N);
}

// The column pass of k_cols for column x of field f (0 pump, 1 SH) of solve d, lane t of the
// column's G lanes; the TC columns of a group transpose through sc (interleaved, stride TC)
// and synchronise the block (BS) or, when the group is one warp, the warp.
template <int N, int TC, bool BS>
__device__ __forceinline__ void cols_body(const InstDesc &d, int x, int f, int t, float2 *sc) {
    constexpr int G = LineShape<N>::G, E = N / G;
    const float2 *__restrict__ tab = g_twiddle + N;
    float2 *F = f == 0 ? d.P : d.S;
    const float2 *__restrict__ H = f == 0 ? d.Hp : d.Hs;
    constexpr size_t NN = (size_t)N * N;
    // propagator values first: their latency overlaps the transform
    float2 h[E];
    hprop_load<N>(H, x, t, h);
    float2 v[E];
#pragma unroll
    for (int j = 0; j < E; ++j) v[j] = SHG_AT(F, (size_t)(t + G * j) * N + x, NN, kChkColsGlobal);
    fft_nat_to_spec<N, G, +1, BS, TC, G>(v, t, sc, tab);
#pragma unroll
    for (int r = 0; r < E; ++r) v[r] = c_mul(v[r], h[r]);
    fft_spec_to_nat<N, G, -1, BS, TC, G>(v, t, sc, tab);
#pragma unroll
    for (int j = 0; j < E; ++j) SHG_AT(F, (size_t)(t + G * j) * N + x, NN, kChkColsGlobal) = v[j];
}

// Column pass. Block = TC columns x G threads (lane = column + TC * t) so that every
// load and store is a run of TC consecutive complex values; blockIdx.y = field (pump, SH).
template <int N, int TC>
__global__ void __launch_bounds__(TC * LineShape<N>::G) k_cols(const InstDesc *__restrict__ inst, const int *__restrict__ list) {
    constexpr int G = LineShape<N>::G, E = N / G, BPI = N / TC;
    __shared__ float2 scratch[TC * E * G];
    const int c = threadIdx.x % TC;
    const InstDesc &d = inst[list[blockIdx.x / BPI]];
    if (!SHG_REQUIRE(d.n == N, kChkDescriptor, d.n)) return;
    cols_body<N, TC, true>(d, (blockIdx.x % BPI) * TC + c, blockIdx.y, threadIdx.x / TC, scratch + c);
}

// ---------------------------------------------------------------------------------------
// Persistent march of one solve on a cooperative grid: the row and column passes of the
// streaming kernels (rows_pt_body, cols_body: the same arithmetic, bit-identical results)
// in one launch, separated by grid-wide barriers instead of kernel boundaries. A lone solve
// otherwise pays two dependent launches per z-step.

// Grid barrier, CoopShape and cols_body_h: shg_coop.cuh.
static_assert(CoopShape<64>::TPB == PtRowShape<64>::TPB && CoopShape<256>::ROW_UNITS == PtRowShape<256>::BPI &&
                  CoopShape<16>::TPB == PtRowShape<16>::TPB,
              "the persistent grid's row units are the row pass's blocks");

// Grid of B blocks of TPB threads; block b runs row units b, b + B, ... and column groups
// b + B w (warp w < col_warps), whose propagator values stay in registers for the whole run.
// Dynamic shared memory: col_warps scratch regions of TC * N float2. bar: zeroed arrival
// counter; err: zeroed error word of the run.
template <int N>
__global__ void __launch_bounds__(CoopShape<N>::TPB) k_march_coop(const InstDesc *__restrict__ inst,
                                                                 const int *__restrict__ list, unsigned *bar,
                                                                 int *err, int col_warps) {
    using Sh = PtRowShape<N>;
    using C = CoopShape<N>;
    constexpr int G = Sh::G;
    __shared__ float2 scratch[2 * Sh::LPB * LineScratch<N, G>::SIZE];
    __shared__ float2 lines[2][Sh::LPB * N];
    __shared__ __align__(16) float2 tws[N];  // the split's twiddle pairs, staged once per launch
    extern __shared__ float2 cscr[];
    const InstDesc &d = inst[list[0]];
    // every block of the grid leaves together (before its first barrier) on a bad descriptor
    if (!check_solve<N>(d, 0)) return;
    {
        const float2 *src = twiddle_split<N, G>(g_twiddle + N);
        for (int i = threadIdx.x; i < N; i += blockDim.x) tws[i] = src[i];
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int K = d.nsteps;
    const int u = blockIdx.x + gridDim.x * warp;
    const bool colw = warp < col_warps && u < C::COL_UNITS;
    const int f = u / (N / C::TC), x = (u % (N / C::TC)) * C::TC + lane % C::TC, t = lane / C::TC;
    float2 h[C::E];
    if (colw) hprop_load<N>(f == 0 ? d.Hp : d.Hs, x, t, h);
    unsigned target = 0;
    for (int s = 0; s <= K; ++s) {
        for (int r = blockIdx.x; r < C::ROW_UNITS; r += gridDim.x) {
            rows_pt_body<N, true>(d, r * Sh::LPB, s, scratch, lines[0], lines[1], tws);
            __syncthreads();  // the block's line buffers are reused by its next unit
        }
        if (s == K) break;
        target += gridDim.x;
        if (!grid_barrier(bar, target, err)) return;
        if (colw) cols_body_h<N, C::TC>(d, x, f, t, cscr + (size_t)warp * C::TC * N + lane % C::TC, h, tws);
        target += gridDim.x;
        if (!grid_barrier(bar, target, err)) return;
    }
}

template <int N>
static cudaError_t launch_coop_t(const InstDesc *inst, const int *list, unsigned *bar, int *err, cudaStream_t st,
                                 int *blocks_out) {
    using C = CoopShape<N>;
    constexpr int warps = C::TPB / 32;
    auto k = k_march_coop<N>;
    int dev = 0, sms = 0, per_sm = 0;
    cudaError_t e;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    // one column group per block where that many blocks fit co-resident (the column pass
    // then spreads over the most SMs), else the fewest blocks that hold every row unit
    int blocks = 0, col_warps = 0;
    size_t smem = 0;
    for (int pass = 0; pass < 2 && !blocks; ++pass) {
        int b = C::ROW_UNITS;
        if (pass == 0 && C::COL_UNITS > b) b = C::COL_UNITS;
        if ((C::COL_UNITS + warps - 1) / warps > b) b = (C::COL_UNITS + warps - 1) / warps;
        const int cw = (C::COL_UNITS + b - 1) / b;
        const size_t sm = (size_t)cw * C::TC * N * sizeof(float2);
        if ((e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm)) != cudaSuccess) return e;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, C::TPB, sm)) != cudaSuccess) return e;
        if (per_sm * sms >= b) {
            blocks = b;
            col_warps = cw;
            smem = sm;
        }
    }
    if (!blocks) return cudaErrorCooperativeLaunchTooLarge;
    if (blocks_out) *blocks_out = blocks;
    if (!inst) return cudaSuccess;  // fit check only
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(blocks, 1, 1);
    cfg.blockDim = dim3(C::TPB, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k, inst, list, bar, err, col_warps);
}

cudaError_t launch_coop(int n, const InstDesc *inst, const int *list, unsigned *bar, int *err, cudaStream_t st,
                        int *blocks) {
    switch (n) {
        case 16: return launch_coop_t<16>(inst, list, bar, err, st, blocks);
        case 32: return launch_coop_t<32>(inst, list, bar, err, st, blocks);
        case 64: return launch_coop_t<64>(inst, list, bar, err, st, blocks);
        case 128: return launch_coop_t<128>(inst, list, bar, err, st, blocks);
        case 256: return launch_coop_t<256>(inst, list, bar, err, st, blocks);
        default: return cudaErrorInvalidValue;
    }
}

// ---------------------------------------------------------------------------------------
// Standalone unnormalised 2D DFT (component tests): rows, then columns in place on out.
template <int N, int SIGN>
__global__ void __launch_bounds__(RowShape<N>::TPB) k_dft_rows(const float2 *__restrict__ in, float2 *out) {
    constexpr int G = LineShape<N>::G, E = N / G, LPB = RowShape<N>::LPB;
    constexpr int SC = LineScratch<N, G>::SIZE;
    __shared__ float2 scratch[LPB * SC];
    const float2 *__restrict__ tab = g_twiddle + N;
    const int line = blockIdx.x * LPB + threadIdx.x / G, t = threadIdx.x % G;
    float2 *sc = scratch + (threadIdx.x / G) * SC;
    float2 v[E];
#pragma unroll
    for (int j = 0; j < E; ++j) v[j] = in[(size_t)line * N + t + G * j];
    fft_nat_to_spec<N, G, SIGN>(v, t, sc, tab);
#pragma unroll
    for (int r = 0; r < E; ++r) out[(size_t)line * N + spec_index<N, G>(t, r)] = v[r];
}

template <int N, int SIGN>
__global__ void __launch_bounds__(16 * LineShape<N>::G) k_dft_cols(float2 *out) {
    constexpr int G = LineShape<N>::G, E = N / G, TC = 16;
    __shared__ float2 scratch[TC * E * G];
    const float2 *__restrict__ tab = g_twiddle + N;
    const int c = threadIdx.x % TC, t = threadIdx.x / TC, x = blockIdx.x * TC + c;
    float2 v[E];
#pragma unroll
    for (int j = 0; j < E; ++j) v[j] = out[(size_t)(t + G * j) * N + x];
    fft_nat_to_spec<N, G, SIGN, true, TC, G>(v, t, scratch + c, tab);
    __syncthreads();
#pragma unroll
    for (int r = 0; r < E; ++r) out[(size_t)spec_index<N, G>(t, r) * N + x] = v[r];
}

template <int N>
static cudaError_t launch_dft2d_t(int sign, const float2 *in, float2 *out, cudaStream_t st) {
    constexpr int G = LineShape<N>::G, TC = 16;
    constexpr int rb = RowShape<N>::BPI, tpb = RowShape<N>::TPB;
    if (sign < 0) {
        k_dft_rows<N, -1><<<rb, tpb, 0, st>>>(in, out);
        k_dft_cols<N, -1><<<N / TC, TC * G, 0, st>>>(out);
    } else {
        k_dft_rows<N, +1><<<rb, tpb, 0, st>>>(in, out);
        k_dft_cols<N, +1><<<N / TC, TC * G, 0, st>>>(out);
    }
    return cudaGetLastError();
}

template <int N>
static cudaError_t launch_dft_rows_t(int sign, const float2 *in, float2 *out, int fields, cudaStream_t st) {
    const int blocks = RowShape<N>::BPI * fields;  // fields stored back to back: n*fields rows
    if (sign < 0)
        k_dft_rows<N, -1><<<blocks, RowShape<N>::TPB, 0, st>>>(in, out);
    else
        k_dft_rows<N, +1><<<blocks, RowShape<N>::TPB, 0, st>>>(in, out);
    return cudaGetLastError();
}

cudaError_t launch_dft_rows(int n, int sign, const float2 *in, float2 *out, cudaStream_t st, int fields) {
    switch (n) {
        case 16: return launch_dft_rows_t<16>(sign, in, out, fields, st);
        case 32: return launch_dft_rows_t<32>(sign, in, out, fields, st);
        case 64: return launch_dft_rows_t<64>(sign, in, out, fields, st);
        case 128: return launch_dft_rows_t<128>(sign, in, out, fields, st);
        case 256: return launch_dft_rows_t<256>(sign, in, out, fields, st);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_dft2d(int n, int sign, const float2 *in, float2 *out, cudaStream_t st) {
    switch (n) {
        case 16: return launch_dft2d_t<16>(sign, in, out, st);
        case 32: return launch_dft2d_t<32>(sign, in, out, st);
        case 64: return launch_dft2d_t<64>(sign, in, out, st);
        case 128: return launch_dft2d_t<128>(sign, in, out, st);
        case 256: return launch_dft2d_t<256>(sign, in, out, st);
        default: return cudaErrorInvalidValue;
    }
}

// ---------------------------------------------------------------------------------------
// Host-side launchers.

int rows_threads() { return 256; }

template <int N>
static cudaError_t launch_rows_t(const InstDesc *inst, const int *list, int count, int s, cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
    if (count >= 4)
        k_rows<N><<<count * RowShape<N>::BPI, RowShape<N>::TPB, 0, st>>>(inst, list, s);
    else
        k_rows_pt<N><<<count * PtRowShape<N>::BPI, PtRowShape<N>::TPB, 0, st>>>(inst, list, s);
    return cudaGetLastError();
}

// 16-column tiles when several solves fill the GPU; 4-column tiles (four times the blocks)
// for one to three solves, where the launch would otherwise cover a few SMs.
template <int N>
static cudaError_t launch_cols_t(const InstDesc *inst, const int *list, int count, cudaStream_t st) {
    constexpr int G = LineShape<N>::G;
    if (count <= 0) return cudaSuccess;
    if (count >= 4)
        k_cols<N, 16><<<dim3(count * (N / 16), 2), 16 * G, 0, st>>>(inst, list);
    else
        k_cols<N, 4><<<dim3(count * (N / 4), 2), 4 * G, 0, st>>>(inst, list);
    return cudaGetLastError();
}

cudaError_t launch_rows(int n, const InstDesc *inst, const int *list, int count, int s, cudaStream_t st) {
    switch (n) {
        case 16: return launch_rows_t<16>(inst, list, count, s, st);
        case 32: return launch_rows_t<32>(inst, list, count, s, st);
        case 64: return launch_rows_t<64>(inst, list, count, s, st);
        case 128: return launch_rows_t<128>(inst, list, count, s, st);
        case 256: return launch_rows_t<256>(inst, list, count, s, st);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_cols(int n, const InstDesc *inst, const int *list, int count, cudaStream_t st) {
    switch (n) {
        case 16: return launch_cols_t<16>(inst, list, count, st);
        case 32: return launch_cols_t<32>(inst, list, count, st);
        case 64: return launch_cols_t<64>(inst, list, count, st);
        case 128: return launch_cols_t<128>(inst, list, count, st);
        case 256: return launch_cols_t<256>(inst, list, count, st);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_setup(const InstDesc *inst, int n_inst, int max_nn, int max_nz, cudaStream_t st) {
    if (n_inst <= 0) return cudaSuccess;
    k_setup_steps<<<n_inst, 256, (size_t)max_nz * sizeof(float), st>>>(inst, n_inst);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    dim3 grid((max_nn + 1023) / 1024, n_inst);
    k_setup_fields<<<grid, 256, 0, st>>>(inst);
    return cudaGetLastError();
}

bool line_length_supported(int n) { return n == 16 || n == 32 || n == 64 || n == 128 || n == 256; }

}  // namespace shg
