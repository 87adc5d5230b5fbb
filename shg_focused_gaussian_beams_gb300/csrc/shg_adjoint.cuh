// Device helpers shared by the adjoint kernels of the plain and the thermal z-march.
#pragma once

#include <cuda_runtime.h>

#include "shg_march.cuh"

namespace shg {

// Adds the block's k partial sums (k <= 6) to dst[0..k) with one FP64 atomic each.
__device__ __forceinline__ void block_sum_doubles(double *v, int k, double *dst) {
    __shared__ double red[32][6];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    for (int j = 0; j < k; ++j)
        for (int o = 16; o > 0; o >>= 1) v[j] += __shfl_xor_sync(0xffffffffu, v[j], o);
    __syncthreads();
    if (l == 0)
        for (int j = 0; j < k; ++j) red[w][j] = v[j];
    __syncthreads();
    if (w == 0) {
        for (int j = 0; j < k; ++j) {
            double x = (l < (int)(blockDim.x >> 5)) ? red[l][j] : 0.0;
            for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
            if (l == 0 && x != 0.0) atomicAdd(dst + j, x);
        }
    }
}

// Adds the block's k per-thread FP32 partial sums (k <= 5, blockDim <= 512) to dst[0..k)
// in FP64: the partials are staged in shared memory and warp j sums quantity j in double,
// so a thread converts 512/32 values of one quantity instead of reducing five doubles.
__device__ __forceinline__ void block_sum_f2d(const float *v, int k, double *dst) {
    __shared__ float stage[5][512];
    const int tid = threadIdx.x, w = tid >> 5, l = tid & 31, nt = blockDim.x;
    __syncthreads();  // earlier users of the stage are done
    for (int j = 0; j < k; ++j) stage[j][tid] = v[j];
    __syncthreads();
    if (w < k) {
        double a = 0.0;
        for (int i = l; i < nt; i += 32) a += (double)stage[w][i];
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if (l == 0 && a != 0.0) atomicAdd(dst + w, a);
    }
}

// Reverse mode of one dA/dz evaluation at (P, S) with output cotangents (u, v); adds the
// input cotangents to (cp, cs) and the parameter sensitivities to acc (T = double, or
// float for the per-point partial sums that a block then reduces in FP64).
template <typename T>
__device__ __forceinline__ void dadz_vjp(float2 P, float2 S, float2 u, float2 v, float4 c, float hp, float tpa0,
                                         float tpa1, float2 &cp, float2 &cs, T *acc) {
    const float2 aP = make_float2(c.x, c.y), aS = make_float2(c.z, c.w);
    // c_P = -hp u + aP S conj(u) + 2 conj(aS) conj(P) v
    const float2 aPS = c_mul(aP, S);
    const float2 t1 = c_mulc(aPS, u);                      // aP S conj(u)
    const float2 cPv = c_mulc(v, c_mul(aS, P));            // v conj(aS P) = conj(aS) conj(P) v
    cp.x += -hp * u.x + t1.x + 2.0f * cPv.x;
    cp.y += -hp * u.y + t1.y + 2.0f * cPv.y;
    // c_S = conj(aP) P u - (tpa0 + 2 tpa1 |S|^2) v - tpa1 S^2 conj(v)
    const float a2 = fmaf(S.x, S.x, S.y * S.y);
    const float2 t2 = c_mulc(c_mul(P, u), aP);             // P u conj(aP)
    const float2 S2 = c_mul(S, S);
    const float2 t3 = c_mulc(S2, v);                       // S^2 conj(v)
    const float g = fmaf(2.0f * tpa1, a2, tpa0);
    cs.x += t2.x - g * v.x - tpa1 * t3.x;
    cs.y += t2.y - g * v.y - tpa1 * t3.y;
    // sensitivities: sum conj(S conj(P)) u, sum conj(P^2) v, sum Re(conj(v) (-|S|^2 S))
    const float2 gP = c_mulc(S, P);                        // S conj(P)
    const float2 hS = c_mul(P, P);
    const float2 eP = c_mulc(u, gP);                       // u conj(g)
    const float2 eS = c_mulc(v, hS);                       // v conj(h)
    acc[0] += (T)eP.x;
    acc[1] += (T)eP.y;
    acc[2] += (T)eS.x;
    acc[3] += (T)eS.y;
    acc[4] += -(T)a2 * ((T)v.x * (T)S.x + (T)v.y * (T)S.y);
}

// RK4^T of Solver.h:216-228 at the base state (P, S) with step constants c: (cP, cS) hold
// the cotangent of the RK4 output on entry and of its input on exit; acc[0..4] += the
// step's sensitivities.
template <typename T>
__device__ __forceinline__ void rk4_vjp_point(float2 P, float2 S, float2 &cP, float2 &cS, float4 c, float hp,
                                              float t0, float t1, float w6, T *acc) {
    // forward stages
    float2 k1p, k1s, k2p, k2s, k3p, k3s;
    dadz_point(P, S, c, hp, t0, t1, k1p, k1s);
    const float2 B2p = make_float2(fmaf(0.5f, k1p.x, P.x), fmaf(0.5f, k1p.y, P.y));
    const float2 B2s = make_float2(fmaf(0.5f, k1s.x, S.x), fmaf(0.5f, k1s.y, S.y));
    dadz_point(B2p, B2s, c, hp, t0, t1, k2p, k2s);
    const float2 B3p = make_float2(fmaf(0.5f, k2p.x, P.x), fmaf(0.5f, k2p.y, P.y));
    const float2 B3s = make_float2(fmaf(0.5f, k2s.x, S.x), fmaf(0.5f, k2s.y, S.y));
    dadz_point(B3p, B3s, c, hp, t0, t1, k3p, k3s);
    const float2 B4p = c_add(P, k3p), B4s = c_add(S, k3s);
    // reverse
    const float2 op = cP, os = cS;
    float2 cap = op, cas = os;
    float2 ck3p = make_float2(2.0f * w6 * op.x, 2.0f * w6 * op.y), ck3s = make_float2(2.0f * w6 * os.x, 2.0f * w6 * os.y);
    float2 ck2p = ck3p, ck2s = ck3s;
    float2 ck1p = make_float2(w6 * op.x, w6 * op.y), ck1s = make_float2(w6 * os.x, w6 * os.y);
    const float2 ck4p = ck1p, ck4s = ck1s;
    float2 bp = make_float2(0.f, 0.f), bs = make_float2(0.f, 0.f);
    dadz_vjp(B4p, B4s, ck4p, ck4s, c, hp, t0, t1, bp, bs, acc);
    cap = c_add(cap, bp);
    cas = c_add(cas, bs);
    ck3p = c_add(ck3p, bp);
    ck3s = c_add(ck3s, bs);
    bp = bs = make_float2(0.f, 0.f);
    dadz_vjp(B3p, B3s, ck3p, ck3s, c, hp, t0, t1, bp, bs, acc);
    cap = c_add(cap, bp);
    cas = c_add(cas, bs);
    ck2p = make_float2(fmaf(0.5f, bp.x, ck2p.x), fmaf(0.5f, bp.y, ck2p.y));
    ck2s = make_float2(fmaf(0.5f, bs.x, ck2s.x), fmaf(0.5f, bs.y, ck2s.y));
    bp = bs = make_float2(0.f, 0.f);
    dadz_vjp(B2p, B2s, ck2p, ck2s, c, hp, t0, t1, bp, bs, acc);
    cap = c_add(cap, bp);
    cas = c_add(cas, bs);
    ck1p = make_float2(fmaf(0.5f, bp.x, ck1p.x), fmaf(0.5f, bp.y, ck1p.y));
    ck1s = make_float2(fmaf(0.5f, bs.x, ck1s.x), fmaf(0.5f, bs.y, ck1s.y));
    bp = bs = make_float2(0.f, 0.f);
    dadz_vjp(P, S, ck1p, ck1s, c, hp, t0, t1, bp, bs, acc);
    cP = c_add(cap, bp);
    cS = c_add(cas, bs);
}

// Fused row passes for one solve, one thread per point (block = LPB lines x N threads; the
// x-transforms of the pump and SH lines run on two groups of LPB * G threads). Between two
// column passes a row pass finishes one diffraction along x, applies the pointwise RK4 (or
// RK4^T) work of the step boundary, and starts the next diffraction along x, so a z-step
// costs one row and one column launch. The working state A / cotangent C holds the pump
// then the SH field (n*n each); the column passes (k_colpass) see rows in natural
// frequency order, as after launch_dft_rows(+1).
template <int N>
struct AdjRowShape {
    static constexpr int G = LineShape<N>::G;
    static constexpr int LPB = (512 / N < N) ? 512 / N : N;
    static constexpr int TPB = LPB * N;
    static constexpr int BPI = N / LPB;
    static constexpr int FT = LPB * G;  // transform threads per field
    static_assert(FT % 32 == 0 && 2 * FT <= TPB && N % LPB == 0, "transform threads fill whole warps");
};

// Shared state of a fused row pass: line buffers and the roles of this thread.
template <int N>
struct AdjRowCtx {
    using Sh = AdjRowShape<N>;
    static constexpr int G = Sh::G, E = N / G, LPB = Sh::LPB, FT = Sh::FT, SC = LineScratch<N, G>::SIZE;
    float2 *fline, *fsc;  // transform role: this thread's line buffer and FFT scratch
    int t;
    bool xf;
    size_t frow;          // offset of the transformed row in A (field included)
    size_t i2;            // point role: index of the point in one field
    int lx;               // point role: offset in a line buffer
    __device__ AdjRowCtx(float2 (*lines)[LPB * N], float2 *scratch) {
        const int tid = threadIdx.x, line0 = blockIdx.x * LPB;
        xf = tid < 2 * FT;
        const int f = (tid / FT) & 1, fl = (tid % FT) / G;
        t = tid % G;
        fline = lines[f] + fl * N;
        fsc = scratch + (size_t)(f * LPB + fl) * SC;
        frow = (size_t)f * N * N + (size_t)(line0 + fl) * N;
        const int l = tid / N, x = tid % N;
        i2 = (size_t)(line0 + l) * N + x;
        lx = l * N + x;
    }
    // rows of A (natural frequency order) -> line buffers in real space (natural x order)
    __device__ void finish(const float2 *A, const float2 *tab) {
        if (xf) {
            float2 v[E];
#pragma unroll
            for (int j = 0; j < E; ++j) v[j] = A[frow + t + G * j];
            fft_nat_to_spec<N, G, -1>(v, t, fsc, tab);
#pragma unroll
            for (int r = 0; r < E; ++r) fline[spec_index<N, G>(t, r)] = v[r];
        }
    }
    // line buffers (real space) -> rows of A in natural frequency order
    __device__ void start(float2 *A, const float2 *tab) {
        if (xf) {
            float2 v[E];
#pragma unroll
            for (int r = 0; r < E; ++r) v[r] = fline[spec_index<N, G>(t, r)];
            fft_spec_to_nat<N, G, +1>(v, t, fsc, tab);
#pragma unroll
            for (int j = 0; j < E; ++j) A[frow + t + G * j] = v[j];
        }
    }
};

}  // namespace shg
