// Line FFTs for the transverse diffraction step (replaces the fftwf_plan_dft_2d /
// fftwf_execute calls of Solver.h:161-187).
//
// A line of N complex points is held by a group of G threads, E = N/G points per thread,
// and transformed in two register stages with one shared-memory transpose between them
// (N = E * G, x = t + G*j on input):
//
//   stage 1: each thread runs an E-point DFT over its registers (compile-time twiddles),
//   twiddle:  multiply by w_N^(t*k2) from a table evaluated in double and rounded once
//             (stored per split as 16-byte pairs, see g_twiddle),
//   transpose through shared memory,
//   stage 2: each thread runs E/G DFTs of G points.
//
// Two register layouts matter to callers:
//   natural  L_in : thread t, register j          <-> index t + G*j
//   spectral L_out: thread t, register m*G + k1   <-> index (t*(E/G) + m) + E*k1
// `fft_nat_to_spec` maps L_in data to its DFT in L_out; `fft_spec_to_nat` maps L_out
// data to its DFT in L_in (the transposed factorisation of the same symmetric DFT
// matrix). Pointwise work between a transform and the next one in the other direction
// (propagator products, the RK4 coupling) therefore never reorders data.
//
// SIGN = -1 is FFTW_FORWARD (exp(-2 pi i jk/N)), SIGN = +1 is FFTW_BACKWARD.
#pragma once

#include <cuda_runtime.h>

#include <utility>

#include "shg_check.cuh"

namespace shg {

constexpr int kMaxLine = 256;

// Threads per line for each supported line length (E = N/G points per thread).
template <int N>
struct LineShape;
template <> struct LineShape<16> { static constexpr int G = 4; };
template <> struct LineShape<32> { static constexpr int G = 4; };
template <> struct LineShape<64> { static constexpr int G = 8; };
template <> struct LineShape<128> { static constexpr int G = 8; };
template <> struct LineShape<256> { static constexpr int G = 16; };
template <> struct LineShape<512> { static constexpr int G = 16; };

// Inter-stage twiddles w_N^(t*k2) = exp(-2 pi i (t*k2 mod N) / N) of the split N = E x G,
// for N = 16..kMaxLine, stored as 16-byte pairs: word (j*G + t) holds the twiddles of
// k2 = 2j and 2j+1 for thread t (j < E/2), so the E - 1 twiddles of a thread take E/2
// vector loads and the lanes of consecutive t read consecutive words. The table of line
// length N for the default split G = LineShape<N>::G sits at float2 offset [N, 2N), the
// one for G = LineShape<N>::G / 2 (N >= 64) at [2*kMaxLine + N, 2*kMaxLine + 2N). Each
// translation unit that launches line FFTs has its own copy (internal linkage) whose
// address the host looks up; the host fills every copy once per device.
static __device__ __align__(16) float2 g_twiddle[4 * kMaxLine];

__device__ __forceinline__ float2 c_add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 c_sub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 c_mul(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// a * conj(b)
__device__ __forceinline__ float2 c_mulc(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.y, b.x, -a.x * b.y));
}

template <int... Is, class F>
__device__ __forceinline__ void sfor_impl(std::integer_sequence<int, Is...>, F &&f) {
    (f(std::integral_constant<int, Is>{}), ...);
}
// Compile-time unrolled loop: f(std::integral_constant<int, i>) for i in [0, N).
template <int N, class F>
__device__ __forceinline__ void sfor(F &&f) {
    sfor_impl(std::make_integer_sequence<int, N>{}, f);
}

__host__ __device__ constexpr int ilog2(int n) { return n <= 1 ? 0 : 1 + ilog2(n / 2); }
__host__ __device__ constexpr int bitrev(int i, int bits) {
    int r = 0;
    for (int b = 0; b < bits; ++b)
        if (i & (1 << b)) r |= 1 << (bits - 1 - b);
    return r;
}

// cos / sin of 2*pi*m/32, m < 16, evaluated in double and rounded to float.
struct W32 {
    static constexpr float c[16] = {1.0f, 0.9807852506637573f, 0.9238795042037964f, 0.8314695954322815f,
                                    0.7071067690849304f, 0.5555702447891235f, 0.3826834261417389f,
                                    0.19509032368659973f, 0.0f, -0.19509032368659973f, -0.3826834261417389f,
                                    -0.5555702447891235f, -0.7071067690849304f, -0.8314695954322815f,
                                    -0.9238795042037964f, -0.9807852506637573f};
    static constexpr float s[16] = {0.0f, 0.19509032368659973f, 0.3826834261417389f, 0.5555702447891235f,
                                    0.7071067690849304f, 0.8314695954322815f, 0.9238795042037964f,
                                    0.9807852506637573f, 1.0f, 0.9807852506637573f, 0.9238795042037964f,
                                    0.8314695954322815f, 0.7071067690849304f, 0.5555702447891235f,
                                    0.3826834261417389f, 0.19509032368659973f};
};

// tan(pi m / 16) for m = 0..4, evaluated in double and rounded to float.
struct TanPi16 {
    static constexpr float t[5] = {0.0f, 0.19891236737965800691f, 0.41421356237309504880f, 0.66817863791929891999f,
                                   1.0f};
};

// Radix-2 butterfly (x, y) -> (x + w y, x - w y), w = exp(SIGN * 2 pi i M / 32). A
// non-trivial w y is formed as f * u with f = cos or sin of the angle (whichever is larger
// in magnitude) and u = y rotated by the ratio of the other to it (|ratio| <= 1), so that
// f multiplies inside the output FMAs: six instructions instead of eight for the
// product-then-add form.
template <int SIGN, int M>
__device__ __forceinline__ void bfly_const(float2 &a, float2 &b) {
    const float2 x = a, y = b;
    if constexpr (M == 0) {
        a = c_add(x, y);
        b = c_sub(x, y);
    } else if constexpr (M == 8) {
        const float2 wy = SIGN > 0 ? make_float2(-y.y, y.x) : make_float2(y.y, -y.x);
        a = c_add(x, wy);
        b = c_sub(x, wy);
    } else if constexpr (M <= 4 || M >= 12) {
        // w y = c (y.x - tau y.y, y.y + tau y.x), tau = SIGN tan(angle), |tau| <= 1
        constexpr float c = W32::c[M];
        constexpr float tau = (SIGN > 0 ? 1.0f : -1.0f) * (M <= 4 ? TanPi16::t[M] : -TanPi16::t[16 - M]);
        const float ux = fmaf(-tau, y.y, y.x), uy = fmaf(tau, y.x, y.y);
        a = make_float2(fmaf(c, ux, x.x), fmaf(c, uy, x.y));
        b = make_float2(fmaf(-c, ux, x.x), fmaf(-c, uy, x.y));
    } else {
        // w y = s (kappa y.x - y.y, kappa y.y + y.x), s = SIGN sin(angle), kappa = SIGN cot(angle)
        constexpr float sg = SIGN > 0 ? 1.0f : -1.0f;
        constexpr float s = sg * W32::s[M];
        constexpr float kappa = sg * (M < 8 ? TanPi16::t[8 - M] : -TanPi16::t[M - 8]);
        const float ux = fmaf(kappa, y.x, -y.y), uy = fmaf(kappa, y.y, y.x);
        a = make_float2(fmaf(s, ux, x.x), fmaf(s, uy, x.y));
        b = make_float2(fmaf(-s, ux, x.x), fmaf(-s, uy, x.y));
    }
}

// In-register DFT of E <= 32 points held in v[OFF .. OFF+E), natural order in and out
// (radix-2 decimation in time over a bit-reversed copy; the permutations are renamings).
template <int E, int SIGN, int OFF = 0, int NV>
__device__ __forceinline__ void dft_reg(float2 (&v)[NV]) {
    static_assert(E >= 1 && E <= 32 && (E & (E - 1)) == 0, "register DFT size");
    if constexpr (E == 1) return;
    constexpr int LG = ilog2(E);
    float2 t[E];
    sfor<E>([&](auto I) { t[bitrev(decltype(I)::value, LG)] = v[OFF + decltype(I)::value]; });
    sfor<LG>([&](auto S) {
        constexpr int len = 2 << decltype(S)::value;
        constexpr int half = len / 2;
        sfor<E / 2>([&](auto B) {
            constexpr int grp = decltype(B)::value / half, k = decltype(B)::value % half;
            constexpr int a = grp * len + k, b = a + half;
            bfly_const<SIGN, k * (32 / len)>(t[a], t[b]);
        });
    });
    sfor<E>([&](auto I) { v[OFF + decltype(I)::value] = t[decltype(I)::value]; });
}

// The pair table of split (N, G) within the line length's block tab = g_twiddle + N.
template <int N, int G>
__device__ __forceinline__ const float2 *twiddle_split(const float2 *tab) {
    static_assert(G == LineShape<N>::G || (N >= 64 && 2 * G == LineShape<N>::G), "no twiddle table for this split");
    return G == LineShape<N>::G ? tab : tab + 2 * kMaxLine;
}

// Inter-stage twiddle multiply of thread t: v[k2] *= w_N^(SIGN-direction t*k2), k2 >= 1,
// from the pair table of split (N, G). tab: the line length's block g_twiddle + N, or with
// TS a copy of the split's own table (N float2) in shared memory.
template <int N, int G, int SIGN, bool TS = false>
__device__ __forceinline__ void twiddle_mul(float2 (&v)[N / G], int t, const float2 *__restrict__ tab) {
    constexpr int E = N / G;
    const float4 *__restrict__ w4 = reinterpret_cast<const float4 *>(TS ? tab : twiddle_split<N, G>(tab)) + t;
#pragma unroll
    for (int j = 0; j < E / 2; ++j) {
        const float4 q = TS ? w4[j * G] : __ldg(w4 + j * G);  // SIGN = +1 uses the conjugates
        if (j > 0) v[2 * j] = c_mul(v[2 * j], make_float2(q.x, SIGN > 0 ? -q.y : q.y));
        v[2 * j + 1] = c_mul(v[2 * j + 1], make_float2(q.z, SIGN > 0 ? -q.w : q.w));
    }
}

// Per-line shared scratch: E rows of G entries padded to G+1, plus a line pad.
__host__ __device__ constexpr int pad_to_8_mod_16(int s) {
    while (s % 16 != 8) ++s;
    return s;
}
template <int N, int G>
struct LineScratch {
    static constexpr int E = N / G;
    static constexpr int GP = G + 1;
    static constexpr int SIZE = pad_to_8_mod_16(E * GP);
};

// Lines whose G threads sit in one warp synchronise the warp; lines spread over warps
// (BS = true) synchronise the block.
template <bool BS>
__device__ __forceinline__ void group_sync() {
    if constexpr (BS) __syncthreads();
    else __syncwarp();
}

// Shared-scratch geometry of one line: element (row e < E, column g < G) lives at
// sc[(e * GP + g) * STRIDE]. Lines held by consecutive lanes (FAST passes) use STRIDE = 1,
// GP = G + 1 and a padded per-line base; lines interleaved across lanes (column passes)
// use STRIDE = lines per block, GP = G and base = scratch + line.
// L_in -> DFT in L_out.
template <int N, int G, int SIGN, bool BS = false, int STRIDE = 1, int GP = G + 1, bool TS = false>
__device__ __forceinline__ void fft_nat_to_spec(float2 (&v)[N / G], int t, float2 *sc, const float2 *__restrict__ tab) {
    constexpr int E = N / G, Q = E / G;
    static_assert(E % G == 0, "need G <= E with G | E");
    dft_reg<E, SIGN>(v);
    twiddle_mul<N, G, SIGN, TS>(v, t, tab);
    group_sync<BS>();
#pragma unroll
    for (int k2 = 0; k2 < E; ++k2) sc[(k2 * GP + t) * STRIDE] = v[k2];
    group_sync<BS>();
#pragma unroll
    for (int m = 0; m < Q; ++m)
#pragma unroll
        for (int tt = 0; tt < G; ++tt) v[m * G + tt] = sc[((t * Q + m) * GP + tt) * STRIDE];
    sfor<Q>([&](auto M) { dft_reg<G, SIGN, decltype(M)::value * G>(v); });
}

// L_out -> DFT in L_in.
template <int N, int G, int SIGN, bool BS = false, int STRIDE = 1, int GP = G + 1, bool TS = false>
__device__ __forceinline__ void fft_spec_to_nat(float2 (&v)[N / G], int t, float2 *sc, const float2 *__restrict__ tab) {
    constexpr int E = N / G, Q = E / G;
    static_assert(E % G == 0, "need G <= E with G | E");
    sfor<Q>([&](auto M) { dft_reg<G, SIGN, decltype(M)::value * G>(v); });
    group_sync<BS>();
#pragma unroll
    for (int m = 0; m < Q; ++m)
#pragma unroll
        for (int tt = 0; tt < G; ++tt) sc[((t * Q + m) * GP + tt) * STRIDE] = v[m * G + tt];
    group_sync<BS>();
#pragma unroll
    for (int k2 = 0; k2 < E; ++k2) v[k2] = sc[(k2 * GP + t) * STRIDE];
    twiddle_mul<N, G, SIGN, TS>(v, t, tab);
    dft_reg<E, SIGN>(v);
}

// Index of register r of thread t in the spectral layout L_out.
template <int N, int G>
__device__ __forceinline__ int spec_index(int t, int r) {
    constexpr int E = N / G, Q = E / G;
    const int m = r / G, k1 = r % G;
    return (t * Q + m) + E * k1;
}

// Propagator storage order. The column transforms (G = LineShape<N>::G threads per column,
// E = N / G registers each) multiply register r of thread t by the propagator of spectral
// row k = spec_index<N, G>(t, r) and column x. Registers r = 2j, 2j+1 of thread t form one
// 16-byte word, and the words of consecutive columns are adjacent: word (t * E/2 + j) * N + x.
// A warp over consecutive columns then reads whole segments with E/2 loads per thread
// instead of E.
__host__ __device__ inline int line_threads(int n) { return n <= 32 ? 4 : (n <= 128 ? 8 : 16); }

__host__ __device__ inline size_t hprop_index_rt(int n, int k, int x) {
    const int G = line_threads(n), E = n / G, Q = E / G;
    const int rem = k % E, k1 = k / E;
    const int t = rem / Q, r = (rem % Q) * G + k1;
    return (((size_t)t * (E / 2) + (r >> 1)) * n + x) * 2 + (r & 1);
}

template <int N>
__device__ __forceinline__ size_t hprop_index(int k, int x) {
    constexpr int G = LineShape<N>::G, E = N / G, Q = E / G;
    const int rem = k % E, k1 = k / E;
    const int t = rem / Q, r = (rem % Q) * G + k1;
    return (((size_t)t * (E / 2) + (r >> 1)) * N + x) * 2 + (r & 1);
}

// The E propagator values of column x for thread t of a column transform with
// G = LineShape<N>::G (H 16-byte aligned).
template <int N>
__device__ __forceinline__ void hprop_load(const float2 *__restrict__ H, int x, int t,
                                           float2 (&h)[N / LineShape<N>::G]) {
    constexpr int G = LineShape<N>::G, E = N / G;
    static_assert(E % 2 == 0, "pairs of values per 16-byte load");
    const float4 *p = reinterpret_cast<const float4 *>(H);
#pragma unroll
    for (int j = 0; j < E / 2; ++j) {
        const float4 q = __ldg(&SHG_AT(p, ((size_t)t * (E / 2) + j) * N + x, (size_t)N * N / 2, kChkPropagator));
        h[2 * j] = make_float2(q.x, q.y);
        h[2 * j + 1] = make_float2(q.z, q.w);
    }
}

}  // namespace shg
