// Adjoint of the plain z-march (reverse-mode through Solver.h:193-276).
//
// One SSFM step maps X_s -> Y = RK4(X_s; z_s) -> W = D(Y) -> X_{s+1} = RK4(W; z_s), with
// D(Y) = F_fwd(H' . F_bwd(Y)) (H' the shifted propagator over NX*NY). For a real loss L,
// the cotangent of a complex field A is c_A = dL/dRe(A) + i dL/dIm(A) (Wirtinger form).
// The reverse step is
//   c_W = RK4^T(W)[c_{X_{s+1}}],  c_Y = D^H c_W = F_fwd(conj(H') . F_bwd(c_W)),
//   c_{X_s} = RK4^T(X_s)[c_Y],
// where RK4^T recomputes the stage states of Solver.h:216-228 pointwise and applies
// c_x = conj(dy/dx) c_y + (dy/dconj x) conj(c_y) through each dA/dz evaluation.
// Per-step sums (FP64) of the sensitivities to the complex coupling constants, to the
// two-photon-absorption factor and to the propagator wavenumbers give the parameter
// gradients (oven temperature, poling period) on the host.
#include <cuda_runtime.h>

#include "shg_adjoint.cuh"
#include "shg_internal.h"
#include "shg_march.cuh"

namespace shg {

const float2 *twiddle_symbol_address_adjoint() {
    void *p = nullptr;
    cudaGetSymbolAddress(&p, g_twiddle);
    return static_cast<const float2 *>(p);
}

// Forward RK4 on a plain state (Solver.h:216-228 with the step constants folded).
__global__ void k_rk4_state(float2 *P, float2 *S, int nn, const float4 *__restrict__ stepc, int s,
                            const InstDesc *__restrict__ dd) {
    const InstDesc &d = *dd;
    const float4 c = stepc[s];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += gridDim.x * blockDim.x) {
        float2 p = P[i], q = S[i];
        rk4_point(p, q, c, d);
        P[i] = p;
        S[i] = q;
    }
}

// RK4^T at the base state (P0, S0): (cP, cS) hold the cotangent of the RK4 output on
// entry and of its input on exit. acc_step[0..4] += the step's sensitivities.
__global__ void k_rk4_vjp(const float2 *__restrict__ P0, const float2 *__restrict__ S0, float2 *cP, float2 *cS,
                          int nn, const float4 *__restrict__ stepc, int s, const InstDesc *__restrict__ dd,
                          double *acc_step) {
    const InstDesc &d = *dd;
    const float4 c = stepc[s];
    const float hp = d.hp, t0 = d.tpa0, t1 = d.tpa1, w6 = d.dz6;
    double acc[5] = {0, 0, 0, 0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += gridDim.x * blockDim.x) {
        const float2 P = P0[i], S = S0[i];
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
        const float2 op = cP[i], os = cS[i];
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
        cP[i] = c_add(cap, bp);
        cS[i] = c_add(cas, bs);
    }
    block_sum_doubles(acc, 5, acc_step);
}

// Column pass of the diffraction step on one field of one solve (after the row transform
// along x with sign +1): backward transform along y, then either
//   MODE 0 (forward):  store the 2D spectrum F (if Fst), multiply by H', forward along y;
//   MODE 1 (adjoint):  acc += sum Re(F conj(X) i H' q2), multiply by conj(H'), forward,
// where X is the transformed cotangent and q2 = dfX^2 tx^2 + dfY^2 ty^2 of the propagator
// phase (Efields.h:121), so that acc * dz * g / k is the derivative of L w.r.t. the
// wavenumber k = 2 pi n / lambda of that field.
//   MODE 2 (adjoint, no sums): multiply by conj(H'), forward.
// All fields of all solves in one launch: blockIdx.y = 2*solve + {0 pump (Hp), 1 SH (Hs)};
// A and Fst hold the fields back to back (solve-major), acc[blockIdx.y] receives the sums.
template <int N, int MODE>
__global__ void __launch_bounds__(16 * LineShape<N>::G) k_colpass(float2 *A0, float2 *Fst0,
                                                             const InstDesc *__restrict__ dd, double *acc0) {
    constexpr int G = LineShape<N>::G, E = N / G, TC = 16;
    __shared__ float2 scratch[TC * E * G];
    const float2 *__restrict__ tab = g_twiddle + N;
    const int f = blockIdx.y;
    const InstDesc &d = dd[f >> 1];
    const size_t nn = (size_t)N * N;
    float2 *A = A0 + f * nn;
    float2 *Fst = Fst0 ? Fst0 + f * nn : nullptr;
    const float2 *__restrict__ H = (f & 1) ? d.Hs : d.Hp;
    double *acc = acc0 ? acc0 + f : nullptr;
    const int c = threadIdx.x % TC, t = threadIdx.x / TC, x = blockIdx.x * TC + c;
    float2 v[E];
#pragma unroll
    for (int j = 0; j < E; ++j) v[j] = A[(size_t)(t + G * j) * N + x];
    fft_nat_to_spec<N, G, +1, true, TC, G>(v, t, scratch + c, tab);
    double a = 0.0;
#pragma unroll
    for (int r = 0; r < E; ++r) {
        const int k = spec_index<N, G>(t, r);
        const size_t i = (size_t)k * N + x;
        const float2 h = __ldg(H + i);
        if (MODE == 0) {
            if (Fst) Fst[i] = v[r];
            v[r] = c_mul(v[r], h);
        } else if (MODE == 2) {
            v[r] = c_mulc(v[r], h);
        } else {
            const int ux = (x + N / 2) & (N - 1), uy = (k + N / 2) & (N - 1);
            const float tx = (float)ux - d.uX, ty = (float)uy - d.uY;
            const float q2 = d.dfX2 * (tx * tx) + d.dfY2 * (ty * ty);
            const float2 fx = c_mulc(Fst[i], v[r]);   // F conj(X)
            const float2 fh = c_mul(fx, h);
            a += -(double)fh.y * (double)q2;          // Re(i z) = -Im(z)
            v[r] = c_mulc(v[r], h);                   // conj(H') X
        }
    }
    fft_spec_to_nat<N, G, -1, true, TC, G>(v, t, scratch + c, tab);
#pragma unroll
    for (int j = 0; j < E; ++j) A[(size_t)(t + G * j) * N + x] = v[j];
    if (MODE == 1) {
        double b[1] = {a};
        block_sum_doubles(b, 1, acc);
    }
}

// sum |S|^2 of a field (FP64).
__global__ void k_abs2_sum(const float2 *__restrict__ S, int nn, double *out) {
    double a[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += gridDim.x * blockDim.x) {
        const float2 v = S[i];
        a[0] += (double)v.x * v.x + (double)v.y * v.y;
    }
    block_sum_doubles(a, 1, out);
}

// c_S = g * S (the cotangent of g/2 * sum |S|^2), c_P = 0; g read from device memory.
__global__ void k_seed_cotangent(const float2 *__restrict__ S, float2 *cP, float2 *cS, int nn, const double *gd) {
    const float g = (float)*gd;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += gridDim.x * blockDim.x) {
        const float2 v = S[i];
        cS[i] = make_float2(g * v.x, g * v.y);
        cP[i] = make_float2(0.f, 0.f);
    }
}

static int grid_for(int nn) {
    int b = (nn + 255) / 256;
    return b < 1216 ? b : 1216;
}

cudaError_t launch_rk4_state(float2 *P, float2 *S, int nn, const float4 *stepc, int s, const InstDesc *d,
                             cudaStream_t st) {
    k_rk4_state<<<grid_for(nn), 256, 0, st>>>(P, S, nn, stepc, s, d);
    return cudaGetLastError();
}

cudaError_t launch_rk4_vjp(const float2 *P0, const float2 *S0, float2 *cP, float2 *cS, int nn, const float4 *stepc,
                           int s, const InstDesc *d, double *acc_step, cudaStream_t st) {
    k_rk4_vjp<<<grid_for(nn), 256, 0, st>>>(P0, S0, cP, cS, nn, stepc, s, d, acc_step);
    return cudaGetLastError();
}

template <int N>
static cudaError_t launch_colpass_t(int mode, float2 *A, float2 *F, const InstDesc *d, double *acc, int solves,
                                    cudaStream_t st) {
    constexpr int G = LineShape<N>::G, TC = 16;
    const dim3 grid(N / TC, 2 * solves);
    if (mode == 0)
        k_colpass<N, 0><<<grid, TC * G, 0, st>>>(A, F, d, acc);
    else if (mode == 1)
        k_colpass<N, 1><<<grid, TC * G, 0, st>>>(A, F, d, acc);
    else
        k_colpass<N, 2><<<grid, TC * G, 0, st>>>(A, F, d, acc);
    return cudaGetLastError();
}

cudaError_t launch_colpass(int n, int mode, float2 *A, float2 *F, const InstDesc *d, double *acc, cudaStream_t st,
                           int solves) {
    if (solves < 1 || solves > 32767) return cudaErrorInvalidValue;
    switch (n) {
        case 16: return launch_colpass_t<16>(mode, A, F, d, acc, solves, st);
        case 32: return launch_colpass_t<32>(mode, A, F, d, acc, solves, st);
        case 64: return launch_colpass_t<64>(mode, A, F, d, acc, solves, st);
        case 128: return launch_colpass_t<128>(mode, A, F, d, acc, solves, st);
        case 256: return launch_colpass_t<256>(mode, A, F, d, acc, solves, st);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_abs2_sum(const float2 *S, int nn, double *out, cudaStream_t st) {
    k_abs2_sum<<<grid_for(nn), 256, 0, st>>>(S, nn, out);
    return cudaGetLastError();
}

cudaError_t launch_seed_cotangent(const float2 *S, float2 *cP, float2 *cS, int nn, const double *g, cudaStream_t st) {
    k_seed_cotangent<<<grid_for(nn), 256, 0, st>>>(S, cP, cS, nn, g);
    return cudaGetLastError();
}

}  // namespace shg
