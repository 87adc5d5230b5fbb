// Adjoint of the THERMAL z-march with the temperature field held fixed, batched over solves.
//
// With T fixed, step s of Solver::CWES (-DTHERMAL, Solver.h:245-276) maps
//   X_s -> RK4_th(X_s; s) -> D -> RK4_th(.; s) = X_{s+1},
// where RK4_th is Solver.h:193-233 with the per-pixel coupling of Solver.h:44-63: n_p, n_s
// from T(x,y,s) and the phase DKint_s*(dz*inc + (s+1)*dz)/(s+1), DKint_s the running sum of
// delta-k(T) over slices 0..s (PhaseMatching.h:12-38), inc = 0, 0.25, 0.25, 0.5 per stage.
// Both RK4 calls of step s use slice s. Per voxel the solve keeps a float4 table
// (kp, ks, tpa1, DKint) built once from T; the stage constants are re-derived from it on
// the fly (three sincosf per pixel and RK4 call).
//
// Batch layout: solve b owns states X + b*2*nn (pump then SH), tables coef + b*K*nn (slice
// s at s*nn); one launch covers every solve (blockIdx.y = b).
#include <cuda_runtime.h>

#include "shg_adjoint.cuh"
#include "shg_adjoint_th.h"
#include "shg_thermal.cuh"

namespace shg {

// coef[s*nn + i] = (kp, ks, tpa1, DKint_s) of pixel i for s < K; the running sum follows
// the order of the thermal row pass (DKint_0 = DK_0, DKint_s = DKint_{s-1} + DK_s).
__global__ void k_th_coef_table(const float *__restrict__ NP, const float *__restrict__ NS,
                                const float *__restrict__ DK, float4 *coef, int nn, int K, const ThermDesc th) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += gridDim.x * blockDim.x) {
        float dk = 0.0f;
        for (int s = 0; s < K; ++s) {
            const size_t j = (size_t)s * nn + i;
            dk = s == 0 ? DK[j] : dk + DK[j];
            const float np = NP[j], ns = NS[j];
            coef[j] = make_float4(th_kp(th, np), th_ks(th, ns), th.tpa_c * ns, dk);
        }
    }
}

__device__ __forceinline__ ThCoef th_coef_of(float4 cf, int s, float dz) {
    return th_coef_k(cf.x, cf.y, cf.z, cf.w, s, dz);
}

// RK4_th^T of one point at the base state (P, S) with stage constants k: (cp, cs) hold the
// cotangent of the RK4 output on entry and of its input on exit (stages 1..4 use the
// constants c0, c1, c1, c2).
__device__ __forceinline__ void th_vjp_point(const float2 P, const float2 S, float2 &cp, float2 &cs, const ThCoef &k,
                                             float hp, float t0, float w6) {
    const float t1 = k.tpa1;
    float unused[5];  // parameter sensitivities are not needed here
    float2 k1p, k1s, k2p, k2s, k3p, k3s;
    dadz_point(P, S, k.c0, hp, t0, t1, k1p, k1s);
    const float2 B2p = make_float2(fmaf(0.5f, k1p.x, P.x), fmaf(0.5f, k1p.y, P.y));
    const float2 B2s = make_float2(fmaf(0.5f, k1s.x, S.x), fmaf(0.5f, k1s.y, S.y));
    dadz_point(B2p, B2s, k.c1, hp, t0, t1, k2p, k2s);
    const float2 B3p = make_float2(fmaf(0.5f, k2p.x, P.x), fmaf(0.5f, k2p.y, P.y));
    const float2 B3s = make_float2(fmaf(0.5f, k2s.x, S.x), fmaf(0.5f, k2s.y, S.y));
    dadz_point(B3p, B3s, k.c1, hp, t0, t1, k3p, k3s);
    const float2 B4p = c_add(P, k3p), B4s = c_add(S, k3s);
    const float2 op = cp, os = cs;
    float2 cap = op, cas = os;
    float2 ck3p = make_float2(2.0f * w6 * op.x, 2.0f * w6 * op.y), ck3s = make_float2(2.0f * w6 * os.x, 2.0f * w6 * os.y);
    float2 ck2p = ck3p, ck2s = ck3s;
    float2 ck1p = make_float2(w6 * op.x, w6 * op.y), ck1s = make_float2(w6 * os.x, w6 * os.y);
    const float2 ck4p = ck1p, ck4s = ck1s;
    float2 bp = make_float2(0.f, 0.f), bs = make_float2(0.f, 0.f);
    dadz_vjp(B4p, B4s, ck4p, ck4s, k.c2, hp, t0, t1, bp, bs, unused);
    cap = c_add(cap, bp);
    cas = c_add(cas, bs);
    ck3p = c_add(ck3p, bp);
    ck3s = c_add(ck3s, bs);
    bp = bs = make_float2(0.f, 0.f);
    dadz_vjp(B3p, B3s, ck3p, ck3s, k.c1, hp, t0, t1, bp, bs, unused);
    cap = c_add(cap, bp);
    cas = c_add(cas, bs);
    ck2p = make_float2(fmaf(0.5f, bp.x, ck2p.x), fmaf(0.5f, bp.y, ck2p.y));
    ck2s = make_float2(fmaf(0.5f, bs.x, ck2s.x), fmaf(0.5f, bs.y, ck2s.y));
    bp = bs = make_float2(0.f, 0.f);
    dadz_vjp(B2p, B2s, ck2p, ck2s, k.c1, hp, t0, t1, bp, bs, unused);
    cap = c_add(cap, bp);
    cas = c_add(cas, bs);
    ck1p = make_float2(fmaf(0.5f, bp.x, ck1p.x), fmaf(0.5f, bp.y, ck1p.y));
    ck1s = make_float2(fmaf(0.5f, bs.x, ck1s.x), fmaf(0.5f, bs.y, ck1s.y));
    bp = bs = make_float2(0.f, 0.f);
    dadz_vjp(P, S, ck1p, ck1s, k.c0, hp, t0, t1, bp, bs, unused);
    cp = c_add(cap, bp);
    cs = c_add(cas, bs);
}

// Step boundary of the forward march in one pass over every solve's state X: RK4_th of step
// sp (its second call, slice sp; skipped for sp < 0) with its input stored to save_w, then
// the state stored to save_x, then RK4_th of step sn (its first call, slice sn; skipped for
// sn < 0): the state crosses memory once per step boundary.
__global__ void k_th_rk4_pair(float2 *X, float2 *save_w, float2 *save_x, const float4 *__restrict__ coef, int nn,
                              int K, int sp, int sn, const InstDesc *__restrict__ dd) {
    const int b = blockIdx.y;
    const InstDesc &d = dd[b];
    float2 *P = X + (size_t)b * 2 * nn, *S = P + nn;
    const size_t o = (size_t)b * 2 * nn;
    const float4 *__restrict__ cp = coef + ((size_t)b * K + (sp < 0 ? 0 : sp)) * nn;
    const float4 *__restrict__ cn = coef + ((size_t)b * K + (sn < 0 ? 0 : sn)) * nn;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += gridDim.x * blockDim.x) {
        float2 p = P[i], q = S[i];
        if (sp >= 0) {
            if (save_w) {
                save_w[o + i] = p;
                save_w[o + nn + i] = q;
            }
            rk4_point_th(p, q, th_coef_of(cp[i], sp, d.dz), d);
        }
        if (save_x) {
            save_x[o + i] = p;
            save_x[o + nn + i] = q;
        }
        if (sn >= 0) rk4_point_th(p, q, th_coef_of(cn[i], sn, d.dz), d);
        P[i] = p;
        S[i] = q;
    }
}

// Step boundary of the reverse sweep in one pass over every solve's cotangent: RK4_th^T of
// step sa at its first call's input Xa (skipped for sa < 0), then RK4_th^T of step sb at its
// second call's input Wb (skipped for sb < 0).
__global__ void k_th_vjp_pair(const float2 *__restrict__ Xa, const float2 *__restrict__ Wb, float2 *cot,
                              const float4 *__restrict__ coef, int nn, int K, int sa, int sb,
                              const InstDesc *__restrict__ dd) {
    const int b = blockIdx.y;
    const InstDesc &d = dd[b];
    const size_t o = (size_t)b * 2 * nn;
    float2 *cP = cot + o, *cS = cP + nn;
    const float4 *__restrict__ ca = coef + ((size_t)b * K + (sa < 0 ? 0 : sa)) * nn;
    const float4 *__restrict__ cb = coef + ((size_t)b * K + (sb < 0 ? 0 : sb)) * nn;
    const float hp = d.hp, t0 = d.tpa0, w6 = d.dz6;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += gridDim.x * blockDim.x) {
        float2 a = cP[i], c = cS[i];
        if (sa >= 0) th_vjp_point(Xa[o + i], Xa[o + nn + i], a, c, th_coef_of(ca[i], sa, d.dz), hp, t0, w6);
        if (sb >= 0) th_vjp_point(Wb[o + i], Wb[o + nn + i], a, c, th_coef_of(cb[i], sb, d.dz), hp, t0, w6);
        cP[i] = a;
        cS[i] = c;
    }
}

// out[b] += sum |field|^2 of solve b's field at X + b*2*nn + off (FP64).
__global__ void k_abs2_sum_b(const float2 *__restrict__ X, int nn, int off, double *out) {
    const float2 *A = X + (size_t)blockIdx.y * 2 * nn + off;
    double a[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += gridDim.x * blockDim.x) {
        const float2 v = A[i];
        a[0] += (double)v.x * v.x + (double)v.y * v.y;
    }
    block_sum_doubles(a, 1, out + blockIdx.y);
}

// Cotangent of L_b = seed_b/2 * sum |S_b|^2: c_S = seed_b * S_b, c_P = 0.
__global__ void k_seed_b(const float2 *__restrict__ X, float2 *cot, int nn, const double *__restrict__ seed) {
    const size_t o = (size_t)blockIdx.y * 2 * nn;
    const float g = (float)seed[blockIdx.y];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += gridDim.x * blockDim.x) {
        const float2 v = X[o + nn + i];
        cot[o + nn + i] = make_float2(g * v.x, g * v.y);
        cot[o + i] = make_float2(0.f, 0.f);
    }
}

static dim3 grid_b(int nn, int solves) { return dim3((unsigned)((nn + 255) / 256 < 64 ? (nn + 255) / 256 : 64), solves); }

cudaError_t launch_th_coef_table(const float *NP, const float *NS, const float *DK, float4 *coef, int nn, int K,
                                 const ThermDesc &th, cudaStream_t st) {
    k_th_coef_table<<<(nn + 255) / 256, 256, 0, st>>>(NP, NS, DK, coef, nn, K, th);
    return cudaGetLastError();
}

cudaError_t launch_th_rk4_pair(float2 *X, float2 *save_w, float2 *save_x, const float4 *coef, int nn, int K, int sp,
                               int sn, const InstDesc *d, int solves, cudaStream_t st) {
    if (sp >= K || sn >= K) return cudaErrorInvalidValue;
    k_th_rk4_pair<<<grid_b(nn, solves), 256, 0, st>>>(X, save_w, save_x, coef, nn, K, sp, sn, d);
    return cudaGetLastError();
}

cudaError_t launch_th_vjp_pair(const float2 *Xa, const float2 *Wb, float2 *cot, const float4 *coef, int nn, int K,
                               int sa, int sb, const InstDesc *d, int solves, cudaStream_t st) {
    if (sa >= K || sb >= K || (sa >= 0 && !Xa) || (sb >= 0 && !Wb)) return cudaErrorInvalidValue;
    k_th_vjp_pair<<<grid_b(nn, solves), 256, 0, st>>>(Xa, Wb, cot, coef, nn, K, sa, sb, d);
    return cudaGetLastError();
}

cudaError_t launch_abs2_sum_b(const float2 *X, int nn, int off, double *out, int solves, cudaStream_t st) {
    k_abs2_sum_b<<<grid_b(nn, solves), 256, 0, st>>>(X, nn, off, out);
    return cudaGetLastError();
}

cudaError_t launch_seed_b(const float2 *X, float2 *cot, int nn, const double *seed, int solves, cudaStream_t st) {
    k_seed_b<<<grid_b(nn, solves), 256, 0, st>>>(X, cot, nn, seed);
    return cudaGetLastError();
}

}  // namespace shg
