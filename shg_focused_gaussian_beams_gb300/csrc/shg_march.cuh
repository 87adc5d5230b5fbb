// Device-side descriptors and pointwise physics of the plain SSFM z-march.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "shg_check.cuh"
#include "shg_fft.cuh"

namespace shg {

// One solve on the device. Fields use the reference layout IDX(x, y) = y*NX + x
// (Common.h:27-29) with NX = NY = n.
struct InstDesc {
    float2 *P, *S;          // working pump / SH fields
    float2 *Pout, *Sout;    // state at the top of slice nz-1 (Solver.h:250-255)
    float2 *Hp, *Hs;        // shifted propagators (Efields.h:107-126, 186-192) times 1/(n*n)
    float4 *stepc;          // per slice s: (kp*sin, kp*cos, -ks*sin, ks*cos) of z_s*dk
    double *acc;            // [0] sum |P_in|^2, [1] sum |S_out|^2, [2] sum |P_out|^2
    float2 *slices;         // optional: state at the top of every slice s >= 1, P then S
                            // (2*n*n per slice; the caller fills slice 0 with the input)
    int n;                  // NX = NY
    int nz;                 // slices
    int nsteps;             // SSFM steps run before the capture (nz - 1)
    int pump_given;         // 1: P already holds the input pump; 0: Gaussian built on device
    float dz, dz6;          // dz and dz/6
    float hp;               // 0.5*alpha_p
    float tpa0, tpa1;       // 0.5*alpha_s, 0.25*beta_s*C*EPS0*n_s
    float kp, ks;           // pi*dQ/(n_p*lp), 0.5*pi*dQ/(n_s*ls)
    float dk;               // phase mismatch (PhaseMatching.h:57-70), float
    // Gaussian pump (Efields.h:74-104): exact float operands of the reference.
    float uX, uY, dx, dy;
    float2 amp;             // Ap0 / MX
    float2 wM;              // wX2 * MX
    float wM_den;           // |wM|^2 as operator/(real, complex) forms it
    // Propagator phase (Efields.h:121-122): -dz*(g*(dfX^2 tx^2 + dfY^2 ty^2) + lin*tx)
    float gp, gs;           // 2*PI^2 / k
    float dfX2, dfY2;       // dfX*dfX, dfY*dfY
    float linp, lins;       // 2*PI*dfX*tan(rho)
    float mdz;              // -dz
    float inv_nn;           // 1/(n*n), exact for power-of-two n
};

// dA/dz of Solver.h:65-83 for one point, with the per-slice constants folded:
//   dP = (i kp e^{-i z dk}) * S * conj(P) - 0.5 alpha_p P
//   dS = (i ks e^{+i z dk}) * P * P - (0.5 alpha_s + 0.25 beta_s C EPS0 n_s |S|^2) S
__device__ __forceinline__ void dadz_point(float2 P, float2 S, float4 c, float hp, float tpa0, float tpa1,
                                           float2 &dP, float2 &dS) {
    const float tr = fmaf(S.x, P.x, S.y * P.y);
    const float ti = fmaf(S.y, P.x, -S.x * P.y);
    dP.x = fmaf(tr, c.x, fmaf(-ti, c.y, -hp * P.x));
    dP.y = fmaf(tr, c.y, fmaf(ti, c.x, -hp * P.y));
    const float xr = fmaf(P.x, P.x, -P.y * P.y);
    const float xh = P.x * P.y;                      // half the imaginary part of P^2
    const float a2 = fmaf(S.x, S.x, S.y * S.y);
    const float coef = fmaf(tpa1, a2, tpa0);
    dS.x = fmaf(xr, c.z, fmaf(-2.0f * xh, c.w, -coef * S.x));
    dS.y = fmaf(xr, c.w, fmaf(2.0f * xh, c.z, -coef * S.y));
}

// One solverRK4 call (Solver.h:193-233, plain branch): stage offsets 0.5, 0.5, 1 without a
// dz factor, and the update A + (k1 + 2 k2 + 2 k3 + k4) dz/6; every stage uses the same z.
__device__ __forceinline__ void rk4_point(float2 &P, float2 &S, float4 c, const InstDesc &d) {
    float2 kp, ks, ap, as, accp, accs;
    dadz_point(P, S, c, d.hp, d.tpa0, d.tpa1, kp, ks);
    accp = kp;
    accs = ks;
    ap = make_float2(fmaf(0.5f, kp.x, P.x), fmaf(0.5f, kp.y, P.y));
    as = make_float2(fmaf(0.5f, ks.x, S.x), fmaf(0.5f, ks.y, S.y));
    dadz_point(ap, as, c, d.hp, d.tpa0, d.tpa1, kp, ks);
    accp = make_float2(fmaf(2.0f, kp.x, accp.x), fmaf(2.0f, kp.y, accp.y));
    accs = make_float2(fmaf(2.0f, ks.x, accs.x), fmaf(2.0f, ks.y, accs.y));
    ap = make_float2(fmaf(0.5f, kp.x, P.x), fmaf(0.5f, kp.y, P.y));
    as = make_float2(fmaf(0.5f, ks.x, S.x), fmaf(0.5f, ks.y, S.y));
    dadz_point(ap, as, c, d.hp, d.tpa0, d.tpa1, kp, ks);
    accp = make_float2(fmaf(2.0f, kp.x, accp.x), fmaf(2.0f, kp.y, accp.y));
    accs = make_float2(fmaf(2.0f, ks.x, accs.x), fmaf(2.0f, ks.y, accs.y));
    ap = c_add(P, kp);
    as = c_add(S, ks);
    dadz_point(ap, as, c, d.hp, d.tpa0, d.tpa1, kp, ks);
    accp = c_add(accp, kp);
    accs = c_add(accs, ks);
    P = make_float2(fmaf(accp.x, d.dz6, P.x), fmaf(accp.y, d.dz6, P.y));
    S = make_float2(fmaf(accs.x, d.dz6, S.x), fmaf(accs.y, d.dz6, S.y));
}

}  // namespace shg
