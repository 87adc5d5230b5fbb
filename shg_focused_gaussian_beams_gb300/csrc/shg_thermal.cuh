// THERMAL path (-DTHERMAL of the reference): device descriptors.
#pragma once

#include <cuda_runtime.h>

#include "shg_march.cuh"

namespace shg {

// Coefficients of the steady heat stencil (Tfield.h:118-125) with the reference's
// rounding; the three *_K terms are the double constants 0.5*T_inf*(Bi+Bi) of the edge
// formulas (Tfield.h:162-195).
struct HeatCoef {
    float Bix, Biy, Biz, ax, ay, az, bx, by, bz, av, bv, cv, V, ah, bh, ch, H, ad, bd, cd, D, AV, BV, CV, BiD, GV,
        L2, dx2, dy2, dz2;
    float den_x, den_y, den_z;   // 1 + 2a + 2b + Bi of the three face families
    float tinf;
    double KV, KH, KD;           // 0.5*T_inf*(Bix+Biz), 0.5*T_inf*(Biy+Biz), 0.5*T_inf*(Bix+Biy)
    float tinfBix, tinfBiy, tinfBiz, tinfBiD;
    // Division of the interior stencil by dx^2, dy^2, dz^2: when fast_div is set, a / d is
    // formed as q = a*r, q + (a - q*d)*r with r = 1/d rounded, which was checked against
    // IEEE division for every float a with biased exponent in [kDivExpLo, kDivExpHi]
    // (verify_fast_division); other numerators use IEEE division.
    float rdx2, rdy2, rdz2;
    int fast_div;
};

constexpr unsigned kDivExpLo = 27, kDivExpHi = 227;  // |a| in [2^-100, 2^101)

// Thermal extension of one solve.
struct ThermDesc {
    int nx, ny, nz;
    const float *NP, *NS, *DK;   // n(lp, T), n(ls, T), delta-k(T) per voxel (PhaseMatching.h:41-54)
    float *DKint;                // running sum over slices (PhaseMatching.h:25-38), n*n
    float *QK;                   // heat source divided by the conductivity, per voxel
    float pidq, hpidq;           // fl(PI*dQ), fl(dQ*fl(0.5*PI)) (Solver.h:55-57)
    float lp, ls;
    float qc;                    // 0.5*C*EPS0 (Tfield.h:284)
    float alpha_p, alpha_s, beta_s, kth;
    float tpa_c;                 // 0.25*beta_s*EPS0*C for the TPA factor per unit n_s
};

// Per-pixel constants of one thermal RK4 call (Solver.h:44-63): n from T(x,y,slice),
// phase DKint*(dz*inc + (s+1)*dz)/(s+1) with inc = 0, 0.25, 0.25, 0.5 for the four stages.
struct ThCoef {
    float4 c0, c1, c2;  // stage constants for inc = 0, 0.25 (stages 2, 3), 0.5 (stage 4)
    float tpa1;
};

// Stage constants from the per-pixel coupling factors kp = pi dQ / (n_p lp),
// ks = 0.5 pi dQ / (n_s ls), the TPA factor and the running delta-k sum of slice s.
__device__ __forceinline__ ThCoef th_coef_k(float kp, float ks, float tpa1, float dkint, int s, float dz) {
    ThCoef r;
    const float sp1 = (float)(s + 1);
    const float base = sp1 * dz;
    const float ph0 = (dkint * base) / sp1;
    const float ph1 = (dkint * (dz * 0.25f + base)) / sp1;
    const float ph2 = (dkint * (dz * 0.5f + base)) / sp1;
    float sn, cs;
    sincosf(ph0, &sn, &cs);
    r.c0 = make_float4(kp * sn, kp * cs, -ks * sn, ks * cs);
    sincosf(ph1, &sn, &cs);
    r.c1 = make_float4(kp * sn, kp * cs, -ks * sn, ks * cs);
    sincosf(ph2, &sn, &cs);
    r.c2 = make_float4(kp * sn, kp * cs, -ks * sn, ks * cs);
    r.tpa1 = tpa1;
    return r;
}

__device__ __forceinline__ float th_kp(const ThermDesc &t, float np) { return t.pidq / (np * t.lp); }
__device__ __forceinline__ float th_ks(const ThermDesc &t, float ns) { return t.hpidq / (ns * t.ls); }

__device__ __forceinline__ ThCoef th_coef(const ThermDesc &t, float np, float ns, float dkint, int s, float dz) {
    return th_coef_k(th_kp(t, np), th_ks(t, ns), t.tpa_c * ns, dkint, s, dz);
}

__device__ __forceinline__ void rk4_point_th(float2 &P, float2 &S, const ThCoef &k, const InstDesc &d) {
    float2 kp, ks, ap, as, accp, accs;
    dadz_point(P, S, k.c0, d.hp, d.tpa0, k.tpa1, kp, ks);
    accp = kp;
    accs = ks;
    ap = make_float2(fmaf(0.5f, kp.x, P.x), fmaf(0.5f, kp.y, P.y));
    as = make_float2(fmaf(0.5f, ks.x, S.x), fmaf(0.5f, ks.y, S.y));
    dadz_point(ap, as, k.c1, d.hp, d.tpa0, k.tpa1, kp, ks);
    accp = make_float2(fmaf(2.0f, kp.x, accp.x), fmaf(2.0f, kp.y, accp.y));
    accs = make_float2(fmaf(2.0f, ks.x, accs.x), fmaf(2.0f, ks.y, accs.y));
    ap = make_float2(fmaf(0.5f, kp.x, P.x), fmaf(0.5f, kp.y, P.y));
    as = make_float2(fmaf(0.5f, ks.x, S.x), fmaf(0.5f, ks.y, S.y));
    dadz_point(ap, as, k.c1, d.hp, d.tpa0, k.tpa1, kp, ks);
    accp = make_float2(fmaf(2.0f, kp.x, accp.x), fmaf(2.0f, kp.y, accp.y));
    accs = make_float2(fmaf(2.0f, ks.x, accs.x), fmaf(2.0f, ks.y, accs.y));
    ap = c_add(P, kp);
    as = c_add(S, ks);
    dadz_point(ap, as, k.c2, d.hp, d.tpa0, k.tpa1, kp, ks);
    accp = c_add(accp, kp);
    accs = c_add(accs, ks);
    P = make_float2(fmaf(accp.x, d.dz6, P.x), fmaf(accp.y, d.dz6, P.y));
    S = make_float2(fmaf(accs.x, d.dz6, S.x), fmaf(accs.y, d.dz6, S.y));
}

}  // namespace shg
