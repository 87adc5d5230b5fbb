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

// ---- one voxel of the heat stencil (shared by the sweep kernels) ----------------------

// a / d for the interior stencil: the corrected product where it was verified equal to the
// IEEE quotient, IEEE division otherwise. The corrected product is the textbook FMA
// quotient-correction step (P. Markstein, "Computation of elementary functions on the IBM
// RISC System/6000 processor", IBM J. Res. Dev. 34(1), 1990): q = a * r with r = 1/d
// rounded, the residual a - q*d formed exactly by one FMA, then q + residual * r. It is
// not correctly rounded for every a, which is why verify_fast_division compares it with
// IEEE division for every numerator of the exponent range used before it is enabled.
__device__ __forceinline__ float div_const(float a, float d, float r, int fast) {
    const unsigned e = (__float_as_uint(a) >> 23) & 0xffu;
    if (fast && e - kDivExpLo <= kDivExpHi - kDivExpLo) {
        const float q = a * r;
        const float rem = fmaf(-q, d, a);
        return fmaf(rem, r, q);
    }
    return __fdiv_rn(a, d);
}

// One voxel of Tfield.h:113-258 from its six face neighbours (only those the formula of
// the voxel's class uses are read): xm/xp, ym/yp, zm/zp = T at x-1/x+1, y-1/y+1, z-1/z+1.
// Returns false for voxels the reference never writes.
template <int BC>
__device__ __forceinline__ bool heat_voxel(const HeatCoef &c, int x, int y, int z, int nx, int ny, int nz, float xm,
                                           float xp, float ym, float yp, float zm, float zp, float qk, float &out) {
    const bool xi = x > 0 && x < nx - 1, yi = y > 0 && y < ny - 1, zi = z > 0 && z < nz - 1;
    if (xi && yi && zi) {
        const float a = div_const(__fadd_rn(xp, xm), c.dx2, c.rdx2, c.fast_div);
        const float b = div_const(__fadd_rn(yp, ym), c.dy2, c.rdy2, c.fast_div);
        const float d = div_const(__fadd_rn(zp, zm), c.dz2, c.rdz2, c.fast_div);
        out = __fmul_rn(c.L2, __fadd_rn(__fadd_rn(__fadd_rn(a, b), d), qk));
        return true;
    }
    const float tzn = z == 0 ? zp : zm;
    if (xi && yi) {  // back / front faces
        float s = __fadd_rn(tzn, __fmul_rn(c.az, __fadd_rn(xp, xm)));
        s = __fadd_rn(s, __fmul_rn(c.bz, __fadd_rn(yp, ym)));
        s = __fadd_rn(s, c.tinfBiz);
        out = __fdiv_rn(s, c.den_z);
        return true;
    }
    if (BC != 0) return false;
    const bool xe = x == 0 || x == nx - 1, ze = z == 0 || z == nz - 1, ytop = y == ny - 1;
    const float txn = x == 0 ? xp : xm;
    if (xe && yi && zi) {
        float s = __fadd_rn(txn, __fmul_rn(c.ax, __fadd_rn(yp, ym)));
        s = __fadd_rn(s, __fmul_rn(c.bx, __fadd_rn(zp, zm)));
        s = __fadd_rn(s, c.tinfBix);
        out = __fdiv_rn(s, c.den_x);
    } else if (xi && ytop && zi) {
        float s = __fadd_rn(ym, __fmul_rn(c.ay, __fadd_rn(xp, xm)));
        s = __fadd_rn(s, __fmul_rn(c.by, __fadd_rn(zp, zm)));
        s = __fadd_rn(s, c.tinfBiy);
        out = __fdiv_rn(s, c.den_y);
    } else if (xe && yi && ze) {
        const float s = __fadd_rn(__fadd_rn(__fmul_rn(c.av, txn), __fmul_rn(c.bv, tzn)), __fmul_rn(c.cv, __fadd_rn(yp, ym)));
        out = __double2float_rn(__dmul_rn(__dadd_rn((double)s, c.KV), (double)c.V));
    } else if (ytop && xi && ze) {
        const float s = __fadd_rn(__fadd_rn(__fmul_rn(c.ah, ym), __fmul_rn(c.bh, tzn)), __fmul_rn(c.ch, __fadd_rn(xm, xp)));
        out = __double2float_rn(__dmul_rn(__dadd_rn((double)s, c.KH), (double)c.H));
    } else if (xe && ytop && zi) {
        const float s = __fadd_rn(__fadd_rn(__fmul_rn(c.ad, ym), __fmul_rn(c.bd, txn)), __fmul_rn(c.cd, __fadd_rn(zp, zm)));
        out = __double2float_rn(__dmul_rn(__dadd_rn((double)s, c.KD), (double)c.D));
    } else if (xe && ytop && ze) {
        float s = __fadd_rn(__fmul_rn(c.AV, txn), __fmul_rn(c.BV, ym));
        s = __fadd_rn(s, __fmul_rn(c.CV, tzn));
        s = __fadd_rn(s, c.tinfBiD);
        out = __fmul_rn(s, c.GV);
    } else {
        return false;
    }
    return true;
}

// Interior voxel (Tfield.h:132) with the three divisions by dx^2, dy^2, dz^2 taken as
// corrected products when all three numerators lie in the verified exponent range (one
// combined test), else through div_const: bit-identical to heat_voxel's interior branch.
// Biased exponent in [kDivExpLo, kDivExpHi] is |a| in [2^-100, 2^101): two float compares
// (NaN and infinity fail them, as their exponent 255 fails the range).
static_assert(kDivExpLo == 27 && kDivExpHi == 227, "div_in_range bounds follow the exponent range");
__device__ __forceinline__ bool div_in_range(float a) {
    const float m = fabsf(a);
    return m >= 0x1p-100f && m < 0x1p101f;
}

// All three in range at once: the smallest magnitude >= 2^-100 and the largest < 2^101
// (a NaN may pass through fminf/fmaxf, but then both paths give NaN).
__device__ __forceinline__ bool div_in_range3(float a, float b, float c) {
    const float lo = fminf(fminf(fabsf(a), fabsf(b)), fabsf(c));
    const float hi = fmaxf(fmaxf(fabsf(a), fabsf(b)), fabsf(c));
    return lo >= 0x1p-100f && hi < 0x1p101f;
}

__device__ __forceinline__ float interior_voxel(const HeatCoef &c, float xm, float xp, float ym, float yp, float zm,
                                                float zp, float qk) {
    const float sx = __fadd_rn(xp, xm), sy = __fadd_rn(yp, ym), sz = __fadd_rn(zp, zm);
    float a, b, d;
    if (c.fast_div && div_in_range3(sx, sy, sz)) {
        const float qa = sx * c.rdx2, qb = sy * c.rdy2, qd = sz * c.rdz2;
        a = fmaf(fmaf(-qa, c.dx2, sx), c.rdx2, qa);
        b = fmaf(fmaf(-qb, c.dy2, sy), c.rdy2, qb);
        d = fmaf(fmaf(-qd, c.dz2, sz), c.rdz2, qd);
    } else {
        a = div_const(sx, c.dx2, c.rdx2, c.fast_div);
        b = div_const(sy, c.dy2, c.rdy2, c.fast_div);
        d = div_const(sz, c.dz2, c.rdz2, c.fast_div);
    }
    return __fmul_rn(c.L2, __fadd_rn(__fadd_rn(__fadd_rn(a, b), d), qk));
}

}  // namespace shg
