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

}  // namespace shg
