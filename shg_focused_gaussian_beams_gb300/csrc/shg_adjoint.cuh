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

// Reverse mode of one dA/dz evaluation at (P, S) with output cotangents (u, v); adds the
// input cotangents to (cp, cs) and the parameter sensitivities to acc.
__device__ __forceinline__ void dadz_vjp(float2 P, float2 S, float2 u, float2 v, float4 c, float hp, float tpa0,
                                         float tpa1, float2 &cp, float2 &cs, double *acc) {
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
    acc[0] += (double)eP.x;
    acc[1] += (double)eP.y;
    acc[2] += (double)eS.x;
    acc[3] += (double)eS.y;
    acc[4] += -(double)a2 * ((double)v.x * S.x + (double)v.y * S.y);
}

}  // namespace shg
