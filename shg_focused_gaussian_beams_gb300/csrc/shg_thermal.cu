// THERMAL kernels (-DTHERMAL of the reference): temperature set-up, the steady heat
// Jacobi sweep, its convergence sum, the Sellmeier / delta-k(T) tables, and the thermal
// row pass of the z-march (per-pixel coupling from T, running delta-k sum, heat source).
//
// The heat sweep reproduces Tfield.h:113-258 bit for bit: the same float operations in
// the same order with no contraction (__fadd_rn / __fmul_rn / __fdiv_rn), and the double
// sub-expressions of the edge formulas in double. The Sellmeier index is evaluated in
// double exactly as Crystal.h:116-132 does on the host (the reference's own arithmetic),
// so delta-k(T) is bit-identical too.
#include <cuda_runtime.h>

#include "shg_internal.h"
#include "shg_thermal.cuh"

namespace shg {

const float2 *twiddle_symbol_address_thermal() {
    void *p = nullptr;
    cudaGetSymbolAddress(&p, g_twiddle);
    return static_cast<const float2 *>(p);
}

// ---------------------------------------------------------------------------------------
// Tfield.h:31-110: T = Temp everywhere, then the oven faces (bc 0: y = 0 plane; bc 1: all
// four lateral faces), T1 for z < NZ/2 and T2 otherwise.
__global__ void k_init_temperature(float *T, int nx, int ny, int nz, float temp, float t1, float t2, int bc) {
    const size_t total = (size_t)nx * ny * nz;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(i % nx), y = (int)((i / nx) % ny), z = (int)(i / ((size_t)nx * ny));
        const bool oven = bc == 0 ? (y == 0) : (y == 0 || y == ny - 1 || x == 0 || x == nx - 1);
        const double half = (double)(float)nz / 2.0;
        T[i] = oven ? ((double)z < half ? t1 : t2) : temp;
    }
}

// One Jacobi sweep Tf <- stencil(Ti). Voxels the reference never writes are left alone;
// both ping-pong buffers start equal, so they hold the same value.
template <int BC>
__global__ void __launch_bounds__(256) k_heat(float *__restrict__ Tf, const float *__restrict__ Ti,
                                              const float *__restrict__ QK, const HeatCoef c, int nx, int ny, int nz) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    if (x >= nx || y >= ny) return;
    const size_t sxy = (size_t)nx * ny;
    const size_t i = (size_t)z * sxy + (size_t)y * nx + x;
    const bool xi = x > 0 && x < nx - 1, yi = y > 0 && y < ny - 1, zi = z > 0 && z < nz - 1;
    const float *t = Ti + i;
    const long long X = 1, Y = nx, Z = (long long)sxy;
    if (xi && yi && zi) {
        const float a = __fdiv_rn(__fadd_rn(t[X], t[-X]), c.dx2);
        const float b = __fdiv_rn(__fadd_rn(t[Y], t[-Y]), c.dy2);
        const float d = __fdiv_rn(__fadd_rn(t[Z], t[-Z]), c.dz2);
        Tf[i] = __fmul_rn(c.L2, __fadd_rn(__fadd_rn(__fadd_rn(a, b), d), QK[i]));
        return;
    }
    if (xi && yi) {  // z = 0 or z = NZ-1 (back / front faces)
        const long long zn = z == 0 ? Z : -Z;
        float s = __fadd_rn(t[zn], __fmul_rn(c.az, __fadd_rn(t[X], t[-X])));
        s = __fadd_rn(s, __fmul_rn(c.bz, __fadd_rn(t[Y], t[-Y])));
        s = __fadd_rn(s, c.tinfBiz);
        Tf[i] = __fdiv_rn(s, c.den_z);
        return;
    }
    if (BC != 0) return;  // oven surrounded: lateral faces are fixed
    const bool xe = x == 0 || x == nx - 1, ze = z == 0 || z == nz - 1, ytop = y == ny - 1;
    const long long xn = x == 0 ? X : -X;
    const long long zn = z == 0 ? Z : -Z;
    if (xe && yi && zi) {  // left / right faces
        float s = __fadd_rn(t[xn], __fmul_rn(c.ax, __fadd_rn(t[Y], t[-Y])));
        s = __fadd_rn(s, __fmul_rn(c.bx, __fadd_rn(t[Z], t[-Z])));
        s = __fadd_rn(s, c.tinfBix);
        Tf[i] = __fdiv_rn(s, c.den_x);
    } else if (xi && ytop && zi) {  // top face
        float s = __fadd_rn(t[-Y], __fmul_rn(c.ay, __fadd_rn(t[X], t[-X])));
        s = __fadd_rn(s, __fmul_rn(c.by, __fadd_rn(t[Z], t[-Z])));
        s = __fadd_rn(s, c.tinfBiy);
        Tf[i] = __fdiv_rn(s, c.den_y);
    } else if (xe && yi && ze) {  // vertical sides
        const float s = __fadd_rn(__fadd_rn(__fmul_rn(c.av, t[xn]), __fmul_rn(c.bv, t[zn])),
                                  __fmul_rn(c.cv, __fadd_rn(t[Y], t[-Y])));
        Tf[i] = __double2float_rn(__dmul_rn(__dadd_rn((double)s, c.KV), (double)c.V));
    } else if (ytop && xi && ze) {  // horizontal sides
        const float s = __fadd_rn(__fadd_rn(__fmul_rn(c.ah, t[-Y]), __fmul_rn(c.bh, t[zn])),
                                  __fmul_rn(c.ch, __fadd_rn(t[-X], t[X])));
        Tf[i] = __double2float_rn(__dmul_rn(__dadd_rn((double)s, c.KH), (double)c.H));
    } else if (xe && ytop && zi) {  // depth sides
        const float s = __fadd_rn(__fadd_rn(__fmul_rn(c.ad, t[-Y]), __fmul_rn(c.bd, t[xn])),
                                  __fmul_rn(c.cd, __fadd_rn(t[Z], t[-Z])));
        Tf[i] = __double2float_rn(__dmul_rn(__dadd_rn((double)s, c.KD), (double)c.D));
    } else if (xe && ytop && ze) {  // vertices
        float s = __fadd_rn(__fmul_rn(c.AV, t[xn]), __fmul_rn(c.BV, t[-Y]));
        s = __fadd_rn(s, __fmul_rn(c.CV, t[zn]));
        s = __fadd_rn(s, c.tinfBiD);
        Tf[i] = __fmul_rn(s, c.GV);
    }
}

// sum over voxels of fl((Tf - Ti)^2) accumulated in double (Tfield.h:13-28 sums in float
// sequentially; the stop rule reads this sum rounded to float).
__global__ void k_sq_diff_sum(const float *__restrict__ Tf, const float *__restrict__ Ti, size_t n, double *out) {
    double acc = 0.0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float d = __fsub_rn(Tf[i], Ti[i]);
        acc += (double)__fmul_rn(d, d);
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    __shared__ double red[32];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) red[w] = acc;
    __syncthreads();
    if (w == 0) {
        acc = l < (int)(blockDim.x >> 5) ? red[l] : 0.0;
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (l == 0 && acc != 0.0) atomicAdd(out, acc);
    }
}

// Crystal.h:116-132 in double with no contraction: bit-identical to the host evaluation.
__device__ __forceinline__ float sellmeier_dev(float L, float T) {
    const float A = 4.502483f, B = 0.007294f, C = 0.185087f, D = -0.02357f;
    const float E = 0.073423f, F = 0.199595f, G = 0.001f, H = 7.99724f;
    const double tk = __dadd_rn((double)T, 273.15);
    const double tk2 = __dmul_rn(tk, tk);
    const float b = __double2float_rn(__dmul_rn(3.483933e-8, tk2));
    const float c = __double2float_rn(__dmul_rn(1.607839e-8, tk2));
    const double L2 = __dmul_rn((double)L, (double)L);
    const float Cc = __fadd_rn(C, c), Bb = __fadd_rn(B, b);
    const double t1 = __ddiv_rn((double)Bb, __dsub_rn(L2, __dmul_rn((double)Cc, (double)Cc)));
    const double t2 = __ddiv_rn((double)E, __dsub_rn(L2, __dmul_rn((double)F, (double)F)));
    const double t3 = __ddiv_rn((double)G, __dsub_rn(L2, __dmul_rn((double)H, (double)H)));
    const double t4 = __dmul_rn((double)D, L2);
    const double n2 = __dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn((double)A, t1), t2), t3), t4);
    return __double2float_rn(__dsqrt_rn(n2));
}

// PhaseMatching.h:41-54 per voxel, plus the two indices the thermal z-march needs.
__global__ void k_sellmeier_tables(const float *__restrict__ T, float *NP, float *NS, float *DK, size_t n, float lp,
                                   float ls, float two_pi, float inv_lambda) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float t = T[i];
        const float np = sellmeier_dev(lp, t), ns = sellmeier_dev(ls, t);
        NP[i] = np;
        NS[i] = ns;
        DK[i] = __fmul_rn(two_pi, __fadd_rn(__fsub_rn(__fdiv_rn(__fmul_rn(2.0f, np), lp), __fdiv_rn(ns, ls)), inv_lambda));
    }
}

// ---------------------------------------------------------------------------------------
// Thermal row pass. Stage s of K = nz steps:
//   s == 0        : DKint = DK(slice 0); RK4 of step 0 (slice 0); backward FFT along x;
//   0 < s < nz    : forward FFT; second RK4 of step s-1; heat source of slice s-1;
//                   [capture at s == nz-1]; DKint += DK(slice s); first RK4 of step s;
//                   backward FFT;
//   s == nz       : forward FFT; second RK4 of step nz-1; heat source of slice nz-1.
// The coupling per pixel follows Solver.h:44-63: n from T(x,y,slice), phase
// DKint*(dz*inc + (s+1)*dz)/(s+1) with inc = 0, 0.25, 0.25, 0.5 for the four stages.

struct ThCoef {
    float4 c0, c1, c2;  // stage constants for inc = 0, 0.25 (stages 2, 3), 0.5 (stage 4)
    float tpa1;
};

__device__ __forceinline__ ThCoef th_coef(const ThermDesc &t, float np, float ns, float dkint, int s, float dz) {
    ThCoef r;
    const float kp = t.pidq / (np * t.lp);
    const float ks = t.hpidq / (ns * t.ls);
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
    r.tpa1 = t.tpa_c * ns;
    return r;
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

__device__ __forceinline__ void block_add_double_th(double v, double *dst) {
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

template <int N>
struct ThRowShape {
    static constexpr int G = LineShape<N>::G;
    static constexpr int TPB = (N * G < 256) ? N * G : 256;
    static constexpr int LPB = TPB / G;
    static constexpr int BPI = N / LPB;
};

template <int N>
__global__ void __launch_bounds__(ThRowShape<N>::TPB) k_rows_th(const InstDesc *__restrict__ dd, const ThermDesc th, int s) {
    constexpr int G = LineShape<N>::G, E = N / G, LPB = ThRowShape<N>::LPB;
    constexpr int SC = LineScratch<N, G>::SIZE;
    __shared__ float2 scratch[LPB * SC];
    const InstDesc &d = *dd;
    const float2 *__restrict__ tab = g_twiddle + N;
    const int y = blockIdx.x * LPB + threadIdx.x / G;
    const int t = threadIdx.x % G;
    float2 *sc = scratch + (threadIdx.x / G) * SC;
    const size_t base = (size_t)y * N;
    const size_t nxy = (size_t)N * N;
    float2 vp[E], vs[E];
#pragma unroll
    for (int j = 0; j < E; ++j) {
        vp[j] = d.P[base + t + G * j];
        vs[j] = d.S[base + t + G * j];
    }
    if (s == 0) {
#pragma unroll
        for (int j = 0; j < E; ++j) {
            const size_t i2 = base + t + G * j;
            const float dkint = th.DK[i2];
            th.DKint[i2] = dkint;
            const ThCoef k = th_coef(th, th.NP[i2], th.NS[i2], dkint, 0, d.dz);
            rk4_point_th(vp[j], vs[j], k, d);
        }
        fft_nat_to_spec<N, G, +1>(vp, t, sc, tab);
        fft_nat_to_spec<N, G, +1>(vs, t, sc, tab);
#pragma unroll
        for (int r = 0; r < E; ++r) {
            const int kx = spec_index<N, G>(t, r);
            d.P[base + kx] = vp[r];
            d.S[base + kx] = vs[r];
        }
        return;
    }
    fft_nat_to_spec<N, G, -1>(vp, t, sc, tab);
    fft_nat_to_spec<N, G, -1>(vs, t, sc, tab);
    const bool capture = (s == th.nz - 1);
    double aS = 0.0, aP = 0.0;
#pragma unroll
    for (int r = 0; r < E; ++r) {
        const int x = spec_index<N, G>(t, r);
        const size_t i2 = base + x, i3 = (size_t)(s - 1) * nxy + i2;
        const float np1 = th.NP[i3], ns1 = th.NS[i3];
        const float dkint = th.DKint[i2];
        const ThCoef k1 = th_coef(th, np1, ns1, dkint, s - 1, d.dz);
        rk4_point_th(vp[r], vs[r], k1, d);
        // Tfield.h:277-290: heat source of slice s-1 from the fields after step s-1
        const float a2p = fmaf(vp[r].x, vp[r].x, vp[r].y * vp[r].y);
        const float a2s = fmaf(vs[r].x, vs[r].x, vs[r].y * vs[r].y);
        const float Ip = th.qc * np1 * a2p, Is = th.qc * ns1 * a2s;
        const float Q = th.alpha_p * Ip + th.alpha_s * Is + th.beta_s * (Is * Is);
        th.QK[i3] = Q / th.kth;
        if (capture) {
            d.Pout[i2] = vp[r];
            d.Sout[i2] = vs[r];
            aS += (double)a2s;
            aP += (double)a2p;
        }
        if (s < th.nz) {
            const size_t i3n = (size_t)s * nxy + i2;
            const float dk2 = dkint + th.DK[i3n];
            th.DKint[i2] = dk2;
            const ThCoef k2 = th_coef(th, th.NP[i3n], th.NS[i3n], dk2, s, d.dz);
            rk4_point_th(vp[r], vs[r], k2, d);
        }
    }
    if (capture) {
        block_add_double_th(aS, d.acc + 1);
        block_add_double_th(aP, d.acc + 2);
    }
    if (s == th.nz) {
#pragma unroll
        for (int r = 0; r < E; ++r) {
            const int kx = spec_index<N, G>(t, r);
            d.P[base + kx] = vp[r];
            d.S[base + kx] = vs[r];
        }
        return;
    }
    fft_spec_to_nat<N, G, +1>(vp, t, sc, tab);
    fft_spec_to_nat<N, G, +1>(vs, t, sc, tab);
#pragma unroll
    for (int j = 0; j < E; ++j) {
        d.P[base + t + G * j] = vp[j];
        d.S[base + t + G * j] = vs[j];
    }
}

// ---------------------------------------------------------------------------------------
// Launchers.

cudaError_t launch_init_temperature(float *T, int nx, int ny, int nz, float temp, float t1, float t2, int bc,
                                    cudaStream_t st) {
    k_init_temperature<<<1024, 256, 0, st>>>(T, nx, ny, nz, temp, t1, t2, bc);
    return cudaGetLastError();
}

cudaError_t launch_heat(float *Tf, const float *Ti, const float *QK, const HeatCoef &c, int nx, int ny, int nz,
                        int bc, cudaStream_t st) {
    dim3 blk(32, 8, 1);
    dim3 grd((nx + 31) / 32, (ny + 7) / 8, nz);
    if (bc == 0)
        k_heat<0><<<grd, blk, 0, st>>>(Tf, Ti, QK, c, nx, ny, nz);
    else
        k_heat<1><<<grd, blk, 0, st>>>(Tf, Ti, QK, c, nx, ny, nz);
    return cudaGetLastError();
}

cudaError_t launch_sq_diff_sum(const float *Tf, const float *Ti, size_t n, double *out, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double), st);
    if (e != cudaSuccess) return e;
    k_sq_diff_sum<<<1216, 256, 0, st>>>(Tf, Ti, n, out);
    return cudaGetLastError();
}

cudaError_t launch_sellmeier_tables(const float *T, float *NP, float *NS, float *DK, size_t n, float lp, float ls,
                                    float two_pi, float inv_lambda, cudaStream_t st) {
    k_sellmeier_tables<<<2432, 256, 0, st>>>(T, NP, NS, DK, n, lp, ls, two_pi, inv_lambda);
    return cudaGetLastError();
}

template <int N>
static cudaError_t launch_rows_th_t(const InstDesc *d, const ThermDesc &th, int s, cudaStream_t st) {
    k_rows_th<N><<<ThRowShape<N>::BPI, ThRowShape<N>::TPB, 0, st>>>(d, th, s);
    return cudaGetLastError();
}

cudaError_t launch_rows_th(int n, const InstDesc *d, const ThermDesc &th, int s, cudaStream_t st) {
    switch (n) {
        case 16: return launch_rows_th_t<16>(d, th, s, st);
        case 32: return launch_rows_th_t<32>(d, th, s, st);
        case 64: return launch_rows_th_t<64>(d, th, s, st);
        case 128: return launch_rows_th_t<128>(d, th, s, st);
        case 256: return launch_rows_th_t<256>(d, th, s, st);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace shg
