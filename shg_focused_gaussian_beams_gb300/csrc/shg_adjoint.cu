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
SHG_CHECK_TU(adjoint)

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
// TC columns per block: 16 when several solves fill the GPU, 4 for one to three solves
// (N >= 64, so that a block holds whole warps).
template <int N, int MODE, int TC>
__global__ void __launch_bounds__(TC * LineShape<N>::G) k_colpass(float2 *A0, float2 *Fst0,
                                                             const InstDesc *__restrict__ dd, double *acc0) {
    constexpr int G = LineShape<N>::G, E = N / G;
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
    // propagator values (and the stored spectrum) first: their latency overlaps the transform
    float2 hv[E], fv[MODE == 1 ? E : 1];
    hprop_load<N>(H, x, t, hv);
    if constexpr (MODE == 2) {  // conj(H') applied as a plain product (mode 0's code path)
#pragma unroll
        for (int r = 0; r < E; ++r) hv[r].y = -hv[r].y;
    }
    if constexpr (MODE == 1) {
#pragma unroll
        for (int r = 0; r < E; ++r) fv[r] = Fst[(size_t)spec_index<N, G>(t, r) * N + x];
    }
    float2 v[E];
#pragma unroll
    for (int j = 0; j < E; ++j) v[j] = A[(size_t)(t + G * j) * N + x];
    fft_nat_to_spec<N, G, +1, true, TC, G>(v, t, scratch + c, tab);
    float a = 0.0f;  // this thread's E terms; FP64 across threads
#pragma unroll
    for (int r = 0; r < E; ++r) {
        const int k = spec_index<N, G>(t, r);
        const size_t i = (size_t)k * N + x;
        const float2 h = hv[r];
        if (MODE == 0) {
            if (Fst) Fst[i] = v[r];
            v[r] = c_mul(v[r], h);
        } else if (MODE == 2) {
            v[r] = c_mul(v[r], h);  // h = conj(H')
        } else {
            const int ux = (x + N / 2) & (N - 1), uy = (k + N / 2) & (N - 1);
            const float tx = (float)ux - d.uX, ty = (float)uy - d.uY;
            const float q2 = d.dfX2 * (tx * tx) + d.dfY2 * (ty * ty);
            const float2 fx = c_mulc(fv[MODE == 1 ? r : 0], v[r]);   // F conj(X)
            const float2 fh = c_mul(fx, h);
            a = fmaf(-fh.y, q2, a);                   // Re(i z) = -Im(z)
            v[r] = c_mulc(v[r], h);                   // conj(H') X
        }
    }
    fft_spec_to_nat<N, G, -1, true, TC, G>(v, t, scratch + c, tab);
#pragma unroll
    for (int j = 0; j < E; ++j) A[(size_t)(t + G * j) * N + x] = v[j];
    if (MODE == 1) block_sum_f2d(&a, 1, acc);
}

// ---------------------------------------------------------------------------------------
// Fused row passes for one solve (row roles: AdjRowShape / AdjRowCtx, shg_adjoint.cuh).

// Forward row pass at step boundary s (0 <= s <= K):
//   finish (s > 0): W_{s-1} = end of the diffraction of step s-1 -> w_out; X_s = RK4(W_{s-1})
//   else          : X_s = (inP, inS)
//   X_s -> x_out, ck_out (when given); start (s < K): Y_s = RK4(X_s), begin the diffraction
//   of step s; else X_K -> final_out.
// Stored states hold the pump then the SH field, natural layout.
template <int N>
__global__ void __launch_bounds__(AdjRowShape<N>::TPB)
    k_adj_rows_fwd(const InstDesc *__restrict__ dd, float2 *A, int s, int finish, int start, const float2 *inP,
                   const float2 *inS, float2 *w_out, float2 *x_out, float2 *ck_out, float2 *final_out) {
    using Cx = AdjRowCtx<N>;
    __shared__ float2 scratch[2 * Cx::LPB * Cx::SC];
    __shared__ float2 lines[2][Cx::LPB * N];
    const InstDesc &d = *dd;
    if (!SHG_REQUIRE(d.n == N && (!finish || (s >= 1 && s - 1 < d.nz)) && (!start || (s >= 0 && s < d.nz)),
                     kChkAdjoint, s))
        return;  // block-uniform
    const float2 *__restrict__ tab = g_twiddle + N;
    const size_t nn = (size_t)N * N;
    Cx cx(lines, scratch);
    float2 p, q;
    if (finish) {
        cx.finish(A, tab);
        __syncthreads();
        p = lines[0][cx.lx];
        q = lines[1][cx.lx];
        if (w_out) {
            w_out[cx.i2] = p;
            w_out[nn + cx.i2] = q;
        }
        rk4_point(p, q, d.stepc[s - 1], d);
    } else {
        p = inP[cx.i2];
        q = inS[cx.i2];
    }
    if (x_out) {
        x_out[cx.i2] = p;
        x_out[nn + cx.i2] = q;
    }
    if (ck_out) {
        ck_out[cx.i2] = p;
        ck_out[nn + cx.i2] = q;
    }
    if (!start) {
        final_out[cx.i2] = p;
        final_out[nn + cx.i2] = q;
        return;
    }
    rk4_point(p, q, d.stepc[s], d);
    lines[0][cx.lx] = p;  // each point thread rewrites only the entry it read
    lines[1][cx.lx] = q;
    __syncthreads();
    cx.start(A, tab);
}

// Backward row pass at step boundary s (-1 <= s < K), cotangent C:
//   finish: end of the adjoint diffraction of step s+1, then c_{X_{s+1}} = RK4^T(X_{s+1})[c]
//           (sums into acc_fin, the step s+1 row of acc_step)
//   else  : c = C (natural layout)
//   start : c_{W_s} = RK4^T(W_s)[c] (sums into acc_start), begin the adjoint diffraction of
//           step s; else c -> C (natural layout).
template <int N>
__global__ void __launch_bounds__(AdjRowShape<N>::TPB)
    k_adj_rows_bwd(const InstDesc *__restrict__ dd, float2 *C, int s, int finish, int start,
                   const float2 *__restrict__ Xn, const float2 *__restrict__ Wn, double *acc_fin, double *acc_start) {
    using Cx = AdjRowCtx<N>;
    __shared__ float2 scratch[2 * Cx::LPB * Cx::SC];
    __shared__ float2 lines[2][Cx::LPB * N];
    const InstDesc &d = *dd;
    if (!SHG_REQUIRE(d.n == N && (!finish || (s + 1 >= 0 && s + 1 < d.nz)) && (!start || (s >= 0 && s < d.nz)),
                     kChkAdjoint, s))
        return;  // block-uniform
    const float2 *__restrict__ tab = g_twiddle + N;
    const size_t nn = (size_t)N * N;
    const float hp = d.hp, t0 = d.tpa0, t1 = d.tpa1, w6 = d.dz6;
    Cx cx(lines, scratch);
    float a1[5] = {0, 0, 0, 0, 0}, a2[5] = {0, 0, 0, 0, 0};  // this point's sums, FP64 across points
    // the stored states of this point first: their latency overlaps the transform
    float2 xp = make_float2(0.f, 0.f), xs = xp, wp = xp, ws = xp;
    if (finish) {
        xp = Xn[cx.i2];
        xs = Xn[nn + cx.i2];
    }
    if (start) {
        wp = Wn[cx.i2];
        ws = Wn[nn + cx.i2];
    }
    float2 cp, cs;
    if (finish) {
        cx.finish(C, tab);
        __syncthreads();
        cp = lines[0][cx.lx];
        cs = lines[1][cx.lx];
        rk4_vjp_point(xp, xs, cp, cs, d.stepc[s + 1], hp, t0, t1, w6, a1);
    } else {
        cp = C[cx.i2];
        cs = C[nn + cx.i2];
    }
    if (start) {
        rk4_vjp_point(wp, ws, cp, cs, d.stepc[s], hp, t0, t1, w6, a2);
        lines[0][cx.lx] = cp;  // each point thread rewrites only the entry it read
        lines[1][cx.lx] = cs;
        __syncthreads();
        cx.start(C, tab);
    } else {
        C[cx.i2] = cp;
        C[nn + cx.i2] = cs;
    }
    if (finish) block_sum_f2d(a1, 5, acc_fin);
    if (start) block_sum_f2d(a2, 5, acc_start);
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

// Parameter sensitivities of the focused Gaussian pump of Efields.h:74-104 (setPump),
//   G = (Ap0 / M) exp(X),  X = -r^2 / (w^2 M),  M = 1 - i f / zR,
//   Ap0 = sqrt(4 P / (eps0 c pi n w^2)),  zR = pi n w^2 / lp,
// evaluated in FP64 per grid point: with the input A = G * factor and the cotangent g of A
// (dL/dRe + i dL/dIm), out[k] += sum Re(conj(g) dA/dtheta_k) for theta = (f, w, P, n):
//   dG/dM = G (-1/M + r^2/(w^2 M^2)),  dM/df = -i/zR,  dM/dw = 2 i f/(zR w),  dM/dn = i f/(zR n),
//   dG/dw = G (-1/w + 2 r^2/(w^3 M)) + dG/dM dM/dw,  dG/dP = G/(2P),  dG/dn = -G/(2n) + dG/dM dM/dn.
// r^2 uses the reference's centre (0.5 NX, 0.5 NY) and float coordinates ((i - u) dx).
struct PumpParams {
    int n;
    float uX, uY, dx, dy;
    double ap0, zr, w, f, power, nidx;
};

__device__ __forceinline__ double2 z_mul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 z_div(double2 a, double2 b) {
    const double d = b.x * b.x + b.y * b.y;
    return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}

__global__ void k_pump_param_sums(const float2 *__restrict__ g, const float2 *__restrict__ factor, PumpParams p,
                                  double *out) {
    double a[4] = {0.0, 0.0, 0.0, 0.0};
    const int nn = p.n * p.n;
    const double2 M = make_double2(1.0, -p.f / p.zr);
    const double2 one = make_double2(1.0, 0.0);
    const double2 invM = z_div(one, M), invM2 = z_mul(invM, invM);
    const double w2 = p.w * p.w;
    const double2 dMf = make_double2(0.0, -1.0 / p.zr);
    const double2 dMw = make_double2(0.0, 2.0 * p.f / (p.zr * p.w));
    const double2 dMn = make_double2(0.0, p.f / (p.zr * p.nidx));
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += gridDim.x * blockDim.x) {
        const int ix = i % p.n, iy = i / p.n;
        const double x = (double)((float)ix - p.uX) * (double)p.dx, y = (double)((float)iy - p.uY) * (double)p.dy;
        const double r2 = x * x + y * y;
        // G = Ap0/M exp(-r^2/(w^2 M))
        const double2 X = make_double2(-r2 / w2 * invM.x, -r2 / w2 * invM.y);
        const double ex = exp(X.x);
        double sn, cs;
        sincos(X.y, &sn, &cs);
        const double2 G = z_mul(make_double2(p.ap0 * invM.x, p.ap0 * invM.y), make_double2(ex * cs, ex * sn));
        // dG/dM = G (-1/M + r^2/(w^2 M^2))
        const double2 q = make_double2(-invM.x + r2 / w2 * invM2.x, -invM.y + r2 / w2 * invM2.y);
        const double2 dGdM = z_mul(G, q);
        const double2 dGf = z_mul(dGdM, dMf);
        const double2 tw = make_double2(-1.0 / p.w + 2.0 * r2 / (w2 * p.w) * invM.x, 2.0 * r2 / (w2 * p.w) * invM.y);
        const double2 dGw0 = z_mul(G, tw), dGw1 = z_mul(dGdM, dMw);
        const double2 dGw = make_double2(dGw0.x + dGw1.x, dGw0.y + dGw1.y);
        const double2 dGP = make_double2(G.x / (2.0 * p.power), G.y / (2.0 * p.power));
        const double2 dGn1 = z_mul(dGdM, dMn);
        const double2 dGn = make_double2(-G.x / (2.0 * p.nidx) + dGn1.x, -G.y / (2.0 * p.nidx) + dGn1.y);
        const float2 fc = factor ? factor[i] : make_float2(1.f, 0.f);
        const double2 fd = make_double2(fc.x, fc.y);
        const float2 gv = g[i];
        const double2 ds[4] = {z_mul(dGf, fd), z_mul(dGw, fd), z_mul(dGP, fd), z_mul(dGn, fd)};
#pragma unroll
        for (int k = 0; k < 4; ++k) a[k] += (double)gv.x * ds[k].x + (double)gv.y * ds[k].y;
    }
    block_sum_doubles(a, 4, out);
}

// A *= factor (complex), elementwise.
__global__ void k_cmul_inplace(float2 *A, const float2 *__restrict__ factor, int nn) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += gridDim.x * blockDim.x) A[i] = c_mul(A[i], factor[i]);
}

static int grid_for(int nn) {
    int b = (nn + 255) / 256;
    return b < 1216 ? b : 1216;
}

template <int N, int TC>
static cudaError_t launch_colpass_tc(int mode, float2 *A, float2 *F, const InstDesc *d, double *acc, int solves,
                                     cudaStream_t st) {
    constexpr int G = LineShape<N>::G;
    const dim3 grid(N / TC, 2 * solves);
    if (mode == 0)
        k_colpass<N, 0, TC><<<grid, TC * G, 0, st>>>(A, F, d, acc);
    else if (mode == 1)
        k_colpass<N, 1, TC><<<grid, TC * G, 0, st>>>(A, F, d, acc);
    else
        k_colpass<N, 2, TC><<<grid, TC * G, 0, st>>>(A, F, d, acc);
    return cudaGetLastError();
}

template <int N>
static cudaError_t launch_colpass_t(int mode, float2 *A, float2 *F, const InstDesc *d, double *acc, int solves,
                                    cudaStream_t st) {
    // narrow tiles only where a block still fills a warp (the sums use full-warp shuffles)
    if (solves >= 4 || 4 * LineShape<N>::G < 32) return launch_colpass_tc<N, 16>(mode, A, F, d, acc, solves, st);
    return launch_colpass_tc<N, 4>(mode, A, F, d, acc, solves, st);
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

template <int N>
static cudaError_t launch_adj_rows_fwd_t(const InstDesc *d, float2 *A, int s, int finish, int start, const float2 *inP,
                                         const float2 *inS, float2 *w_out, float2 *x_out, float2 *ck_out,
                                         float2 *final_out, cudaStream_t st) {
    k_adj_rows_fwd<N><<<AdjRowShape<N>::BPI, AdjRowShape<N>::TPB, 0, st>>>(d, A, s, finish, start, inP, inS, w_out,
                                                                            x_out, ck_out, final_out);
    return cudaGetLastError();
}

template <int N>
static cudaError_t launch_adj_rows_bwd_t(const InstDesc *d, float2 *C, int s, int finish, int start,
                                         const float2 *Xn, const float2 *Wn, double *acc_fin, double *acc_start,
                                         cudaStream_t st) {
    k_adj_rows_bwd<N><<<AdjRowShape<N>::BPI, AdjRowShape<N>::TPB, 0, st>>>(d, C, s, finish, start, Xn, Wn, acc_fin,
                                                                            acc_start);
    return cudaGetLastError();
}

cudaError_t launch_adj_rows_fwd(int n, const InstDesc *d, float2 *A, int s, int finish, int start, const float2 *inP,
                                const float2 *inS, float2 *w_out, float2 *x_out, float2 *ck_out, float2 *final_out,
                                cudaStream_t st) {
    if ((!finish && (!inP || !inS)) || (!start && !final_out)) return cudaErrorInvalidValue;
    switch (n) {
        case 16: return launch_adj_rows_fwd_t<16>(d, A, s, finish, start, inP, inS, w_out, x_out, ck_out, final_out, st);
        case 32: return launch_adj_rows_fwd_t<32>(d, A, s, finish, start, inP, inS, w_out, x_out, ck_out, final_out, st);
        case 64: return launch_adj_rows_fwd_t<64>(d, A, s, finish, start, inP, inS, w_out, x_out, ck_out, final_out, st);
        case 128: return launch_adj_rows_fwd_t<128>(d, A, s, finish, start, inP, inS, w_out, x_out, ck_out, final_out, st);
        case 256: return launch_adj_rows_fwd_t<256>(d, A, s, finish, start, inP, inS, w_out, x_out, ck_out, final_out, st);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_adj_rows_bwd(int n, const InstDesc *d, float2 *C, int s, int finish, int start, const float2 *Xn,
                                const float2 *Wn, double *acc_fin, double *acc_start, cudaStream_t st) {
    if ((finish && (!Xn || !acc_fin)) || (start && (!Wn || !acc_start))) return cudaErrorInvalidValue;
    switch (n) {
        case 16: return launch_adj_rows_bwd_t<16>(d, C, s, finish, start, Xn, Wn, acc_fin, acc_start, st);
        case 32: return launch_adj_rows_bwd_t<32>(d, C, s, finish, start, Xn, Wn, acc_fin, acc_start, st);
        case 64: return launch_adj_rows_bwd_t<64>(d, C, s, finish, start, Xn, Wn, acc_fin, acc_start, st);
        case 128: return launch_adj_rows_bwd_t<128>(d, C, s, finish, start, Xn, Wn, acc_fin, acc_start, st);
        case 256: return launch_adj_rows_bwd_t<256>(d, C, s, finish, start, Xn, Wn, acc_fin, acc_start, st);
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

cudaError_t launch_pump_param_sums(const float2 *g, const float2 *factor, int n, float uX, float uY, float dx, float dy,
                                   double ap0, double zr, double w, double f, double power, double nidx, double *out,
                                   cudaStream_t st) {
    const PumpParams p{n, uX, uY, dx, dy, ap0, zr, w, f, power, nidx};
    cudaError_t e = cudaMemsetAsync(out, 0, 4 * sizeof(double), st);
    if (e != cudaSuccess) return e;
    k_pump_param_sums<<<grid_for(n * n), 256, 0, st>>>(g, factor, p, out);
    return cudaGetLastError();
}

cudaError_t launch_cmul_inplace(float2 *A, const float2 *factor, int nn, cudaStream_t st) {
    k_cmul_inplace<<<grid_for(nn), 256, 0, st>>>(A, factor, nn);
    return cudaGetLastError();
}

}  // namespace shg
