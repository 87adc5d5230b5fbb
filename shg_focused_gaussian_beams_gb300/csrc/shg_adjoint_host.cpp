// Gradient of the output SH power of a plain solve (adjoint z-march with checkpoints).
//
// Forward: the solve is marched once, saving the state every L steps (L = ceil(K/C) for
// C checkpoints, K = NZ-1 steps). Backward: segment by segment from the last, the segment
// is replayed from its checkpoint (keeping the step-start state X_s, the diffraction
// output W_s and the spectrum F_s), then the cotangent is carried back through
// RK4^T(W_s), the adjoint diffraction, and RK4^T(X_s). Parameter gradients come from
// per-step FP64 sums: the coupling constants i*kappa*exp(-+i z dk) carry dk (hence the
// poling period and T), kappa_p,s = pi dQ / (n lambda) and the TPA factor carry n(T), the
// propagators carry k = 2 pi n / lambda. The oven temperature enters through n_p(T) and
// n_s(T) (Sellmeier, Crystal.h:116-132, differentiated analytically); the input fields are
// held fixed.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/shg.h"
#include "shg_adjoint.h"
#include "shg_internal.h"

namespace shg {

#define AD_CUDA(call)                                                                                  \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess) {                                                                       \
            set_error(std::string("adjoint: ") + #call + ": " + cudaGetErrorString(e_));              \
            return e_ == cudaErrorMemoryAllocation ? SHG_ERR_NOMEM : SHG_ERR_CUDA;                     \
        }                                                                                              \
    } while (0)

AdjointWork::~AdjointWork() {
    release();
    if (cap) cudaStreamDestroy(cap);
    if (side) cudaStreamDestroy(side);
    if (ev) cudaEventDestroy(ev);
}

void AdjointWork::release() {
    if (graph) cudaGraphExecDestroy(graph);
    graph = nullptr;
    for (auto &k : graph_key) k = nullptr;
    if (mem) cudaFree(mem);
    mem = nullptr;
    bytes = 0;
}

// Layout: X, cot (one state each: P then S), nck checkpoint states, and L segment states
// for each of X_s, W_s, F_s (two sets of L when checkpointing, so that the replay of one
// segment overlaps the backward sweep of the next); then per-step sums (K x 8 doubles) and
// 8 global doubles ([0..1] propagator sums, [2] sum |S_out|^2, [3] seed scale).
int AdjointWork::ensure(int n_, int K_, int L_, int nck_) {
    if (mem && n == n_ && K == K_ && L == L_ && nck == nck_) return SHG_OK;
    release();
    n = n_;
    K = K_;
    L = L_;
    nck = nck_;
    const size_t nn = (size_t)n * n;
    const size_t st = 2 * nn;
    const size_t sets = nck > 0 ? 2 : 1;
    bytes = sizeof(float2) * (st * (2 + (size_t)nck + 3 * sets * (size_t)L)) + sizeof(double) * (8 * (size_t)K + 8);
    {
        const int rc = device_fits(bytes, "gradient work space");
        if (rc) return rc;
    }
    AD_CUDA(cudaMalloc(&mem, bytes));
    float2 *p = reinterpret_cast<float2 *>(mem);
    X = p;
    p += st;
    cot = p;
    p += st;
    ck = p;
    p += st * nck;
    Xs = p;
    p += st * L * sets;
    Ws = p;
    p += st * L * sets;
    Fs = p;
    p += st * L * sets;
    acc_step = reinterpret_cast<double *>(p);
    acc_glob = acc_step + 8 * (size_t)K;
    return SHG_OK;
}

// dn/dT of the crystal's index in double (the smooth model behind the float index):
// Crystal.h:116-132 (MgO:sPPLT) or the LiNbO3 fit of sellmeier_ln (PPLN).
double crystal_index_dT(int crystal, double L, double T) {
    if (crystal == SHG_CRYSTAL_PPLN) {
        const double a1 = 5.35583, a2 = 0.100473, a3 = 0.20692, a4 = 100.0, a5 = 11.34927, a6 = 1.5334e-2;
        const double b1 = 4.629e-7, b2 = 3.862e-8, b3 = -0.89e-8, b4 = 2.657e-5;
        const double L2 = L * L, f = (T - 24.5) * (T + 570.82), df = 2.0 * T + 546.32;
        const double c3 = a3 + b3 * f, den1 = L2 - c3 * c3, den2 = L2 - a5 * a5;
        const double n2 = a1 + b1 * f + (a2 + b2 * f) / den1 + (a4 + b4 * f) / den2 - a6 * L2;
        const double dn2 = (b1 + b2 / den1 + (a2 + b2 * f) * 2.0 * c3 * b3 / (den1 * den1) + b4 / den2) * df;
        return dn2 / (2 * std::sqrt(n2));
    }
    return sellmeier_dT(L, T);
}

// dn/dT of Crystal.h:116-132 in double (the smooth model behind the float index).
double sellmeier_dT(double L, double T) {
    const double A = 4.502483, B = 0.007294, C = 0.185087, D = -0.02357, E = 0.073423, F = 0.199595, G = 0.001,
                 H = 7.99724;
    const double tk = T + 273.15;
    const double b = 3.483933e-8 * tk * tk, c = 1.607839e-8 * tk * tk;
    const double db = 2 * 3.483933e-8 * tk, dc = 2 * 1.607839e-8 * tk;
    const double L2 = L * L;
    const double den = L2 - (C + c) * (C + c);
    const double n2 = A + (B + b) / den + E / (L2 - F * F) + G / (L2 - H * H) + D * L2;
    const double dn2 = db / den + (B + b) * 2 * (C + c) * dc / (den * den);
    return dn2 / (2 * std::sqrt(n2));
}

// The whole gradient pass on `st`, from the input fields in h.P / h.S to the cotangent of
// the inputs in w.cot and the sums in w.acc_step / w.acc_glob (seed scale read from
// w.acc_glob[3]). Each z-step is one fused row launch and one column launch per direction
// (launch_adj_rows_fwd / launch_adj_rows_bwd around launch_colpass). Segments of L steps;
// with store_all the forward pass keeps every step's X_s, W_s, F_s and the backward pass
// needs no replay.
static int enqueue_pass(const InstDesc &h, const InstDesc *d, AdjointWork &w, int L, int nseg, bool store_all,
                        cudaStream_t st) {
    const int n = h.n, K = h.nsteps;
    const size_t nn = (size_t)n * n, st2 = 2 * nn;
    int rc;
    AD_CUDA(cudaMemsetAsync(w.acc_step, 0, sizeof(double) * (8 * (size_t)K + 3), st));
    // Checkpointed: segment seg's X_s, W_s, F_s go to slot set seg & 1, replayed there from
    // its checkpoint, or, for the last two segments, written by the forward pass itself
    // (the two slot sets hold them; no replay). store_all: slot s of one set of K.
    auto slot = [&](int s) -> size_t {
        return store_all ? (size_t)s * st2 : (size_t)((s / L) & 1) * L * st2 + (size_t)(s % L) * st2;
    };
    auto stored = [&](int seg) -> bool { return store_all || seg >= nseg - 2; };
    // forward from the inputs (X_K into w.X), keeping what the backward pass reads
    for (int s = 0; s <= K; ++s) {
        const bool fin = s > 0, start = s < K;
        float2 *w_out = (fin && stored((s - 1) / L)) ? w.Ws + slot(s - 1) : nullptr;
        float2 *x_out = (start && stored(s / L)) ? w.Xs + slot(s) : nullptr;
        float2 *ck_out = (start && !stored(s / L) && s % L == 0) ? w.ck + (size_t)(s / L) * st2 : nullptr;
        AD_CUDA(launch_adj_rows_fwd(n, d, w.X, s, fin, start, h.P, h.S, w_out, x_out, ck_out, start ? nullptr : w.X,
                                    st));
        if (start)
            AD_CUDA(launch_colpass(n, 0, w.X, stored(s / L) ? w.Fs + slot(s) : nullptr, d, nullptr, st));
    }
    AD_CUDA(launch_abs2_sum(w.X + nn, (int)nn, w.acc_glob + 2, st));
    AD_CUDA(launch_seed_cotangent(w.X + nn, w.cot, w.cot + nn, (int)nn, w.acc_glob + 3, st));
    // backward, segment by segment from the last; the cotangent of X_{s1} enters each
    // segment in natural layout in w.cot. Boundary s: finish step s+1 (RK4^T at X_{s+1}),
    // start step s (RK4^T at W_s).
    auto backward = [&](int s0, int s1, size_t set) -> int {
        float2 *Xs = w.Xs + set, *Ws = w.Ws + set, *Fs = w.Fs + set;
        for (int s = s1 - 1; s >= s0 - 1; --s) {
            const bool fin = s < s1 - 1, start = s >= s0;
            const float2 *Xn = fin ? Xs + (size_t)(s + 1 - s0) * st2 : nullptr;
            const float2 *Wn = start ? Ws + (size_t)(s - s0) * st2 : nullptr;
            double *af = fin ? w.acc_step + 8 * (size_t)(s + 1) : nullptr;
            double *as = start ? w.acc_step + 8 * (size_t)s : nullptr;
            AD_CUDA(launch_adj_rows_bwd(n, d, w.cot, s, fin, start, Xn, Wn, af, as, st));
            if (start) AD_CUDA(launch_colpass(n, 1, w.cot, Fs + (size_t)(s - s0) * st2, d, w.acc_glob, st));
        }
        return SHG_OK;
    };
    if (store_all) return backward(0, K, 0);
    // replay of segment seg from its checkpoint on the side branch, keeping X_s, W_s, F_s for
    // s0 <= s < s1 in slot set seg & 1 (X_{s1} is not needed and lands in w.X)
    auto replay = [&](int seg) -> int {
        const int s0 = seg * L, s1 = std::min(K, s0 + L);
        const size_t set = (size_t)(seg & 1) * L * st2;
        float2 *Xs = w.Xs + set, *Ws = w.Ws + set, *Fs = w.Fs + set;
        const float2 *ckp = w.ck + (size_t)seg * st2;
        for (int s = s0; s <= s1; ++s) {
            const bool fin = s > s0, start = s < s1;
            float2 *w_out = fin ? Ws + (size_t)(s - 1 - s0) * st2 : nullptr;
            float2 *x_out = start ? Xs + (size_t)(s - s0) * st2 : nullptr;
            AD_CUDA(launch_adj_rows_fwd(n, d, w.X, s, fin, start, ckp, ckp + nn, w_out, x_out, nullptr,
                                        start ? nullptr : w.X, w.side));
            if (start) AD_CUDA(launch_colpass(n, 0, w.X, Fs + (size_t)(s - s0) * st2, d, nullptr, w.side));
        }
        return SHG_OK;
    };
    // branch b waits for everything enqueued so far on branch a
    auto join = [&](cudaStream_t a, cudaStream_t b) -> int {
        AD_CUDA(cudaEventRecord(w.ev, a));
        AD_CUDA(cudaStreamWaitEvent(b, w.ev, 0));
        return SHG_OK;
    };
    for (int seg = nseg - 1; seg >= 0; --seg) {
        if (!stored(seg) && (rc = join(w.side, st))) return rc;  // replay(seg) done
        // replay(seg-1) reuses the slot set of backward(seg+1), which st has finished
        if (seg >= 1 && !stored(seg - 1) && ((rc = join(st, w.side)) || (rc = replay(seg - 1)))) return rc;
        const int s0 = seg * L, s1 = std::min(K, s0 + L);
        if ((rc = backward(s0, s1, (size_t)(seg & 1) * L * st2))) return rc;
    }
    return SHG_OK;
}

int adjoint_run(const shg_config &cfg, const InstDesc &h, const InstDesc *d, float temp, int checkpoints,
                AdjointWork &w, cudaStream_t st, float2 *grad_pump, float2 *grad_sh, double *out) {
    const int n = h.n, K = h.nsteps;
    const size_t nn = (size_t)n * n;
    if (checkpoints < 1) checkpoints = 1;
    const bool store_all = checkpoints >= K;
    if (checkpoints > K) checkpoints = K;
    const int L = store_all ? K : (K + checkpoints - 1) / checkpoints;
    const int nseg = store_all ? 1 : (K + L - 1) / L;
    int rc = w.ensure(n, K, L, store_all ? 0 : nseg);
    if (rc) return rc;
    // loss scale: P_SH = 1/2 eps0 c n_s dx dy sum |S_out|^2; the seed is 2 * that scale
    const float lp = cfg.lp, ls = (float)(0.5 * (double)lp);
    const float ns = crystal_index(cfg.crystal, ls, temp), np = crystal_index(cfg.crystal, lp, temp);
    const double kl = field_power(1.0, ns, h.dx, h.dy);
    const double seed = 2.0 * kl;
    AD_CUDA(cudaMemcpyAsync(w.acc_glob + 3, &seed, sizeof(double), cudaMemcpyHostToDevice, st));
    // the pass is captured once per (grid, steps, segments, solve) and replayed
    const void *key[4] = {d, h.P, h.S, h.stepc};
    if (!w.graph || std::memcmp(key, w.graph_key, sizeof(key)) != 0) {
        if (w.graph) cudaGraphExecDestroy(w.graph);
        w.graph = nullptr;
        // the reverse sweep (captured on w.cap) is the pass's critical path: its nodes get the
        // higher block-scheduling priority, the replay branch (w.side) the lower one
        int prio_lo = 0, prio_hi = 0;
        AD_CUDA(cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi));
        if (!w.cap) AD_CUDA(cudaStreamCreateWithPriority(&w.cap, cudaStreamNonBlocking, prio_hi));
        if (!w.side) AD_CUDA(cudaStreamCreateWithPriority(&w.side, cudaStreamNonBlocking, prio_lo));
        if (!w.ev) AD_CUDA(cudaEventCreateWithFlags(&w.ev, cudaEventDisableTiming));
        cudaGraph_t g = nullptr;
        AD_CUDA(cudaStreamBeginCapture(w.cap, cudaStreamCaptureModeThreadLocal));
        rc = enqueue_pass(h, d, w, L, nseg, store_all, w.cap);
        cudaError_t e = cudaStreamEndCapture(w.cap, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        AD_CUDA(e);
        e = cudaGraphInstantiate(&w.graph, g, cudaGraphInstantiateFlagUseNodePriority);
        cudaGraphDestroy(g);
        AD_CUDA(e);
        std::memcpy(w.graph_key, key, sizeof(key));
    }
    AD_CUDA(cudaGraphLaunch(w.graph, st));
    if (grad_pump) AD_CUDA(cudaMemcpyAsync(grad_pump, w.cot, nn * sizeof(float2), cudaMemcpyDeviceToDevice, st));
    if (grad_sh) AD_CUDA(cudaMemcpyAsync(grad_sh, w.cot + nn, nn * sizeof(float2), cudaMemcpyDeviceToDevice, st));
    // parameter gradients on the host
    std::vector<double> acc(8 * (size_t)K + 8);
    std::vector<float4> stepc(K);
    AD_CUDA(cudaMemcpyAsync(acc.data(), w.acc_step, acc.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    AD_CUDA(cudaMemcpyAsync(stepc.data(), h.stepc, K * sizeof(float4), cudaMemcpyDeviceToHost, st));
    AD_CUDA(cudaStreamSynchronize(st));
    const double *g = acc.data() + 8 * (size_t)K;
    const double loss = kl * g[2];
    double dL_ddk = 0, dL_dkp = 0, dL_dks = 0, dL_dtpa = 0;
    float z = 0.0f;
    for (int s = 0; s < K; ++s) {
        const double *a = acc.data() + 8 * (size_t)s;
        const double aPr = stepc[s].x, aPi = stepc[s].y, aSr = stepc[s].z, aSi = stepc[s].w;
        // d alpha_P / d theta = -i alpha_P, d alpha_S / d theta = i alpha_S
        const double dth = (a[0] * aPi + a[1] * (-aPr)) + (a[2] * (-aSi) + a[3] * aSr);
        dL_ddk += (double)z * dth;
        dL_dkp += a[0] * aPr + a[1] * aPi;
        dL_dks += a[2] * aSr + a[3] * aSi;
        dL_dtpa += a[4];
        z += h.dz;
    }
    dL_dkp /= (double)h.kp;
    dL_dks /= (double)h.ks;
    const double kpw = 2.0 * 3.14159265358979323846 * (double)np / (double)lp;
    const double ksw = 2.0 * 3.14159265358979323846 * (double)ns / (double)ls;
    const double dL_dkpw = g[0] * (double)h.dz * (double)h.gp / kpw;
    const double dL_dksw = g[1] * (double)h.dz * (double)h.gs / ksw;
    const double dnp = crystal_index_dT(cfg.crystal, lp, temp), dns = crystal_index_dT(cfg.crystal, ls, temp);
    const double two_pi = 2.0 * 3.14159265358979323846;
    const double ddk_dT = two_pi * (2.0 * dnp / lp - dns / ls);
    const double dT = dL_ddk * ddk_dT + dL_dkp * (-(double)h.kp / np) * dnp + dL_dks * (-(double)h.ks / ns) * dns +
                      dL_dtpa * ((double)h.tpa1 / ns) * dns + dL_dkpw * (two_pi / lp) * dnp +
                      dL_dksw * (two_pi / ls) * dns + loss / ns * dns;
    const double lam = (double)cfg.lambda_qpm;
    out[0] = loss;
    out[1] = dT;
    out[2] = dL_ddk * (-two_pi / (lam * lam));
    out[3] = dL_ddk;
    return SHG_OK;
}

int pump_param_gradients(const shg_config &cfg, const InstDesc &h, float power, float waist, float focal, float temp,
                         const float2 *factor, AdjointWork &w, cudaStream_t st, double *out4) {
    // Efields.h:74-104 constants in double from the float index the reference uses
    const double PI = 3.14159265358979323846;
    const double eps0 = (double)(float)(8.8541878128E-12 * 1E12 / 1E6), c = (double)(float)(299792458 * 1E6 / 1E12);
    const double np = (double)crystal_index(cfg.crystal, cfg.lp, temp);
    const double w_ = waist, w2 = w_ * w_;
    const double zr = PI * np * w2 / (double)cfg.lp;
    const double ap0 = std::sqrt(4.0 * (double)power / (eps0 * c * PI * np * w2));
    double *sums = w.acc_glob + 4;  // [4..7] free in the global sums
    AD_CUDA(launch_pump_param_sums(w.cot, factor, h.n, h.uX, h.uY, h.dx, h.dy, ap0, zr, w_, (double)focal,
                                   (double)power, np, sums, st));
    double r[4];
    AD_CUDA(cudaMemcpyAsync(r, sums, sizeof(r), cudaMemcpyDeviceToHost, st));
    AD_CUDA(cudaStreamSynchronize(st));
    out4[0] = r[0];
    out4[1] = r[1];
    out4[2] = r[2];
    out4[3] = r[3] * crystal_index_dT(cfg.crystal, cfg.lp, temp);
    return SHG_OK;
}

}  // namespace shg
